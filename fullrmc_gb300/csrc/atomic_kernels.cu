// Atomic distance constraints (Extensions/atomic_distances.pyx): for atom
// rows against every other atom, the pairs whose distance falls inside (or
// outside) per-element-pair limits are counted, and their distance -- or its
// difference to the nearest / upper / lower limit -- is summed, into
// [ne][ne] intra- and inter-molecular accumulators.
//
// The counts are integers and order-free, but the sums are float32 additions
// in the reference's loop order (rows in the order given, then columns in
// increasing index), and float32 addition is not associative.  So the pairs
// are evaluated in parallel and every contributing pair is listed in that
// order, then one warp adds the listed values in list order:
//   k_atomic_pairs<true>   one CTA per (row, chunk of kAtomicCols columns):
//                          the number of contributing pairs of its block;
//   k_scan_*               exclusive scan of those numbers (block offsets);
//   k_atomic_pairs<false>  the same blocks list their contributors, in column
//                          order, at their offsets;
//   k_atomic_sum           adds the list in order into the accumulators.
// Contributing pairs are few for the limits these constraints use (contacts
// closer than a few Angstrom), so the ordered walk is short.
#include <cstdint>

#include "frmc_math.cuh"
#include "frmc_runtime.h"

namespace frmc {

constexpr int kAtomicThreads = 256;
constexpr int kAtomicPerThread = 4;
constexpr int kAtomicCols = kAtomicThreads * kAtomicPerThread;

enum AtomicFlags {
    AF_INTER = 1,
    AF_INTRA = 2,
    AF_WITHIN = 4,
    AF_RED_UPPER = 8,
    AF_RED_LOWER = 16,
    AF_RED = 32,
};

struct AtomicParams {
    const float *coords;  // (n, 3) box coordinates, or null when dists is given
    const float *dists;   // (n, K) distances, column k for row k (or null)
    const int *rows;      // (K,) atom index of each row
    int K, n, nchunks, allAtoms, flags, ne;
    Basis B;
    int bm;
    const int *mol, *el;
    const float *lower, *upper;  // (ne, ne) limits, indexed [el(column)][el(row)]
    long long *block_count;      // per (row, chunk): contributors, then their list offset
    int *list_bucket;            // contributors: (0 intra / 1 inter) * ne*ne + el(row) * ne + el(column)
    float *list_value;           // their values
};

template <int BM>
__device__ __forceinline__ bool atomic_pair(const AtomicParams &p, int ela, int mola, float ax, float ay, float az,
                                            int k, int j, float &value, int &bucket)
{
    const int molj = p.mol[j];
    const bool same = molj == mola;
    if (!(p.flags & AF_INTRA) && same)
        return false;
    if (!(p.flags & AF_INTER) && !same)
        return false;
    float d;
    if (p.dists) {
        d = p.dists[(long long)j * p.K + k];
    } else {
        const float *c = p.coords + 3ll * j;
        d = __fsqrt_rn(pair_s<BM>(ax, ay, az, c[0], c[1], c[2], p.B));
    }
    const int elj = p.el[j];
    const float lower = p.lower[elj * p.ne + ela];
    const float upper = p.upper[elj * p.ne + ela];
    if (p.flags & AF_WITHIN) {
        if (d < lower || d >= upper)
            return false;
    } else if (d >= lower && d < upper) {
        return false;
    }
    if (p.flags & AF_RED_UPPER) {
        d = fabsf(__fsub_rn(upper, d));
    } else if (p.flags & AF_RED_LOWER) {
        d = fabsf(__fsub_rn(lower, d));
    } else if (p.flags & AF_RED) {
        d = d > __fdiv_rn(__fadd_rn(lower, upper), 2.0f) ? fabsf(__fsub_rn(upper, d)) : fabsf(__fsub_rn(lower, d));
    }
    value = d;
    bucket = (same ? 0 : p.ne * p.ne) + ela * p.ne + elj;
    return true;
}

template <int BM, bool COUNT>
__global__ void __launch_bounds__(kAtomicThreads) k_atomic_pairs(AtomicParams p)
{
    __shared__ int s_warp[kAtomicThreads / 32];
    const long long blk = blockIdx.x;
    const int k = (int)(blk / p.nchunks);
    const int chunk = (int)(blk % p.nchunks);
    const int a = p.rows[k];
    const int start = p.allAtoms ? 0 : a;
    const int j0 = chunk * kAtomicCols;
    const int ela = p.el[a], mola = p.mol[a];
    float ax = 0.f, ay = 0.f, az = 0.f;
    if (!p.dists) {
        ax = p.coords[3ll * a];
        ay = p.coords[3ll * a + 1];
        az = p.coords[3ll * a + 2];
    }
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    // each thread takes kAtomicPerThread consecutive columns, so the block's
    // column order is (thread, column) order
    bool hit[kAtomicPerThread];
    float val[kAtomicPerThread];
    int bkt[kAtomicPerThread];
    int mine = 0;
#pragma unroll
    for (int u = 0; u < kAtomicPerThread; ++u) {
        const int j = j0 + threadIdx.x * kAtomicPerThread + u;
        hit[u] = false;
        if (j < p.n && j >= start && j != a)
            hit[u] = atomic_pair<BM>(p, ela, mola, ax, ay, az, k, j, val[u], bkt[u]);
        mine += hit[u];
    }
    int incl = mine;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, off);
        if ((int)lane >= off)
            incl += v;
    }
    if (lane == 31)
        s_warp[warp] = incl;
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < kAtomicThreads / 32; ++w) {
        const int c = s_warp[w];
        if (w < (int)warp)
            before += c;
        total += c;
    }
    if (COUNT) {
        if (threadIdx.x == 0)
            p.block_count[blk] = total;
        return;
    }
    long long pos = p.block_count[blk] + before + incl - mine;
#pragma unroll
    for (int u = 0; u < kAtomicPerThread; ++u)
        if (hit[u]) {
            p.list_bucket[pos] = bkt[u];
            p.list_value[pos] = val[u];
            ++pos;
        }
}

// Exclusive scan of v[0..n) in place (int64), three launches: each CTA of
// 1024 scans its segment and stores the segment total; one CTA scans the
// totals; the totals' prefix is added back.
__global__ void __launch_bounds__(1024) k_scan_segments(long long *v, long long n, long long *totals)
{
    __shared__ long long s[1024];
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    const long long x = i < n ? v[i] : 0;
    s[threadIdx.x] = x;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const long long t = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n)
        v[i] = s[threadIdx.x] - x;
    if (threadIdx.x == 1023)
        totals[blockIdx.x] = s[1023];
}

__global__ void __launch_bounds__(1024) k_scan_totals(long long *totals, long long m, long long *grand)
{
    __shared__ long long s[1024];
    __shared__ long long carry;
    if (threadIdx.x == 0)
        carry = 0;
    __syncthreads();
    for (long long c0 = 0; c0 < m; c0 += 1024) {
        const long long i = c0 + threadIdx.x;
        const long long x = i < m ? totals[i] : 0;
        s[threadIdx.x] = x;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const long long t = threadIdx.x >= (unsigned)off ? s[threadIdx.x - off] : 0;
            __syncthreads();
            s[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < m)
            totals[i] = carry + s[threadIdx.x] - x;
        __syncthreads();
        if (threadIdx.x == 0)
            carry += s[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        *grand = carry;
}

__global__ void k_scan_add(long long *v, long long n, const long long *totals)
{
    const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
    if (i < n)
        v[i] += totals[blockIdx.x];
}

// One warp adds the list in order: 32 entries are loaded at a time and lane 0
// adds them one after the other.  dsum and nsum are (2, ne, ne) and start
// from the caller's values.
__global__ void k_atomic_sum(const int *list_bucket, const float *list_value, long long len, float *dsum, int *nsum,
                             int nb)
{
    __shared__ float sd[2 * 16 * 16];
    __shared__ int sn[2 * 16 * 16];
    const unsigned lane = threadIdx.x & 31u;
    for (int b = lane; b < nb; b += 32) {
        sd[b] = dsum[b];
        sn[b] = nsum[b];
    }
    __syncwarp();
    for (long long i0 = 0; i0 < len; i0 += 32) {
        const long long i = i0 + lane;
        const int bk = i < len ? list_bucket[i] : 0;
        const float v = i < len ? list_value[i] : 0.f;
        const int m = (int)min(32ll, len - i0);
        for (int t = 0; t < m; ++t) {
            const int b = __shfl_sync(0xffffffffu, bk, t);
            const float x = __shfl_sync(0xffffffffu, v, t);
            if (lane == 0) {
                sd[b] = __fadd_rn(sd[b], x);
                sn[b] += 1;
            }
        }
    }
    __syncwarp();
    for (int b = lane; b < nb; b += 32) {
        dsum[b] = sd[b];
        nsum[b] = sn[b];
    }
}

// pair_elements_stats (atomic_distances.pyx:632-672): for i < j, count
// [el(i)][el(j)] intra (same molecule) or inter.  One CTA per row i; lanes
// with the same counter are merged with __match_any_sync before the shared
// atomic, and each CTA adds its counts to the result once.
__global__ void __launch_bounds__(256) k_pair_stats(const int *el, const int *mol, int n, int ne, int *nintra,
                                                   int *ninter)
{
    extern __shared__ int cnt[];  // [2][ne][ne]
    const int total = 2 * ne * ne;
    for (int k = threadIdx.x; k < total; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    const int i = blockIdx.x;
    const int ei = el[i], mi = mol[i];
    const unsigned lane = threadIdx.x & 31u;
    for (int jb = i + 1; jb < n; jb += blockDim.x) {
        const int j = jb + threadIdx.x;
        const int off = j < n ? (mol[j] == mi ? 0 : ne * ne) + ei * ne + el[j] : -1;
        const unsigned same = __match_any_sync(0xffffffffu, off);
        if (off >= 0 && lane == (unsigned)(__ffs(same) - 1))
            atomicAdd(cnt + off, __popc(same));
    }
    __syncthreads();
    for (int k = threadIdx.x; k < total; k += blockDim.x) {
        const int v = cnt[k];
        if (v)
            atomicAdd((k < ne * ne ? nintra + k : ninter + (k - ne * ne)), v);
    }
}

// The whole pipeline for one call: lists the contributors (device buffers
// grown as needed) and adds them in order into dsum / nsum (device, (2, ne,
// ne), holding the starting values).
static int atomic_distances_device(AtomicParams p, DevBuf &counts, DevBuf &totals, DevBuf &list_b, DevBuf &list_v,
                                   float *dsum, int *nsum, cudaStream_t st)
{
    p.nchunks = (p.n + kAtomicCols - 1) / kAtomicCols;
    const long long nblocks = (long long)p.K * p.nchunks;
    if (nblocks <= 0)
        return FRMC_OK;
    if (nblocks > 0x7fffffffll)
        return set_error(FRMC_E_ARG, "atomic distances: too many rows x columns");
    if (p.ne > 16)
        return set_error(FRMC_E_ARG, "atomic distances: at most 16 elements");
    const long long nseg = (nblocks + 1023) / 1024;
    FRMC_TRY(counts.ensure(8 * (size_t)nblocks));
    FRMC_TRY(totals.ensure(8 * (size_t)(nseg + 1)));
    p.block_count = counts.as<long long>();
    const unsigned g = (unsigned)nblocks;
#define FRMC_ATOMIC_LAUNCH(C)                                                                                        \
    switch (p.bm) {                                                                                              \
    case BM_IBC: k_atomic_pairs<BM_IBC, C><<<g, kAtomicThreads, 0, st>>>(p); break;                            \
    case BM_DIAG: k_atomic_pairs<BM_DIAG, C><<<g, kAtomicThreads, 0, st>>>(p); break;                          \
    case BM_XYTRI: k_atomic_pairs<BM_XYTRI, C><<<g, kAtomicThreads, 0, st>>>(p); break;                        \
    case BM_LOWER: k_atomic_pairs<BM_LOWER, C><<<g, kAtomicThreads, 0, st>>>(p); break;                        \
    default: k_atomic_pairs<BM_GENERAL, C><<<g, kAtomicThreads, 0, st>>>(p); break;                            \
    }
    FRMC_ATOMIC_LAUNCH(true);
    FRMC_CUDA(cudaGetLastError());
    long long *tot = totals.as<long long>();
    k_scan_segments<<<(unsigned)nseg, 1024, 0, st>>>(p.block_count, nblocks, tot);
    k_scan_totals<<<1, 1024, 0, st>>>(tot, nseg, tot + nseg);
    k_scan_add<<<(unsigned)nseg, 1024, 0, st>>>(p.block_count, nblocks, tot);
    FRMC_CUDA(cudaGetLastError());
    long long len = 0;
    FRMC_CUDA(cudaMemcpyAsync(&len, tot + nseg, 8, cudaMemcpyDeviceToHost, st));
    FRMC_CUDA(cudaStreamSynchronize(st));
    if (len > 0) {
        FRMC_TRY(list_b.ensure(4 * (size_t)len));
        FRMC_TRY(list_v.ensure(4 * (size_t)len));
        p.list_bucket = list_b.as<int>();
        p.list_value = list_v.as<float>();
        FRMC_ATOMIC_LAUNCH(false);
        FRMC_CUDA(cudaGetLastError());
        k_atomic_sum<<<1, 32, 0, st>>>(p.list_bucket, p.list_value, len, dsum, nsum, 2 * p.ne * p.ne);
        FRMC_CUDA(cudaGetLastError());
    }
#undef FRMC_ATOMIC_LAUNCH
    return FRMC_OK;
}

int atomic_distances_run(Context *c, const float *coords, const float *dists, const int *rows, int K, int n,
                         int allAtoms, int flags, int ne, const float *basis_host, int isPBC, const int *mol,
                         const int *el, const float *lower, const float *upper, float *dsum, int *nsum,
                         cudaStream_t st)
{
    static const float kId[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    AtomicParams p{};
    p.coords = coords;
    p.dists = dists;
    p.rows = rows;
    p.K = K;
    p.n = n;
    p.allAtoms = allAtoms;
    p.flags = flags;
    p.ne = ne;
    const float *B = isPBC && basis_host ? basis_host : kId;
    p.bm = basis_mode(B, isPBC);
    p.B = make_basis(B);
    p.mol = mol;
    p.el = el;
    p.lower = lower;
    p.upper = upper;
    return atomic_distances_device(p, c->buf[BUF_ATOMIC_COUNTS], c->buf[BUF_ATOMIC_TOTALS], c->buf[BUF_ATOMIC_LIST_B],
                                   c->buf[BUF_ATOMIC_LIST_V], dsum, nsum, st);
}

int launch_pair_stats(const int *el, const int *mol, int n, int ne, int *nintra, int *ninter, cudaStream_t st)
{
    if (n < 2)
        return FRMC_OK;
    k_pair_stats<<<n - 1, 256, 8 * ne * ne, st>>>(el, mol, n, ne, nintra, ninter);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

}  // namespace frmc
