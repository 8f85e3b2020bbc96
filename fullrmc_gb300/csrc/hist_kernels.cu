// Per-species-pair distance histograms (fullrmc Extensions/pairs_histograms.pyx).
//
// k_full_tiles: the all-pairs (i < j) histogram of full_pairs_histograms_coords
//   (pairs_histograms.pyx:289-335).  Persistent CTAs walk the upper triangle of
//   (row tile, column tile) pairs.  Row atoms live in registers; each column
//   tile (float4 x, y, z, el and int mol) is staged into shared memory by a
//   1-D bulk copy (TMA engine) on an mbarrier, double-buffered so the next
//   tile streams in while the current one is processed.  The inter-molecular
//   counts are privatised per CTA in shared memory and merged once at the end;
//   the rare intra-molecular counts go straight to global atomics.
//
//   Rejection uses exact squared-distance limits (s >= s_lo && s < s_hi is
//   the same predicate as d >= min && d < max for d = sqrtf(s)), so the IEEE
//   sqrt and division run only for accepted pairs.  When few pairs are
//   accepted, accepted pairs are appended to a per-thread queue in shared
//   memory and binned warp-synchronously, so the expensive tail runs with
//   full lanes instead of diverging.
//
// k_rows_vs_all: explicit row atoms against every column atom (the per-step
//   multiple_pairs_histograms_coords call, pairs_histograms.pyx:150-217).
//
// k_dists_hist: histogram of given distance rows (single_pairs_histograms,
//   multiple_/full_pairs_histograms_dists; pairs_histograms.pyx:36-141,225-383).
//
// Counts are uint32 and converted to the reference's float32 values by
// k_counts_to_f32, which reproduces sequential float32 additions of 1.0.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "frmc_math.cuh"
#include "frmc_ptx.cuh"
#include "frmc_runtime.h"

namespace frmc {

// ----------------------------------------------------------------- helpers
__device__ __forceinline__ void bin_count(float s, float minD, float binw, long long rowbase, int elj, int hs,
                                          long long total, bool same_mol, unsigned *intra, unsigned *inter_g,
                                          unsigned *inter_s)
{
    int bin = pair_bin(s, minD, binw);
    long long flat = (rowbase + elj) * (long long)hs + bin;
    if ((unsigned long long)flat < (unsigned long long)total) {
        if (same_mol)
            atomicAdd(intra + flat, 1u);
        else if (inter_s)
            atomicAdd(inter_s + flat, 1u);
        else
            atomicAdd(inter_g + flat, 1u);
    }
}

template <int R, class T>
__device__ __forceinline__ T pick(const T (&a)[R], int r)
{
    T v = a[0];
#pragma unroll
    for (int k = 1; k < R; ++k)
        if (r == k) v = a[k];
    return v;
}

// ------------------------------------------------------------ full (i < j)
struct FullParams {
    const float4 *atoms;
    const int *mol;
    int n;
    Basis B;
    float s_lo, s_hi, minD, binw;
    int ne, hs;
    long long total;
    unsigned *intra;
    unsigned *inter;
    uint32_t *status;
    int T;        // atoms per tile (= blockDim * R)
    int nt;       // number of tiles
    long long item_begin;  // this launch walks items [item_begin, nitems)
    long long nitems;
    int qcap;
    int smem_hist;
    int agg;      // warp-aggregated binning of queued pairs
};

// Item t of the row-major upper triangle (I <= J) of an nt x nt tile grid.
__device__ __forceinline__ void decode_item(long long t, int nt, int &I, int &J)
{
    // off(I) = I*nt - I*(I-1)/2 items precede row I.
    float a = 2.0f * nt + 1.0f;
    float disc = a * a - 8.0f * (float)t;
    int i = (int)floorf((a - sqrtf(fmaxf(disc, 0.0f))) * 0.5f);
    i = max(0, min(i, nt - 1));
    auto off = [nt](long long k) { return k * nt - k * (k - 1) / 2; };
    while (i > 0 && off(i) > t) --i;
    while (i + 1 < nt && off(i + 1) <= t) ++i;
    I = i;
    J = i + (int)(t - off(i));
}

struct FullSmem {
    uint64_t *bar;
    float4 *tile[2];
    int *tmol[2];
    unsigned *hist;
    uint2 *queue;
};

__device__ __forceinline__ FullSmem full_smem_layout(unsigned char *smem, const FullParams &p, int nthr)
{
    FullSmem s;
    size_t off = 0;
    s.bar = reinterpret_cast<uint64_t *>(smem);
    off = 16;
    s.tile[0] = reinterpret_cast<float4 *>(smem + off);
    off += (size_t)p.T * 16;
    s.tile[1] = reinterpret_cast<float4 *>(smem + off);
    off += (size_t)p.T * 16;
    s.tmol[0] = reinterpret_cast<int *>(smem + off);
    off += (size_t)p.T * 4;
    s.tmol[1] = reinterpret_cast<int *>(smem + off);
    off += (size_t)p.T * 4;
    s.hist = reinterpret_cast<unsigned *>(smem + off);
    if (p.smem_hist)
        off += ((size_t)p.total * 4 + 15) & ~(size_t)15;
    s.queue = reinterpret_cast<uint2 *>(smem + off);
    return s;
}

// Issue the column tile of item t into buffer b (thread 0 issues the bulk
// copies; threads 1..3 copy the up-to-3 molecule indexes that do not fill a
// 16-byte chunk with plain loads).
__device__ __forceinline__ void issue_tile(const FullParams &p, FullSmem &s, long long t, int b)
{
    int I, J;
    decode_item(t, p.nt, I, J);
    int col0 = J * p.T;
    int ncol = min(p.T, p.n - col0);
    int nmol4 = ncol & ~3;
    int tid = threadIdx.x;
    if (tid == 0) {
        uint32_t bytes = (uint32_t)ncol * 16u + (uint32_t)nmol4 * 4u;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&s.bar[b], bytes);
        bulk_g2s(s.tile[b], p.atoms + col0, (uint32_t)ncol * 16u, &s.bar[b]);
        if (nmol4)
            bulk_g2s(s.tmol[b], p.mol + col0, (uint32_t)nmol4 * 4u, &s.bar[b]);
    } else if (tid <= 3) {
        int k = nmol4 + tid - 1;
        if (k < ncol)
            s.tmol[b][k] = p.mol[col0 + k];
    }
}

template <int R>
struct RowRegs {
    float x[R], y[R], z[R];
    long long rb[R];  // el_i * ne
    int mol[R];
    int li[R];        // local row index within the tile
};

template <int R>
__device__ __forceinline__ void flush_queue(const FullParams &p, uint2 *&qp, uint2 *qb, int nthr, const float4 *tb,
                                            const int *tm, const RowRegs<R> &rr, unsigned *shist)
{
    while (__any_sync(0xffffffffu, qp != qb)) {
        if (p.agg) {
            // lanes that bin into the same counter add once, with the group's size
            const unsigned lane = threadIdx.x & 31u;
            unsigned long long key = ~0ull - lane;  // unique for lanes without a pair
            unsigned *dst = nullptr;
            long long flat = 0;
            if (qp != qb) {
                qp -= nthr;
                uint2 e = *qp;
                int jl = (int)(e.y >> 2);
                int r = (int)(e.y & 3u);
                int elj = __float_as_int(tb[jl].w);
                bool same = pick<R>(rr.mol, r) == tm[jl];
                int bin = pair_bin(__uint_as_float(e.x), p.minD, p.binw);
                flat = (pick<R>(rr.rb, r) + elj) * (long long)p.hs + bin;
                if ((unsigned long long)flat < (unsigned long long)p.total) {
                    dst = same ? p.intra : (shist ? shist : p.inter);
                    key = ((unsigned long long)flat << 1) | (same ? 1ull : 0ull);
                }
            }
            const unsigned grp = __match_any_sync(0xffffffffu, key);
            if (dst && (unsigned)(__ffs(grp) - 1) == lane)
                atomicAdd(dst + flat, (unsigned)__popc(grp));
        } else if (qp != qb) {
            qp -= nthr;
            uint2 e = *qp;
            int jl = (int)(e.y >> 2);
            int r = (int)(e.y & 3u);
            int elj = __float_as_int(tb[jl].w);
            bool same = pick<R>(rr.mol, r) == tm[jl];
            bin_count(__uint_as_float(e.x), p.minD, p.binw, pick<R>(rr.rb, r), elj, p.hs, p.total, same, p.intra,
                      p.inter, shist);
        }
    }
}

template <int BM, int R, bool QUEUED, bool DIAG>
__device__ __forceinline__ void tile_pairs(const FullParams &p, const float4 *__restrict__ tb, const int *tm, int ncol,
                                           const RowRegs<R> &rr, uint2 *&qp, uint2 *qb, uint2 *qlim, int nthr,
                                           unsigned *shist)
{
    const float s_lo = p.s_lo, s_hi = p.s_hi;
#pragma unroll 2
    for (int jl = 0; jl < ncol; ++jl) {
        float4 c = tb[jl];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float s = pair_s<BM>(rr.x[r], rr.y[r], rr.z[r], c.x, c.y, c.z, p.B);
            bool acc = (s >= s_lo) & (s < s_hi);
            if (DIAG)
                acc &= (jl > rr.li[r]);
            if (QUEUED) {
                *qp = make_uint2(__float_as_uint(s), ((unsigned)jl << 2) | (unsigned)r);
                if (acc)
                    qp += nthr;
            } else if (acc) {
                bin_count(s, p.minD, p.binw, rr.rb[r], __float_as_int(c.w), p.hs, p.total, rr.mol[r] == tm[jl],
                          p.intra, p.inter, shist);
            }
        }
        if (QUEUED && (jl & 1)) {
            if (__any_sync(0xffffffffu, qp >= qlim))
                flush_queue<R>(p, qp, qb, nthr, tb, tm, rr, shist);
        }
    }
}

template <int BM, int R, bool QUEUED>
__global__ void __launch_bounds__(1024) k_full_tiles(FullParams p)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int nthr = blockDim.x;
    FullSmem s = full_smem_layout(smem, p, nthr);
    unsigned *shist = p.smem_hist ? s.hist : nullptr;

    if (shist)
        for (long long k = tid; k < p.total; k += nthr) shist[k] = 0u;
    if (tid == 0) {
        mbar_init(&s.bar[0], 1);
        mbar_init(&s.bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();

    uint2 *qb = s.queue + tid;
    uint2 *qp = qb;
    uint2 *qlim = qb + (size_t)(p.qcap - 2 * R) * nthr;
    uint32_t par0 = 0u, par1 = 0u;
    bool ok = true;

    long long t = p.item_begin + blockIdx.x;
    if (t < p.nitems)
        issue_tile(p, s, t, 0);
    __syncthreads();

    for (int it = 0; t < p.nitems; t += gridDim.x, ++it) {
        const int b = it & 1;
        const long long tn = t + gridDim.x;
        if (tn < p.nitems)
            issue_tile(p, s, tn, b ^ 1);

        int I, J;
        decode_item(t, p.nt, I, J);
        RowRegs<R> rr;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            int li = r * nthr + tid;
            int i = I * p.T + li;
            rr.li[r] = li;
            if (i < p.n) {
                float4 a = p.atoms[i];
                rr.x[r] = a.x; rr.y[r] = a.y; rr.z[r] = a.z;
                rr.rb[r] = (long long)__float_as_int(a.w) * p.ne;
                rr.mol[r] = p.mol[i];
            } else {
                // NaN coordinates make every comparison false: no pair counts.
                rr.x[r] = rr.y[r] = rr.z[r] = __int_as_float(0x7fc00000);
                rr.rb[r] = 0;
                rr.mol[r] = 0;
            }
        }
        const int col0 = J * p.T;
        const int ncol = min(p.T, p.n - col0);

        ok = mbar_wait(&s.bar[b], b ? par1 : par0, p.status);
        if (b) par1 ^= 1u; else par0 ^= 1u;
        // Every thread takes the same path below (warp votes need all lanes).
        ok = __syncthreads_and(ok) != 0;
        if (!ok)
            break;
        if (I == J)
            tile_pairs<BM, R, QUEUED, true>(p, s.tile[b], s.tmol[b], ncol, rr, qp, qb, qlim, nthr, shist);
        else
            tile_pairs<BM, R, QUEUED, false>(p, s.tile[b], s.tmol[b], ncol, rr, qp, qb, qlim, nthr, shist);
        if (QUEUED)
            flush_queue<R>(p, qp, qb, nthr, s.tile[b], s.tmol[b], rr, shist);
        __syncthreads();
    }
    // A CTA that gave up on a barrier drains its copies still in flight
    // (bounded waits) before it exits, so no bulk copy outlives the CTA.
    if (!ok && tid == 0) {
        mbar_wait(&s.bar[0], par0, nullptr);
        mbar_wait(&s.bar[1], par1, nullptr);
    }
    __syncthreads();
    if (shist) {
        for (long long k = tid; k < p.total; k += nthr) {
            unsigned v = shist[k];
            if (v)
                atomicAdd(p.inter + k, v);
        }
    }
}

// ------------------------------------------------------------ rows vs all
struct RowsParams {
    const float *coords;
    const int *el;
    const int *mol;
    int n;
    const int *rows;
    int K;
    int allAtoms;
    Basis B;
    float s_lo, s_hi, minD, binw;
    int ne, hs;
    long long total;
    unsigned *intra;
    unsigned *inter;
};

constexpr int kRowChunk = 64;

template <int BM>
__global__ void __launch_bounds__(256) k_rows_vs_all(RowsParams p)
{
    __shared__ float sx[kRowChunk], sy[kRowChunk], sz[kRowChunk];
    __shared__ int sa[kRowChunk], smol[kRowChunk];
    __shared__ long long srb[kRowChunk];
    const int k0 = blockIdx.y * kRowChunk;
    const int kc = min(kRowChunk, p.K - k0);
    for (int k = threadIdx.x; k < kc; k += blockDim.x) {
        int a = p.rows ? p.rows[k0 + k] : k0 + k;
        sa[k] = a;
        sx[k] = p.coords[3 * (long long)a + 0];
        sy[k] = p.coords[3 * (long long)a + 1];
        sz[k] = p.coords[3 * (long long)a + 2];
        smol[k] = p.mol[a];
        srb[k] = (long long)p.el[a] * p.ne;
    }
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= p.n)
        return;
    // identity rows without allAtoms: columns below every row of the chunk
    if (!p.rows && !p.allAtoms && j < k0)
        return;
    const float cx = p.coords[3 * (long long)j + 0];
    const float cy = p.coords[3 * (long long)j + 1];
    const float cz = p.coords[3 * (long long)j + 2];
    const int elj = p.el[j];
    const int molj = p.mol[j];
    for (int k = 0; k < kc; ++k) {
        const int a = sa[k];
        if (j == a || (!p.allAtoms && j < a))
            continue;
        float s = pair_s<BM>(sx[k], sy[k], sz[k], cx, cy, cz, p.B);
        if ((s >= p.s_lo) & (s < p.s_hi))
            bin_count(s, p.minD, p.binw, srb[k], elj, p.hs, p.total, smol[k] == molj, p.intra, p.inter, nullptr);
    }
}

// --------------------------------------------------- a group move's delta
// The change of fullrmc's before/after-move data for a moved group
// (PairDistributionConstraints.py:1044-1129): after - before of M - F, with M
// the group's rows against all atoms (allAtoms, multiple_pairs_histograms_
// coords on the group) and F the group's own pairs (full_pairs_histograms_
// coords on the group's coordinates), before with every atom at `coords`,
// after with the group's atoms at `newc`.  Every pair takes the reference's
// float32 order (pair_s, pair_bin); counts are signed.
struct GroupDeltaParams {
    const float *coords;  // (n, 3) box coordinates before the move
    const float *newc;    // (K, 3) the group's box coordinates after, in group order
    const int *el;
    const int *mol;
    const int *rows;      // (K) the group's atoms, group order
    const int *sorted;    // (2K) the group's atoms in increasing order, then their group positions
    int n, K, nchunk;
    Basis B;
    float s_lo, s_hi, minD, binw;
    int ne, hs;
    long long total;
    int *intra, *inter;
};

__device__ __forceinline__ void delta_count(const GroupDeltaParams &p, float s, long long rowbase, int elj,
                                            bool same_mol, int v)
{
    if (!((s >= p.s_lo) & (s < p.s_hi)))
        return;
    const long long flat = (rowbase + elj) * (long long)p.hs + pair_bin(s, p.minD, p.binw);
    if ((unsigned long long)flat < (unsigned long long)p.total)
        atomicAdd((same_mol ? p.intra : p.inter) + flat, v);
}

constexpr int kGroupDeltaMax = 1024;  // atoms of a group in one call at most

template <int BM>
__global__ void __launch_bounds__(256) k_group_delta(GroupDeltaParams p)
{
    __shared__ int sidx[kGroupDeltaMax], spos[kGroupDeltaMax];
    __shared__ float ox[kRowChunk], oy[kRowChunk], oz[kRowChunk], nx[kRowChunk], ny[kRowChunk], nz[kRowChunk];
    __shared__ int sa[kRowChunk], smol[kRowChunk];
    __shared__ long long srb[kRowChunk];
    if ((int)blockIdx.y == p.nchunk) {
        // F: the group's own pairs (positions q < r), at [el(q)][el(r)]:
        // + before, - after
        const long long npair = (long long)p.K * (p.K - 1) / 2;
        for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < npair;
             t += (long long)gridDim.x * blockDim.x) {
            int r = 1;
            long long q = t;
            while (q >= r) {
                q -= r;
                ++r;
            }
            const int a = p.rows[q], b = p.rows[r];
            const long long rb = (long long)p.el[a] * p.ne;
            const bool same = p.mol[a] == p.mol[b];
            const float s0 = pair_s<BM>(p.coords[3 * (long long)a], p.coords[3 * (long long)a + 1],
                                        p.coords[3 * (long long)a + 2], p.coords[3 * (long long)b],
                                        p.coords[3 * (long long)b + 1], p.coords[3 * (long long)b + 2], p.B);
            const float s1 = pair_s<BM>(p.newc[3 * q], p.newc[3 * q + 1], p.newc[3 * q + 2], p.newc[3 * (long long)r],
                                        p.newc[3 * (long long)r + 1], p.newc[3 * (long long)r + 2], p.B);
            delta_count(p, s0, rb, p.el[b], same, 1);
            delta_count(p, s1, rb, p.el[b], same, -1);
        }
        return;
    }
    // M: the group's rows of this chunk against every column j != row atom,
    // - before, + after (column j after the move: its new position when it is
    // in the group)
    for (int k = threadIdx.x; k < p.K; k += blockDim.x) {
        sidx[k] = p.sorted[k];
        spos[k] = p.sorted[p.K + k];
    }
    const int k0 = blockIdx.y * kRowChunk;
    const int kc = min(kRowChunk, p.K - k0);
    for (int k = threadIdx.x; k < kc; k += blockDim.x) {
        const int a = p.rows[k0 + k];
        sa[k] = a;
        ox[k] = p.coords[3 * (long long)a];
        oy[k] = p.coords[3 * (long long)a + 1];
        oz[k] = p.coords[3 * (long long)a + 2];
        nx[k] = p.newc[3 * (long long)(k0 + k)];
        ny[k] = p.newc[3 * (long long)(k0 + k) + 1];
        nz[k] = p.newc[3 * (long long)(k0 + k) + 2];
        smol[k] = p.mol[a];
        srb[k] = (long long)p.el[a] * p.ne;
    }
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= p.n)
        return;
    const float cx = p.coords[3 * (long long)j], cy = p.coords[3 * (long long)j + 1],
                cz = p.coords[3 * (long long)j + 2];
    float ax = cx, ay = cy, az = cz;
    {
        int lo = 0, hi = p.K;  // first sorted entry >= j
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (sidx[mid] < j)
                lo = mid + 1;
            else
                hi = mid;
        }
        if (lo < p.K && sidx[lo] == j) {
            const int m = spos[lo];
            ax = p.newc[3 * (long long)m];
            ay = p.newc[3 * (long long)m + 1];
            az = p.newc[3 * (long long)m + 2];
        }
    }
    const int elj = p.el[j], molj = p.mol[j];
    for (int k = 0; k < kc; ++k) {
        if (j == sa[k])
            continue;
        const bool same = smol[k] == molj;
        delta_count(p, pair_s<BM>(ox[k], oy[k], oz[k], cx, cy, cz, p.B), srb[k], elj, same, -1);
        delta_count(p, pair_s<BM>(nx[k], ny[k], nz[k], ax, ay, az, p.B), srb[k], elj, same, 1);
    }
}

int launch_group_delta(const float *coords, const float *newc, const int *el, const int *mol, int n, const int *rows,
                       const int *sorted, int K, int bm, const Basis &B, float minD, float maxD, float binw, int ne,
                       int hs, int *intra, int *inter, cudaStream_t st)
{
    if (K <= 0 || n <= 0)
        return FRMC_OK;
    if (K > kGroupDeltaMax)
        return set_error(FRMC_E_ARG, "a group move of %d atoms (at most %d)", K, kGroupDeltaMax);
    GroupDeltaParams p;
    p.coords = coords;
    p.newc = newc;
    p.el = el;
    p.mol = mol;
    p.rows = rows;
    p.sorted = sorted;
    p.n = n;
    p.K = K;
    p.nchunk = (K + kRowChunk - 1) / kRowChunk;
    p.B = B;
    sq_limits(minD, maxD, &p.s_lo, &p.s_hi);
    p.minD = minD;
    p.binw = binw;
    p.ne = ne;
    p.hs = hs;
    p.total = (long long)ne * ne * hs;
    p.intra = intra;
    p.inter = inter;
    // blocks (column tile, row chunk) for M, and one more row of blocks for F
    const long long npair = (long long)K * (K - 1) / 2;
    const long long gx = std::max<long long>((n + 255) / 256, std::min<long long>((npair + 255) / 256, 4096));
    dim3 grid((unsigned)gx, (unsigned)(p.nchunk + 1));
    switch (bm) {
    case BM_IBC: k_group_delta<BM_IBC><<<grid, 256, 0, st>>>(p); break;
    case BM_DIAG: k_group_delta<BM_DIAG><<<grid, 256, 0, st>>>(p); break;
    case BM_XYTRI: k_group_delta<BM_XYTRI><<<grid, 256, 0, st>>>(p); break;
    case BM_LOWER: k_group_delta<BM_LOWER><<<grid, 256, 0, st>>>(p); break;
    default: k_group_delta<BM_GENERAL><<<grid, 256, 0, st>>>(p); break;
    }
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

// ------------------------------------------------------------ given distances
__global__ void __launch_bounds__(256) k_dists_hist(const float *__restrict__ dists, int n, int K,
                                                    const int *__restrict__ rows, const int *__restrict__ el,
                                                    const int *__restrict__ mol, int allAtoms, float minD, float maxD,
                                                    float binw, int ne, int hs, long long total, unsigned *intra,
                                                    unsigned *inter)
{
    const int k = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    const int a = rows[k];
    if (j == a || (!allAtoms && j < a))
        return;
    const float d = dists[(long long)j * K + k];
    if (d < minD)
        return;
    if (d >= maxD)
        return;
    const float q = __fdiv_rn(__fsub_rn(d, minD), binw);
    if (!(q < 2147483648.0f))
        return;
    const long long flat = ((long long)el[a] * ne + el[j]) * hs + __float2int_rz(q);
    if ((unsigned long long)flat < (unsigned long long)total) {
        if (mol[j] == mol[a])
            atomicAdd(intra + flat, 1u);
        else
            atomicAdd(inter + flat, 1u);
    }
}

// --------------------------------------------------------- counts -> float32
__global__ void k_counts_to_f32(const unsigned *__restrict__ counts, const float *__restrict__ h0,
                                float *__restrict__ out, long long total)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        unsigned c = counts[k];
        float h = h0 ? h0[k] : 0.0f;
        if (c) {
            if (h == truncf(h) && fabsf(h) <= 16777216.0f) {
                long long v = (long long)h + (long long)c;
                h = v >= 16777216LL ? 16777216.0f : (float)v;
            } else {
                for (unsigned t = 0; t < c; ++t) {
                    float nh = __fadd_rn(h, 1.0f);
                    if (nh == h)
                        break;
                    h = nh;
                }
            }
        }
        out[k] = h;
    }
}

__global__ void k_pack_atoms(const float *__restrict__ coords, const int *__restrict__ el, int n,
                             float4 *__restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = make_float4(coords[3 * (long long)i], coords[3 * (long long)i + 1], coords[3 * (long long)i + 2],
                             __int_as_float(el[i]));
}

__global__ void k_unpack_atoms(const float4 *__restrict__ atoms, int n, float *__restrict__ coords,
                               int *__restrict__ el)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float4 a = atoms[i];
        coords[3 * (long long)i] = a.x;
        coords[3 * (long long)i + 1] = a.y;
        coords[3 * (long long)i + 2] = a.z;
        el[i] = __float_as_int(a.w);
    }
}

// ================================================================ launchers
template <int BM, int R, bool Q>
static int launch_full_typed(const FullParams &p, int threads, int grid, size_t smem, cudaStream_t st)
{
    auto kern = k_full_tiles<BM, R, Q>;
    FRMC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, threads, smem, st>>>(p);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

template <int BM>
static int launch_full_bm(const FullParams &p, int R, bool Q, int threads, int grid, size_t smem, cudaStream_t st)
{
    if (R == 1)
        return Q ? launch_full_typed<BM, 1, true>(p, threads, grid, smem, st)
                 : launch_full_typed<BM, 1, false>(p, threads, grid, smem, st);
    return Q ? launch_full_typed<BM, 2, true>(p, threads, grid, smem, st)
             : launch_full_typed<BM, 2, false>(p, threads, grid, smem, st);
}

long long full_hist_items(int n, const FullTune *tune)
{
    FullTune tn = tune ? *tune : FullTune();
    const int R = tn.rows == 1 ? 1 : 2;
    const long long T = (long long)tn.threads * R;
    const long long nt = (n + T - 1) / T;
    return nt * (nt + 1) / 2;
}

int launch_full_hist(const float4 *atoms, const int *mol, int n, int bm, const Basis &B, float minD, float maxD,
                     float binw, int ne, int hs, unsigned *intra, unsigned *inter, uint32_t *status,
                     double accept_fraction, const FullTune *tune, cudaStream_t st, long long item_begin,
                     long long item_end)
{
    if (n < 2)
        return FRMC_OK;
    Context *ctx;
    int rc = get_context(&ctx);
    if (rc)
        return rc;
    return launch_full_hist_on(ctx->sms, ctx->max_smem_optin, atoms, mol, n, bm, B, minD, maxD, binw, ne, hs, intra,
                               inter, status, accept_fraction, tune, st, item_begin, item_end);
}

int launch_full_hist_on(int sms, int max_smem_optin, const float4 *atoms, const int *mol, int n, int bm,
                        const Basis &B, float minD, float maxD, float binw, int ne, int hs, unsigned *intra,
                        unsigned *inter, uint32_t *status, double accept_fraction, const FullTune *tune,
                        cudaStream_t st, long long item_begin, long long item_end)
{
    if (n < 2)
        return FRMC_OK;
    FullTune tn = tune ? *tune : FullTune();
    const int R = tn.rows == 1 ? 1 : 2;
    const int threads = tn.threads;
    if (threads % 32 || threads < 64 || threads > 1024)
        return set_error(FRMC_E_ARG, "full histogram: threads must be a multiple of 32 in [64, 1024]");
    bool queued = tn.queued < 0 ? accept_fraction < 0.2 : tn.queued != 0;
    FullParams p;
    p.atoms = atoms;
    p.mol = mol;
    p.n = n;
    p.B = B;
    sq_limits(minD, maxD, &p.s_lo, &p.s_hi);
    p.minD = minD;
    p.binw = binw;
    p.ne = ne;
    p.hs = hs;
    p.total = (long long)ne * ne * hs;
    p.intra = intra;
    p.inter = inter;
    p.status = status;
    p.T = threads * R;
    p.nt = (n + p.T - 1) / p.T;
    p.nitems = (long long)p.nt * (p.nt + 1) / 2;
    if (item_end >= 0 && item_end < p.nitems)
        p.nitems = item_end;
    p.item_begin = item_begin < 0 ? 0 : item_begin;
    if (p.item_begin >= p.nitems)
        return FRMC_OK;
    p.qcap = tn.qcap < 2 * R + 2 ? 2 * R + 2 : tn.qcap;
    p.agg = tn.aggregate ? 1 : 0;
    const size_t base = 16 + (size_t)p.T * 40;
    const size_t hist_bytes = ((size_t)p.total * 4 + 15) & ~(size_t)15;
    const size_t queue_bytes = queued ? (size_t)p.qcap * threads * 8 : 0;
    p.smem_hist = (base + hist_bytes + queue_bytes) <= (size_t)max_smem_optin ? 1 : 0;
    size_t smem = base + (p.smem_hist ? hist_bytes : 0) + queue_bytes;
    if (smem > (size_t)max_smem_optin)
        return set_error(FRMC_E_ARG, "full histogram: tile configuration needs %zu bytes of shared memory", smem);
    long long grid = (long long)sms * (tn.ctas_per_sm > 0 ? tn.ctas_per_sm : 1);
    if (grid > p.nitems - p.item_begin)
        grid = p.nitems - p.item_begin;
    switch (bm) {
    case BM_IBC: return launch_full_bm<BM_IBC>(p, R, queued, threads, (int)grid, smem, st);
    case BM_DIAG: return launch_full_bm<BM_DIAG>(p, R, queued, threads, (int)grid, smem, st);
    case BM_XYTRI: return launch_full_bm<BM_XYTRI>(p, R, queued, threads, (int)grid, smem, st);
    case BM_LOWER: return launch_full_bm<BM_LOWER>(p, R, queued, threads, (int)grid, smem, st);
    default: return launch_full_bm<BM_GENERAL>(p, R, queued, threads, (int)grid, smem, st);
    }
}

int launch_rows_hist(const float *coords, const int *el, const int *mol, int n, const int *rows, int K,
                     int allAtoms, int bm, const Basis &B, float minD, float maxD, float binw, int ne, int hs,
                     unsigned *intra, unsigned *inter, cudaStream_t st)
{
    if (K <= 0 || n <= 0)
        return FRMC_OK;
    RowsParams p;
    p.coords = coords;
    p.el = el;
    p.mol = mol;
    p.n = n;
    p.rows = rows;
    p.K = K;
    p.allAtoms = allAtoms;
    p.B = B;
    sq_limits(minD, maxD, &p.s_lo, &p.s_hi);
    p.minD = minD;
    p.binw = binw;
    p.ne = ne;
    p.hs = hs;
    p.total = (long long)ne * ne * hs;
    p.intra = intra;
    p.inter = inter;
    dim3 grid((n + 255) / 256, (K + kRowChunk - 1) / kRowChunk);
    if (grid.y > 65535)
        return set_error(FRMC_E_ARG, "too many rows (%d)", K);
    switch (bm) {
    case BM_IBC: k_rows_vs_all<BM_IBC><<<grid, 256, 0, st>>>(p); break;
    case BM_DIAG: k_rows_vs_all<BM_DIAG><<<grid, 256, 0, st>>>(p); break;
    case BM_XYTRI: k_rows_vs_all<BM_XYTRI><<<grid, 256, 0, st>>>(p); break;
    case BM_LOWER: k_rows_vs_all<BM_LOWER><<<grid, 256, 0, st>>>(p); break;
    default: k_rows_vs_all<BM_GENERAL><<<grid, 256, 0, st>>>(p); break;
    }
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

int launch_dists_hist(const float *dists, int n, int K, const int *rows, const int *el, const int *mol,
                      int allAtoms, float minD, float maxD, float binw, int ne, int hs, unsigned *intra,
                      unsigned *inter, cudaStream_t st)
{
    if (K <= 0 || n <= 0)
        return FRMC_OK;
    if (K > 65535)
        return set_error(FRMC_E_ARG, "too many distance columns (%d)", K);
    dim3 grid((n + 255) / 256, K);
    k_dists_hist<<<grid, 256, 0, st>>>(dists, n, K, rows, el, mol, allAtoms, minD, maxD, binw, ne, hs,
                                       (long long)ne * ne * hs, intra, inter);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

// Both histograms of fresh counts (no starting values: a count c becomes
// min(c, 2^24) as float32, as sequential float32 additions of 1.0 from zero
// give) into two separate outputs, and the counts reset to zero for the next
// call.
__global__ void k_counts_pair_to_f32_zero(unsigned *__restrict__ counts, long long total, float *__restrict__ out0,
                                          float *__restrict__ out1)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < 2 * total;
         k += (long long)gridDim.x * blockDim.x) {
        const unsigned c = counts[k];
        const float h = c >= 16777216u ? 16777216.0f : (float)c;
        if (k < total)
            out0[k] = h;
        else
            out1[k - total] = h;
        if (c)
            counts[k] = 0u;
    }
}

int launch_counts_pair_to_f32_zero(unsigned *counts, int64_t total, float *out0, float *out1, cudaStream_t st)
{
    if (total <= 0)
        return FRMC_OK;
    long long blocks = (2 * total + 255) / 256;
    if (blocks > 4096)
        blocks = 4096;
    k_counts_pair_to_f32_zero<<<(int)blocks, 256, 0, st>>>(counts, total, out0, out1);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

int launch_counts_to_f32(const unsigned *counts, const float *h0, float *out, int64_t total, cudaStream_t st)
{
    if (total <= 0)
        return FRMC_OK;
    long long blocks = (total + 255) / 256;
    if (blocks > 4096)
        blocks = 4096;
    k_counts_to_f32<<<(int)blocks, 256, 0, st>>>(counts, h0, out, total);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

int launch_unpack_atoms(const float4 *atoms, int n, float *coords, int *el, cudaStream_t st)
{
    if (n <= 0)
        return FRMC_OK;
    k_unpack_atoms<<<(n + 255) / 256, 256, 0, st>>>(atoms, n, coords, el);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

int launch_pack_atoms(const float *coords, const int *el, int n, float4 *out, cudaStream_t st)
{
    if (n <= 0)
        return FRMC_OK;
    k_pack_atoms<<<(n + 255) / 256, 256, 0, st>>>(coords, el, n, out);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

}  // namespace frmc
