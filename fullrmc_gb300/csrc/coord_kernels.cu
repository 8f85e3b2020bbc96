// Coordination numbers (Extensions/atomic_coordination.pyx, used by
// AtomicCoordinationNumberConstraint).  Every entry point of that module is a
// sequence of terms
//     coordNumData[def] += count{ j in list : lower[def] <= d(row, j) <= upper[def] }
// where d is the minimum-image distance of two atoms (or an entry of a
// caller's distance row) and the count is a float32 sum of ones
// (atomic_coordination.pyx:31-44), so it is exact below 2^24 and stops at
// 2^24 above.  The additions into coordNumData are float32 and happen in term
// order (atomic_coordination.pyx:184-198, 220-240), which only matters when a
// partial sum is not an integer below 2^24.
//
//   k_coord_count       one CTA per (term, chunk of kCoordChunk list entries):
//                       distances, window test, one integer atomicAdd per CTA;
//   k_coord_accumulate  one warp per definition: the sum of its terms' counts
//                       when every partial sum is an exact integer, else the
//                       float32 additions one by one in term order.
#include <cstdint>

#include "frmc_math.cuh"
#include "frmc_runtime.h"

namespace frmc {

constexpr int kCoordThreads = 256;
constexpr int kCoordPerThread = 4;
constexpr int kCoordChunk = kCoordThreads * kCoordPerThread;
constexpr int kCoordSaturate = 1 << 24;  // 2^24 + 1 rounds back to 2^24 in float32

struct CoordParams {
    const float *coords;         // (n, 3) box coordinates, or null for distance rows
    const float *dists;          // concatenated distance rows
    const long long *dist_off;   // start of row r in dists
    const int *dist_len;         // length of row r
    int n;
    Basis B;
    const int *lists;            // concatenated index lists
    const CoordTerm *terms;
    const int2 *items;           // (term, first list entry of the chunk)
    const float *lower, *upper;  // per definition
    int *counts;                 // per term, zeroed before the launch
};

template <int BM>
__global__ void __launch_bounds__(kCoordThreads) k_coord_count(CoordParams p)
{
    __shared__ int s_warp[kCoordThreads / 32];
    const int2 it = p.items[blockIdx.x];
    const CoordTerm t = p.terms[it.x];
    const float lo = p.lower[t.def], up = p.upper[t.def];
    float ax = 0.f, ay = 0.f, az = 0.f;
    const float *row = nullptr;
    int rowlen;
    if (p.coords) {
        ax = p.coords[3ll * t.row];
        ay = p.coords[3ll * t.row + 1];
        az = p.coords[3ll * t.row + 2];
        rowlen = p.n;
    } else {
        row = p.dists + p.dist_off[t.row];
        rowlen = p.dist_len[t.row];
    }
    int hits = 0;
#pragma unroll
    for (int u = 0; u < kCoordPerThread; ++u) {
        const int e = it.y + u * kCoordThreads + (int)threadIdx.x;
        if (e < t.len) {
            int j = p.lists[t.begin + e];
            if (j < 0)  // numpy indexing of the list (checked on the host)
                j += rowlen;
            float d;
            if (p.coords)
                d = __fsqrt_rn(pair_s<BM>(ax, ay, az, p.coords[3ll * j], p.coords[3ll * j + 1], p.coords[3ll * j + 2],
                                          p.B));
            else
                d = row[j];
            hits += (lo <= d && d <= up) ? 1 : 0;
        }
    }
    hits = __reduce_add_sync(0xffffffffu, hits);
    if ((threadIdx.x & 31u) == 0)
        s_warp[threadIdx.x >> 5] = hits;
    __syncthreads();
    if (threadIdx.x == 0) {
        int total = 0;
#pragma unroll
        for (int w = 0; w < kCoordThreads / 32; ++w) total += s_warp[w];
        if (total)
            atomicAdd(p.counts + it.x, total);
    }
}

__device__ __forceinline__ int coord_saturate(int c)
{
    return c < kCoordSaturate ? c : kCoordSaturate;
}

// def_ids[u]: the u-th definition touched; its terms, in call order, are
// def_terms[def_off[u] .. def_off[u+1]).
__global__ void k_coord_accumulate(const int *counts, const int *def_ids, const int *def_off, const int *def_terms,
                                   int ndefs, float *data)
{
    const int u = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const unsigned lane = threadIdx.x & 31u;
    if (u >= ndefs)
        return;
    const int b = def_off[u], e = def_off[u + 1];
    long long total = 0;
    for (int i = b + (int)lane; i < e; i += 32) total += coord_saturate(counts[def_terms[i]]);
#pragma unroll
    for (int off = 16; off; off >>= 1) total += __shfl_xor_sync(0xffffffffu, total, off);
    if (lane)
        return;
    const int def = def_ids[u];
    const float c0 = data[def];
    // all partial sums c0 + k lie in [c0, c0 + total]: exact when that range
    // holds only integers of magnitude <= 2^24
    if (c0 == rintf(c0) && fabsf(c0) <= (float)kCoordSaturate && (double)c0 + (double)total <= (double)kCoordSaturate) {
        data[def] = (float)((long long)c0 + total);
        return;
    }
    float c = c0;
    for (int i = b; i < e; ++i) c = __fadd_rn(c, (float)coord_saturate(counts[def_terms[i]]));
    data[def] = c;
}

int coordination_run(const CoordLaunch &L, cudaStream_t st)
{
    if (L.nitems > 0) {
        CoordParams p{};
        p.coords = L.coords;
        p.dists = L.dists;
        p.dist_off = L.dist_off;
        p.dist_len = L.dist_len;
        p.n = L.n;
        static const float kId[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        const float *B = L.isPBC && L.basis ? L.basis : kId;
        const int bm = L.coords ? basis_mode(B, L.isPBC) : BM_IBC;
        p.B = make_basis(B);
        p.lists = L.lists;
        p.terms = L.terms;
        p.items = L.items;
        p.lower = L.lower;
        p.upper = L.upper;
        p.counts = L.counts;
        const unsigned g = (unsigned)L.nitems;
        switch (bm) {
        case BM_IBC: k_coord_count<BM_IBC><<<g, kCoordThreads, 0, st>>>(p); break;
        case BM_DIAG: k_coord_count<BM_DIAG><<<g, kCoordThreads, 0, st>>>(p); break;
        case BM_XYTRI: k_coord_count<BM_XYTRI><<<g, kCoordThreads, 0, st>>>(p); break;
        case BM_LOWER: k_coord_count<BM_LOWER><<<g, kCoordThreads, 0, st>>>(p); break;
        default: k_coord_count<BM_GENERAL><<<g, kCoordThreads, 0, st>>>(p); break;
        }
        FRMC_CUDA(cudaGetLastError());
    }
    if (L.ndefs > 0) {
        const int threads = 128;
        const unsigned g = (unsigned)(((long long)L.ndefs * 32 + threads - 1) / threads);
        k_coord_accumulate<<<g, threads, 0, st>>>(L.counts, L.def_ids, L.def_off, L.def_terms, L.ndefs, L.data);
        FRMC_CUDA(cudaGetLastError());
    }
    return FRMC_OK;
}

int coordination_chunk()
{
    return kCoordChunk;
}

}  // namespace frmc
