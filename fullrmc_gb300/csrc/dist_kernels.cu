// Distances, differences and coordinate transforms
// (fullrmc Extensions/pairs_distances.pyx and
//  Extensions/boundary_conditions_collection.pyx:88-110).
//
// One thread per (atom i, point k).  Distances use the same squared-distance
// arithmetic as the histogram kernels followed by an IEEE sqrt; differences
// keep every basis term so that even signed zeros match the reference.
#include "frmc_math.cuh"
#include "frmc_runtime.h"

namespace frmc {

struct PointSrc {
    const float *pts;  // explicit points: component c of point k at pts[c*ps + k]
    long long ps;
    const int *idx;    // or atom indexes into coords
};

__device__ __forceinline__ void point_of(const PointSrc &src, const float *coords, int k, float &px, float &py,
                                         float &pz, int &atom)
{
    if (src.idx) {
        atom = src.idx[k];
        px = coords[3 * (long long)atom];
        py = coords[3 * (long long)atom + 1];
        pz = coords[3 * (long long)atom + 2];
    } else {
        atom = -1;
        px = src.pts[k];
        py = src.pts[src.ps + k];
        pz = src.pts[2 * src.ps + k];
    }
}

template <int BM>
__global__ void __launch_bounds__(256) k_distances(const float *__restrict__ coords, int n, PointSrc src, int K,
                                                   int fromIndex, Basis B, float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (i >= n)
        return;
    float px, py, pz;
    int atom;
    point_of(src, coords, k, px, py, pz, atom);
    if (fromIndex && i < atom)
        return;
    float s = pair_s<BM>(px, py, pz, coords[3 * (long long)i], coords[3 * (long long)i + 1],
                         coords[3 * (long long)i + 2], B);
    out[(long long)i * K + k] = __fsqrt_rn(s);
}

__global__ void __launch_bounds__(256) k_differences(const float *__restrict__ coords, int n, PointSrc src, int K,
                                                     int fromIndex, Basis B, int isPBC, float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (i >= n)
        return;
    float px, py, pz;
    int atom;
    point_of(src, coords, k, px, py, pz, atom);
    if (fromIndex && i < atom)
        return;
    float ox, oy, oz;
    pair_diff(px, py, pz, coords[3 * (long long)i], coords[3 * (long long)i + 1], coords[3 * (long long)i + 2], B,
              isPBC, ox, oy, oz);
    out[((long long)i * 3 + 0) * K + k] = ox;
    out[((long long)i * 3 + 1) * K + k] = oy;
    out[((long long)i * 3 + 2) * K + k] = oz;
}

// out[i] = bc(to[i] - from[i])  (pairs_distances.pyx:71-93, :113-126)
__global__ void __launch_bounds__(256) k_from_to(const float *__restrict__ from, const float *__restrict__ to, int n,
                                                 Basis B, int isPBC, float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float ox, oy, oz;
    pair_diff(to[3 * (long long)i], to[3 * (long long)i + 1], to[3 * (long long)i + 2], from[3 * (long long)i],
              from[3 * (long long)i + 1], from[3 * (long long)i + 2], B, isPBC, ox, oy, oz);
    out[3 * (long long)i] = ox;
    out[3 * (long long)i + 1] = oy;
    out[3 * (long long)i + 2] = oz;
}

// out[i] = coords[i] . M in the reference's order
// (boundary_conditions_collection.pyx:104-106).
__global__ void __launch_bounds__(256) k_transform(Basis M, const float *__restrict__ coords, int n,
                                                   float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float x = coords[3 * (long long)i], y = coords[3 * (long long)i + 1], z = coords[3 * (long long)i + 2];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        out[3 * (long long)i + c] =
            __fadd_rn(__fadd_rn(__fmul_rn(x, M.b[c]), __fmul_rn(y, M.b[3 + c])), __fmul_rn(z, M.b[6 + c]));
}

int launch_distances(const float *coords, int n, const float *pts, long long ps, const int *idx, int K,
                     int fromIndex, int isPBC, const float *basis, float *out, cudaStream_t st)
{
    if (n <= 0 || K <= 0)
        return FRMC_OK;
    if (K > 65535)
        return set_error(FRMC_E_ARG, "too many points (%d)", K);
    PointSrc src{pts, ps, idx};
    Basis B = make_basis(basis);
    dim3 grid((n + 255) / 256, K);
    switch (basis_mode(basis, isPBC)) {
    case BM_IBC: k_distances<BM_IBC><<<grid, 256, 0, st>>>(coords, n, src, K, fromIndex, B, out); break;
    case BM_DIAG: k_distances<BM_DIAG><<<grid, 256, 0, st>>>(coords, n, src, K, fromIndex, B, out); break;
    case BM_XYTRI: k_distances<BM_XYTRI><<<grid, 256, 0, st>>>(coords, n, src, K, fromIndex, B, out); break;
    case BM_LOWER: k_distances<BM_LOWER><<<grid, 256, 0, st>>>(coords, n, src, K, fromIndex, B, out); break;
    default: k_distances<BM_GENERAL><<<grid, 256, 0, st>>>(coords, n, src, K, fromIndex, B, out); break;
    }
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

int launch_differences(const float *coords, int n, const float *pts, long long ps, const int *idx, int K,
                       int fromIndex, int isPBC, const float *basis, float *out, cudaStream_t st)
{
    if (n <= 0 || K <= 0)
        return FRMC_OK;
    if (K > 65535)
        return set_error(FRMC_E_ARG, "too many points (%d)", K);
    PointSrc src{pts, ps, idx};
    dim3 grid((n + 255) / 256, K);
    k_differences<<<grid, 256, 0, st>>>(coords, n, src, K, fromIndex, make_basis(basis), isPBC, out);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

int launch_from_to(const float *from, const float *to, int n, int isPBC, const float *basis, float *out,
                   cudaStream_t st)
{
    if (n <= 0)
        return FRMC_OK;
    k_from_to<<<(n + 255) / 256, 256, 0, st>>>(from, to, n, make_basis(basis), isPBC, out);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

int launch_transform(const float *M, const float *coords, int n, float *out, cudaStream_t st)
{
    if (n <= 0)
        return FRMC_OK;
    k_transform<<<(n + 255) / 256, 256, 0, st>>>(make_basis(M), coords, n, out);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

}  // namespace frmc
