// FP64 sine transforms between real and reciprocal space
// (fullrmc Extensions/reciprocal_space.pyx, recomputed in double precision).
//
//   gr_to_sq  (reciprocal_space.pyx:42-73):
//       S(q) = 1 + 4 pi rho / q * sum_r dr r (g(r) - 1) sin(q r)
//   Gr_to_sq  (reciprocal_space.pyx:82-109):
//       S(q) = 1 + 1 / q * sum_r dr G(r) sin(q r)
//   sq_to_Gr  (reciprocal_space.pyx:118-145):
//       G(r) = 2 / pi * sum_q dq q (S(q) - 1) sin(q r)
//
// The float32 inputs are promoted exactly, so every sine argument q*r is the
// exact double product; only the summation order differs from a float64
// numpy evaluation.  One thread per output point; the summation grid is
// staged through shared memory in chunks.
#include <cmath>

#include "frmc_runtime.h"

namespace frmc {

enum SineKind : int { SK_GR_TO_SQ = 0, SK_BIGGR_TO_SQ = 1, SK_SQ_TO_GR = 2 };

constexpr int kSineChunk = 256;

__global__ void __launch_bounds__(256) k_sine(int kind, const float *__restrict__ xs, int nx,
                                              const float *__restrict__ ys, const float *__restrict__ f, int ny,
                                              double rho, double *__restrict__ out)
{
    __shared__ double sy[kSineChunk], sw[kSineChunk];
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const double x = m < nx ? (double)xs[m] : 0.0;
    const double dy = (double)ys[1] - (double)ys[0];
    double acc = 0.0;
    for (int l0 = 0; l0 < ny; l0 += kSineChunk) {
        __syncthreads();
        for (int l = threadIdx.x; l < kSineChunk && l0 + l < ny; l += blockDim.x) {
            const double y = (double)ys[l0 + l];
            const double v = (double)f[l0 + l];
            double w;
            if (kind == SK_GR_TO_SQ)
                w = dy * y * (v - 1.0);
            else if (kind == SK_BIGGR_TO_SQ)
                w = dy * v;
            else
                w = dy * y * (v - 1.0);
            sy[l] = y;
            sw[l] = w;
        }
        __syncthreads();
        const int lc = min(kSineChunk, ny - l0);
        for (int l = 0; l < lc; ++l) acc = fma(sw[l], sin(x * sy[l]), acc);
    }
    if (m >= nx)
        return;
    if (kind == SK_GR_TO_SQ)
        out[m] = 1.0 + (4.0 * M_PI * rho) * (acc / x);
    else if (kind == SK_BIGGR_TO_SQ)
        out[m] = 1.0 + acc / x;
    else
        out[m] = (2.0 / M_PI) * acc;
}

int launch_sine(int kind, const float *xs, int nx, const float *ys, const float *f, int ny, double rho, double *out,
                cudaStream_t st)
{
    if (nx <= 0)
        return FRMC_OK;
    if (ny < 2)
        return set_error(FRMC_E_ARG, "sine transform needs at least two grid points");
    k_sine<<<(nx + 255) / 256, 256, 0, st>>>(kind, xs, nx, ys, f, ny, rho, out);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

}  // namespace frmc
