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
// numpy evaluation.  One CTA per output point (k_sine_rows), so a grid of a
// few thousand points fills every SM.
#include <cmath>

#include "frmc_runtime.h"

namespace frmc {

enum SineKind : int { SK_GR_TO_SQ = 0, SK_BIGGR_TO_SQ = 1, SK_SQ_TO_GR = 2 };

// ----------------------------------------------------------------- shape function
// fullrmc's ShapeFunction (Constraints/Collection.py:15-160) on the device in
// FP64: a StructureFactorConstraint's total G(r) from all-pairs counts
// (StructureFactorConstraints.py:836-896), its S(q) (:302-312, 772-773) and
// G(r) back from S(q) (Collection.py:131-139).

// G(b) = 4 pi r_b rho0 (g(b) - 1), g(b) = sum_p coef_p n_p(b) / vol_b with
// n_p the pair's intra + inter counts (both orientations for unlike
// elements) and coef_p = w_p V / N_p; also w1[b] = dr G(b) for S(q).
__global__ void k_shape_G(const unsigned *__restrict__ counts, int ne, int hs, int npairs, const int *__restrict__ pi,
                          const int *__restrict__ pj, const double *__restrict__ pc, const double *__restrict__ r,
                          const double *__restrict__ vol, double rho0, double dr, double *__restrict__ G,
                          double *__restrict__ w1)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= hs)
        return;
    const long long total = (long long)ne * ne * hs;
    const unsigned *intra = counts, *inter = counts + total;
    double g = 0.0;
    for (int q = 0; q < npairs; ++q) {
        const int i = pi[q], j = pj[q];
        const long long ij = ((long long)i * ne + j) * hs + b;
        long long n = (long long)intra[ij] + inter[ij];
        if (i != j) {
            const long long ji = ((long long)j * ne + i) * hs + b;
            n += (long long)intra[ji] + inter[ji];
        }
        g += pc[q] * (double)n;
    }
    g /= vol[b];
    const double Gb = (4.0 * M_PI * r[b] * rho0) * (g - 1.0);
    G[b] = Gb;
    w1[b] = dr * Gb;
}

// w2[k] = dq q_k (S(q_k) - 1), the weights of the transform back to r.
__global__ void k_shape_wq(const double *__restrict__ q, const double *__restrict__ S, int nq, double dq,
                           double *__restrict__ w2)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nq)
        w2[k] = dq * q[k] * (S[k] - 1.0);
}

// out[m] = add + mul * sum_l w[l] sin(x_m y_l) (divided by x_m when div): one
// CTA per output point; thread t sums l = t, t + 128, ... in order, and a
// fixed tree combines the 128 partial sums, so the result does not depend on
// anything but the inputs.
constexpr int kSineRowThreads = 128;
__global__ void __launch_bounds__(kSineRowThreads) k_sine_rows(const double *__restrict__ x,
                                                               const double *__restrict__ y,
                                                               const double *__restrict__ w, int ny, double add,
                                                               double mul, int div, double *__restrict__ out)
{
    __shared__ double part[kSineRowThreads / 32];
    const int m = blockIdx.x;
    const double xm = x[m];
    double acc = 0.0;
    for (int l = threadIdx.x; l < ny; l += kSineRowThreads) acc = fma(w[l], sin(xm * y[l]), acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31u) == 0)
        part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        const double s = (part[0] + part[1]) + (part[2] + part[3]);
        out[m] = add + mul * (div ? s / xm : s);
    }
}

// The sine transforms with one CTA per output point (k_sine_rows): the
// float32 grids are promoted exactly and the summand weights formed first.
__global__ void k_sine_prep(int kind, const float *__restrict__ xs, int nx, const float *__restrict__ ys,
                            const float *__restrict__ f, int ny, double *__restrict__ xd, double *__restrict__ yd,
                            double *__restrict__ w)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nx)
        xd[i] = (double)xs[i];
    if (i < ny) {
        const double dy = (double)ys[1] - (double)ys[0];
        const double y = (double)ys[i], v = (double)f[i];
        yd[i] = y;
        w[i] = kind == SK_BIGGR_TO_SQ ? dy * v : dy * y * (v - 1.0);
    }
}

int launch_sine(int kind, const float *xs, int nx, const float *ys, const float *f, int ny, double rho, double *out,
                double *scratch, cudaStream_t st)
{
    if (nx <= 0)
        return FRMC_OK;
    if (ny < 2)
        return set_error(FRMC_E_ARG, "sine transform needs at least two grid points");
    double *xd = scratch, *yd = xd + nx, *w = yd + ny;
    const int n = nx > ny ? nx : ny;
    k_sine_prep<<<(n + 255) / 256, 256, 0, st>>>(kind, xs, nx, ys, f, ny, xd, yd, w);
    if (kind == SK_GR_TO_SQ)
        k_sine_rows<<<nx, kSineRowThreads, 0, st>>>(xd, yd, w, ny, 1.0, 4.0 * M_PI * rho, 1, out);
    else if (kind == SK_BIGGR_TO_SQ)
        k_sine_rows<<<nx, kSineRowThreads, 0, st>>>(xd, yd, w, ny, 1.0, 1.0, 1, out);
    else
        k_sine_rows<<<nx, kSineRowThreads, 0, st>>>(xd, yd, w, ny, 0.0, 2.0 / M_PI, 0, out);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

int launch_shape_function(const unsigned *counts, int ne, int hs, int npairs, const int *pi, const int *pj,
                          const double *pc, const double *r, const double *vol, double rho0, double dr,
                          const double *q, int nq, double dq, const double *rv, int nr, double *G, double *S,
                          double *Gs, double *w1, double *w2, cudaStream_t st)
{
    if (hs < 1 || nq < 1)
        return FRMC_OK;
    k_shape_G<<<(hs + 255) / 256, 256, 0, st>>>(counts, ne, hs, npairs, pi, pj, pc, r, vol, rho0, dr, G, w1);
    k_sine_rows<<<nq, kSineRowThreads, 0, st>>>(q, r, w1, hs, 1.0, 1.0, 1, S);
    k_shape_wq<<<(nq + 255) / 256, 256, 0, st>>>(q, S, nq, dq, w2);
    if (nr > 0)
        k_sine_rows<<<nr, kSineRowThreads, 0, st>>>(rv, q, w2, nq, 0.0, 2.0 / M_PI, 0, Gs);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

}  // namespace frmc
