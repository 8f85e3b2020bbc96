// Per-pair float32 arithmetic shared by every kernel of the library.
//
// The operation order is fullrmc's (Extensions/pairs_distances.pyx:375-386,
// :443-471 and Extensions/pairs_histograms.pyx:53-68), written with explicit
// round-to-nearest intrinsics so that no multiply-add is ever contracted:
//
//   diff = a - b
//   box  = diff - round(diff),  round(x) = x > 0 ? floor(x + .5) : ceil(x - .5)
//   real = (box_x*B[0][k] + box_y*B[1][k]) + box_z*B[2][k]
//   s    = (rx*rx + ry*ry) + rz*rz,   d = sqrt(s)   (IEEE, round to nearest)
//
// round(): for x > 0, x + .5 > 0 so floor == trunc; for x < 0, x - .5 < 0
// so ceil == trunc; hence round(x) == trunc(x + copysign(.5, x)) for every x
// except x == +0, where the two differ only in the sign of a zero that is
// then subtracted from zero (both give box == +0).  That is one LOP3, one
// FADD and one FRND instead of a compare, two adds, floor, ceil and a select.
//
// Basis sparsity: a product with an exactly-zero basis entry is +-0, and
// adding +-0 to a non-zero float returns it unchanged, so for *distances*
// (which square every component) the terms with a zero basis entry may be
// dropped without changing a single bit of d.  Differences keep every term.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace frmc {

// Basis shapes, chosen on the host from the exact zero pattern of B.
enum BasisMode : int {
    BM_IBC = 0,      // infinite boundary conditions: real coordinates
    BM_DIAG = 1,     // orthorhombic: only B00, B11, B22
    BM_XYTRI = 2,    // a || x, b in xy, c || z: B00, B10, B11, B22
    BM_LOWER = 3,    // a || x, b in xy, c general: B01 = B02 = B12 = 0
    BM_GENERAL = 4,  // any basis
};

struct Basis {
    float b[9];  // row-major B[row][col]; rows are the box vectors
};

__device__ __forceinline__ float box_wrap(float x)
{
    return __fsub_rn(x, truncf(__fadd_rn(x, copysignf(0.5f, x))));
}

// Squared minimum-image distance s for the pair (a, b), a - b order.
template <int BM>
__device__ __forceinline__ float pair_s(float ax, float ay, float az,
                                        float bx, float by, float bz,
                                        const Basis &B)
{
    float dx = __fsub_rn(ax, bx);
    float dy = __fsub_rn(ay, by);
    float dz = __fsub_rn(az, bz);
    float rx, ry, rz;
    if (BM == BM_IBC) {
        rx = dx; ry = dy; rz = dz;
    } else {
        dx = box_wrap(dx);
        dy = box_wrap(dy);
        dz = box_wrap(dz);
        if (BM == BM_DIAG) {
            rx = __fmul_rn(dx, B.b[0]);
            ry = __fmul_rn(dy, B.b[4]);
            rz = __fmul_rn(dz, B.b[8]);
        } else if (BM == BM_XYTRI) {
            rx = __fadd_rn(__fmul_rn(dx, B.b[0]), __fmul_rn(dy, B.b[3]));
            ry = __fmul_rn(dy, B.b[4]);
            rz = __fmul_rn(dz, B.b[8]);
        } else if (BM == BM_LOWER) {
            rx = __fadd_rn(__fadd_rn(__fmul_rn(dx, B.b[0]), __fmul_rn(dy, B.b[3])), __fmul_rn(dz, B.b[6]));
            ry = __fadd_rn(__fmul_rn(dy, B.b[4]), __fmul_rn(dz, B.b[7]));
            rz = __fmul_rn(dz, B.b[8]);
        } else {
            rx = __fadd_rn(__fadd_rn(__fmul_rn(dx, B.b[0]), __fmul_rn(dy, B.b[3])), __fmul_rn(dz, B.b[6]));
            ry = __fadd_rn(__fadd_rn(__fmul_rn(dx, B.b[1]), __fmul_rn(dy, B.b[4])), __fmul_rn(dz, B.b[7]));
            rz = __fadd_rn(__fadd_rn(__fmul_rn(dx, B.b[2]), __fmul_rn(dy, B.b[5])), __fmul_rn(dz, B.b[8]));
        }
    }
    return __fadd_rn(__fadd_rn(__fmul_rn(rx, rx), __fmul_rn(ry, ry)), __fmul_rn(rz, rz));
}

// Full real-space difference (every basis term, a - b order): used by the
// *_differences_* entry points, whose outputs keep signed zeros.
__device__ __forceinline__ void pair_diff(float ax, float ay, float az,
                                          float bx, float by, float bz,
                                          const Basis &B, int isPBC,
                                          float &ox, float &oy, float &oz)
{
    float dx = __fsub_rn(ax, bx);
    float dy = __fsub_rn(ay, by);
    float dz = __fsub_rn(az, bz);
    if (!isPBC) {
        ox = dx; oy = dy; oz = dz;
        return;
    }
    dx = box_wrap(dx);
    dy = box_wrap(dy);
    dz = box_wrap(dz);
    ox = __fadd_rn(__fadd_rn(__fmul_rn(dx, B.b[0]), __fmul_rn(dy, B.b[3])), __fmul_rn(dz, B.b[6]));
    oy = __fadd_rn(__fadd_rn(__fmul_rn(dx, B.b[1]), __fmul_rn(dy, B.b[4])), __fmul_rn(dz, B.b[7]));
    oz = __fadd_rn(__fadd_rn(__fmul_rn(dx, B.b[2]), __fmul_rn(dy, B.b[5])), __fmul_rn(dz, B.b[8]));
}

// Histogram bin of an accepted pair: (int)((sqrt(s) - min) / bin) with IEEE
// sqrt and division (pairs_histograms.pyx:63).  The caller has already
// established d >= min, so the quotient is >= 0 and truncation is floor.
__device__ __forceinline__ int pair_bin(float s, float minD, float binw)
{
    float d = __fsqrt_rn(s);
    float q = __fdiv_rn(__fsub_rn(d, minD), binw);
    return __float2int_rz(q);
}

}  // namespace frmc
