// Device-resident RMC engines: many independent fullrmc-style Metropolis
// chains advanced by one persistent kernel per step.
//
// One chain follows fullrmc's step (Engine.py:3278-3344) with a single
// PairDistributionConstraint (PairDistributionConstraints.py:1044-1166):
//   1. moved atom a: new real coordinates = real + v, new box coordinates =
//      transform(reciprocal basis, new real) (boundary_conditions_collection.pyx:88-110);
//   2. delta histograms of a against every other atom j, before and after the
//      move, oriented [el(a)][el(j)] as multiple_pairs_histograms_coords does
//      (the F term of compute_before/after_move is empty for one atom);
//   3. G(r) of data - before + after (PairDistributionConstraints.py:847-895)
//      and chi2 = sum w (exp - G)^2 / varianceSquared, in FP64;
//   4. reject iff chi2_new > chi2_old and u > tolerance (Engine.py:3310-3317);
//      on accept the counts and coordinates are committed.
//
// Layout in HBM: one allocation per engine holding float4 box (x, y, z, el
// bits) and float4 real coordinates, int mol, int32 oriented counts and deltas
// [2][ne][ne][hs], the FP64 per-bin tables, the element-pair table, a ring of
// moves, a ring of step results and the chain state.  A descriptor array
// holds each engine's pointers and constants.
//
// The step kernel walks a work list of (engine, atom tile) items; persistent
// CTAs claim items from an atomic counter (the last CTA to leave resets it).
// Each item adds +-1 to its engine's oriented delta, to its element-pair delta
// and to a touched list with global atomics; the CTA that completes an
// engine's last item (threadfence + counter, no waiting) then evaluates,
// decides and commits that engine while the other CTAs keep claiming items.
// The FP64 evaluation is incremental: G(r) of the current configuration is
// kept, and only bins whose element-pair counts changed do FP64 work.
// Nothing spins, so the kernel cannot hang; a chain's arithmetic depends only
// on its own data and every reduction has a fixed order, so a chain gives
// bit-identical results alone or batched with any other chains, under any
// tile or CTA configuration.  Engines with a StructureFactorConstraint term
// finish their step in a second persistent kernel (k_sq_fused, below), whose
// items wait only for items listed before them, with bounded waits.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include "frmc_gpu_engine.h"
#include "frmc_math.cuh"
#include "frmc_ptx.cuh"
#include "frmc_runtime.h"
#include "frmc_tc.cuh"

namespace frmc {

struct EState {
    double chi2;        // sd / varianceSquared (+ sd_sq / sq varianceSquared)
    double sd;          // sum w (exp - G)^2 of the current configuration
    double sd_sq;       // sum w (S_exp - S)^2 of the current configuration
    double dsd;         // change of sd proposed this step (engines with S(Q))
    long long step;
    long long accepted;
    unsigned long long swept;  // columns swept by one-CTA steps (all atoms, or the selected cells')
    unsigned done;      // items of the current step finished
    unsigned tcount;    // entries in the touched-bin list of the current step
    unsigned sq_done;   // S(Q) tiles of the current step finished (engines with S(Q))
    unsigned sq_ydone;  // S(Q) row items of the current step finished
    int fmt;            // touched-list format of the step: 1 = (flat << 1) | sign, 0 = flat
    double sf;          // scale factor of the current configuration (dense engines)
    double sf_prop;     // scale factor of this step's proposal (dense engines with S(Q))
    // The next step's single-atom move as a fused step stages it while it
    // runs: the ring entry and the moved atom's data at the end of the step.
    // The next step uses it, instead of two dependent loads through the
    // ring, while nx_step is its step and nx_gen the ring's generation `gen`
    // (every write of the move ring raises gen once its data have landed).
    unsigned gen;
    unsigned nx_gen;
    long long nx_step;
    int nx_atom;
    float nx_v[3];
    float nx_u;
    int nx_mol;
    int2 nx_csl;
    float4 nx_box, nx_real;
};

// Work scheduler of one engine set: CTAs claim items with an atomic counter;
// the last CTA to leave a launch resets it for the next launch.
struct Sched {
    unsigned long long claimed;
    unsigned finished;
    unsigned status;  // DeviceStatus bits raised by the kernels (a bounded wait gave up)
};

struct EMove {
    int atom;    // the moved atom (the first atom of a moved group)
    float v[3];  // its real-space displacement (every atom's, for a group translation)
    float u;     // uniform number of the tolerance test
};

// Group moves (engines with group > 1; fullrmc's TranslationGenerator and
// RotationGenerator on molecule groups, Generators/Translations.py,
// Generators/Rotations.py): the other atoms of the group and the kind of move.
// A rotation takes every atom x of the group to (x - c) rot + c, c the
// group's centroid (float32, atoms added in group order, divided by the
// group size), with row-vector products summed as (x0 r0k + x1 r1k) + x2 r2k.
constexpr int kMaxGroup = 16;
constexpr int kMaxCells = 512;  // cells of an engine's column grid
struct EGroup {
    int kind;       // 0: translation by the move's v, 1: rotation
    float rot[9];   // row-major 3 x 3
    int atoms[kMaxGroup - 1];
};

// The moved atoms of the current step, in shared memory.
struct MovedGroup {
    int n;
    int atom[kMaxGroup];
    int el[kMaxGroup];
    int mol[kMaxGroup];
    float o[kMaxGroup][3];   // box coordinates before the move
    float nw[kMaxGroup][3];  // box coordinates after
    float nr[kMaxGroup][3];  // real coordinates after
    int slot[kMaxGroup];     // cell-sorted position and cell of each moved atom (engines with a grid)
    int cell[kMaxGroup];
    float u;                 // the move's uniform number
    long long step;          // the engine's step, accepted count, sd and chi2 before this step
    long long accepted;
    double sd, chi2;
};

struct EResult {
    double chi2_new;
    int accepted;
    int atom;
};

struct EDesc {
    int n, ne, hs, bm, npairs, ntiles, move_cap, has_dw;
    long long total;  // ne*ne*hs
    float minD, maxD, binw, s_lo, s_hi;
    Basis B, RB;
    double var2, tol;
    float4 *box, *real;
    int *mol, *counts, *delta, *pi, *pj;
    int *dP;      // [npairs][hs] per-step change of the element-pair counts
    int *pidx;    // [ne][ne] element pair -> index into the pair table (-1: none)
    int *tlist;   // oriented bins touched this step (2 n + 8 entries)
    double *rfac, *invvol, *expd, *dw, *pc;
    double *R;    // [hs] rfac * invvol: G(b) = R(b) sum_p pair_coef_p n_p(b) - rfac(b)
    double *A;    // [hs] w R^2
    double *Bq;   // [hs] 2 w R (exp - G) of the current configuration
    double *Sb;   // [hs] S(b) = sum_p pair_coef_p dP_p(b) proposed this step (large hs, S(Q) or dense)
    // Dense engines (scale factor != 1, a fitted scale factor or a window):
    // every step evaluates window * (s G') over all bins, G' = Gc + R S.
    int dense, wlen, fit_freq;
    double sf0, fit_min, fit_max;
    double *Gc;   // [hs] G of the current configuration (before scale factor and window)
    double *fnum; // [hs] fit numerator weights times the fit target
    double *fden; // [hs] fit denominator weights
    double *win;  // [wlen] window
    // S(Q) term (sq = 1): with x(b) = Rq(b) S(b) the change of the S(Q)
    // shells' G, d(sd_sq) = x^T y - x^T h, y = K x, K = M W M^T,
    // h = 2 M W (S_exp - S).  y is computed exactly in integers from the
    // element-pair deltas: y(b) = yscale sum_p pair_coef_p z_p(b),
    // z_p(b) = sum_c T[c][b] dP_p(c), T[c][b] = round(K[c][b] R0(c) 2^s).
    int sq, nq;
    double var2q;
    double yscale;      // rho0 2^-s
    const double *M;    // [hs][nq] G -> S(Q) table (shared)
    const long long *T; // [hs][hs] fixed-point K R0 (shared)
    const double *wq;   // [nq] data weights or null (shared)
    double *Rq;         // [hs] 4 pi r rho0 / shell volume of the S(Q) shells
    double *rfacq;      // [hs] 4 pi r rho0 of the S(Q) shells
    double *sqexp;      // [nq] experimental S(Q)
    double *h;          // [hs] 2 M W (S_exp - S) of the current configuration
    double *y;          // [hs] K x of this step
    double *gsq;        // [hs] G on the S(Q) shells of the current counts (set-up and reports)
    double *sqpart;     // [hs / kSqRows rounded up] this step's shares of x (y - h), per 128-bin row block
    double *sqv;        // [nq] S(Q) written by the evaluation kernel
    int *evl;           // [npairs][hs] this step's non-zero element-pair deltas, per pair
    int *evn;           // [npairs] their counts n (-1 - n: a delta beyond kSqGemmMaxDelta or a column
                        // sum beyond kSqMaxL1, sum the list exactly; INT_MIN: a delta beyond 16 bits,
                        // sum the deltas dP), in the table's per-column array
    // y on the tensor cores: X holds this step's element-pair deltas as fp16
    // (column q of the engine at X + q xld, bins down the column); the S(Q)
    // kernel multiplies the table's kSqLimbs balanced base-4096 digit planes
    // by every engine's columns (exact integers in fp32) into Zf, kept as
    // [plane][row block][table column][kSqRows]: bin b of plane l of column q
    // at Zf + ((l hsp / kSqRows + b / kSqRows) zcap + q) kSqRows + b % kSqRows;
    // wide columns go to Zi (column q at Zi + q hsp) by the exact integer path.
    __half *X;
    float *Zf;
    long long *Zi;
    int xld, hsp, zcap;
    int sq_gemm_max;    // largest |delta| taken through the product (kSqGemmMaxDelta; lower values,
                        // down to 0 = never and -1 = the dense integer loop, exist for tests)
    // Column grid (nc > 0): the atoms sorted by cell, so that a step sweeps
    // only the cells whose bounding box may come within maxD of a moved atom.
    // cbox / cmol mirror box / mol in cell order, csl[i] = (position, cell)
    // of atom i, cstart[c] the first position of cell c; clo / chi bound the
    // box coordinates of each cell's atoms and only grow (an accepted move
    // widens its atom's cell).  The lower bound of the minimum-image distance
    // from per-axis gaps m (fractional, or real for free boundaries) is
    // sum_k (m_k cw_k)^2 (cmode 0: orthorhombic box, free boundaries) or
    // max(max_k (m_k cw_k)^2, clam2 |m|^2) (cmode 1: cw_k the cell's
    // perpendicular widths, clam2 the smallest eigenvalue of B B^T).
    int nc, cmode, cpbc;
    float cw[3], clam2, cthr2;
    // one-CTA steps keep the element-pair deltas as biased 16-bit halves of
    // 32-bit words (dpk = 1) when no delta can pass 32767 in magnitude
    // (atoms x moved atoms + moved-atom pairs < 32000)
    int dpk;
    float4 *cbox, *clo, *chi;
    int *cmol, *cstart;
    int2 *csl;
    EMove *moves;
    EGroup *groups;     // [move_cap] (group > 1)
    int group;          // atoms per move
    EResult *results;
    EState *st;
};

// The fields the per-column loops read, copied into registers once per item
// (through a const reference every access would be a global load that the
// compiler must repeat after each store, since the stores might alias it).
struct ColView {
    Basis B;
    float s_lo, s_hi, minD, binw;
    int n, ne, hs, dpk;
    long long total;
    const float4 *__restrict__ box;
    const int *__restrict__ mol;
    const int *__restrict__ pidx;
    int *__restrict__ tlist;
};

__device__ __forceinline__ ColView col_view(const EDesc &D)
{
    ColView v;
    v.B = D.B;
    v.s_lo = D.s_lo;
    v.s_hi = D.s_hi;
    v.minD = D.minD;
    v.binw = D.binw;
    v.n = D.n;
    v.ne = D.ne;
    v.hs = D.hs;
    v.dpk = D.dpk;
    v.total = D.total;
    v.box = D.box;
    v.mol = D.mol;
    v.pidx = D.pidx;
    v.tlist = D.tlist;
    return v;
}

struct StepParams {
    const EDesc *desc;
    const EDesc *fdesc;  // fused launches: the descriptors in work-list order (fdesc[k] is item k's engine)
    const int2 *items;
    int nitems;
    int tile;
    int eval_only;      // 1: compute G(r) and chi2 of the current counts, no move
    int fused_dp_ints;  // fused launches: ints of the element-pair deltas (a multiple of 4)
    int fused_bins;     // fused launches: doubles of each of A and Bq (even)
    Sched *sched;
    // host-buffer steps of fused engines (else null): item k's move is
    // hmoves[fpos[k]] and its result goes to hres[fpos[k]], both in mapped
    // pinned host memory
    const EMove *hmoves;
    EResult *hres;
    const int *fpos;
    // one-CTA launches with one item per CTA: per item, the SM that ran it
    // (bits 48..63) and its CTA's time on the item in ns, or null
    unsigned long long *place;
};

constexpr int kRedLanes = 64;

// transform_coordinates row-vector product (boundary_conditions_collection.pyx:104-106)
__device__ __forceinline__ float3 to_box(const Basis &RB, float x, float y, float z)
{
    float3 r;
    r.x = __fadd_rn(__fadd_rn(__fmul_rn(x, RB.b[0]), __fmul_rn(y, RB.b[3])), __fmul_rn(z, RB.b[6]));
    r.y = __fadd_rn(__fadd_rn(__fmul_rn(x, RB.b[1]), __fmul_rn(y, RB.b[4])), __fmul_rn(z, RB.b[7]));
    r.z = __fadd_rn(__fadd_rn(__fmul_rn(x, RB.b[2]), __fmul_rn(y, RB.b[5])), __fmul_rn(z, RB.b[8]));
    return r;
}

// The moved atoms of `step` into shared memory: box coordinates before, real
// and box coordinates after the move (new box = transform(reciprocal basis,
// new real), boundary_conditions_collection.pyx:88-110).  All threads of the
// CTA call it; the caller synchronises before use.  A single atom is done by
// thread 0 alone.
__device__ void load_moved_group(const EDesc &D, long long step, MovedGroup &g, const EMove *staged = nullptr)
{
    const int G = D.group;
    if (G == 1) {
        if (threadIdx.x == 0) {
            // the move and the moved atom as the previous step staged them
            // (read with the state: one load hop), else through the ring
            const EState &S = *D.st;
            const long long nxs = S.nx_step;
            const unsigned nxg = S.nx_gen, gen = S.gen;
            int a = S.nx_atom, mol = S.nx_mol;
            float v0 = S.nx_v[0], v1 = S.nx_v[1], v2 = S.nx_v[2], u = S.nx_u;
            float4 ob = S.nx_box, orl = S.nx_real;
            int2 sl = S.nx_csl;
            g.accepted = S.accepted;
            g.sd = S.sd;
            g.chi2 = S.chi2;
            if (staged || nxs != step || nxg != gen) {
                const EMove &m = staged ? *staged : D.moves[step % D.move_cap];
                a = m.atom;
                v0 = m.v[0]; v1 = m.v[1]; v2 = m.v[2]; u = m.u;
                ob = D.box[a];
                orl = D.real[a];
                mol = D.mol[a];
                if (D.nc > 0)
                    sl = D.csl[a];
            }
            const float rx = __fadd_rn(orl.x, v0), ry = __fadd_rn(orl.y, v1), rz = __fadd_rn(orl.z, v2);
            const float3 nw = D.bm == BM_IBC ? make_float3(rx, ry, rz) : to_box(D.RB, rx, ry, rz);
            g.u = u;
            g.step = step;
            g.n = 1;
            g.atom[0] = a;
            g.el[0] = __float_as_int(ob.w);
            g.mol[0] = mol;
            g.o[0][0] = ob.x; g.o[0][1] = ob.y; g.o[0][2] = ob.z;
            g.nw[0][0] = nw.x; g.nw[0][1] = nw.y; g.nw[0][2] = nw.z;
            g.nr[0][0] = rx; g.nr[0][1] = ry; g.nr[0][2] = rz;
            if (D.nc > 0) {
                g.slot[0] = sl.x;
                g.cell[0] = sl.y;
            }
        }
        return;
    }
    const EMove &m = staged ? *staged : D.moves[step % D.move_cap];
    if (threadIdx.x == 0) {
        g.u = m.u;
        g.step = step;
        g.accepted = D.st->accepted;
        g.sd = D.st->sd;
        g.chi2 = D.st->chi2;
    }
    const EGroup &gm = D.groups[step % D.move_cap];
    const int t = threadIdx.x;
    if (t < G) {
        const int a = t == 0 ? m.atom : gm.atoms[t - 1];
        const float4 ob = D.box[a];
        const float4 orl = D.real[a];
        g.atom[t] = a;
        g.el[t] = __float_as_int(ob.w);
        g.mol[t] = D.mol[a];
        g.o[t][0] = ob.x; g.o[t][1] = ob.y; g.o[t][2] = ob.z;
        g.nr[t][0] = orl.x; g.nr[t][1] = orl.y; g.nr[t][2] = orl.z;
        if (D.nc > 0) {
            const int2 sl = D.csl[a];
            g.slot[t] = sl.x;
            g.cell[t] = sl.y;
        }
    }
    if (t == 0)
        g.n = G;
    __syncthreads();
    __shared__ float s_c[3];
    const bool rot = gm.kind == 1;
    if (rot && t == 0) {
        float cx = g.nr[0][0], cy = g.nr[0][1], cz = g.nr[0][2];
        for (int k = 1; k < G; ++k) {
            cx = __fadd_rn(cx, g.nr[k][0]);
            cy = __fadd_rn(cy, g.nr[k][1]);
            cz = __fadd_rn(cz, g.nr[k][2]);
        }
        const float fg = (float)G;
        s_c[0] = __fdiv_rn(cx, fg);
        s_c[1] = __fdiv_rn(cy, fg);
        s_c[2] = __fdiv_rn(cz, fg);
    }
    __syncthreads();
    if (t < G) {
        const float x = g.nr[t][0], y = g.nr[t][1], z = g.nr[t][2];
        float rx, ry, rz;
        if (rot) {
            const float *R = gm.rot;
            const float dx = __fsub_rn(x, s_c[0]), dy = __fsub_rn(y, s_c[1]), dz = __fsub_rn(z, s_c[2]);
            rx = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, R[0]), __fmul_rn(dy, R[3])), __fmul_rn(dz, R[6])), s_c[0]);
            ry = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, R[1]), __fmul_rn(dy, R[4])), __fmul_rn(dz, R[7])), s_c[1]);
            rz = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, R[2]), __fmul_rn(dy, R[5])), __fmul_rn(dz, R[8])), s_c[2]);
        } else {
            rx = __fadd_rn(x, m.v[0]);
            ry = __fadd_rn(y, m.v[1]);
            rz = __fadd_rn(z, m.v[2]);
        }
        const float3 nw = D.bm == BM_IBC ? make_float3(rx, ry, rz) : to_box(D.RB, rx, ry, rz);
        g.nr[t][0] = rx; g.nr[t][1] = ry; g.nr[t][2] = rz;
        g.nw[t][0] = nw.x; g.nw[t][1] = nw.y; g.nw[t][2] = nw.z;
    }
}

// Commit of an accepted move: the moved atoms' coordinates, their copies in
// cell order and their cells' bounds (one thread, as atoms of a group may
// share a cell).
// cb: the bounds of atom 0's cell as cell selection read them (single-atom
// steps with a grid), or null to read them here.
__device__ void commit_moved_group(const EDesc &D, const MovedGroup &g, const float4 *cb = nullptr)
{
    for (int t = threadIdx.x; t < g.n; t += blockDim.x) {
        const int a = g.atom[t];
        const float4 nb = make_float4(g.nw[t][0], g.nw[t][1], g.nw[t][2], __int_as_float(g.el[t]));
        D.box[a] = nb;
        D.real[a] = make_float4(g.nr[t][0], g.nr[t][1], g.nr[t][2], 0.0f);
        if (D.nc > 0)
            D.cbox[g.slot[t]] = nb;
    }
    if (D.nc > 0 && threadIdx.x == 0) {
        for (int t = 0; t < g.n; ++t) {
            const int c = g.cell[t];
            float4 lo = (cb && t == 0) ? cb[0] : D.clo[c], hi = (cb && t == 0) ? cb[1] : D.chi[c];
            lo.x = fminf(lo.x, g.nw[t][0]);
            lo.y = fminf(lo.y, g.nw[t][1]);
            lo.z = fminf(lo.z, g.nw[t][2]);
            hi.x = fmaxf(hi.x, g.nw[t][0]);
            hi.y = fmaxf(hi.y, g.nw[t][1]);
            hi.z = fmaxf(hi.z, g.nw[t][2]);
            D.clo[c] = lo;
            D.chi[c] = hi;
        }
    }
}

// Element-pair index and bin of an oriented flat index.  A count past the
// last bin lands in bin 0.. of the next oriented row of the C-contiguous
// array, as with the reference's unchecked index.
template <class V>
__device__ __forceinline__ void pair_of_flat(const V &D, int flat, int ra, int rb, int bin, int &p, int &b)
{
    if (bin >= D.hs) {
        const int row = flat / D.hs;
        bin = flat - row * D.hs;
        ra = row / D.ne;
        rb = row - ra * D.ne;
    }
    p = D.pidx[ra * D.ne + rb];
    b = bin;
}

// Bins of column j before and after the move: flat oriented indexes f0, f1
// (-1 when out of range or unchanged), `half` (0 intra, total inter), bins and
// the column's element.  32-bit indexes: 2 * ne * ne * hs < 2^31 is checked
// when an engine is created.
// Bins of one column from its squared distances to the moved atom before
// (s0) and after (s1) the move; `valid` is false for a column past the end or
// the moved atom itself.  The squared distances of all columns of a batch are
// computed first, without branches, so their independent chains interleave.
template <class V>
__device__ __forceinline__ void column_bins(const V &D, float s0, float s1, bool valid, float4 c, int mj, int arow,
                                            int mola, int &f0, int &f1, int &half, int &b0, int &b1, int &elj)
{
    f0 = f1 = -1;
    const bool a0 = valid & (s0 >= D.s_lo) & (s0 < D.s_hi);
    const bool a1 = valid & (s1 >= D.s_lo) & (s1 < D.s_hi);
    if (a0 | a1) {
        elj = __float_as_int(c.w);
        half = mj == mola ? 0 : (int)D.total;
        const long long rowb = (long long)(arow + elj) * D.hs;
        if (a0) {
            b0 = pair_bin(s0, D.minD, D.binw);
            const long long f = rowb + b0;
            if ((unsigned long long)f < (unsigned long long)D.total) f0 = (int)f;
        }
        if (a1) {
            b1 = pair_bin(s1, D.minD, D.binw);
            const long long f = rowb + b1;
            if ((unsigned long long)f < (unsigned long long)D.total) f1 = (int)f;
        }
        if (f0 == f1)
            f0 = f1 = -1;
    }
}

constexpr int kItemUnroll = 4;

// One item of the split path: the moved atom against atoms
// [t*tile, (t+1)*tile).  For every column j the pair before and after the
// move is binned; a changed bin adds -1 / +1 to the engine's global oriented
// delta and element-pair delta, and its oriented index is appended to the
// touched list (one list reservation per warp and column).  Coordinates of
// kItemUnroll columns are loaded before any is used.
template <int BM>
__device__ void item_delta(const EDesc &Dg, int tile, const MovedGroup &g, int t)
{
    const ColView D = col_view(Dg);
    int *__restrict__ delta = Dg.delta;
    int *__restrict__ dP = Dg.dP;
    unsigned *tcount = &Dg.st->tcount;
    const int j0 = t * tile;
    const int j1 = min(D.n, j0 + tile);
    const int G = g.n;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt = (1u << lane) - 1u;
    for (int jb = j0; jb < j1; jb += kItemUnroll * blockDim.x) {
        float4 c[kItemUnroll];
        int mj[kItemUnroll];
        bool valid[kItemUnroll];
#pragma unroll
        for (int u = 0; u < kItemUnroll; ++u) {
            const int j = jb + u * blockDim.x + threadIdx.x;
            c[u] = j < j1 ? D.box[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            mj[u] = j < j1 ? D.mol[j] : 0;
            bool ok = j < j1;
            for (int q = 0; q < G; ++q) ok &= j != g.atom[q];
            valid[u] = ok;
        }
        for (int gi = 0; gi < G; ++gi) {
            const float3 o = make_float3(g.o[gi][0], g.o[gi][1], g.o[gi][2]);
            const float3 nw = make_float3(g.nw[gi][0], g.nw[gi][1], g.nw[gi][2]);
            const int ela = g.el[gi], mola = g.mol[gi], arow = ela * D.ne;
            float s0[kItemUnroll], s1[kItemUnroll];
#pragma unroll
            for (int u = 0; u < kItemUnroll; ++u) {
                s0[u] = pair_s<BM>(o.x, o.y, o.z, c[u].x, c[u].y, c[u].z, D.B);
                s1[u] = pair_s<BM>(nw.x, nw.y, nw.z, c[u].x, c[u].y, c[u].z, D.B);
            }
#pragma unroll
            for (int u = 0; u < kItemUnroll; ++u) {
                int f0 = -1, f1 = -1, half = 0, b0 = 0, b1 = 0, elj = 0;
                column_bins(D, s0[u], s1[u], valid[u], c[u], mj[u], arow, mola, f0, f1, half, b0, b1, elj);
                const unsigned m0 = __ballot_sync(0xffffffffu, f0 >= 0);
                const unsigned m1 = __ballot_sync(0xffffffffu, f1 >= 0);
                if ((m0 | m1) == 0u)
                    continue;
                unsigned base = 0;
                if (lane == 0)
                    base = atomicAdd(tcount, __popc(m0) + __popc(m1));
                base = __shfl_sync(0xffffffffu, base, 0);
                unsigned pos = base + __popc(m0 & lt) + __popc(m1 & lt);
                if (f0 >= 0) {
                    atomicSub(delta + half + f0, 1);
                    D.tlist[pos++] = half + f0;
                    int p, b;
                    pair_of_flat(D, f0, ela, elj, b0, p, b);
                    if (p >= 0)
                        atomicSub(dP + p * D.hs + b, 1);
                }
                if (f1 >= 0) {
                    atomicAdd(delta + half + f1, 1);
                    D.tlist[pos] = half + f1;
                    int p, b;
                    pair_of_flat(D, f1, ela, elj, b1, p, b);
                    if (p >= 0)
                        atomicAdd(dP + p * D.hs + b, 1);
                }
            }
        }
    }
}

// FP64 reductions with a fixed order that does not depend on the CTA size:
// bin b's contribution c(b) is computed by any thread into shared memory,
// then lane L (0 .. kRedLanes - 1) sums the contributions of bins b = L (mod
// kRedLanes) in increasing order and a fixed binary tree combines the lanes.
constexpr int kChunk = 2048;    // bins per shared-memory chunk

__device__ void lanes_zero(double *red)
{
    for (int L = threadIdx.x; L < kRedLanes; L += blockDim.x) red[L] = 0.0;
}

__device__ void lanes_add_chunk(double *red, const double *cb, int c0, int cn)
{
    __syncthreads();
    for (int L = threadIdx.x; L < kRedLanes; L += blockDim.x) {
        int b = c0 + ((L - c0 % kRedLanes) + kRedLanes) % kRedLanes;
        double acc = red[L];
        for (; b < c0 + cn; b += kRedLanes) acc += cb[b - c0];
        red[L] = acc;
    }
    __syncthreads();
}

// The lanes are combined by warp 0: each group of 32 lanes by a fixed
// shuffle tree, then the group sums by a fixed pairwise tree.
__device__ double lanes_total(double *red)
{
    constexpr int G = kRedLanes / 32;
    static_assert((G & (G - 1)) == 0, "lane groups must be a power of two");
    __shared__ double s_total;
    __syncthreads();  // every lane's partial sum is written
    if (threadIdx.x < 32) {
        double g[G];
#pragma unroll
        for (int k = 0; k < G; ++k) {
            double v = red[32 * k + threadIdx.x];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            g[k] = v;
        }
#pragma unroll
        for (int w = G / 2; w > 0; w >>= 1)
#pragma unroll
            for (int i = 0; i < w; ++i) g[i] += g[i + w];
        if (threadIdx.x == 0)
            s_total = g[0];
    }
    __syncthreads();
    return s_total;
}

// -2 x by exponent and sign arithmetic (exact; x is a sum of a few pair
// coefficients times small integers, so it is zero or a normal number).
__device__ __forceinline__ double neg_twice(double x)
{
    const long long b = __double_as_longlong(x);
    const long long e = (b & 0x7ff0000000000000ll) ? (1ll << 52) : 0ll;
    return __longlong_as_double((b ^ (long long)0x8000000000000000ull) + e);
}

// Element-pair count n_p(b) from the oriented counts (intra + inter, both
// orientations for unlike elements; PairDistributionConstraints.py:864-878).
__device__ __forceinline__ long long pair_count(const EDesc &D, int q, int b)
{
    const int i = D.pi[q], j = D.pj[q];
    const long long kij = (long long)(i * D.ne + j) * D.hs + b;
    long long c = (long long)D.counts[kij] + D.counts[D.total + kij];
    if (i != j) {
        const long long kji = (long long)(j * D.ne + i) * D.hs + b;
        c += (long long)D.counts[kji] + D.counts[D.total + kji];
    }
    return c;
}

// G(r) of the current counts and its sum of squared deviations (set-up):
// G(b) = R(b) sum_p pair_coef_p n_p(b) - rfac(b)  (PairDistributionConstraints.py:864-884);
// also the per-bin state Bq(b) = 2 w R (exp - G).
__device__ double eval_full(const EDesc &D, double *red, double *cb)
{
    lanes_zero(red);
    for (int c0 = 0; c0 < D.hs; c0 += kChunk) {
        const int cn = min(kChunk, D.hs - c0);
        for (int b = c0 + threadIdx.x; b < c0 + cn; b += blockDim.x) {
            double S = 0.0;
            for (int q = 0; q < D.npairs; ++q) S = fma(D.pc[q], (double)pair_count(D, q, b), S);
            const double G = fma(D.R[b], S, -D.rfac[b]);
            const double e = D.expd[b] - G;
            const double w = D.has_dw ? D.dw[b] : 1.0;
            D.Bq[b] = 2.0 * (w * D.R[b]) * e;
            cb[b - c0] = (w * e) * e;
            if (D.dense)
                D.Gc[b] = G;
        }
        lanes_add_chunk(red, cb, c0, cn);
    }
    return lanes_total(red);
}

// Dense engines (scale factor, fitted scale factor, window): the proposed G'
// = Gc + R S over all bins (with_step = false: the current G), the scale
// factor s -- fitted, s = clamp(sum fnum G' / sum fden G'^2), when `fit`,
// else the current one (Core/Constraint.py:1363-1424) -- and
// sd' = sum w (exp - window * (s G'))^2 with numpy.convolve's 'same' window
// (PairDistributionConstraints.py:884-893).  Every sum is taken in the fixed
// lane order.  Thread 0 stores s in *s_sf.
__device__ __forceinline__ double dense_G(const EDesc &D, int b, bool with_step)
{
    return with_step ? fma(D.R[b], __ldcg(D.Sb + b), D.Gc[b]) : D.Gc[b];
}

__device__ double eval_dense(const EDesc &D, double *red, double *cb, bool with_step, bool fit, double sf,
                             double *s_sf)
{
    if (fit) {
        double nd[2];
        for (int pass = 0; pass < 2; ++pass) {
            lanes_zero(red);
            for (int c0 = 0; c0 < D.hs; c0 += kChunk) {
                const int cn = min(kChunk, D.hs - c0);
                for (int b = c0 + threadIdx.x; b < c0 + cn; b += blockDim.x) {
                    const double G = dense_G(D, b, with_step);
                    cb[b - c0] = pass == 0 ? D.fnum[b] * G : D.fden[b] * (G * G);
                }
                lanes_add_chunk(red, cb, c0, cn);
            }
            nd[pass] = lanes_total(red);
        }
        if (nd[1] > 0.0)
            sf = fmin(fmax(nd[0] / nd[1], D.fit_min), D.fit_max);
    }
    const int L = D.wlen, c = (L - 1) / 2;
    lanes_zero(red);
    for (int c0 = 0; c0 < D.hs; c0 += kChunk) {
        const int cn = min(kChunk, D.hs - c0);
        for (int b = c0 + threadIdx.x; b < c0 + cn; b += blockDim.x) {
            double u;
            if (L > 0) {
                u = 0.0;
                for (int k = 0; k < L; ++k) {
                    const int j = b + c - k;
                    if (j >= 0 && j < D.hs)
                        u = fma(D.win[k], sf * dense_G(D, j, with_step), u);
                }
            } else {
                u = sf * dense_G(D, b, with_step);
            }
            const double e = D.expd[b] - u;
            const double w = D.has_dw ? D.dw[b] : 1.0;
            cb[b - c0] = (w * e) * e;
        }
        lanes_add_chunk(red, cb, c0, cn);
    }
    const double sd = lanes_total(red);
    if (threadIdx.x == 0)
        *s_sf = sf;
    return sd;
}

// On accept a dense engine's G moves to G' (the bins whose S changed).
__device__ void dense_commit(const EDesc &D)
{
    for (int b = threadIdx.x; b < D.hs; b += blockDim.x) {
        const double S = __ldcg(D.Sb + b);
        if (S != 0.0)
            D.Gc[b] = fma(D.R[b], S, D.Gc[b]);
    }
}

// Change of the sum of squared deviations for this step.  With
// dG(b) = R(b) S(b), S(b) = sum_p pair_coef_p dP_p(b):
//   d(sd) = sum_b w [(exp - G - dG)^2 - (exp - G)^2] = sum_b S (A S - Bq).
// Each thread takes bins b = tid, tid + blockDim, ...; all loads of a bin are
// issued before any is used and FP64 work is done only where some dP is
// non-zero.  The element-pair deltas are cleared as they are read; S is kept
// in shared memory (chunk) or global memory (Sb) for the commit.  Sums use the
// fixed lane order, so the result does not depend on the CTA size.
constexpr int kMaxP = 10;  // element pairs loaded with unrolled loads (ne <= 4)
// T in kSqLimbs balanced base-4096 digits t_l in [-2048, 2047] (4 digits
// cover |T| < 2^47; T stays below 2^46).  fp16 holds every integer up to 2048,
// so a delta column goes through the tensor-core product when its entries are
// at most kSqGemmMaxDelta in magnitude and their absolute sum is at most
// kSqMaxL1: every partial sum of a digit product, over any subset of the bins,
// is then an integer of magnitude <= 2048 * 2^13 = 2^24, which fp32
// accumulation (and fp32 addition of such partial sums) holds exactly.
constexpr int kSqLimbs = 4;
constexpr int kSqDigitBits = 12;
constexpr int kSqGemmMaxDelta = 2048;
constexpr int kSqMaxL1 = 1 << 13;

// SMEM: the element-pair deltas are this CTA's shared-memory copy (one CTA per
// engine); otherwise they are the engine's global array, filled by several
// CTAs, read through L2 and cleared as they are read (engines with an S(Q)
// term leave them for the S(Q) kernel, which clears them, and list them per
// element pair as (bin << 16) | (delta & 0xffff)).
//
// The bins whose element-pair counts changed are first listed, chunk by
// chunk, in increasing bin order (sbin[k]); the FP64 work then runs on the
// list only, so each warp-level FP64 instruction -- the FP64 pipe is narrow
// on this GPU -- serves up to 32 changed bins.  Lane L of the fixed-order
// reduction sums the list entries k = L (mod kRedLanes) in increasing k.  For
// hs <= kChunk the list, its -2 S values (sbs[k]) and its length (*s_nchg)
// stay in shared memory for the commit; larger histograms, and engines with
// an S(Q) term, also keep S in the global Sb (zero for unchanged bins).
// pair_coef_p * v for |v| <= 4 comes from a small table, so a changed bin
// costs one FP64 add per non-zero element-pair delta.
// Element-pair delta idx of a CTA's shared deltas (either layout).
__device__ __forceinline__ int delta_get(const int *sdP, int idx, int dpk)
{
    if (dpk)
        return (int)((reinterpret_cast<const unsigned *>(sdP)[idx >> 1] >> ((unsigned)(idx & 1) << 4)) & 0xffffu) -
               32768;
    return sdP[idx];
}

template <bool SMEM>
__device__ double eval_delta(const EDesc &Dg, int *dP, const double *Ab, const double *Bqb, double *red, double *cb,
                             double *sbs, int *sbin, int *s_nchg, double *coef, const int *nz)
{
    const int hs = Dg.hs;
    const double *__restrict__ A = Ab;
    const double *__restrict__ Bq = Bqb;
    double *__restrict__ Sb = Dg.Sb;
    const int np = Dg.npairs;
    const bool sq = Dg.sq != 0;
    int *__restrict__ gdP = Dg.dP;
    int *__restrict__ evl = Dg.evl;
    __shared__ int s_evn[kMaxP];
    __shared__ int s_l1[kMaxP];  // sum of |delta| per element pair (S(Q) product bound)
    __shared__ int s_wide;
    __shared__ int s_cnt[kChunk / 32];  // changed bins per 32-bin group, then their list offsets
    __shared__ double tabv[kMaxP * 9];  // pair_coef_q * v, v = -4..4
    if (sq) {
        for (int q = threadIdx.x; q < kMaxP; q += blockDim.x) {
            s_evn[q] = 0;
            s_l1[q] = 0;
        }
        if (threadIdx.x == 0)
            s_wide = 0;
    }
    if (!SMEM) {
        for (int q = threadIdx.x; q < np; q += blockDim.x) coef[q] = Dg.pc[q];
        __syncthreads();
    }
    for (int i = threadIdx.x; i < min(np, kMaxP) * 9; i += blockDim.x) {
        const int v = i % 9 - 4;
        const double cf = coef[i / 9];
        tabv[i] = v == 1 ? cf : (v == -1 ? -cf : cf * (double)v);
    }
    lanes_zero(red);
    __syncthreads();
    const bool big = hs > kChunk;
    const unsigned lane = threadIdx.x & 31u;
    const int dpk = Dg.dpk;
    auto delta_at = [&](int q, int b) -> int {
        return SMEM ? delta_get(dP, q * hs + b, dpk) : __ldcg(dP + (long long)q * hs + b);
    };
    for (int c0 = 0; c0 < hs; c0 += kChunk) {
        const int cn = min(kChunk, hs - c0);
        const int span = (cn + 31) & ~31;  // whole 32-bin groups, so every ballot has full warps
        // 1. which bins changed
        unsigned long long mine = 0;  // bit r: this thread's bin of round r changed
        int r = 0;
        for (int i = threadIdx.x; i < span; i += blockDim.x, ++r) {
            bool any = false;
            if (i < cn) {
                const int b = c0 + i;
                if (nz) {
                    any = nz[b] != 0;
                } else {
#pragma unroll
                    for (int q = 0; q < kMaxP; ++q)
                        if (q < np)
                            any |= delta_at(q, b) != 0;
                    for (int q = kMaxP; q < np; ++q) any |= delta_at(q, b) != 0;
                }
                if ((sq || big || Dg.dense) && !any)
                    Sb[b] = 0.0;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, any);
            if (lane == 0)
                s_cnt[i >> 5] = __popc(bal);
            if (any)
                mine |= 1ull << r;
        }
        __syncthreads();
        // 2. every warp scans the (at most 64) group counts in registers:
        // ex0 / ex1 are the list offsets of groups `lane` and 32 + `lane`
        const int ngroups = span >> 5;
        const int v0 = (int)lane < ngroups ? s_cnt[lane] : 0;
        const int v1 = (int)lane + 32 < ngroups ? s_cnt[lane + 32] : 0;
        int i0 = v0, i1 = v1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t0 = __shfl_up_sync(0xffffffffu, i0, o);
            const int t1 = __shfl_up_sync(0xffffffffu, i1, o);
            if ((int)lane >= o) {
                i0 += t0;
                i1 += t1;
            }
        }
        const int tot0 = __shfl_sync(0xffffffffu, i0, 31);
        const int ex0 = i0 - v0, ex1 = tot0 + i1 - v1;
        const int n = tot0 + __shfl_sync(0xffffffffu, i1, 31);
        if (threadIdx.x == 0)
            *s_nchg = n;
        // 3. the list, in increasing bin order (a warp's bins of one round are
        // one group, so its offset comes from the lane that holds the group)
        r = 0;
        for (int i = threadIdx.x; i < span; i += blockDim.x, ++r) {
            const int gi = i >> 5;
            const int base = gi < 32 ? __shfl_sync(0xffffffffu, ex0, gi) : __shfl_sync(0xffffffffu, ex1, gi - 32);
            const bool any = (mine >> r) & 1ull;
            const unsigned bal = __ballot_sync(0xffffffffu, any);
            if (any)
                sbin[base + __popc(bal & ((1u << lane) - 1u))] = c0 + i;
        }
        __syncthreads();
        // 4. FP64 on the listed bins
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            const int b = sbin[k];
            const double a = A[b];
            const double bq = Bq[b];
            double S = 0.0;
            bool wide_v = false;  // a delta beyond the table's -4..4 (one CTA's shared deltas)
#pragma unroll
            for (int q = 0; q < kMaxP; ++q) {
                if (q >= np)
                    break;
                const int v = delta_at(q, b);
                if (v) {
                    if (!SMEM && !sq)
                        dP[(long long)q * hs + b] = 0;
                    if (sq) {
                        if (SMEM)
                            gdP[q * hs + b] = v;
                        evl[q * hs + atomicAdd(&s_evn[q], 1)] = (b << 16) | (v & 0xffff);
                        Dg.X[q * Dg.xld + b] = __int2half_rn(v);
                        atomicAdd(&s_l1[q], v < 0 ? -v : v);
                        if (v > Dg.sq_gemm_max || v < -Dg.sq_gemm_max)
                            s_wide = (v > 32767 || v < -32768 || Dg.sq_gemm_max < 0) ? 2 : max(s_wide, 1);
                    }
                    if (SMEM) {
                        // the table only: the product below would otherwise be
                        // formed for every delta and discarded
                        if ((unsigned)(v + 4) <= 8u)
                            S += tabv[q * 9 + v + 4];
                        else
                            wide_v = true;
                    } else {
                        S += (unsigned)(v + 4) <= 8u ? tabv[q * 9 + v + 4] : coef[q] * (double)v;
                    }
                }
            }
            if (SMEM && __any_sync(__activemask(), wide_v) && wide_v) {
                // a rare delta beyond -4..4: the sum again, in the same order
                // (the shared deltas are still in place)
                S = 0.0;
#pragma unroll
                for (int q = 0; q < kMaxP; ++q) {
                    if (q >= np)
                        break;
                    const int v = delta_at(q, b);
                    if (v)
                        S += (unsigned)(v + 4) <= 8u ? tabv[q * 9 + v + 4] : coef[q] * (double)v;
                }
            }
            for (int q = kMaxP; q < np; ++q) {
                const int v = delta_at(q, b);
                if (v) {
                    if (!SMEM)
                        dP[(long long)q * hs + b] = 0;
                    const double cf = coef[q];
                    S += v == 1 ? cf : (v == -1 ? -cf : cf * (double)v);
                }
            }
            cb[k] = S * fma(a, S, -bq);
            sbs[k] = neg_twice(S);
            if (big || sq || Dg.dense)
                Sb[b] = S;
        }
        lanes_add_chunk(red, cb, 0, n);
    }
    const double total = lanes_total(red);
    if (sq && (int)threadIdx.x < np) {
        // per element pair: n (tensor-core product), -1 - n (exact sum over
        // the list of deltas) or INT_MIN (exact sum over the dense deltas)
        const int n = s_evn[threadIdx.x];
        const bool wide = s_wide == 1 || s_l1[threadIdx.x] > kSqMaxL1;
        Dg.evn[threadIdx.x] = s_wide == 2 ? INT_MIN : (wide ? -1 - n : n);
    }
    return total;
}

// Pairs inside a moved group.  fullrmc's before/after-move data is M - F
// (PairDistributionConstraints.py:1044-1129): M counts each group atom
// against all atoms, so a pair (a, b) of the group (a before b in group
// order) appears at [el(a)][el(b)] and [el(b)][el(a)], and F counts the group
// alone once, at [el(a)][el(b)]: one count per pair remains, at [el(b)][el(a)].
// Pair t of the G(G-1)/2 pairs gives its before/after bins like a column.
template <int BM, class V>
__device__ __forceinline__ void group_pair_bins(const V &D, const MovedGroup &g, int t, int &f0, int &f1, int &half,
                                                int &b0, int &b1, int &ela, int &elj)
{
    int b = 1, a = t;
    while (a >= b) {
        a -= b;
        ++b;
    }
    const float s0 = pair_s<BM>(g.o[b][0], g.o[b][1], g.o[b][2], g.o[a][0], g.o[a][1], g.o[a][2], D.B);
    const float s1 = pair_s<BM>(g.nw[b][0], g.nw[b][1], g.nw[b][2], g.nw[a][0], g.nw[a][1], g.nw[a][2], D.B);
    ela = g.el[b];
    half = b0 = b1 = elj = 0;
    column_bins(D, s0, s1, true, make_float4(0.f, 0.f, 0.f, __int_as_float(g.el[a])), g.mol[a], ela * D.ne, g.mol[b],
                f0, f1, half, b0, b1, elj);
}

// One +-1 on the shared element-pair delta at (pair row idx - b, bin b), and
// the bin's count of non-zero deltas kept exact: the thread that moves a delta
// away from zero adds one, the thread that brings it back removes one.
__device__ __forceinline__ void delta_add(int *sdP, int *nz, int idx, int b, int v, int dpk)
{
    int old;
    if (dpk) {
        // delta idx is the half (idx & 1) of word idx >> 1, stored + 32768, so
        // adding v << 16 or v never carries or borrows across the halves
        const unsigned sh = (unsigned)(idx & 1) << 4;
        const unsigned w = atomicAdd(reinterpret_cast<unsigned *>(sdP) + (idx >> 1), (unsigned)v << sh);
        old = (int)((w >> sh) & 0xffffu) - 32768;
    } else {
        old = atomicAdd(sdP + idx, v);
    }
    if (old == 0)
        atomicAdd(nz + b, 1);
    else if (old + v == 0)
        atomicSub(nz + b, 1);
}

// The fused path's share of the group's internal pairs (shared-memory deltas).
template <int BM>
__device__ void fused_group_internal(const EDesc &Dg, int *sdP, int *nz, unsigned *s_tcount, const MovedGroup &g,
                                     const int *pidx)
{
    ColView D = col_view(Dg);
    D.pidx = pidx;
    const int npair = g.n * (g.n - 1) / 2;
    for (int t = threadIdx.x; t < npair; t += blockDim.x) {
        int f0, f1, half, b0, b1, ela, elj;
        group_pair_bins<BM>(D, g, t, f0, f1, half, b0, b1, ela, elj);
        const unsigned cnt = (f0 >= 0) + (f1 >= 0);
        if (!cnt)
            continue;
        unsigned pos = atomicAdd(s_tcount, cnt);
        if (f0 >= 0) {
            D.tlist[pos++] = (half + f0) << 1;
            int p, bb;
            pair_of_flat(D, f0, ela, elj, b0, p, bb);
            if (p >= 0)
                delta_add(sdP, nz, p * D.hs + bb, bb, -1, D.dpk);
        }
        if (f1 >= 0) {
            D.tlist[pos] = ((half + f1) << 1) | 1;
            int p, bb;
            pair_of_flat(D, f1, ela, elj, b1, p, bb);
            if (p >= 0)
                delta_add(sdP, nz, p * D.hs + bb, bb, 1, D.dpk);
        }
    }
}

// The split path's share (global deltas; run by the CTA that evaluates).
template <int BM>
__device__ void split_group_internal(const EDesc &Dg, const MovedGroup &g)
{
    const ColView D = col_view(Dg);
    const int npair = g.n * (g.n - 1) / 2;
    for (int t = threadIdx.x; t < npair; t += blockDim.x) {
        int f0, f1, half, b0, b1, ela, elj;
        group_pair_bins<BM>(D, g, t, f0, f1, half, b0, b1, ela, elj);
        const unsigned cnt = (f0 >= 0) + (f1 >= 0);
        if (!cnt)
            continue;
        unsigned pos = atomicAdd(&Dg.st->tcount, cnt);
        if (f0 >= 0) {
            atomicSub(Dg.delta + half + f0, 1);
            D.tlist[pos++] = half + f0;
            int p, bb;
            pair_of_flat(D, f0, ela, elj, b0, p, bb);
            if (p >= 0)
                atomicSub(Dg.dP + p * D.hs + bb, 1);
        }
        if (f1 >= 0) {
            atomicAdd(Dg.delta + half + f1, 1);
            D.tlist[pos] = half + f1;
            int p, bb;
            pair_of_flat(D, f1, ela, elj, b1, p, bb);
            if (p >= 0)
                atomicAdd(Dg.dP + p * D.hs + bb, 1);
        }
    }
}

constexpr int kCommitUnroll = 4;

__device__ void finish_engine(const EDesc &D, const MovedGroup &g, double *red, double *cb, double *sbs, int *sbin,
                              int *s_nchg, double *coef, int *s_flag)
{
    if (g.n > 1) {
        switch (D.bm) {
        case BM_IBC: split_group_internal<BM_IBC>(D, g); break;
        case BM_DIAG: split_group_internal<BM_DIAG>(D, g); break;
        case BM_XYTRI: split_group_internal<BM_XYTRI>(D, g); break;
        case BM_LOWER: split_group_internal<BM_LOWER>(D, g); break;
        default: split_group_internal<BM_GENERAL>(D, g); break;
        }
        __syncthreads();
    }
    double dsd = eval_delta<false>(D, D.dP, D.A, D.Bq, red, cb, sbs, sbin, s_nchg, coef, nullptr);
    __shared__ double s_sf;
    double sd_dense = 0.0;
    if (D.dense) {
        // the whole model: scale factor (fitted when due) and window
        const EState &S0 = *D.st;
        const bool fit = D.fit_freq > 0 && S0.accepted % D.fit_freq == 0;
        sd_dense = eval_dense(D, red, cb, true, fit, S0.sf, &s_sf);
        dsd = sd_dense - S0.sd;
        __syncthreads();
    }
    if (D.sq) {
        // the S(Q) kernel evaluates its term, decides and commits
        if (threadIdx.x == 0) {
            EState &S = *D.st;
            S.dsd = dsd;
            S.fmt = 0;
            S.done = 0u;
            if (D.dense)
                S.sf_prop = s_sf;
        }
        return;
    }
    const EState &S0 = *D.st;
    double sd_new = 0.0, chi2_new = 0.0;  // thread 0's
    if (threadIdx.x == 0) {
        sd_new = D.dense ? sd_dense : S0.sd + dsd;
        chi2_new = sd_new / D.var2;
        const EMove &m = D.moves[S0.step % D.move_cap];
        const bool reject = (chi2_new > S0.chi2) && (m.u > D.tol);
        *s_flag = reject ? 0 : 1;
    }
    __syncthreads();
    const bool accept = *s_flag != 0;
    // commit (or drop) the oriented delta through the touched list; duplicates
    // are harmless: atomicExch hands each bin's delta to exactly one entry
    const unsigned nt = __ldcg(&D.st->tcount);
    for (unsigned k0 = threadIdx.x; k0 < nt; k0 += kCommitUnroll * blockDim.x) {
        int f[kCommitUnroll], d[kCommitUnroll];
#pragma unroll
        for (int u = 0; u < kCommitUnroll; ++u) {
            const unsigned k = k0 + u * blockDim.x;
            f[u] = k < nt ? __ldcg(D.tlist + k) : -1;
        }
#pragma unroll
        for (int u = 0; u < kCommitUnroll; ++u) d[u] = f[u] >= 0 ? atomicExch(D.delta + f[u], 0) : 0;
        if (accept) {
#pragma unroll
            for (int u = 0; u < kCommitUnroll; ++u)
                if (d[u]) D.counts[f[u]] += d[u];
        }
    }
    // on accept G += R S, hence Bq -= 2 A S on the bins that changed
    if (accept) {
        if (D.hs > kChunk) {
            for (int b = threadIdx.x; b < D.hs; b += blockDim.x) {
                const double S = D.Sb[b];
                if (S != 0.0)
                    D.Bq[b] = fma(-2.0 * D.A[b], S, D.Bq[b]);
            }
        } else {
            const int n = *s_nchg;
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                const int b = sbin[k];
                D.Bq[b] = fma(D.A[b], sbs[k], D.Bq[b]);
            }
        }
    }
    if (accept) {
        commit_moved_group(D, g);
        if (D.dense)
            dense_commit(D);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        EState &S = *D.st;
        EResult &r = D.results[S.step % D.move_cap];
        r.chi2_new = chi2_new;
        r.accepted = accept ? 1 : 0;
        r.atom = g.atom[0];
        if (accept) {
            S.chi2 = chi2_new;
            S.sd = sd_new;
            S.accepted += 1;
            if (D.dense)
                S.sf = s_sf;
        }
        S.step += 1;
        S.done = 0u;
        S.tcount = 0u;
    }
}

// Fused path: one CTA advances one engine by one step.  The element-pair
// deltas live in this CTA's shared memory (sdP: npairs * hs ints, or biased
// 16-bit halves of words), changes are listed as (oriented bin, sign) in the
// engine's touched list, and an accepted move is committed with
// fire-and-forget atomics on the counts.  No other CTA touches the engine
// during the step, so there is no cross-CTA hand-off.
// Columns of the fused path.  Batches of kItemUnroll * blockDim columns are
// software-pipelined: the next batch's coordinates are loaded before the
// current batch's squared distances are taken against each moved atom; the
// columns in range go to a per-thread queue that whole warps bin.  Columns
// that belong to the moved group are left to group_internal (fullrmc's M - F).
// Per-thread queue of accepted columns in the fused path: kColQueue entries
// per thread, entry k of thread t at [k * blockDim + t] (conflict-free).
constexpr int kColQueue = 8;
constexpr int kMaxEngineThreads = 512;  // CTA size limit of the step kernels (128 registers per thread)
// Touched-list entries per thread of the one-CTA step read ahead of the
// decision (a single-atom move touches at most 2 n + 8 oriented bins).
constexpr int kTouchAhead = 8;
// The one-CTA step keeps the column grid's prefix and bases, the warps'
// packed queue lists and the element-pair index table in the evaluation
// scratch cb until the evaluation: ints at [0, kCellInts), the lists, then
// kPidxSmem ints.
constexpr int kCellInts = 2 * kMaxCells + 34, kPidxSmem = 256;
__host__ __device__ constexpr int list_ints(int threads) { return 32 * kColQueue * (threads / 32) / 2; }
// Doubles of the one-CTA step's evaluation scratch cb (and bins of sbs /
// sbin): the changed bins of one chunk, at least the cell, list and table
// ints above.
__host__ __device__ constexpr int fused_bins_cap(int fused_bins) { return fused_bins < kChunk ? fused_bins : kChunk; }
__host__ __device__ constexpr int fused_cb_cap(int fused_bins, int threads)
{
    return fused_bins_cap(fused_bins) > (kCellInts + list_ints(threads) + kPidxSmem + 1) / 2
               ? fused_bins_cap(fused_bins)
               : (kCellInts + list_ints(threads) + kPidxSmem + 1) / 2;
}

struct ColQueue {
    float2 *s;        // squared distances before (x) / after (y) the move
    unsigned *info;   // el(j) | same molecule << 8 | accepted before << 9 | after << 10 | group atom << 11
    int *nz;          // per bin: element pairs whose delta is non-zero
    unsigned short *list;  // per warp: 32 * kColQueue queue indexes, the warp's entries packed
};

// Bins the queued columns of a warp: the lanes' entries are packed into one
// list (a warp scan of the queue lengths), and each pass bins 32 of them, so
// the IEEE sqrt / division and the delta atomics run with full warps however
// unevenly the entries fell on the lanes.
__device__ __forceinline__ void flush_columns(const ColView &D, const MovedGroup &g, int *sdP, int *nz,
                                              unsigned *s_tcount, const ColQueue &q, int &qn)
{
    const unsigned lane = threadIdx.x & 31u;
    unsigned short *lst = q.list + (threadIdx.x >> 5) * (32 * kColQueue);
    int inc = qn;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, o);
        if ((int)lane >= o)
            inc += v;
    }
    const int total = __shfl_sync(0xffffffffu, inc, 31);
    const int ex = inc - qn;
    for (int j = 0; j < qn; ++j) lst[ex + j] = (unsigned short)(j * (int)blockDim.x + (int)threadIdx.x);
    qn = 0;
    __syncwarp();
    for (int e = (int)lane; e < total; e += 32) {
        const int k = lst[e];
        const float2 sk = q.s[k];
        const float s0 = sk.x, s1 = sk.y;
        const unsigned info = q.info[k];
        const int elj = (int)(info & 0xffu);
        const int gi = (int)(info >> 11);
        const int ela = g.el[gi];
        const long long half = (info >> 8) & 1u ? 0 : D.total;
        const long long rowb = (long long)(ela * D.ne + elj) * D.hs;
        int f0 = -1, f1 = -1, b0 = 0, b1 = 0;
        if ((info >> 9) & 1u) {
            b0 = pair_bin(s0, D.minD, D.binw);
            const long long f = rowb + b0;
            if ((unsigned long long)f < (unsigned long long)D.total) f0 = (int)f;
        }
        if ((info >> 10) & 1u) {
            b1 = pair_bin(s1, D.minD, D.binw);
            const long long f = rowb + b1;
            if ((unsigned long long)f < (unsigned long long)D.total) f1 = (int)f;
        }
        if (f0 != f1) {
            unsigned pos = atomicAdd(s_tcount, (unsigned)((f0 >= 0) + (f1 >= 0)));
            if (f0 >= 0) {
                D.tlist[pos++] = (int)((half + f0) << 1);
                int p, bb;
                pair_of_flat(D, f0, ela, elj, b0, p, bb);
                if (p >= 0)
                    delta_add(sdP, nz, p * D.hs + bb, bb, -1, D.dpk);
            }
            if (f1 >= 0) {
                D.tlist[pos] = (int)(((half + f1) << 1) | 1);
                int p, bb;
                pair_of_flat(D, f1, ela, elj, b1, p, bb);
                if (p >= 0)
                    delta_add(sdP, nz, p * D.hs + bb, bb, 1, D.dpk);
            }
        }
    }
    __syncwarp();  // the list and the queue slots are refilled after this
}

// Gap m >= 0 between the ranges [a, b] of coordinate differences and the
// nearest difference the distance can reach: the nearest integer with
// periodic boundaries (the minimum image subtracts round(diff)), zero with
// free boundaries.
__device__ __forceinline__ float cell_gap(float a, float b, int pbc)
{
    if (!pbc)
        return a > 0.f ? a : (b < 0.f ? -b : 0.f);
    const float n = floorf(b);
    return n >= a ? 0.f : fminf(a - n, n + 1.f - b);
}

// The cells of the column grid that a moved atom may reach: for each cell,
// a lower bound of the distance from the bounding box of the moved atoms'
// positions (before and after the move) to the cell's box; a cell whose
// bound is not below maxD + margin holds only columns out of range before
// and after the move, which change no bin.  lo, hi, st0, st1: cell
// threadIdx.x's bounds and start positions, loaded by the caller ahead of
// the barrier.  Writes P[c], the exclusive prefix of the selected cells'
// atom counts (P[nc] = the total), and Bse[c] = cstart[c] - P[c] (wsum: 32
// ints of scratch); returns the number of columns to sweep.  Column v of the sweep is atom
// Bse[c] + v of the cell order, c the last cell with P[c] <= v.
__device__ int cell_select(const EDesc &D, const MovedGroup &g, float4 lo, float4 hi, int st0, int st1, int *P,
                           int *Bse, int *wsum, float4 lo1, float4 hi1, int st01, int st11, float4 *cb0)
{
    float plo[3], phi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        plo[k] = fminf(g.o[0][k], g.nw[0][k]);
        phi[k] = fmaxf(g.o[0][k], g.nw[0][k]);
    }
    for (int t = 1; t < g.n; ++t)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            plo[k] = fminf(plo[k], fminf(g.o[t][k], g.nw[t][k]));
            phi[k] = fmaxf(phi[k], fmaxf(g.o[t][k], g.nw[t][k]));
        }
    const int nc = D.nc;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int carry = 0;
    for (int c0 = 0; c0 < nc; c0 += blockDim.x) {
        const int c = c0 + (int)threadIdx.x;
        if (c0 == (int)blockDim.x) {
            // the second round's cell, read by the caller ahead of the barrier
            lo = lo1;
            hi = hi1;
            st0 = st01;
            st1 = st11;
        } else if (c0 > 0 && c < nc) {
            lo = D.clo[c];
            hi = D.chi[c];
            st0 = D.cstart[c];
            st1 = D.cstart[c + 1];
        }
        if (c < nc && c == g.cell[0]) {
            // the moved atom's cell: its bounds for the commit
            cb0[0] = lo;
            cb0[1] = hi;
        }
        int take = 0;
        if (c < nc && st1 > st0) {
            const float f0 = cell_gap(plo[0] - hi.x, phi[0] - lo.x, D.cpbc);
            const float f1 = cell_gap(plo[1] - hi.y, phi[1] - lo.y, D.cpbc);
            const float f2 = cell_gap(plo[2] - hi.z, phi[2] - lo.z, D.cpbc);
            const float m0 = f0 * D.cw[0], m1 = f1 * D.cw[1], m2 = f2 * D.cw[2];
            float lb2 = m0 * m0 + m1 * m1 + m2 * m2;
            if (D.cmode != 0)
                lb2 = fmaxf(fmaxf(m0 * m0, m1 * m1), fmaxf(m2 * m2, D.clam2 * (f0 * f0 + f1 * f1 + f2 * f2)));
            take = lb2 < D.cthr2 ? st1 - st0 : 0;
        }
        // exclusive scan of the selected counts: warps by shuffles, then
        // every thread adds the totals of the warps before its own
        int inc = take;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, inc, o);
            if ((int)lane >= o)
                inc += v;
        }
        if (lane == 31)
            wsum[warp] = inc;
        __syncthreads();
        int before = carry, total = 0;
        for (unsigned w = 0; w < nw; ++w) {
            const int x = wsum[w];
            before += w < warp ? x : 0;
            total += x;
        }
        if (c < nc) {
            const int ex = before + inc - take;
            P[c] = ex;
            Bse[c] = st0 - ex;
        }
        carry += total;
        if (threadIdx.x == 0 && c0 + (int)blockDim.x >= nc)
            P[nc] = carry;
        __syncthreads();
    }
    return carry;
}

// Position in cell order of sweep column v (P[lo] <= v < P[lo + 1]).
__device__ __forceinline__ int cell_column(const int *P, const int *Bse, int nc, int v)
{
    int lo = 0, hi = nc;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (P[mid] <= v)
            lo = mid;
        else
            hi = mid;
    }
    return Bse[lo] + v;
}

// The fused path's columns: every column j (not a moved atom) against every
// moved atom before and after the move.  Squared distances and the window
// test are branch-free for a batch of columns; accepted columns go to the
// thread's queue, flushed when a queue is full and at the end.
//
// With a column grid (CELL) the sweep runs over the ncol columns of the
// selected cells in cell order (cell_select, cell_column): the copies cbox /
// cmol, and the moved atoms recognised by their cell-order positions.
template <int BM, bool GROUP, bool CELL>
__device__ void fused_columns(const EDesc &Dg, int *sdP, int *nz, unsigned *s_tcount, const MovedGroup &g,
                              const ColQueue &q, int ncol, const int *cP, const int *cB, const int *pidx)
{
    ColView D = col_view(Dg);
    D.pidx = pidx;
    if (CELL) {
        D.box = Dg.cbox;
        D.mol = Dg.cmol;
    }
    const int nc = Dg.nc;
    const int step = kItemUnroll * blockDim.x;
    const int G = GROUP ? g.n : 1;
    const int self0 = CELL ? g.slot[0] : g.atom[0];
    const int mola0 = g.mol[0];
    int qn = 0;
    // a batch: coordinates, molecules (a single atom compares them once, into
    // the bits of `same`, after the next batch's loads are issued) and the
    // bits of `vmask` (column u exists and is not a moved atom): bit masks
    // leave registers to the batch in flight and the flushes
    float4 c[kItemUnroll];
    int mj[kItemUnroll];
    unsigned vmask = 0u, same = 0u;
#pragma unroll
    for (int u = 0; u < kItemUnroll; ++u) {
        const int v = u * blockDim.x + threadIdx.x;
        const int j = v < ncol ? (CELL ? cell_column(cP, cB, nc, v) : v) : -1;
        bool ok = j >= 0 && j != self0;
        if (GROUP)
            for (int t = 1; t < G; ++t) ok &= j != (CELL ? g.slot[t] : g.atom[t]);
        vmask |= (ok ? 1u : 0u) << u;
        c[u] = j >= 0 ? D.box[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        mj[u] = j >= 0 ? D.mol[j] : 0;
    }
    for (int jb = 0; jb < ncol; jb += step) {
        float4 cn[kItemUnroll];
        int mn[kItemUnroll];
        unsigned vmaskn = 0u;
#pragma unroll
        for (int u = 0; u < kItemUnroll; ++u) {
            const int v = jb + step + u * blockDim.x + threadIdx.x;
            const int j = v < ncol ? (CELL ? cell_column(cP, cB, nc, v) : v) : -1;
            bool ok = j >= 0 && j != self0;
            if (GROUP)
                for (int t = 1; t < G; ++t) ok &= j != (CELL ? g.slot[t] : g.atom[t]);
            vmaskn |= (ok ? 1u : 0u) << u;
            cn[u] = j >= 0 ? D.box[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            mn[u] = j >= 0 ? D.mol[j] : 0;
        }
        if (!GROUP) {
            // (after the next batch's loads are issued)
            same = 0u;
#pragma unroll
            for (int u = 0; u < kItemUnroll; ++u) same |= (mj[u] == mola0 ? 1u : 0u) << u;
        }
        for (int gi = 0; gi < G; ++gi) {
            if (__any_sync(0xffffffffu, qn > kColQueue - kItemUnroll))
                flush_columns(D, g, sdP, nz, s_tcount, q, qn);
            const float3 o = make_float3(g.o[gi][0], g.o[gi][1], g.o[gi][2]);
            const float3 nw = make_float3(g.nw[gi][0], g.nw[gi][1], g.nw[gi][2]);
            const int mola = g.mol[gi];
#pragma unroll
            for (int u = 0; u < kItemUnroll; ++u) {
                const bool valid = (vmask >> u) & 1u;
                const float s0 = pair_s<BM>(o.x, o.y, o.z, c[u].x, c[u].y, c[u].z, D.B);
                const float s1 = pair_s<BM>(nw.x, nw.y, nw.z, c[u].x, c[u].y, c[u].z, D.B);
                const bool a0 = valid & (s0 >= D.s_lo) & (s0 < D.s_hi);
                const bool a1 = valid & (s1 >= D.s_lo) & (s1 < D.s_hi);
                const unsigned sm = GROUP ? (mj[u] == mola ? 1u : 0u) : ((same >> u) & 1u);
                const int k = qn * (int)blockDim.x + (int)threadIdx.x;
                q.s[k] = make_float2(s0, s1);
                q.info[k] = ((unsigned)__float_as_int(c[u].w) & 0xffu) | (sm << 8) | ((a0 ? 1u : 0u) << 9) |
                            ((a1 ? 1u : 0u) << 10) | ((unsigned)gi << 11);
                qn += (a0 | a1) ? 1 : 0;
            }
        }
        vmask = vmaskn;
#pragma unroll
        for (int u = 0; u < kItemUnroll; ++u) {
            c[u] = cn[u];
            mj[u] = mn[u];
        }
    }
    flush_columns(D, g, sdP, nz, s_tcount, q, qn);
}

// sA, sBq: shared-memory copies of A and Bq, brought in by bulk copies on
// `bar` while the columns run; parity = this CTA's count of fused items mod 2.
__device__ void engine_fused(const EDesc &D, int *sdP, double *sA, double *sBq, uint64_t *bar, uint32_t parity,
                             uint32_t *status, double *red, double *cb, double *sbs, int *sbin, int *s_nchg,
                             double *coef, int *s_flag, unsigned *s_tcount, MovedGroup &g, const ColQueue &q0,
                             const EMove *hm, EResult *hr)
{
    // the column grid's prefix and bases, the warps' packed queue lists and
    // the element-pair index table (binning reads it per pair) live in cb
    // until the evaluation
    static_assert(sizeof(double) * kChunk >= sizeof(int) * (kCellInts + list_ints(kMaxEngineThreads) + kPidxSmem),
                  "cb too small");
    int *cP = reinterpret_cast<int *>(cb), *cB = cP + kMaxCells + 1;
    ColQueue q = q0;
    q.list = reinterpret_cast<unsigned short *>(cP + kCellInts);
    int *spidx = cP + kCellInts + list_ints(blockDim.x);
    const int nee = D.ne * D.ne;
    const int *pidx = nee <= kPidxSmem ? spidx : D.pidx;
    if (nee <= kPidxSmem)
        for (int k = threadIdx.x; k < nee; k += blockDim.x) spidx[k] = D.pidx[k];
    if (threadIdx.x == 0) {
        // the previous item's reads of sA / sBq are ordered before this
        // item's bulk copies by the barrier at the item boundary
        const uint32_t bytes = (uint32_t)((8 * D.hs + 15) & ~15);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, 2 * bytes);
        bulk_g2s(sA, D.A, bytes, bar);
        bulk_g2s(sBq, D.Bq, bytes, bar);
        *s_tcount = 0u;
    }
    // this thread's cell of the column grid, read ahead of the barrier
    const int nc = D.nc;
    float4 clo = make_float4(0.f, 0.f, 0.f, 0.f), chi = clo;
    int cs0 = 0, cs1 = 0;
    if ((int)threadIdx.x < nc) {
        clo = D.clo[threadIdx.x];
        chi = D.chi[threadIdx.x];
        cs0 = D.cstart[threadIdx.x];
        cs1 = D.cstart[threadIdx.x + 1];
    }
    // and its cell of the second round (grids of up to 2 blockDim cells)
    float4 clo1 = make_float4(0.f, 0.f, 0.f, 0.f), chi1 = clo1;
    int cs01 = 0, cs11 = 0;
    if ((int)(threadIdx.x + blockDim.x) < nc) {
        const int c = threadIdx.x + blockDim.x;
        clo1 = D.clo[c];
        chi1 = D.chi[c];
        cs01 = D.cstart[c];
        cs11 = D.cstart[c + 1];
    }
    load_moved_group(D, D.st->step, g, hm);
    // the next step's move: its ring entry now, the moved atom's data after
    // the sweep, into the state at the commit (single-atom engines whose step
    // ends here and whose moves come from the ring); the ring's generation is
    // read before the entry
    __shared__ __align__(16) struct {
        float4 box, real;
        long long step;
        unsigned gen;
        int atom, mol;
        float v[3], u;
        int2 csl;
    } s_next;
    const bool stage_next = !hm && D.group == 1 && !D.sq;
    if (stage_next && threadIdx.x == 64) {
        const unsigned gen = ld_acquire_u32(&D.st->gen);
        const long long s1 = __ldcg(&D.st->step) + 1;
        const EMove *m = D.moves + s1 % D.move_cap;
        cp_async4(&s_next.atom, &m->atom);
        cp_async4(&s_next.v[0], &m->v[0]);
        cp_async4(&s_next.v[1], &m->v[1]);
        cp_async4(&s_next.v[2], &m->v[2]);
        cp_async4(&s_next.u, &m->u);
        cp_async_commit();
        s_next.step = s1;
        s_next.gen = gen;
    }
    const int np = D.npairs;
    const int nph = np * D.hs;
    if (D.dpk) {
        const int words = (nph + 1) >> 1;
        for (int k = threadIdx.x; k < words; k += blockDim.x) sdP[k] = (int)0x80008000u;
    } else {
        for (int k = threadIdx.x; k < nph; k += blockDim.x) sdP[k] = 0;
    }
    for (int k = threadIdx.x; k < D.hs; k += blockDim.x) q.nz[k] = 0;
    for (int qq = threadIdx.x; qq < np; qq += blockDim.x) coef[qq] = D.pc[qq];
    __syncthreads();
    __shared__ float4 s_cb[2];  // the moved atom's cell bounds (grids), for the commit
    const int ncol = nc > 0 ? cell_select(D, g, clo, chi, cs0, cs1, cP, cB, cB + kMaxCells, clo1, chi1, cs01, cs11, s_cb) : D.n;
    if (threadIdx.x == 0)
        atomicAdd(&D.st->swept, (unsigned long long)ncol);
#define FRMC_COLUMNS(G_, C_)                                                                           \
    switch (D.bm) {                                                                                    \
    case BM_IBC: fused_columns<BM_IBC, G_, C_>(D, sdP, q.nz, s_tcount, g, q, ncol, cP, cB, pidx); break;     \
    case BM_DIAG: fused_columns<BM_DIAG, G_, C_>(D, sdP, q.nz, s_tcount, g, q, ncol, cP, cB, pidx); break;   \
    case BM_XYTRI: fused_columns<BM_XYTRI, G_, C_>(D, sdP, q.nz, s_tcount, g, q, ncol, cP, cB, pidx); break; \
    case BM_LOWER: fused_columns<BM_LOWER, G_, C_>(D, sdP, q.nz, s_tcount, g, q, ncol, cP, cB, pidx); break; \
    default: fused_columns<BM_GENERAL, G_, C_>(D, sdP, q.nz, s_tcount, g, q, ncol, cP, cB, pidx); break;     \
    }
    if (g.n == 1) {
        if (nc > 0) {
            FRMC_COLUMNS(false, true)
        } else {
            FRMC_COLUMNS(false, false)
        }
    } else {
        if (nc > 0) {
            FRMC_COLUMNS(true, true)
        } else {
            FRMC_COLUMNS(true, false)
        }
    }
#undef FRMC_COLUMNS
    if (g.n > 1) {
        switch (D.bm) {
        case BM_IBC: fused_group_internal<BM_IBC>(D, sdP, q.nz, s_tcount, g, pidx); break;
        case BM_DIAG: fused_group_internal<BM_DIAG>(D, sdP, q.nz, s_tcount, g, pidx); break;
        case BM_XYTRI: fused_group_internal<BM_XYTRI>(D, sdP, q.nz, s_tcount, g, pidx); break;
        case BM_LOWER: fused_group_internal<BM_LOWER>(D, sdP, q.nz, s_tcount, g, pidx); break;
        default: fused_group_internal<BM_GENERAL>(D, sdP, q.nz, s_tcount, g, pidx); break;
        }
    }
    __syncthreads();
    if (stage_next && threadIdx.x == 64) {
        cp_async_wait_all();
        const int a = s_next.atom;
        if (a >= 0 && a < D.n) {
            cp_async16(&s_next.box, D.box + a);
            cp_async16(&s_next.real, D.real + a);
            cp_async4(&s_next.mol, D.mol + a);
            if (D.nc > 0)
                cp_async8(&s_next.csl, D.csl + a);
            cp_async_commit();
        } else {
            s_next.step = -1;  // an entry never pushed: nothing to stage
        }
    }
    mbar_wait(bar, parity, status);
    const double dsd = eval_delta<true>(D, sdP, sA, sBq, red, cb, sbs, sbin, s_nchg, coef, q.nz);
    if (D.sq) {
        // the S(Q) kernel evaluates its term, decides and commits
        if (threadIdx.x == 0) {
            EState &S = *D.st;
            S.dsd = dsd;
            S.tcount = *s_tcount;
            S.fmt = 1;
        }
        return;
    }
    // the touched list's first kTouchAhead entries per thread are read (an L2
    // round trip) while thread 0 decides
    const unsigned nt = *s_tcount;
    const int *__restrict__ tl = D.tlist;
    int ta[kTouchAhead];
#pragma unroll
    for (int u = 0; u < kTouchAhead; ++u) {
        const unsigned k = threadIdx.x + u * blockDim.x;
        ta[u] = k < nt ? __ldcg(tl + k) : -1;
    }
    // the state and the move's uniform number were read at set-up; thread 0
    // alone forms the new chi2 (FP64 division) and decides
    double sd_new = 0.0, chi2_new = 0.0;
    if (threadIdx.x == 0) {
        sd_new = g.sd + dsd;
        chi2_new = sd_new / D.var2;
        const bool reject = (chi2_new > g.chi2) && (g.u > D.tol);
        *s_flag = reject ? 0 : 1;
    }
    __syncthreads();
    const bool accept = *s_flag != 0;
    if (accept) {
        int *__restrict__ cnt = D.counts;
#pragma unroll
        for (int u = 0; u < kTouchAhead; ++u)
            if (ta[u] >= 0)
                atomicAdd(cnt + (ta[u] >> 1), (ta[u] & 1) ? 1 : -1);
        // the rest (group moves), four entries' loads in flight before their atomics
        for (unsigned k0 = threadIdx.x + kTouchAhead * blockDim.x; k0 < nt; k0 += 4 * blockDim.x) {
            int e[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const unsigned k = k0 + u * blockDim.x;
                e[u] = k < nt ? __ldcg(tl + k) : -1;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (e[u] >= 0)
                    atomicAdd(cnt + (e[u] >> 1), (e[u] & 1) ? 1 : -1);
        }
        double *__restrict__ Bq = D.Bq;
        if (D.hs > kChunk) {
            const double *__restrict__ Sb = D.Sb;
            for (int b = threadIdx.x; b < D.hs; b += blockDim.x) {
                const double Sv = Sb[b];
                if (Sv != 0.0)
                    Bq[b] = fma(-2.0 * sA[b], Sv, sBq[b]);
            }
        } else {
            const int n = *s_nchg;
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                const int b = sbin[k];
                Bq[b] = fma(sA[b], sbs[k], sBq[b]);
            }
        }
        commit_moved_group(D, g, (nc > 0 && g.n == 1) ? s_cb : nullptr);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        EState &S = *D.st;
        EResult &r = D.results[g.step % D.move_cap];
        r.chi2_new = chi2_new;
        r.accepted = accept ? 1 : 0;
        r.atom = g.atom[0];
        if (hr)
            *hr = r;
        if (accept) {
            S.chi2 = chi2_new;
            S.sd = sd_new;
            S.accepted = g.accepted + 1;
        }
        S.step = g.step + 1;
    }
    if (stage_next && threadIdx.x == 64 && s_next.step >= 0) {
        cp_async_wait_all();
        EState &S = *D.st;
        float4 nb = s_next.box, nr = s_next.real;
        if (accept && s_next.atom == g.atom[0]) {
            // this step moved the same atom: its coordinates as just committed
            nb = make_float4(g.nw[0][0], g.nw[0][1], g.nw[0][2], __int_as_float(g.el[0]));
            nr = make_float4(g.nr[0][0], g.nr[0][1], g.nr[0][2], 0.0f);
        }
        S.nx_atom = s_next.atom;
        S.nx_v[0] = s_next.v[0];
        S.nx_v[1] = s_next.v[1];
        S.nx_v[2] = s_next.v[2];
        S.nx_u = s_next.u;
        S.nx_mol = s_next.mol;
        S.nx_csl = s_next.csl;
        S.nx_box = nb;
        S.nx_real = nr;
        S.nx_gen = s_next.gen;
        S.nx_step = s_next.step;
    }
}

// Warms L2 for a fused item this CTA will probably take later (one grid
// stride ahead): its descriptor, state, move and the moved atom's lines.  Run
// by one thread of the second warp while thread 0 walks the same chain for the
// CTA's current item, so a later item starts from L2 instead of HBM.
__device__ void warm_item(const StepParams &p, long long idx)
{
    if (idx >= p.nitems)
        return;
    const EDesc &D = p.fdesc[idx];
    const long long stp = D.st->step;
    const long long slot = stp % D.move_cap;
    const int a = p.hmoves ? p.hmoves[p.fpos[idx]].atom : D.moves[slot].atom;
    prefetch_l2(D.box + a);
    prefetch_l2(D.real + a);
    prefetch_l2(D.mol + a);
    if (D.group > 1)
        prefetch_l2(D.groups + slot);
    prefetch_l2(D.A);
    prefetch_l2(D.Bq);
}


template <bool FUSED>
__global__ void __launch_bounds__(kMaxEngineThreads, 1) k_engine_step(StepParams p)
{
    __shared__ double red[kRedLanes];
    // the evaluation scratch: static for tile-split steps, in the dynamic
    // layout (sized by the launch's bins) for one-CTA steps
    __shared__ double cb_s[FUSED ? 1 : kChunk];
    __shared__ double sbs_s[FUSED ? 1 : kChunk];
    __shared__ int sbin_s[FUSED ? 1 : kChunk];
    double *cb = cb_s, *sbs = sbs_s;
    int *sbin = sbin_s;
    __shared__ int s_nchg;
    __shared__ double coef[64];
    __shared__ MovedGroup s_group;
    __shared__ unsigned s_tcount;
    __shared__ int s_last, s_flag, s_item;
    __shared__ __align__(8) uint64_t s_bar;
    // fused items read their descriptor from this copy: the sweep streams the
    // engine's columns through L1, which would otherwise evict the descriptor
    // and turn every later field read into an L2 round trip
    __shared__ __align__(16) EDesc s_desc;
    static_assert(sizeof(EDesc) % 8 == 0, "the descriptor is copied in 8-byte words");
    extern __shared__ __align__(16) int sdP[];
    (void)sdP;
    uint32_t fused_items = 0;
    double *sA = nullptr, *sBq = nullptr;
    ColQueue cq{};
    if (FUSED) {
        // dynamic layout: element-pair deltas, then A and Bq (16-byte aligned)
        sA = reinterpret_cast<double *>(sdP + p.fused_dp_ints);
        sBq = sA + p.fused_bins;
        cq.s = reinterpret_cast<float2 *>(sBq + p.fused_bins);  // 8-byte aligned
        cq.info = reinterpret_cast<unsigned *>(cq.s + kColQueue * blockDim.x);
        cq.nz = reinterpret_cast<int *>(cq.info + kColQueue * blockDim.x);
        cb = reinterpret_cast<double *>(cq.nz + p.fused_bins);  // fused_bins is even: 8-byte aligned
        sbs = cb + fused_cb_cap(p.fused_bins, blockDim.x);
        sbin = reinterpret_cast<int *>(sbs + fused_bins_cap(p.fused_bins));
        if (threadIdx.x == 0) {
            mbar_init(&s_bar, 1);
            mbar_fence_init();
        }
        __syncthreads();
    }
    // a fused launch with an item per CTA needs no scheduler: CTA b takes
    // item b and leaves
    const bool one_each = FUSED && p.nitems <= (int)gridDim.x;
    for (;;) {
        if (threadIdx.x == 0) {
            // fused launches: item blockIdx.x first (the list is largest
            // first), then items gridDim.x, gridDim.x + 1, ... by claim
            unsigned long long k;
            if (FUSED)
                k = fused_items == 0 ? blockIdx.x
                                     : (one_each ? (unsigned long long)p.nitems
                                                 : gridDim.x + atomicAdd(&p.sched->claimed, 1ull));
            else
                k = atomicAdd(&p.sched->claimed, 1ull);
            s_item = k < (unsigned long long)p.nitems ? (int)k : -1;
        }
        __syncthreads();
        const int it = s_item;
        if (FUSED && it >= 0) {
            // the previous item's last reads of s_desc came before the
            // barrier that ended it
            const long long *src = reinterpret_cast<const long long *>(p.fdesc + it);
            long long *dst = reinterpret_cast<long long *>(&s_desc);
            for (int k = threadIdx.x; k < (int)(sizeof(EDesc) / 8); k += blockDim.x) dst[k] = src[k];
        }
        __syncthreads();
        if (it < 0)
            break;
        const int2 item = FUSED ? make_int2(0, -1) : p.items[it];
        const EDesc &D = FUSED ? p.fdesc[it] : p.desc[item.x];
        if (FUSED && fused_items == 0 && threadIdx.x == 32)
            warm_item(p, (long long)it + gridDim.x);
        if (FUSED) {
            __shared__ unsigned long long s_titem;  // the item's start (placement record)
            if (p.place && threadIdx.x == 0)
                s_titem = global_ns();
            const int hp = p.hmoves ? p.fpos[it] : 0;
            engine_fused(s_desc, sdP, sA, sBq, &s_bar, fused_items & 1u, &p.sched->status, red, cb, sbs, sbin, &s_nchg,
                         coef, &s_flag, &s_tcount, s_group, cq, p.hmoves ? p.hmoves + hp : nullptr,
                         p.hres ? p.hres + hp : nullptr);
            ++fused_items;
            __syncthreads();
            if (p.place && threadIdx.x == 0) {
                unsigned sm;
                asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
                p.place[it] = ((unsigned long long)sm << 48) | ((global_ns() - s_titem) & 0xffffffffffffull);
            }
            continue;
        }
        if (!FUSED && p.eval_only) {
            double sd = eval_full(D, red, cb);
            if (D.dense) {
                // fullrmc's compute_data fits the scale factor when the
                // accepted count (0 here) is a multiple of the frequency, for
                // the standard error only; the kept scale factor is the initial one
                __shared__ double s_sf0;
                sd = eval_dense(D, red, cb, false, D.fit_freq > 0, D.sf0, &s_sf0);
            }
            if (threadIdx.x == 0) {
                D.st->sf = D.sf0;
                D.st->sd = sd;
                D.st->chi2 = sd / D.var2;
                D.st->done = 0u;
                D.st->tcount = 0u;
            }
            __syncthreads();
            continue;
        }
        load_moved_group(D, D.st->step, s_group);
        __syncthreads();
        switch (D.bm) {
        case BM_IBC: item_delta<BM_IBC>(D, p.tile, s_group, item.y); break;
        case BM_DIAG: item_delta<BM_DIAG>(D, p.tile, s_group, item.y); break;
        case BM_XYTRI: item_delta<BM_XYTRI>(D, p.tile, s_group, item.y); break;
        case BM_LOWER: item_delta<BM_LOWER>(D, p.tile, s_group, item.y); break;
        default: item_delta<BM_GENERAL>(D, p.tile, s_group, item.y); break;
        }
        // Release: the barrier orders every thread's delta atomics and
        // touched-list stores before thread 0's gpu-scope fence, which is
        // cumulative, so they are visible to the CTA that sees the count.
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            const unsigned prev = atomicAdd(&D.st->done, 1u);
            s_last = (prev == (unsigned)D.ntiles - 1u) ? 1 : 0;
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            finish_engine(D, s_group, red, cb, sbs, sbin, &s_nchg, coef, &s_flag);
        }
        __syncthreads();
    }
    // The last CTA to leave resets the scheduler for the next launch.
    if (!one_each && threadIdx.x == 0) {
        __threadfence();
        const unsigned f = atomicAdd(&p.sched->finished, 1u);
        if (f == gridDim.x - 1) {
            p.sched->claimed = 0ull;
            p.sched->finished = 0u;
            __threadfence();
        }
    }
}

// Host-buffer stepping: scatter this step's moves into each engine's ring
// and gather the step's results (one copy each way for all engines).
__global__ void k_scatter_moves(const EDesc *desc, const int *ids, const EMove *staged, int count)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < count) {
        const EDesc &D = desc[ids[k]];
        D.moves[D.st->step % D.move_cap] = staged[k];
        // a move staged for this step from the ring is stale now
        __threadfence();
        atomicAdd(&D.st->gen, 1u);
    }
}

// A write of engine `st`'s move ring has landed (stream order): staged moves
// read before it are stale.
__global__ void k_bump_gen(EState *st) { atomicAdd(&st->gen, 1u); }

__global__ void k_gather_results(const EDesc *desc, const int *ids, EResult *out, int count)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < count) {
        const EDesc &D = desc[ids[k]];
        out[k] = D.results[(D.st->step + D.move_cap - 1) % D.move_cap];
    }
}

// ------------------------------------------------------------------ S(Q) term
// Engines with a StructureFactorConstraint finish every step here.  The
// histogram kernels have left S(b) in Sb, the element-pair deltas dP_p(b) in
// the global dP array (and as fp16 columns of X), the G(r) change in st->dsd
// and the touched list.  With x(b) = Rq(b) S(b) the change of the S(Q)
// shells' G(r), the change of the S(Q) term is
//   d(sd_sq) = sum_Q w [(e - dS)^2 - e^2] = x^T y - x^T h,
// e = S_exp - S, dS = M^T x, y = K x, K = M W M^T, h = 2 M W (S_exp - S).
// y is formed from the integer deltas and the fixed-point table T (K scaled
// by the shells' 4 pi r / volume and 2^s): z_p(b) = sum_c T[c][b] dP_p(c) is
// an exact int64 sum, so its value does not depend on the order of the
// terms, and y(b) = rho0 2^-s sum_p pair_coef_p z_p(b).
//
// k_sq_fused does the whole term in one persistent launch (one CTA per SM)
// over a work list of tile items, then row items, then one commit item per
// engine:
// * a tile item is (block of delta columns, block of kSqRows rows, K split):
//   the block's columns -- whole engines, at most kSqCols -- times the rows'
//   kSqLimbs digit planes of T over the split's bins, on the tensor cores:
//   tcgen05.mma kind::f16 issued by one thread, fp16 operands staged in
//   shared memory by TMA through a ring of kSqStages stages, one fp32
//   accumulator per digit plane in TMEM.  Every accumulator is an exact
//   integer (see kSqLimbs), so the splits' partial sums are added into the
//   table's fp32 digit products Zf by bulk reductions in L2, in any order
//   with the same result.  The tile then counts itself done in its engines'
//   states.
// * a row item (engine, two row blocks) reads S, Rq and h of its bins, waits
//   (bounded) until all tiles of the engine's block are done, combines each
//   bin's digit products into z (int64), forms y and each row block's share
//   of x (y - h) by a fixed-order sum over its kSqRows bins, and clears the
//   bins' deltas, delta columns and digit products.  The FP64 work -- a
//   narrow pipe on this GPU -- is spread over the SMs this way.
// * a commit item reads what does not depend on the row items (S, h, A, Bq,
//   the touched list, the state, the moved group), waits (bounded) until its
//   row items are done, adds the row blocks' shares in block order, decides
//   and commits: counts, Bq -= 2 A S, h -= 2 y, coordinates.
// The items an item waits for are claimed before it by CTAs that are
// running, so every wait ends.
// A column whose deltas are too large for exact fp32 products is summed
// exactly in int64 over its list of deltas (or its dense deltas) by the first
// K split of each row block instead.  Every quantity of an engine depends
// only on that engine's columns, so a chain is the same in any batch and alone.
constexpr int kSqRows = 128;      // rows per tile: the MMA's M, one TMEM lane per row
constexpr int kSqCols = 128;      // delta columns per block at most: kSqLimbs x kSqCols = all 512 TMEM columns
constexpr int kSqK = 32;          // bins per stage: one 64-byte swizzle row of fp16
constexpr int kSqStages = 4;      // stages in flight
constexpr int kSqThreads = 256;
constexpr int kSqMaxBins = 4096;  // histogram bins of an engine with an S(Q) term
constexpr int kSqBits = 46;       // largest |T| is below 2^46 (four balanced base-4096 digits hold 2^47)
constexpr int kSqPlaneBytes = kSqRows * kSqK * 2;        // one digit plane of a stage: 8 KB
constexpr int kSqABytes = kSqLimbs * kSqPlaneBytes;      // 32 KB
constexpr int kSqBBytes = kSqCols * kSqK * 2;            // 8 KB
constexpr int kSqStageBytes = kSqABytes + kSqBBytes;     // 40 KB
constexpr int kSqRingBytes = kSqStages * kSqStageBytes;  // 160 KB
constexpr int kSqSmemBytes = kSqRingBytes + 1024;        // + the 1024-byte alignment of the swizzled tiles
constexpr int kSqTmemCols = kSqLimbs * kSqCols;          // 512
constexpr unsigned long long kSqWaitNs = 2000000000ull;  // a bounded wait gives up after 2 s
static_assert(kSqTmemCols == 512, "one CTA per SM holds all of its TMEM");
static_assert(2 * kSqCols * kSqRows * 4 <= kSqRingBytes, "the epilogue's two plane buffers fit the ring");
static_assert(5 * kSqMaxBins * 8 <= kSqRingBytes, "a commit's per-bin arrays fit the ring");
static_assert(kSqThreads % kSqRows == 0 && kSqRows % 32 == 0, "a row item holds whole row blocks of whole warps");
static_assert(kSqThreads >= kSqCols && kSqThreads >= kSqRows, "one thread per column and per row");

// A block of delta columns: engines of one table, adjacent in its X.
struct SqBlock {
    const CUtensorMap *tm;  // the table's tensor maps: [0] digit planes of T, [1] delta columns X
    float *Zf;              // the table's fp32 digit products [plane][row block][zcap columns][kSqRows]
    long long *Zi;          // the table's exact products of wide columns: column c at c hsp
    const int *cmode;       // the block's product modes (the engines' evn), one per column
    int col0, ncol, hsp, hs, zcap;
    int nrb, nsplit, nk;    // row blocks, K splits, K chunks of kSqK bins
    int e0, neng;           // its engines: engs[e0 .. e0 + neng)
};

// What a tile needs of one engine of its block: its completion counter and,
// for the exact path of wide columns, its delta lists, deltas and table.
struct SqEng {
    const int *evl, *dP;
    const long long *T;
    unsigned *done;
    int hs, np, lc, pad;
};

struct SqParams {
    const EDesc *desc;
    const SqBlock *blocks;
    const SqEng *engs;
    // work items (kind, ...): tiles (0, block, row block * nsplit + split),
    // then row items (1, engine id, first row block << 16 | row blocks, its
    // block's tiles), then commits (2, engine id, its row items)
    const int4 *items;
    int nitems;
    Sched *sched;
    unsigned *status;
};

// A CTA's tile pipeline: stage barriers, the accumulator barrier and TMEM.
// The barriers' phases follow from the CTA's running counts of chunks and
// tiles, so every wait names the exact phase it needs.
struct SqPipe {
    uint64_t full[kSqStages];   // TMA -> MMA: the stage's operands have landed
    uint64_t empty[kSqStages];  // MMA -> TMA: the MMAs reading the stage have completed
    uint64_t acc;               // MMA -> epilogue: the tile's accumulators are final
    uint32_t tmem;              // TMEM base address (lane 0, first column)
    int fail;                   // a bounded wait gave up: the CTA stops taking items
};

__device__ __forceinline__ void tmap_acquire(const CUtensorMap *m)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(m) : "memory");
}

// Wide columns of a tile's block (ks == 0 only): z = sum_c T[c][b] dP(c) in
// int64 for the tile's rows, over the column's list of deltas (or its dense
// deltas), into Zi.
__device__ void sq_tile_exact(const SqParams &p, const SqBlock &bk, int row0)
{
    for (int k = 0; k < bk.neng; ++k) {
        const SqEng e = p.engs[bk.e0 + k];
        for (int q = 0; q < e.np; ++q) {
            const int n = __ldcg(bk.cmode + e.lc + q);
            if (n >= 0)
                continue;
            const int b = row0 + (int)threadIdx.x;
            if ((int)threadIdx.x >= kSqRows || b >= e.hs)
                continue;
            long long z = 0;
            if (n != INT_MIN) {
                const int *__restrict__ ev = e.evl + q * e.hs;
                for (int i = 0; i < -1 - n; ++i) {
                    const int v = __ldcg(ev + i);
                    z += (long long)(short)(v & 0xffff) * __ldg(e.T + (size_t)(v >> 16) * e.hs + b);
                }
            } else {
                const int *__restrict__ dq = e.dP + q * e.hs;
                for (int c = 0; c < e.hs; ++c) {
                    const int v = __ldcg(dq + c);
                    if (v)
                        z += (long long)v * __ldg(e.T + (size_t)c * e.hs + b);
                }
            }
            bk.Zi[(size_t)(bk.col0 + e.lc + q) * bk.hsp + b] = z;
        }
    }
}

// One tile item: rows [rb kSqRows, +kSqRows) of the block's digit products
// over K split ks.  `chunks` and `tiles` are the CTA's running counts.
__device__ void sq_tile(const SqParams &p, const SqBlock &bk, int rb, int ks, unsigned char *ring, SqPipe &pp,
                        uint32_t &chunks, uint32_t &tiles)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int kb = ks * bk.nk / bk.nsplit, n = (ks + 1) * bk.nk / bk.nsplit - kb;
    const int row0 = rb * kSqRows;
    const uint32_t npad = (uint32_t)((bk.ncol + 15) & ~15);
    // the block's product modes (read now, used after the product)
    const int mode = (int)threadIdx.x < bk.ncol ? __ldcg(bk.cmode + threadIdx.x) : 0;
    if (n > 0) {
        if (warp == 0) {
            if (lane == 0) {
                // producer and MMA issuer: chunk i of the tile is the CTA's
                // chunk g0 + i, in stage (g0 + i) % kSqStages
                const CUtensorMap *tmA = bk.tm, *tmB = bk.tm + 1;
                tmap_acquire(tmA);
                tmap_acquire(tmB);
                const uint32_t idesc = idesc_f16_m128(npad);
                const uint32_t g0 = chunks;
                int issued = 0;
                auto load = [&](int i) {
                    const uint32_t s = (g0 + i) % kSqStages;
                    unsigned char *st = ring + s * kSqStageBytes;
                    mbar_arrive_expect_tx(&pp.full[s], kSqStageBytes);
                    const int x = (kb + i) * kSqK;
                    tma_load_3d(st, tmA, x, row0, 0, &pp.full[s]);
                    tma_load_2d(st + kSqABytes, tmB, x, bk.col0, &pp.full[s]);
                    issued = i + 1;
                };
                auto wait_empty = [&](int i) {
                    const uint32_t g = g0 + i;
                    return mbar_wait_ns(&pp.empty[g % kSqStages], (g / kSqStages) & 1u, kSqWaitNs, p.status);
                };
                for (int i = 0; i < min(n, kSqStages); ++i) load(i);
                int done = 0;
                for (int i = 0; i < n; ++i) {
                    const uint32_t g = g0 + i, s = g % kSqStages;
                    if (!mbar_wait_ns(&pp.full[s], (g / kSqStages) & 1u, kSqWaitNs, p.status)) {
                        pp.fail = 1;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a0 = smem_addr(ring + s * kSqStageBytes), b0 = a0 + kSqABytes;
#pragma unroll
                    for (int kk = 0; kk < kSqK / 16; ++kk)
#pragma unroll
                        for (int l = 0; l < kSqLimbs; ++l)
                            tc_mma_f16(pp.tmem + (uint32_t)(l * kSqCols),
                                       sdesc_k_sw64(a0 + (uint32_t)(l * kSqPlaneBytes + kk * 32)),
                                       sdesc_k_sw64(b0 + (uint32_t)(kk * 32)), idesc, (uint32_t)(i | kk));
                    tc_commit(&pp.empty[s]);
                    done = i + 1;
                    // refill the previous chunk's stage once its MMAs are done
                    if (i >= 1 && i - 1 + kSqStages < n) {
                        if (!wait_empty(i - 1)) {
                            pp.fail = 1;
                            break;
                        }
                        load(i - 1 + kSqStages);
                    }
                }
                tc_commit(&pp.acc);
                // the stages whose MMAs were not waited for above (every
                // chunk's completion is consumed once, in order)
                if (!pp.fail)
                    for (int i = max(0, n - kSqStages); i < n; ++i)
                        if (!wait_empty(i)) {
                            pp.fail = 1;
                            break;
                        }
                if (pp.fail) {
                    // let the copies in flight land before the CTA stops
                    for (int i = done; i < issued; ++i) {
                        const uint32_t g = g0 + i;
                        mbar_wait_ns(&pp.full[g % kSqStages], (g / kSqStages) & 1u, kSqWaitNs, nullptr);
                    }
                }
            }
            __syncwarp();
        }
        chunks += (uint32_t)n;
        if (!mbar_wait_ns(&pp.acc, tiles & 1u, kSqWaitNs, p.status))
            pp.fail = 1;
        tiles += 1;
        tc_fence_after();
        __syncthreads();
        if (pp.fail)
            return;
        // epilogue, one digit plane at a time: warps w and w + 4 share TMEM
        // lanes 32 (w % 4) .. + 31 (the tile's rows) and split the columns;
        // the accumulators go TMEM -> registers -> a plane buffer in the ring
        // (column-major, kSqRows per column, the block's columns adjacent as
        // in Zf) -> one bulk fp32 reduction into Zf in L2 (exact integers:
        // any order of the splits' additions gives the same sums)
        const int quarter = warp & 3, part = warp >> 2;
        const uint32_t half = npad >> 1;  // a multiple of 8
        const size_t zrb = (size_t)bk.zcap * kSqRows;
        const size_t zplane = (size_t)(bk.hsp / kSqRows) * zrb;
        float *planes = reinterpret_cast<float *>(ring);
        for (int l = 0; l < kSqLimbs; ++l) {
            float *buf = planes + (l & 1) * (kSqCols * kSqRows);
            if (l >= 2) {
                if (threadIdx.x == 0)
                    bulk_wait_read<1>();  // plane l - 2's reduction has read this buffer
                __syncthreads();
            }
            // up to kSqCols / 2 columns per thread: every load before one wait
            uint32_t r[kSqCols / 16][8];
            const uint32_t c0 = part * half, taddr = pp.tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(l * kSqCols) + c0;
#pragma unroll
            for (int k = 0; k < kSqCols / 16; ++k)
                if ((uint32_t)(8 * k) < half)
                    tmem_ld8(taddr + 8 * k, r[k]);
            tmem_ld_wait();
#pragma unroll
            for (int k = 0; k < kSqCols / 16; ++k)
                if ((uint32_t)(8 * k) < half)
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        buf[(c0 + 8 * k + j) * kSqRows + 32 * quarter + lane] = __uint_as_float(r[k][j]);
            fence_proxy_async_smem();
            __syncthreads();
            if (threadIdx.x == 0) {
                // the block's columns are adjacent: one reduction per plane
                bulk_reduce_add_f32(bk.Zf + (size_t)l * zplane + (size_t)rb * zrb + (size_t)bk.col0 * kSqRows, buf,
                                    (uint32_t)bk.ncol * kSqRows * 4u);
                bulk_commit_group();
            }
        }
        tc_fence_before();  // the TMEM reads come before the next tile's MMAs
        if (threadIdx.x == 0) {
            bulk_wait<0>();
            fence_proxy_async_global();
        }
    }
    const int wide = __syncthreads_or(mode < 0);
    if (wide && ks == 0) {
        sq_tile_exact(p, bk, row0);
        __syncthreads();
    }
    // release: the barriers above order every Zf / Zi write before the
    // gpu-scope fences of the threads that count the engines' tiles done
    for (int k = threadIdx.x; k < bk.neng; k += kSqThreads) {
        __threadfence();
        atomicAdd(p.engs[bk.e0 + k].done, 1u);
    }
    __syncthreads();  // the ring is reused by the next item
}

// Bounded wait (thread 0) until *counter >= target; false after kSqWaitNs.
__device__ bool sq_wait_count(const unsigned *counter, unsigned target, unsigned *status)
{
    const volatile unsigned *c = counter;
    if (*c >= target)
        return true;
    const unsigned long long t0 = global_ns();
    while (*c < target) {
        if (global_ns() - t0 > kSqWaitNs) {
            atomicOr(status, DS_BARRIER_TIMEOUT);
            return false;
        }
        __nanosleep(128);
    }
    return true;
}

// A row item: bins [rb0 kSqRows, (rb0 + rbn) kSqRows) of one engine (rbn <=
// kSqThreads / kSqRows), one bin per thread, once the `ntiles` tiles of its
// block are done.  y(b) = sum_p coef_p z_p(b) in p order; row block rb's share
// of x (y - h) is summed over its bins by a fixed tree (each warp's shuffle
// tree, then its four warps in order), so it does not depend on how row
// blocks are grouped into items.
__device__ void sq_row_item(const SqParams &p, const EDesc &D, int rb0, int rbn, int ntiles)
{
    __shared__ int s_mode[kMaxP];
    __shared__ double s_coef[kMaxP];
    __shared__ double s_wp[kSqThreads / 32];
    __shared__ int s_ok;
    const int hs = D.hs, np = D.npairs, hsp = D.hsp;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rbl = (int)threadIdx.x / kSqRows, b = (rb0 + rbl) * kSqRows + (int)threadIdx.x % kSqRows;
    const bool row = rbl < rbn && b < hs;
    const size_t zrb = (size_t)D.zcap * kSqRows, zplane = (size_t)(hsp / kSqRows) * zrb;
    // what does not depend on the tiles
    const double sv = row ? __ldcg(D.Sb + b) : 0.0;
    const double rq = row ? __ldg(D.Rq + b) : 0.0;
    const double hb = row ? __ldcg(D.h + b) : 0.0;
    if ((int)threadIdx.x < np) {
        s_mode[threadIdx.x] = __ldcg(D.evn + threadIdx.x);
        s_coef[threadIdx.x] = __ldg(D.pc + threadIdx.x) * D.yscale;
    }
    if (threadIdx.x == 0)
        s_ok = sq_wait_count(&D.st->sq_done, (unsigned)ntiles, p.status) ? 1 : 0;
    __syncthreads();
    if (!s_ok)
        return;
    __threadfence();
    // every load of the bin is issued before any is used
    float *zb = D.Zf + (size_t)(b / kSqRows) * zrb + (b % kSqRows);
    // an element pair without a non-zero delta this step (mode 0) has z = 0 in
    // every bin and nothing to clear: it is skipped (adding its +-0 product
    // would leave y unchanged, y being +0 or non-zero)
    float f[kMaxP][kSqLimbs];
    long long zi[kMaxP];
#pragma unroll
    for (int q = 0; q < kMaxP; ++q) {
        const bool on = row && q < np && s_mode[q] != 0, tc = on && s_mode[q] >= 0;
#pragma unroll
        for (int l = 0; l < kSqLimbs; ++l) f[q][l] = tc ? __ldcg(zb + l * zplane + q * kSqRows) : 0.0f;
        zi[q] = (on && !tc) ? __ldcg(D.Zi + (size_t)q * hsp + b) : 0ll;
    }
    double y = 0.0;
#pragma unroll
    for (int q = 0; q < kMaxP; ++q) {
        if (q >= np)
            break;
        if (s_mode[q] == 0)
            continue;
        long long z = zi[q];
        if (s_mode[q] >= 0) {
            // fp32 -> int32 is exact (|digit product| <= 2^24); planes combine in int64
            unsigned long long u = 0;
#pragma unroll
            for (int l = 0; l < kSqLimbs; ++l)
                u += (unsigned long long)(long long)__float2int_rn(f[q][l]) << (kSqDigitBits * l);
            z = (long long)u;
        }
        y = fma(s_coef[q], (double)z, y);
    }
    double part = 0.0;
    if (row) {
        D.y[b] = y;
        if (sv != 0.0)
            part = (rq * sv) * (y - hb);
        // the bin's deltas, delta columns and digit products are spent
        for (int q = 0; q < np; ++q) {
            if (s_mode[q] == 0)
                continue;
            D.dP[q * hs + b] = 0;
            D.X[q * D.xld + b] = __float2half_rn(0.0f);
#pragma unroll
            for (int l = 0; l < kSqLimbs; ++l) zb[l * zplane + q * kSqRows] = 0.0f;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0)
        s_wp[warp] = part;
    __syncthreads();
    constexpr int kW = kSqRows / 32;  // warps per row block
    if ((int)threadIdx.x < rbn) {
        const double *w = s_wp + threadIdx.x * kW;
        double t = w[0];
#pragma unroll
        for (int k = 1; k < kW; ++k) t += w[k];
        D.sqpart[rb0 + threadIdx.x] = t;
    }
    // release: the barrier orders every y, share and clearing store before
    // the gpu-scope fence of the thread that counts the item done
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&D.st->sq_ydone, 1u);
    }
}

// Decide and commit an engine's step once its `nrow` row items are done.
// What does not depend on them -- the descriptor's fields, S, h, A, Bq, the
// touched list, the state and the moved group -- is read before the wait.
// Shared memory (the ring): S, h, y, then A and Bq where they fit.
__device__ void sq_commit(const SqParams &p, const EDesc &D, int nrow, unsigned char *ring, MovedGroup &g)
{
    constexpr int kTl = 8;  // touched-list entries per thread read before the wait
    __shared__ double s_val[4];
    __shared__ double s_part[kSqMaxBins / kSqRows];
    __shared__ int s_ready, s_flag;
    const int hs = D.hs, hsp = D.hsp;
    const int nrb = (hs + kSqRows - 1) / kSqRows;
    const double var2 = D.var2, var2q = D.var2q, tol = D.tol;
    double *sS = reinterpret_cast<double *>(ring);
    double *sH = sS + hsp, *sY = sH + hsp, *sA = sY + hsp, *sB = sA + hsp;
    // 1. everything that does not depend on the row items
    load_moved_group(D, D.st->step, g);
    for (int b = threadIdx.x; b < hs; b += kSqThreads) {
        sS[b] = __ldcg(D.Sb + b);
        sH[b] = __ldcg(D.h + b);
        sA[b] = __ldcg(D.A + b);
        sB[b] = __ldcg(D.Bq + b);
    }
    const unsigned nt = __ldcg(&D.st->tcount);
    const int fmt = __ldcg(&D.st->fmt);
    int tl[kTl];
#pragma unroll
    for (int i = 0; i < kTl; ++i) {
        const unsigned k = threadIdx.x + i * kSqThreads;
        tl[i] = (fmt && k < nt) ? __ldcg(D.tlist + k) : -1;
    }
    if (threadIdx.x == 32) {
        const EState &S0 = *D.st;
        s_val[0] = S0.sd + S0.dsd;
        s_val[1] = S0.sd_sq;
        s_val[2] = s_val[0] / var2;  // the G(r) term of the new chi2
    }
    // 2. the row items
    if (threadIdx.x == 0)
        s_ready = sq_wait_count(&D.st->sq_ydone, (unsigned)nrow, p.status) ? 1 : 0;
    __syncthreads();
    if (!s_ready)
        return;
    __threadfence();
    for (int k = threadIdx.x; k < nrb; k += kSqThreads) s_part[k] = __ldcg(D.sqpart + k);
    __syncthreads();
    // 3. the row blocks' shares in block order, the decision
    if (threadIdx.x == 0) {
        double dsq = 0.0;
        for (int k = 0; k < nrb; ++k) dsq += s_part[k];
        const double sq_new = s_val[1] + dsq;
        const double chi2_new = s_val[2] + sq_new / var2q;
        const bool reject = (chi2_new > g.chi2) && (g.u > tol);
        s_flag = reject ? 0 : 1;
        s_val[2] = chi2_new;
        s_val[3] = sq_new;
    }
    __syncthreads();
    const bool accept = s_flag != 0;
    // 4. counts
    if (fmt) {
        // one CTA's shared-memory deltas: entries (flat << 1) | sign
        if (accept) {
#pragma unroll
            for (int i = 0; i < kTl; ++i)
                if (tl[i] >= 0)
                    atomicAdd(D.counts + (tl[i] >> 1), (tl[i] & 1) ? 1 : -1);
            for (unsigned k = threadIdx.x + kTl * kSqThreads; k < nt; k += kSqThreads) {
                const int e = __ldcg(D.tlist + k);
                atomicAdd(D.counts + (e >> 1), (e & 1) ? 1 : -1);
            }
        }
    } else {
        // global oriented deltas: atomicExch hands each bin's delta to one entry
        for (unsigned k = threadIdx.x; k < nt; k += kSqThreads) {
            const int f = D.tlist[k];
            const int d = atomicExch(D.delta + f, 0);
            if (accept && d)
                D.counts[f] += d;
        }
    }
    // 5. the accepted step: Bq -= 2 A S, h -= 2 y, coordinates
    if (accept) {
        for (int b = threadIdx.x; b < hs; b += kSqThreads) sY[b] = __ldcg(D.y + b);
        for (int b = threadIdx.x; b < hs; b += kSqThreads) {
            const double sv = sS[b];
            if (sv != 0.0)
                D.Bq[b] = fma(-2.0 * sA[b], sv, sB[b]);
            D.h[b] = fma(-2.0, sY[b], sH[b]);
        }
        commit_moved_group(D, g);
        if (D.dense)
            dense_commit(D);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        EState &S = *D.st;
        EResult &r = D.results[g.step % D.move_cap];
        r.chi2_new = s_val[2];
        r.accepted = accept ? 1 : 0;
        r.atom = g.atom[0];
        if (accept) {
            S.chi2 = s_val[2];
            S.sd = s_val[0];
            S.sd_sq = s_val[3];
            S.accepted += 1;
            if (D.dense)
                S.sf = S.sf_prop;
        }
        S.step += 1;
        S.tcount = 0u;
        S.sq_done = 0u;
        S.sq_ydone = 0u;
        S.dsd = 0.0;
    }
}

__global__ void __launch_bounds__(kSqThreads, 1) k_sq_fused(SqParams p)
{
    extern __shared__ __align__(16) unsigned char sq_smem_raw[];
    // the swizzled operand tiles start on 1024-byte boundaries
    unsigned char *ring = sq_smem_raw + ((1024u - (smem_addr(sq_smem_raw) & 1023u)) & 1023u);
    __shared__ SqPipe pp;
    __shared__ int s_item;
    __shared__ MovedGroup s_group;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kSqStages; ++s) {
            mbar_init(&pp.full[s], 1);
            mbar_init(&pp.empty[s], 1);
        }
        mbar_init(&pp.acc, 1);
        pp.fail = 0;
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(&pp.tmem, kSqTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t chunks = 0, tiles = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long k = atomicAdd(&p.sched->claimed, 1ull);
            s_item = (k < (unsigned long long)p.nitems && !pp.fail) ? (int)k : -1;
        }
        __syncthreads();
        const int it = s_item;
        if (it < 0)
            break;
        const int4 item = p.items[it];
        if (item.x == 0) {
            const SqBlock &bk = p.blocks[item.y];
            sq_tile(p, bk, item.z / bk.nsplit, item.z % bk.nsplit, ring, pp, chunks, tiles);
        } else if (item.x == 1) {
            sq_row_item(p, p.desc[item.y], item.z >> 16, item.z & 0xffff, item.w);
        } else {
            sq_commit(p, p.desc[item.y], item.z, ring, s_group);
        }
        __syncthreads();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(pp.tmem, kSqTmemCols);
    }
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned f = atomicAdd(&p.sched->finished, 1u);
        if (f == gridDim.x - 1) {
            p.sched->claimed = 0ull;
            p.sched->finished = 0u;
            __threadfence();
        }
    }
}

// S(Q) of engine `id`'s current counts (StructureFactorConstraints.py:780-822
// with scale factor 1 and no window), in four short launches so that the
// FP64 work -- GB300's narrow pipe -- spreads over the SMs:
// - k_sq_gs: G_S(b) = Rq(b) sum_p pair_coef_p n_p(b) - rfacq(b) into gsq;
// - k_sq_sv: S(q) = sum_b G_S(b) M[b][q] + 1 into sqv, one thread per q, b in
//   increasing order;
// with commit (set-up), also
// - k_sq_hv: h(b) = 2 sum_q M[b][q] w (S_exp - S), one warp per b (lanes over
//   q, a fixed shuffle tree);
// - k_sq_sd: sd_sq = sum_q w (S_exp - S)^2 (fixed-order lanes) and the
//   chain's chi2.
// Each value is formed by the same operations in the same order wherever
// its thread runs.
__global__ void __launch_bounds__(512) k_sq_gs(const EDesc *desc, int id)
{
    const EDesc &D = desc[id];
    for (int b = threadIdx.x; b < D.hs; b += blockDim.x) {
        double S = 0.0;
        for (int q = 0; q < D.npairs; ++q) S = fma(D.pc[q], (double)pair_count(D, q, b), S);
        D.gsq[b] = fma(D.Rq[b], S, -D.rfacq[b]);
    }
}

__global__ void __launch_bounds__(128) k_sq_sv(const EDesc *desc, int id)
{
    const EDesc &D = desc[id];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= D.nq)
        return;
    const int hs = D.hs, nq = D.nq;
    const double *__restrict__ gs = D.gsq;
    const double *__restrict__ M = D.M;
    double a = 0.0;
    for (int b = 0; b < hs; ++b) a = fma(__ldg(gs + b), __ldg(M + (size_t)b * nq + q), a);
    D.sqv[q] = a + 1.0;
}

__global__ void __launch_bounds__(256) k_sq_hv(const EDesc *desc, int id)
{
    const EDesc &D = desc[id];
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (b >= D.hs)
        return;
    const int nq = D.nq;
    const double *row = D.M + (size_t)b * nq;
    double a = 0.0;
    for (int q = lane; q < nq; q += 32) {
        const double w = D.wq ? D.wq[q] : 1.0;
        a = fma(row[q], w * (D.sqexp[q] - D.sqv[q]), a);
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0)
        D.h[b] = 2.0 * a;
}

__global__ void __launch_bounds__(512) k_sq_sd(const EDesc *desc, int id)
{
    __shared__ double red[kRedLanes];
    __shared__ double cb[kChunk];
    const EDesc &D = desc[id];
    const int nq = D.nq;
    lanes_zero(red);
    for (int c0 = 0; c0 < nq; c0 += kChunk) {
        const int cn = min(kChunk, nq - c0);
        for (int q = c0 + threadIdx.x; q < c0 + cn; q += blockDim.x) {
            const double e = D.sqexp[q] - D.sqv[q];
            const double w = D.wq ? D.wq[q] : 1.0;
            cb[q - c0] = (w * e) * e;
        }
        lanes_add_chunk(red, cb, c0, cn);
    }
    const double sdq = lanes_total(red);
    if (threadIdx.x == 0) {
        EState &S = *D.st;
        S.sd_sq = sdq;
        S.chi2 = S.sd / D.var2 + sdq / D.var2q;
    }
}

// Largest |K[c][b] R0(c)| (non-negative doubles order like their bit patterns).
__global__ void k_sq_absmax(const double *K, const double *R0, int hs, unsigned long long *out)
{
    const long long n = (long long)hs * hs;
    double m = 0.0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        m = fmax(m, fabs(K[k] * R0[k / hs]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// T[c][b] = round(K[c][b] R0(c) 2^s), in place over K.
__global__ void k_sq_quantize(double *K, const double *R0, int hs, int s)
{
    const long long n = (long long)hs * hs;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const double v = ldexp(K[k] * R0[k / hs], s);
        ((long long *)K)[k] = llrint(v);
    }
}

// The product's operand: TD[(l hsp + b) hsp + c] = digit l of T[c][b]
// (balanced base 4096, so T = sum_l 4096^l digit_l), zero outside hs x hs.
__global__ void k_sq_digits(const long long *T, int hs, int hsp, __half *TD)
{
    const long long n = (long long)hsp * hsp;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(k / hsp), c = (int)(k - (long long)b * hsp);
        long long v = (b < hs && c < hs) ? T[(long long)c * hs + b] : 0;
#pragma unroll
        for (int l = 0; l < kSqLimbs; ++l) {
            const long long half = 1ll << (kSqDigitBits - 1);
            const long long d = ((v + half) & ((1ll << kSqDigitBits) - 1)) - half;
            v = (v - d) >> kSqDigitBits;
            TD[(long long)l * n + k] = __int2half_rn((int)d);
        }
    }
}

// K[b][c] = sum_q (M[b][q] M[c][q]) w_q in increasing q: 64 x 64 tiles of K
// per CTA, 4 x 4 per thread, M staged through shared memory 16 Q points at a
// time.  The product M[b][q] M[c][q] is formed before the weight, so K is
// exactly symmetric.
__global__ void __launch_bounds__(256) k_sq_gram(const double *M, const double *w, int hs, int nq, double *K)
{
    __shared__ double A[16][65];
    __shared__ double Bt[16][65];
    const int b0 = blockIdx.y * 64, c0 = blockIdx.x * 64;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
    for (int q0 = 0; q0 < nq; q0 += 16) {
        for (int k = threadIdx.x; k < 64 * 16; k += 256) {
            const int r = k >> 4, qq = k & 15, q = q0 + qq;
            A[qq][r] = (b0 + r < hs && q < nq) ? M[(size_t)(b0 + r) * nq + q] : 0.0;
            Bt[qq][r] = (c0 + r < hs && q < nq) ? M[(size_t)(c0 + r) * nq + q] : 0.0;
        }
        __syncthreads();
        const int qn = min(16, nq - q0);
        for (int qq = 0; qq < qn; ++qq) {
            const double wq = w ? w[q0 + qq] : 1.0;
            double a[4], bb[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = A[qq][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bb[j] = Bt[qq][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i] * bb[j], wq, acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int b = b0 + ty + 16 * i, c = c0 + tx + 16 * j;
            if (b < hs && c < hs)
                K[(size_t)b * hs + c] = acc[i][j];
        }
}

// --------------------------------------------------------------- host side
struct Slot {
    bool live = false;
    bool initialized = false;
    int sq_table = -1;  // S(Q) table of the engine (or -1)
    // cost of a one-CTA step in column units: the columns a step sweeps (all
    // atoms, or with a column grid the estimate, counted 4 times: a grid
    // column is gathered and mostly in range), times the atoms a move moves
    long long cost = 0;
    EDesc d;
    void *blob = nullptr;
    size_t bytes = 0;
};

struct SqTable {
    int hs = 0, nq = 0;
    int s = 0;  // T = round(K R0 2^s)
    void *blob = nullptr;
    double *M = nullptr, *w = nullptr, *R0 = nullptr;
    long long *T = nullptr;
    size_t bytes = 0;
    int hsp = 0;           // hs rounded up to a multiple of kSqRows
    __half *TD = nullptr;  // [kSqLimbs][hsp][hsp] digit planes of T (k_sq_digits)
    // this step's fp16 deltas of every engine on the table (ncols columns of
    // hsp bins), their fp32 digit products (kSqLimbs planes of hsp per
    // column), the exact products of wide columns, the columns' product
    // modes; room for cap columns
    __half *X = nullptr;
    float *Zf = nullptr;
    long long *Zi = nullptr;
    int *cmode = nullptr;
    int ncols = 0, cap = 0;
    CUtensorMap *maps = nullptr;  // device: [0] digit planes (bin, row, plane), [1] X (bin, column)
};

// dynamic shared memory of a one-CTA step at the largest CTA (the static
// part, about 4 KB, comes on top of it within the 227 KB an SM offers)
constexpr long long kFusedDynMax = 221 * 1024;

// Dynamic shared memory of a one-CTA step: element-pair deltas, A and Bq,
// the column queue, the per-bin non-zero counts, the evaluation scratch.
static long long fused_dyn_bytes(long long dp_ints, int bins, int threads)
{
    return 4 * dp_ints + 16ll * bins + (long long)kColQueue * threads * 12 + 4ll * bins +
           8ll * fused_cb_cap(bins, threads) + 12ll * fused_bins_cap(bins);
}

constexpr long long kFusedMaxCost = 49152;  // engines of a higher step cost (Slot::cost) are split over several CTAs
constexpr long long kSoloFusedCost = 16384;  // one-engine steps up to this cost use the fused item

struct EngineSet {
    std::vector<Slot> slots;
    int fused = 1;         // batched steps use one CTA per engine where it fits
    int cells = 1;         // engines added from now on get a column grid where it pays
    int fused_dp_ints = 0; // its layout: element-pair deltas (ints), then A and Bq (fused_bins doubles each)
    int fused_bins = 0;
    int nsolo = 0;         // items [0, nsolo): tiles of every engine (one-engine steps)
    int nbatch = 0;        // items [nsolo, nsolo + nbatch): the batched work list
    int nfused = 0;        // of which the first nfused are one-CTA-per-engine items
    std::vector<int> live;        // live engine ids in work-list order
    std::vector<int> item_first;  // per engine id: first item (or -1)
    std::vector<int> item_count;
    std::vector<int> fused_item;  // per engine id: its one-CTA item in the batched list (or -1)
    int tile = 1024, threads = 256, ctas_per_sm = 2;  // the usual autotuner choice on GB300
    int sq_split_max = 0;  // K splits of an S(Q) row block at most (0: as many as fill the SMs)
    EDesc *ddesc = nullptr;
    int ddesc_cap = 0;
    EDesc *fdesc = nullptr;        // descriptors of the fused items, in work-list order
    int fdesc_cap = 0;
    int *fpos = nullptr;           // per fused item: its engine's index in live order (host-buffer steps)
    int2 *items = nullptr;
    int items_cap = 0;
    int nitems = 0;
    int *dlive = nullptr;
    int dlive_cap = 0;
    // step_host staging, two slots so that a host can submit a step before
    // it reads the previous one's results
    EMove *hstage_m[2] = {nullptr, nullptr};     // pinned
    EResult *hstage_r[2] = {nullptr, nullptr};   // pinned
    EMove *dstage_m[2] = {nullptr, nullptr};
    EResult *dstage_r[2] = {nullptr, nullptr};
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
    bool stage_busy[2] = {false, false};
    int stage_E[2] = {0, 0};       // engines of the step each busy slot holds
    int stage_cap = 0;
    Sched *sched = nullptr;        // [0]: histogram step kernels, [1]: S(Q) kernel
    std::vector<SqTable> tables;
    // S(Q) work lists: the batched list (every block's tiles, then one commit
    // per engine) at [0, sq_nbatch), then each engine's own list (its tiles
    // and its commit) at sq_first[id], sq_count[id] items
    std::vector<int4> sq_host;
    int sq_nbatch = 0;
    std::vector<int> sq_first, sq_count;
    std::vector<int> sq_xcol;      // per engine id: its first delta column in its table's X
    std::vector<SqBlock> sq_hblocks;
    std::vector<SqEng> sq_hengs;
    int4 *sq_items = nullptr;
    int sq_cap = 0;
    SqBlock *sq_blocks = nullptr;
    int sq_blocks_cap = 0;
    SqEng *sq_engs = nullptr;
    int sq_engs_cap = 0;
    cudaStream_t stream = nullptr;
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
    cudaGraphExec_t host_graph[2] = {nullptr, nullptr};  // step_host per slot: copy in, scatter,
    int host_graph_E[2] = {0, 0};                        // step, gather, copy out
    bool dirty = true;
    // Measured placement (frmc_engines_place): the one-CTA batched launch
    // assigns CTA b to an SM the same way every time for a given grid and
    // CTA shape, so recorded steps show which CTAs hold an SM alone and which
    // share one; the work list then gives the lone CTAs the engines that
    // took longest and pairs the rest longest with shortest.
    unsigned long long *place_dev = nullptr;
    int place_cap = 0;
    bool place_rec = false;             // record in the next one-CTA launches
    std::vector<int> place_order;       // engine id per fused item, or empty
    long long place_key = -1;           // the launch shape the order was measured for
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct BlobLayout {
    size_t box, real, mol, counts, delta, rfac, invvol, expd, dw, pc, pi, pj, dP, pidx, tlist, R, A, Bq, Sb, Gc, fnum,
        fden, win, moves,
        results, st, Rq, rfacq, sqexp, h, y, gsq, sqpart, sqv, evl, groups, cbox, cmol, csl, cstart, clo, chi,
        total;
};

static int spec_group(const frmc_engine_spec &sp) { return sp.group_size > 1 ? sp.group_size : 1; }
static double spec_scale(const frmc_engine_spec &sp) { return sp.scale_factor == 0.0 ? 1.0 : sp.scale_factor; }
static bool spec_dense(const frmc_engine_spec &sp)
{
    return spec_scale(sp) != 1.0 || sp.fit_frequency > 0 || sp.window_len > 0;
}

static BlobLayout blob_layout(const frmc_engine_spec &sp)
{
    BlobLayout L;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += align256(bytes);
        return o;
    };
    const size_t n = sp.n, hs = sp.hs, tot = (size_t)sp.ne * sp.ne * sp.hs;
    L.box = take(16 * n);
    L.real = take(16 * n);
    L.mol = take(4 * n);
    L.counts = take(8 * tot);
    L.delta = take(8 * tot);
    L.rfac = take(8 * hs);
    L.invvol = take(8 * hs);
    L.expd = take(8 * hs);
    L.dw = take(sp.data_weights ? 8 * hs : 0);
    L.pc = take(8 * (size_t)sp.npairs);
    L.pi = take(4 * (size_t)sp.npairs);
    L.pj = take(4 * (size_t)sp.npairs);
    L.dP = take(4 * (size_t)sp.npairs * hs);
    L.pidx = take(4 * (size_t)sp.ne * sp.ne);
    const size_t G = spec_group(sp);
    L.tlist = take(4 * (2 * G * n + G * G + 8));
    L.R = take(8 * hs);
    L.A = take(8 * hs);
    L.Bq = take(8 * hs);
    L.Sb = take(8 * hs);
    const bool dense = spec_dense(sp);
    L.Gc = take(dense ? 8 * hs : 0);
    L.fnum = take(dense ? 8 * hs : 0);
    L.fden = take(dense ? 8 * hs : 0);
    L.win = take(dense ? 8 * (size_t)sp.window_len : 0);
    L.moves = take(sizeof(EMove) * (size_t)sp.move_cap);
    L.results = take(sizeof(EResult) * (size_t)sp.move_cap);
    L.st = take(sizeof(EState));
    const bool sq = sp.sq_table >= 0;
    const size_t nq = sq ? (size_t)sp.nq : 0, hq = sq ? hs : 0;
    L.Rq = take(8 * hq);
    L.rfacq = take(8 * hq);
    L.sqexp = take(8 * nq);
    L.h = take(8 * hq);
    L.y = take(8 * hq);
    L.gsq = take(8 * hq);
    L.sqpart = take(sq ? 8 * (size_t)((sp.hs + kSqRows - 1) / kSqRows) : 0);
    L.sqv = take(8 * nq);
    L.evl = take(sq ? 4 * (size_t)sp.npairs * hs : 0);
    L.groups = take(G > 1 ? sizeof(EGroup) * (size_t)sp.move_cap : 0);
    L.cbox = take(16 * n);
    L.cmol = take(4 * n);
    L.csl = take(8 * n);
    L.cstart = take(4 * (size_t)(kMaxCells + 1));
    L.clo = take(16 * (size_t)kMaxCells);
    L.chi = take(16 * (size_t)kMaxCells);
    L.total = off;
    return L;
}

static int check_spec(const frmc_engine_spec &sp)
{
    if (sp.n < 1 || sp.ne < 1 || sp.hs < 1 || sp.npairs < 1 || sp.move_cap < 1 || !sp.box_coords ||
        !sp.real_coords || !sp.el || !sp.mol || !sp.basis || !sp.rbasis || !sp.pair_i || !sp.pair_j ||
        !sp.pair_coef || !sp.rfac || !sp.inv_shell_volume || !sp.experimental || !(sp.variance_squared > 0))
        return set_error(FRMC_E_ARG, "engine spec: missing or invalid field");
    if (sp.group_size < 0 || sp.group_size > kMaxGroup || spec_group(sp) > sp.n)
        return set_error(FRMC_E_ARG, "engine spec: group_size must be in [1, %d] and at most n", kMaxGroup);
    if ((double)sp.ne * sp.ne * sp.hs > 2.0e8)
        return set_error(FRMC_E_ARG, "engine spec: histogram too large (ne*ne*hs must stay below 2e8)");
    if (sp.npairs > 64)
        return set_error(FRMC_E_ARG, "engine spec: at most 64 element pairs (10 elements)");
    for (int q = 0; q < sp.npairs; ++q)
        if (sp.pair_i[q] < 0 || sp.pair_i[q] >= sp.ne || sp.pair_j[q] < 0 || sp.pair_j[q] >= sp.ne)
            return set_error(FRMC_E_ARG, "engine spec: element pair %d out of range", q);
    for (int i = 0; i < sp.n; ++i)
        if (sp.el[i] < 0 || sp.el[i] >= sp.ne)
            return set_error(FRMC_E_ARG, "engine spec: atom %d element out of range", i);
    if (sp.fit_frequency < 0 || (sp.fit_frequency > 0 && (!sp.fit_num || !(sp.fit_min <= sp.fit_max))) ||
        sp.window_len < 0 || sp.window_len > 255 || sp.window_len > sp.hs || (sp.window_len > 0 && !sp.window) ||
        !std::isfinite(sp.scale_factor))
        return set_error(FRMC_E_ARG, "engine spec: invalid scale factor or window fields");
    if (sp.sq_table >= 0) {
        if (sp.nq < 1 || !sp.sq_rfac || !sp.sq_inv_shell_volume || !sp.sq_experimental ||
            !(sp.sq_variance_squared > 0) || !(sp.sq_rho0 > 0))
            return set_error(FRMC_E_ARG, "engine spec: missing or invalid S(Q) field");
        if (sp.hs > kSqMaxBins)
            return set_error(FRMC_E_ARG, "engine spec: an S(Q) term needs hs <= %d", kSqMaxBins);
        if (sp.npairs > kMaxP)
            return set_error(FRMC_E_ARG, "engine spec: an S(Q) term needs at most %d element pairs", kMaxP);
    }
    return FRMC_OK;
}

static void drop_graphs(EngineSet *s)
{
    for (auto &kv : s->graphs) cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
    for (int k = 0; k < 2; ++k) {
        if (s->host_graph[k])
            cudaGraphExecDestroy(s->host_graph[k]);
        s->host_graph[k] = nullptr;
        s->host_graph_E[k] = 0;
    }
}

// A table's TMA operand descriptors: [0] the digit planes as a 3-D tensor
// (bin c, row b, plane l) read in boxes of kSqK x kSqRows x kSqLimbs, [1] the
// delta columns (bin, column) read in boxes of kSqK x kSqCols.  Both use the
// 64-byte swizzle that the MMAs' shared-memory descriptors name; reads past
// the last column fill zeros.
static int sq_encode_maps(SqTable &t)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        FRMC_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
        if (!fn || q != cudaDriverEntryPointSuccess)
            return set_error(FRMC_E_CUDA, "S(Q) table: the driver offers no cuTensorMapEncodeTiled");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    CUtensorMap m[2];
    std::memset(m, 0, sizeof m);
    const cuuint64_t hsp = (cuuint64_t)t.hsp;
    const cuuint32_t unit[3] = {1, 1, 1};
    {
        const cuuint64_t dims[3] = {hsp, hsp, (cuuint64_t)kSqLimbs};
        const cuuint64_t strides[2] = {hsp * 2, hsp * hsp * 2};
        const cuuint32_t box[3] = {(cuuint32_t)kSqK, (cuuint32_t)kSqRows, (cuuint32_t)kSqLimbs};
        const CUresult r = encode(&m[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, t.TD, dims, strides, box, unit,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return set_error(FRMC_E_CUDA, "S(Q) table: digit-plane tensor map (driver error %d)", (int)r);
    }
    if (t.X) {
        const cuuint64_t dims[2] = {hsp, (cuuint64_t)t.cap};
        const cuuint64_t strides[1] = {hsp * 2};
        const cuuint32_t box[2] = {(cuuint32_t)kSqK, (cuuint32_t)kSqCols};
        const CUresult r = encode(&m[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, t.X, dims, strides, box, unit,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return set_error(FRMC_E_CUDA, "S(Q) table: delta-column tensor map (driver error %d)", (int)r);
    }
    if (!t.maps)
        FRMC_CUDA(cudaMalloc(&t.maps, sizeof m));
    FRMC_CUDA(cudaMemcpy(t.maps, m, sizeof m, cudaMemcpyHostToDevice));
    return FRMC_OK;
}

// An engine's entry in an S(Q) block: its device arrays and constants.
static SqEng sq_eng(const EDesc &D, int lc)
{
    SqEng e;
    e.evl = D.evl;
    e.dP = D.dP;
    e.T = D.T;
    e.done = &D.st->sq_done;
    e.hs = D.hs;
    e.np = D.npairs;
    e.lc = lc;
    e.pad = 0;
    return e;
}

// Rebuild the work list over live engines and upload descriptors.
// Placement of n one-CTA items over the CTAs of a launch: CTA b ran on SM
// sm[b] and its item took t[b].  pos[b] = the item that CTA b gets: the CTAs
// that hold an SM alone take the longest items, and on a shared SM the first
// CTA takes the longest remaining item and the others the shortest ones.
static void place_positions(int n, const int *sm, const double *t, int *pos)
{
    std::map<int, std::vector<int>> by_sm;
    for (int b = 0; b < n; ++b) by_sm[sm[b]].push_back(b);
    std::vector<int> items(n);
    for (int b = 0; b < n; ++b) items[b] = b;
    std::stable_sort(items.begin(), items.end(), [t](int a, int b) { return t[a] > t[b]; });
    int lo = 0, hi = n - 1;
    for (auto &g : by_sm)
        if (g.second.size() == 1)
            pos[g.second[0]] = items[lo++];
    for (auto &g : by_sm)
        if (g.second.size() > 1) {
            pos[g.second[0]] = items[lo++];
            for (size_t j = 1; j < g.second.size(); ++j) pos[g.second[j]] = items[hi--];
        }
}

// The launch shape a measured placement belongs to: the one-CTA items, the
// CTA size, CTAs per SM and the dynamic shared memory of the launch.
static long long place_key(const EngineSet *s, int nfused)
{
    return (((long long)nfused * 1031 + s->threads) * 17 + s->ctas_per_sm) * 4194301 +
           fused_dyn_bytes(s->fused_dp_ints, s->fused_bins, s->threads);
}

static int refresh(EngineSet *s)
{
    if (!s->dirty)
        return FRMC_OK;
    const int nslots = (int)s->slots.size();
    std::vector<int2> items;
    s->item_first.assign(nslots, -1);
    s->item_count.assign(nslots, 0);
    for (int id : s->live) {
        EDesc &D = s->slots[id].d;
        D.ntiles = std::max(1, (D.n + s->tile - 1) / s->tile);
        s->item_first[id] = (int)items.size();
        s->item_count[id] = D.ntiles;
        for (int t = 0; t < D.ntiles; ++t) items.push_back(make_int2(id, t));
    }
    s->nsolo = (int)items.size();
    // batched list: fused engines costliest first, then the tiles of the others
    std::vector<int> fused_ids;
    s->fused_dp_ints = 0;
    s->fused_bins = 0;
    for (int id : s->live) {
        const EDesc &D = s->slots[id].d;
        const int dpw = D.dpk ? (D.npairs * D.hs + 1) / 2 : D.npairs * D.hs;  // words of the deltas
        const int dp = (dpw + 3) & ~3, bins = (D.hs + 1) & ~1;
        const int dpi = std::max(s->fused_dp_ints, dp), bi = std::max(s->fused_bins, bins);
        if (s->fused && !D.dense && fused_dyn_bytes(dpi, bi, kMaxEngineThreads) <= kFusedDynMax &&
            s->slots[id].cost <= kFusedMaxCost) {
            fused_ids.push_back(id);
            s->fused_dp_ints = dpi;
            s->fused_bins = bi;
        }
    }
    std::stable_sort(fused_ids.begin(), fused_ids.end(),
                     [s](int a, int b) { return s->slots[a].cost > s->slots[b].cost; });
    {
        // When every fused engine gets its own CTA at launch (CTA b takes
        // item b) and SMs hold more than one CTA, the CTAs past the first wave
        // share SMs with the first: order that second part cheapest first, so
        // that the costliest engines share their SM with the cheapest ones.
        Context *c;
        FRMC_TRY(get_context(&c));
        const int wave = c->sms;
        if (s->ctas_per_sm > 1 && (int)fused_ids.size() > wave &&
            (long long)fused_ids.size() <= (long long)wave * s->ctas_per_sm)
            std::reverse(fused_ids.begin() + wave, fused_ids.end());
    }
    // a measured placement of the same engines and launch shape replaces it
    if (!s->place_order.empty()) {
        std::vector<int> a = fused_ids, b = s->place_order;
        std::sort(a.begin(), a.end());
        std::sort(b.begin(), b.end());
        if (a == b && s->place_key == place_key(s, (int)fused_ids.size()))
            fused_ids = s->place_order;
        else
            s->place_order.clear();
    }
    s->fused_item.assign(nslots, -1);
    for (int id : fused_ids) {
        s->fused_item[id] = (int)items.size();
        items.push_back(make_int2(id, -1));
    }
    s->nfused = (int)fused_ids.size();
    for (int id : s->live) {
        if (std::find(fused_ids.begin(), fused_ids.end(), id) != fused_ids.end())
            continue;
        const EDesc &D = s->slots[id].d;
        for (int t = 0; t < D.ntiles; ++t) items.push_back(make_int2(id, t));
    }
    s->nbatch = (int)items.size() - s->nsolo;
    if ((int)fused_ids.size() > s->fdesc_cap) {
        if (s->fdesc) cudaFree(s->fdesc);
        s->fdesc = nullptr;
        int cap = std::max((int)fused_ids.size(), 2 * s->fdesc_cap);
        FRMC_CUDA(cudaMalloc(&s->fdesc, sizeof(EDesc) * cap));
        if (s->fpos) cudaFree(s->fpos);
        s->fpos = nullptr;
        FRMC_CUDA(cudaMalloc(&s->fpos, sizeof(int) * cap));
        s->fdesc_cap = cap;
    }
    if (nslots > s->ddesc_cap) {
        if (s->ddesc) cudaFree(s->ddesc);
        s->ddesc = nullptr;
        int cap = std::max(nslots, 2 * s->ddesc_cap);
        FRMC_CUDA(cudaMalloc(&s->ddesc, sizeof(EDesc) * cap));
        s->ddesc_cap = cap;
    }
    if ((int)items.size() > s->items_cap) {
        if (s->items) cudaFree(s->items);
        s->items = nullptr;
        int cap = std::max((int)items.size(), 2 * s->items_cap);
        FRMC_CUDA(cudaMalloc(&s->items, sizeof(int2) * cap));
        s->items_cap = cap;
    }
    if ((int)s->live.size() > s->dlive_cap) {
        if (s->dlive) cudaFree(s->dlive);
        s->dlive = nullptr;
        int cap = std::max((int)s->live.size(), 2 * s->dlive_cap);
        FRMC_CUDA(cudaMalloc(&s->dlive, sizeof(int) * cap));
        s->dlive_cap = cap;
    }
    // S(Q) delta columns: each live engine with an S(Q) term owns npairs
    // adjacent fp16 columns of its table's X.  X is all zero between steps
    // (the finisher clears its columns), so columns can be dealt afresh here.
    s->sq_xcol.assign(nslots, -1);
    for (auto &t : s->tables) t.ncols = 0;
    for (int id : s->live) {
        Slot &sl = s->slots[id];
        if (!sl.d.sq)
            continue;
        SqTable &t = s->tables[sl.sq_table];
        s->sq_xcol[id] = t.ncols;
        t.ncols += sl.d.npairs;
    }
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    for (auto &t : s->tables) {
        if (t.ncols <= t.cap)
            continue;
        if (t.X) cudaFree(t.X);
        if (t.Zf) cudaFree(t.Zf);
        if (t.Zi) cudaFree(t.Zi);
        if (t.cmode) cudaFree(t.cmode);
        t.X = nullptr;
        t.Zf = nullptr;
        t.Zi = nullptr;
        t.cmode = nullptr;
        // at least one block's width, so that a column box never passes the end
        const int cap = std::max(std::max(t.ncols, 2 * t.cap), kSqCols);
        const size_t hsp = (size_t)t.hsp;
        FRMC_CUDA(cudaMalloc(&t.X, sizeof(__half) * hsp * cap));
        FRMC_CUDA(cudaMemset(t.X, 0, sizeof(__half) * hsp * cap));
        FRMC_CUDA(cudaMalloc(&t.Zf, sizeof(float) * kSqLimbs * hsp * cap));
        FRMC_CUDA(cudaMemset(t.Zf, 0, sizeof(float) * kSqLimbs * hsp * cap));
        FRMC_CUDA(cudaMalloc(&t.Zi, sizeof(long long) * hsp * cap));
        FRMC_CUDA(cudaMalloc(&t.cmode, sizeof(int) * cap));
        FRMC_CUDA(cudaMemset(t.cmode, 0, sizeof(int) * cap));
        t.cap = cap;
        FRMC_TRY(sq_encode_maps(t));
    }
    for (int id : s->live) {
        Slot &sl = s->slots[id];
        if (!sl.d.sq)
            continue;
        const SqTable &t = s->tables[sl.sq_table];
        const size_t col = (size_t)s->sq_xcol[id];
        sl.d.hsp = t.hsp;
        sl.d.xld = t.hsp;
        sl.d.X = t.X + col * t.hsp;
        sl.d.Zf = t.Zf + col * kSqRows;
        sl.d.zcap = t.cap;
        sl.d.Zi = t.Zi + col * t.hsp;
        sl.d.evn = t.cmode + col;
    }
    // S(Q) work lists.  Blocks of whole engines (at most kSqCols columns, in
    // live order) per table; the batched list is every block's tiles (row
    // blocks x K splits), then one commit per engine; each engine also gets a
    // block of its own and a list of its tiles and commit for steps of that
    // engine alone.  The K splits let a list's tiles about fill the SMs (one
    // CTA each): more splits shorten each tile's product but add partial
    // sums for L2 to reduce.
    s->sq_hblocks.clear();
    s->sq_hengs.clear();
    s->sq_host.clear();
    s->sq_first.assign(nslots, -1);
    s->sq_count.assign(nslots, 0);
    Context *ctx;
    FRMC_TRY(get_context(&ctx));
    auto splits = [&](long long rowblocks, int nk) {
        long long k = std::max<long long>(1, ctx->sms / std::max<long long>(1, rowblocks));
        if (s->sq_split_max > 0)
            k = std::min<long long>(k, s->sq_split_max);
        return (int)std::min<long long>(k, nk);
    };
    auto new_block = [&](const SqTable &t, int col0) {
        SqBlock b{};
        b.tm = t.maps;
        b.Zf = t.Zf;
        b.zcap = t.cap;
        b.Zi = t.Zi;
        b.cmode = t.cmode + col0;
        b.col0 = col0;
        b.hsp = t.hsp;
        b.hs = t.hs;
        b.nrb = (t.hs + kSqRows - 1) / kSqRows;
        b.nk = (t.hs + kSqK - 1) / kSqK;
        b.nsplit = 1;
        b.e0 = (int)s->sq_hengs.size();
        return b;
    };
    std::vector<int> block_of(nslots, -1);
    for (int ti = 0; ti < (int)s->tables.size(); ++ti) {
        const SqTable &t = s->tables[ti];
        SqBlock cur{};
        bool open = false;
        for (int id : s->live) {
            const Slot &sl = s->slots[id];
            if (!sl.d.sq || sl.sq_table != ti)
                continue;
            const int col = s->sq_xcol[id];
            if (open && col + sl.d.npairs - cur.col0 > kSqCols) {
                s->sq_hblocks.push_back(cur);
                open = false;
            }
            if (!open) {
                cur = new_block(t, col);
                open = true;
            }
            block_of[id] = (int)s->sq_hblocks.size();
            s->sq_hengs.push_back(sq_eng(sl.d, col - cur.col0));
            cur.neng += 1;
            cur.ncol = col + sl.d.npairs - cur.col0;
        }
        if (open)
            s->sq_hblocks.push_back(cur);
    }
    {
        long long rowblocks = 0;
        for (const auto &bk : s->sq_hblocks) rowblocks += bk.nrb;
        for (auto &bk : s->sq_hblocks) bk.nsplit = splits(rowblocks, bk.nk);
    }
    // row items: kSqThreads / kSqRows row blocks each
    constexpr int kRowsPerItem = kSqThreads / kSqRows;
    auto push_rows = [&](int id, int nrb, int ntiles) {
        int n = 0;
        for (int rb = 0; rb < nrb; rb += kRowsPerItem, ++n)
            s->sq_host.push_back(make_int4(1, id, (rb << 16) | std::min(kRowsPerItem, nrb - rb), ntiles));
        return n;
    };
    for (int bi = 0; bi < (int)s->sq_hblocks.size(); ++bi) {
        const SqBlock &bk = s->sq_hblocks[bi];
        for (int k = 0; k < bk.nrb * bk.nsplit; ++k) s->sq_host.push_back(make_int4(0, bi, k, 0));
    }
    std::vector<int> nrow(nslots, 0);
    for (int id : s->live)
        if (s->slots[id].d.sq) {
            const SqBlock &bk = s->sq_hblocks[block_of[id]];
            nrow[id] = push_rows(id, bk.nrb, bk.nrb * bk.nsplit);
        }
    for (int id : s->live)
        if (s->slots[id].d.sq)
            s->sq_host.push_back(make_int4(2, id, nrow[id], 0));
    s->sq_nbatch = (int)s->sq_host.size();
    for (int id : s->live) {
        const Slot &sl = s->slots[id];
        if (!sl.d.sq)
            continue;
        const SqTable &t = s->tables[sl.sq_table];
        const int bi = (int)s->sq_hblocks.size();
        SqBlock bk = new_block(t, s->sq_xcol[id]);
        bk.neng = 1;
        bk.ncol = sl.d.npairs;
        bk.nsplit = splits(bk.nrb, bk.nk);
        s->sq_hblocks.push_back(bk);
        s->sq_hengs.push_back(sq_eng(sl.d, 0));
        s->sq_first[id] = (int)s->sq_host.size();
        const int ntiles = bk.nrb * bk.nsplit;
        for (int k = 0; k < ntiles; ++k) s->sq_host.push_back(make_int4(0, bi, k, 0));
        const int nr = push_rows(id, bk.nrb, ntiles);
        s->sq_host.push_back(make_int4(2, id, nr, 0));
        s->sq_count[id] = ntiles + nr + 1;
    }
    if ((int)s->sq_host.size() > s->sq_cap) {
        if (s->sq_items) cudaFree(s->sq_items);
        s->sq_items = nullptr;
        const int cap = std::max((int)s->sq_host.size(), 2 * s->sq_cap);
        FRMC_CUDA(cudaMalloc(&s->sq_items, sizeof(int4) * cap));
        s->sq_cap = cap;
    }
    if ((int)s->sq_hblocks.size() > s->sq_blocks_cap) {
        if (s->sq_blocks) cudaFree(s->sq_blocks);
        s->sq_blocks = nullptr;
        const int cap = std::max((int)s->sq_hblocks.size(), 2 * s->sq_blocks_cap);
        FRMC_CUDA(cudaMalloc(&s->sq_blocks, sizeof(SqBlock) * cap));
        s->sq_blocks_cap = cap;
    }
    if ((int)s->sq_hengs.size() > s->sq_engs_cap) {
        if (s->sq_engs) cudaFree(s->sq_engs);
        s->sq_engs = nullptr;
        const int cap = std::max((int)s->sq_hengs.size(), 2 * s->sq_engs_cap);
        FRMC_CUDA(cudaMalloc(&s->sq_engs, sizeof(SqEng) * cap));
        s->sq_engs_cap = cap;
    }
    if (!s->sq_hblocks.empty())
        FRMC_CUDA(cudaMemcpy(s->sq_blocks, s->sq_hblocks.data(), sizeof(SqBlock) * s->sq_hblocks.size(),
                             cudaMemcpyHostToDevice));
    if (!s->sq_hengs.empty())
        FRMC_CUDA(cudaMemcpy(s->sq_engs, s->sq_hengs.data(), sizeof(SqEng) * s->sq_hengs.size(),
                             cudaMemcpyHostToDevice));
    std::vector<EDesc> hd(nslots);
    for (int k = 0; k < nslots; ++k) hd[k] = s->slots[k].d;
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    if (nslots)
        FRMC_CUDA(cudaMemcpy(s->ddesc, hd.data(), sizeof(EDesc) * nslots, cudaMemcpyHostToDevice));
    if (!fused_ids.empty()) {
        std::vector<EDesc> fd;
        fd.reserve(fused_ids.size());
        for (int id : fused_ids) fd.push_back(s->slots[id].d);
        FRMC_CUDA(cudaMemcpy(s->fdesc, fd.data(), sizeof(EDesc) * fd.size(), cudaMemcpyHostToDevice));
        std::vector<int> live_pos(nslots, -1), fp;
        for (int k = 0; k < (int)s->live.size(); ++k) live_pos[s->live[k]] = k;
        fp.reserve(fused_ids.size());
        for (int id : fused_ids) fp.push_back(live_pos[id]);
        FRMC_CUDA(cudaMemcpy(s->fpos, fp.data(), sizeof(int) * fp.size(), cudaMemcpyHostToDevice));
    }
    if (!items.empty())
        FRMC_CUDA(cudaMemcpy(s->items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice));
    if (!s->live.empty())
        FRMC_CUDA(cudaMemcpy(s->dlive, s->live.data(), sizeof(int) * s->live.size(), cudaMemcpyHostToDevice));
    if (!s->sq_host.empty())
        FRMC_CUDA(cudaMemcpy(s->sq_items, s->sq_host.data(), sizeof(int4) * s->sq_host.size(),
                             cudaMemcpyHostToDevice));
    s->nitems = (int)items.size();
    drop_graphs(s);
    s->dirty = false;
    return FRMC_OK;
}

static int launch_items(EngineSet *s, const int2 *items, int count, int eval_only, cudaStream_t st,
                        int dyn_smem = 0, bool fused = false, const EMove *hmoves = nullptr,
                        EResult *hres = nullptr, int threads = 0)
{
    if (threads <= 0)
        threads = s->threads;
    Context *c;
    FRMC_TRY(get_context(&c));
    int grid = c->sms * s->ctas_per_sm;
    if (grid > count)
        grid = count;
    if (grid < 1)
        return FRMC_OK;
    const long long first = items - (s->items + s->nsolo);
    const EDesc *fd = fused ? s->fdesc + first : nullptr;
    StepParams p{s->ddesc, fd, items, count, s->tile, eval_only, fused ? s->fused_dp_ints : 0,
                 fused ? s->fused_bins : 0, s->sched, nullptr, nullptr, nullptr, nullptr};
    if (fused && s->place_rec && count <= grid && first == 0 && count <= s->place_cap)
        p.place = s->place_dev;
    if (fused && hmoves) {
        p.hmoves = hmoves;
        p.hres = hres;
        p.fpos = s->fpos + first;
    }
    if (fused) {
        FRMC_CUDA(cudaFuncSetAttribute(k_engine_step<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem));
        // all shared memory: two CTAs of 256 threads fit one SM where their layouts do
        FRMC_CUDA(cudaFuncSetAttribute(k_engine_step<true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                       (int)cudaSharedmemCarveoutMaxShared));
        k_engine_step<true><<<grid, threads, dyn_smem, st>>>(p);
    } else {
        k_engine_step<false><<<grid, threads, 0, st>>>(p);
    }
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

// The S(Q) work list items [first, first + count): tiles, then commits.
static int launch_sq(EngineSet *s, int first, int count, cudaStream_t st)
{
    if (count <= 0)
        return FRMC_OK;
    Context *c;
    FRMC_TRY(get_context(&c));
    SqParams p{s->ddesc, s->sq_blocks, s->sq_engs, s->sq_items + first, count, s->sched + 1, &s->sched[0].status};
    FRMC_CUDA(cudaFuncSetAttribute(k_sq_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, kSqSmemBytes));
    // one CTA per SM: it holds the SM's shared-memory ring and all of its TMEM
    const int grid = std::min(count, c->sms);
    k_sq_fused<<<grid, kSqThreads, kSqSmemBytes, st>>>(p);
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

// Dynamic shared memory of a fused launch: element-pair deltas, A, Bq, the
// column queue and the per-bin non-zero counts.
static int fused_dyn_smem(const EngineSet *s)
{
    return (int)fused_dyn_bytes(s->fused_dp_ints, s->fused_bins, s->threads);
}

// The batched work list (every live engine advances one step): the fused
// engines in one launch, then the tiles of the split ones, then the S(Q)
// blocks of the engines that have an S(Q) term.
static int launch_batched(EngineSet *s, cudaStream_t st)
{
    if (s->nfused > 0)
        FRMC_TRY(launch_items(s, s->items + s->nsolo, s->nfused, 0, st, fused_dyn_smem(s), true));
    if (s->nbatch > s->nfused)
        FRMC_TRY(launch_items(s, s->items + s->nsolo + s->nfused, s->nbatch - s->nfused, 0, st));
    FRMC_TRY(launch_sq(s, 0, s->sq_nbatch, st));
    return FRMC_OK;
}

static int launch_sq_eval(EngineSet *s, int id, int commit, cudaStream_t st)
{
    const EDesc &D = s->slots[id].d;
    k_sq_gs<<<1, 512, 0, st>>>(s->ddesc, id);
    k_sq_sv<<<(D.nq + 127) / 128, 128, 0, st>>>(s->ddesc, id);
    if (commit) {
        k_sq_hv<<<(D.hs + 7) / 8, 256, 0, st>>>(s->ddesc, id);
        k_sq_sd<<<1, 512, 0, st>>>(s->ddesc, id);
    }
    FRMC_CUDA(cudaGetLastError());
    return FRMC_OK;
}

// All-pairs counts and initial chi2 of engine `id` (synchronous).
static int init_engine(EngineSet *s, int id)
{
    Context *c;
    FRMC_TRY(get_context(&c));
    EDesc &D = s->slots[id].d;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        FRMC_TRY(c->buf[BUF_STATUS].ensure(16));
        FRMC_TRY(c->buf[BUF_AUX0].ensure(12 * (size_t)D.n + 16));
        FRMC_TRY(c->buf[BUF_AUX1].ensure(4 * (size_t)D.n + 16));
    }
    FRMC_CUDA(cudaMemsetAsync(c->buf[BUF_STATUS].p, 0, 4, s->stream));
    FRMC_CUDA(cudaMemsetAsync(D.counts, 0, sizeof(int) * 2 * D.total, s->stream));
    FRMC_CUDA(cudaMemsetAsync(D.delta, 0, sizeof(int) * 2 * D.total, s->stream));
    FRMC_CUDA(cudaMemsetAsync(D.st, 0, sizeof(EState), s->stream));
    FRMC_CUDA(cudaMemsetAsync(&D.st->nx_step, 0xff, sizeof(long long), s->stream));  // no staged move
    unsigned *cnt = (unsigned *)D.counts;
    FullTune tn;
    if (D.n >= 2) {
        const double pairs = 0.5 * (double)D.n * (D.n - 1);
        if (pairs < tn.min_pairs_tiled) {
            // the row kernel reads AoS float coordinates: unpack once
            std::lock_guard<std::mutex> lk(c->mu);
            FRMC_TRY(launch_unpack_atoms(D.box, D.n, c->buf[BUF_AUX0].as<float>(), c->buf[BUF_AUX1].as<int>(),
                                         s->stream));
            FRMC_TRY(launch_rows_hist(c->buf[BUF_AUX0].as<float>(), c->buf[BUF_AUX1].as<int>(), D.mol, D.n, nullptr,
                                      D.n, 0, D.bm, D.B, D.minD, D.maxD, D.binw, D.ne, D.hs, cnt, cnt + D.total,
                                      s->stream));
            FRMC_CUDA(cudaStreamSynchronize(s->stream));
        } else {
            FRMC_TRY(launch_full_hist(D.box, D.mol, D.n, D.bm, D.B, D.minD, D.maxD, D.binw, D.ne, D.hs, cnt,
                                      cnt + D.total, c->buf[BUF_STATUS].as<uint32_t>(), 0.05, &tn, s->stream));
        }
    }
    FRMC_TRY(refresh(s));
    int2 item = make_int2(id, 0);
    int2 *ditem = nullptr;
    FRMC_CUDA(cudaMalloc(&ditem, sizeof(int2)));
    FRMC_CUDA(cudaMemcpyAsync(ditem, &item, sizeof(int2), cudaMemcpyHostToDevice, s->stream));
    int rc = launch_items(s, ditem, 1, 1, s->stream);
    if (!rc && D.sq)
        rc = launch_sq_eval(s, id, 1, s->stream);
    cudaError_t ce = cudaStreamSynchronize(s->stream);
    cudaFree(ditem);
    if (rc)
        return rc;
    if (ce != cudaSuccess)
        return cuda_fail(ce, "engine init");
    uint32_t status = 0;
    FRMC_CUDA(cudaMemcpy(&status, c->buf[BUF_STATUS].p, 4, cudaMemcpyDeviceToHost));
    if (status)
        return set_error(FRMC_E_TIMEOUT, "engine init: device wait gave up (0x%x)", status);
    s->slots[id].initialized = true;
    return FRMC_OK;
}

// Column grid of an engine (the cell fields of EDesc): the atoms sorted by
// cell of a grid over the range of their box coordinates, with cells of at
// least maxD / 2 across in real space and at most kMaxCells of them; no grid
// where a moved atom would reach most cells anyway.  The distance bound's
// margin (1e-2 A + 1e-4 maxD + a few float32 ulps of the coordinates) is far
// above the float32 rounding of the reference's distance.
struct CellGrid {
    int nc = 0, cmode = 0, cpbc = 0;
    double sweep = 0.0;  // estimated columns a step sweeps (the mean over sample atoms)
    float cw[3] = {1.f, 1.f, 1.f}, clam2 = 0.f, cthr2 = 0.f;
    std::vector<float4> cbox, clo, chi;
    std::vector<int> cmol, cstart;
    std::vector<int2> csl;
};

// Per-axis factors and smallest eigenvalue of the distance bound (see the
// cell fields of EDesc): for a box, w_k = 1 / |column k of B^-1| (cmode 1)
// or |B_kk| for an orthorhombic box (cmode 0); free boundaries: w = 1.
// Returns false for a singular basis.
static bool cell_metric(const float *basis, int bm, double w[3], double *lam, int *mode)
{
    w[0] = w[1] = w[2] = 1.0;
    *lam = 0.0;
    *mode = 0;
    if (bm == BM_IBC)
        return true;
    double B[9];
    for (int k = 0; k < 9; ++k) B[k] = basis[k];
    if (bm == BM_DIAG) {
        for (int k = 0; k < 3; ++k) w[k] = std::fabs(B[4 * k]);
        return w[0] > 0.0 && w[1] > 0.0 && w[2] > 0.0;
    }
    *mode = 1;
    // columns of B^-1 (box = real B^-1): |real| >= |box_k| / |column k|
    const double c00 = B[4] * B[8] - B[5] * B[7], c01 = B[5] * B[6] - B[3] * B[8], c02 = B[3] * B[7] - B[4] * B[6];
    const double det = B[0] * c00 + B[1] * c01 + B[2] * c02;
    if (!(std::fabs(det) > 0.0))
        return false;
    double I[9];  // I[r*3 + c] = (B^-1)[r][c]
    I[0] = c00 / det;
    I[1] = (B[2] * B[7] - B[1] * B[8]) / det;
    I[2] = (B[1] * B[5] - B[2] * B[4]) / det;
    I[3] = c01 / det;
    I[4] = (B[0] * B[8] - B[2] * B[6]) / det;
    I[5] = (B[2] * B[3] - B[0] * B[5]) / det;
    I[6] = c02 / det;
    I[7] = (B[1] * B[6] - B[0] * B[7]) / det;
    I[8] = (B[0] * B[4] - B[1] * B[3]) / det;
    for (int k = 0; k < 3; ++k) w[k] = 1.0 / std::sqrt(I[k] * I[k] + I[3 + k] * I[3 + k] + I[6 + k] * I[6 + k]);
    // smallest eigenvalue of M = B B^T (|real|^2 = box M box^T), by the
    // trigonometric solution of the symmetric 3 x 3 eigenproblem
    double M[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            M[3 * i + j] = B[3 * i] * B[3 * j] + B[3 * i + 1] * B[3 * j + 1] + B[3 * i + 2] * B[3 * j + 2];
    const double p1 = M[1] * M[1] + M[2] * M[2] + M[5] * M[5];
    double l;
    if (p1 == 0.0) {
        l = std::min(M[0], std::min(M[4], M[8]));
    } else {
        const double q = (M[0] + M[4] + M[8]) / 3.0;
        const double p2 = (M[0] - q) * (M[0] - q) + (M[4] - q) * (M[4] - q) + (M[8] - q) * (M[8] - q) + 2 * p1;
        const double pp = std::sqrt(p2 / 6.0);
        double Q[9];
        for (int k = 0; k < 9; ++k) Q[k] = (M[k] - (k % 4 == 0 ? q : 0.0)) / pp;
        double r = 0.5 * (Q[0] * (Q[4] * Q[8] - Q[5] * Q[7]) - Q[1] * (Q[3] * Q[8] - Q[5] * Q[6]) +
                          Q[2] * (Q[3] * Q[7] - Q[4] * Q[6]));
        r = std::max(-1.0, std::min(1.0, r));
        l = q + 2.0 * pp * std::cos(std::acos(r) / 3.0 + 2.0 * M_PI / 3.0);
    }
    *lam = std::max(0.0, 0.999 * l);
    return true;
}

static void build_cells(const frmc_engine_spec &sp, int bm, CellGrid &G)
{
    const int n = sp.n;
    const bool pbc = bm != BM_IBC;
    double w[3], lam;
    int mode;
    if (!cell_metric(sp.basis, bm, w, &lam, &mode))
        return;
    double lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = INFINITY;
        hi[k] = -INFINITY;
    }
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            const double x = sp.box_coords[3 * (size_t)i + k];
            lo[k] = std::min(lo[k], x);
            hi[k] = std::max(hi[k], x);
        }
    const double maxD = sp.maxDistance;
    if (!(maxD > 0.0) || !std::isfinite(lo[0] + lo[1] + lo[2] + hi[0] + hi[1] + hi[2]))
        return;
    double ext[3], vol = 1.0;
    int nk[3];
    const double Lc = std::max(0.5 * maxD, 1e-3);
    for (int k = 0; k < 3; ++k) {
        ext[k] = (hi[k] - lo[k]) * w[k];
        nk[k] = (int)std::max(1.0, std::min(64.0, std::floor(ext[k] / Lc)));
        vol *= std::max(ext[k], 1e-9);
    }
    while (nk[0] * nk[1] * nk[2] > kMaxCells) {
        int k = nk[0] >= nk[1] && nk[0] >= nk[2] ? 0 : (nk[1] >= nk[2] ? 1 : 2);
        --nk[k];
    }
    const int nc = nk[0] * nk[1] * nk[2];
    double diag2 = 0.0;
    for (int k = 0; k < 3; ++k) diag2 += (ext[k] / nk[k]) * (ext[k] / nk[k]);
    const double R = (maxD + 0.5 * std::sqrt(diag2)) * (mode ? 1.1 : 1.0);
    if (nc < 8 || 4.0 / 3.0 * M_PI * R * R * R > 0.6 * vol)
        return;
    std::vector<int> cell(n), count(nc + 1, 0);
    for (int i = 0; i < n; ++i) {
        int ck[3];
        for (int k = 0; k < 3; ++k) {
            const double span = hi[k] - lo[k];
            const double x = sp.box_coords[3 * (size_t)i + k];
            int c = span > 0.0 ? (int)std::floor((x - lo[k]) / span * nk[k]) : 0;
            ck[k] = std::max(0, std::min(nk[k] - 1, c));
        }
        cell[i] = ck[0] + nk[0] * (ck[1] + nk[1] * ck[2]);
        ++count[cell[i]];
    }
    G.cstart.assign(nc + 1, 0);
    for (int c = 0; c < nc; ++c) G.cstart[c + 1] = G.cstart[c] + count[c];
    std::vector<int> fill(G.cstart.begin(), G.cstart.end() - 1);
    G.cbox.resize(n);
    G.cmol.resize(n);
    G.csl.resize(n);
    G.clo.assign(nc, make_float4(INFINITY, INFINITY, INFINITY, 0.f));
    G.chi.assign(nc, make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f));
    for (int i = 0; i < n; ++i) {
        const int c = cell[i], pos = fill[c]++;
        const float x = sp.box_coords[3 * (size_t)i], y = sp.box_coords[3 * (size_t)i + 1],
                    z = sp.box_coords[3 * (size_t)i + 2];
        G.cbox[pos] = make_float4(x, y, z, int_bits_as_float(sp.el[i]));
        G.cmol[pos] = sp.mol[i];
        G.csl[i] = make_int2(pos, c);
        float4 &l = G.clo[c], &h = G.chi[c];
        l.x = std::min(l.x, x); l.y = std::min(l.y, y); l.z = std::min(l.z, z);
        h.x = std::max(h.x, x); h.y = std::max(h.y, y); h.z = std::max(h.z, z);
    }
    for (int c = 0; c < nc; ++c)
        if (!count[c]) {
            G.clo[c] = make_float4(0.f, 0.f, 0.f, 0.f);
            G.chi[c] = G.clo[c];
        }
    double slack = 0.0;
    for (int k = 0; k < 3; ++k) slack += w[k] * std::max(1.0, std::max(std::fabs(lo[k]), std::fabs(hi[k])));
    const double thr = maxD * (1.0 + 1e-4) + 1e-2 + 4e-6 * slack;
    G.nc = nc;
    G.cmode = mode;
    G.cpbc = pbc ? 1 : 0;
    for (int k = 0; k < 3; ++k) G.cw[k] = (float)w[k];
    G.clam2 = (float)lam;
    G.cthr2 = (float)(thr * thr);
    // the columns a step would sweep, averaged over up to 32 atoms taken as
    // the moved atom (the device's test, in double)
    const int ns = std::min(n, 32);
    double sum = 0.0;
    for (int k = 0; k < ns; ++k) {
        const int i = (int)((long long)k * n / ns);
        const double p[3] = {sp.box_coords[3 * (size_t)i], sp.box_coords[3 * (size_t)i + 1],
                             sp.box_coords[3 * (size_t)i + 2]};
        for (int c = 0; c < nc; ++c) {
            if (!count[c])
                continue;
            const double clo[3] = {G.clo[c].x, G.clo[c].y, G.clo[c].z}, chi[3] = {G.chi[c].x, G.chi[c].y, G.chi[c].z};
            double f[3], lb2 = 0.0, mx = 0.0, f2 = 0.0;
            for (int a = 0; a < 3; ++a) {
                const double lo_d = p[a] - chi[a], hi_d = p[a] - clo[a];
                if (!pbc) {
                    f[a] = lo_d > 0 ? lo_d : (hi_d < 0 ? -hi_d : 0.0);
                } else {
                    const double nn = std::floor(hi_d);
                    f[a] = nn >= lo_d ? 0.0 : std::min(lo_d - nn, nn + 1.0 - hi_d);
                }
                const double m = f[a] * w[a];
                lb2 += m * m;
                mx = std::max(mx, m * m);
                f2 += f[a] * f[a];
            }
            if (mode != 0)
                lb2 = std::max(mx, lam * f2);
            if (lb2 < thr * thr)
                sum += count[c];
        }
    }
    G.sweep = sum / ns;
}

static int add_engine(EngineSet *s, const frmc_engine_spec &sp, int *out_id)
{
    FRMC_TRY(check_spec(sp));
    const SqTable *tab = nullptr;
    if (sp.sq_table >= 0) {
        if (sp.sq_table >= (int)s->tables.size())
            return set_error(FRMC_E_ARG, "engine spec: unknown S(Q) table %d", sp.sq_table);
        tab = &s->tables[sp.sq_table];
        if (tab->hs != sp.hs || tab->nq != sp.nq)
            return set_error(FRMC_E_ARG, "engine spec: S(Q) table %d is %d x %d, the engine needs %d x %d",
                             sp.sq_table, tab->hs, tab->nq, sp.hs, sp.nq);
    }
    BlobLayout L = blob_layout(sp);
    Slot sl;
    FRMC_CUDA(cudaMalloc(&sl.blob, L.total));
    sl.bytes = L.total;
    char *b = (char *)sl.blob;
    EDesc &D = sl.d;
    memset(&D, 0, sizeof(D));
    D.n = sp.n;
    D.ne = sp.ne;
    D.hs = sp.hs;
    D.npairs = sp.npairs;
    D.move_cap = sp.move_cap;
    D.bm = sp.isPBC ? basis_mode(sp.basis, 1) : BM_IBC;
    D.B = make_basis(sp.isPBC ? sp.basis : nullptr);
    D.RB = make_basis(sp.isPBC ? sp.rbasis : nullptr);
    D.minD = sp.minDistance;
    D.maxD = sp.maxDistance;
    D.binw = sp.bin;
    sq_limits(sp.minDistance, sp.maxDistance, &D.s_lo, &D.s_hi);
    D.total = (long long)sp.ne * sp.ne * sp.hs;
    D.var2 = sp.variance_squared;
    D.tol = sp.tolerance;
    D.has_dw = sp.data_weights ? 1 : 0;
    {
        const long long G = spec_group(sp);
        D.dpk = (long long)sp.n * G + G * G < 32000 ? 1 : 0;
    }
    D.box = (float4 *)(b + L.box);
    D.real = (float4 *)(b + L.real);
    D.mol = (int *)(b + L.mol);
    D.counts = (int *)(b + L.counts);
    D.delta = (int *)(b + L.delta);
    D.rfac = (double *)(b + L.rfac);
    D.invvol = (double *)(b + L.invvol);
    D.expd = (double *)(b + L.expd);
    D.dw = (double *)(b + L.dw);
    D.pc = (double *)(b + L.pc);
    D.pi = (int *)(b + L.pi);
    D.pj = (int *)(b + L.pj);
    D.dP = (int *)(b + L.dP);
    D.pidx = (int *)(b + L.pidx);
    D.tlist = (int *)(b + L.tlist);
    D.R = (double *)(b + L.R);
    D.A = (double *)(b + L.A);
    D.Bq = (double *)(b + L.Bq);
    D.Sb = (double *)(b + L.Sb);
    if (spec_dense(sp)) {
        D.dense = 1;
        D.wlen = sp.window_len;
        D.fit_freq = sp.fit_frequency;
        D.sf0 = spec_scale(sp);
        D.fit_min = sp.fit_min;
        D.fit_max = sp.fit_max;
        D.Gc = (double *)(b + L.Gc);
        D.fnum = (double *)(b + L.fnum);
        D.fden = (double *)(b + L.fden);
        D.win = (double *)(b + L.win);
    }
    D.moves = (EMove *)(b + L.moves);
    D.group = spec_group(sp);
    D.groups = D.group > 1 ? (EGroup *)(b + L.groups) : nullptr;
    D.results = (EResult *)(b + L.results);
    D.st = (EState *)(b + L.st);
    CellGrid cg;
    if (s->cells)
        build_cells(sp, D.bm, cg);
    D.nc = cg.nc;
    D.cmode = cg.cmode;
    D.cpbc = cg.cpbc;
    for (int k = 0; k < 3; ++k) D.cw[k] = cg.cw[k];
    D.clam2 = cg.clam2;
    D.cthr2 = cg.cthr2;
    D.cbox = (float4 *)(b + L.cbox);
    D.cmol = (int *)(b + L.cmol);
    D.csl = (int2 *)(b + L.csl);
    D.cstart = (int *)(b + L.cstart);
    D.clo = (float4 *)(b + L.clo);
    D.chi = (float4 *)(b + L.chi);
    std::vector<double> Rqt;
    if (tab) {
        D.sq = 1;
        D.nq = sp.nq;
        D.var2q = sp.sq_variance_squared;
        D.M = tab->M;
        D.T = tab->T;
        D.sq_gemm_max = kSqGemmMaxDelta;
        D.wq = tab->w;
        D.yscale = std::ldexp(sp.sq_rho0, -tab->s);
        D.Rq = (double *)(b + L.Rq);
        D.rfacq = (double *)(b + L.rfacq);
        D.sqexp = (double *)(b + L.sqexp);
        D.h = (double *)(b + L.h);
        D.y = (double *)(b + L.y);
        D.gsq = (double *)(b + L.gsq);
        D.sqpart = (double *)(b + L.sqpart);
        D.sqv = (double *)(b + L.sqv);
        D.evl = (int *)(b + L.evl);
        Rqt.resize(sp.hs);
        for (int bb = 0; bb < sp.hs; ++bb) Rqt[bb] = sp.sq_rfac[bb] * sp.sq_inv_shell_volume[bb];
    }
    std::vector<int> pidx((size_t)sp.ne * sp.ne, -1);
    for (int q = 0; q < sp.npairs; ++q) {
        pidx[(size_t)sp.pair_i[q] * sp.ne + sp.pair_j[q]] = q;
        pidx[(size_t)sp.pair_j[q] * sp.ne + sp.pair_i[q]] = q;
    }
    std::vector<double> Rt(sp.hs), At(sp.hs);
    for (int bb = 0; bb < sp.hs; ++bb) {
        Rt[bb] = sp.rfac[bb] * sp.inv_shell_volume[bb];
        const double w = sp.data_weights ? sp.data_weights[bb] : 1.0;
        At[bb] = w * Rt[bb] * Rt[bb];
    }
    std::vector<float4> b4(sp.n), r4(sp.n);
    for (int i = 0; i < sp.n; ++i) {
        b4[i] = make_float4(sp.box_coords[3 * i], sp.box_coords[3 * i + 1], sp.box_coords[3 * i + 2],
                            int_bits_as_float(sp.el[i]));
        r4[i] = make_float4(sp.real_coords[3 * i], sp.real_coords[3 * i + 1], sp.real_coords[3 * i + 2], 0.f);
    }
    int rc = FRMC_OK;
    auto up = [&](void *dst, const void *src, size_t bytes) {
        if (rc || !bytes)
            return;
        cudaError_t ce = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s->stream);
        if (ce != cudaSuccess)
            rc = cuda_fail(ce, "cudaMemcpyAsync");
    };
    up(D.box, b4.data(), 16 * (size_t)sp.n);
    up(D.real, r4.data(), 16 * (size_t)sp.n);
    up(D.mol, sp.mol, 4 * (size_t)sp.n);
    up(D.rfac, sp.rfac, 8 * (size_t)sp.hs);
    up(D.invvol, sp.inv_shell_volume, 8 * (size_t)sp.hs);
    up(D.expd, sp.experimental, 8 * (size_t)sp.hs);
    if (sp.data_weights)
        up(D.dw, sp.data_weights, 8 * (size_t)sp.hs);
    up(D.pc, sp.pair_coef, 8 * (size_t)sp.npairs);
    up(D.pi, sp.pair_i, 4 * (size_t)sp.npairs);
    up(D.pj, sp.pair_j, 4 * (size_t)sp.npairs);
    up(D.pidx, pidx.data(), 4 * pidx.size());
    up(D.R, Rt.data(), 8 * Rt.size());
    up(D.A, At.data(), 8 * At.size());
    if (cg.nc > 0) {
        up(D.cbox, cg.cbox.data(), 16 * cg.cbox.size());
        up(D.cmol, cg.cmol.data(), 4 * cg.cmol.size());
        up(D.csl, cg.csl.data(), 8 * cg.csl.size());
        up(D.cstart, cg.cstart.data(), 4 * cg.cstart.size());
        up(D.clo, cg.clo.data(), 16 * cg.clo.size());
        up(D.chi, cg.chi.data(), 16 * cg.chi.size());
    }
    std::vector<double> fden;
    if (D.dense) {
        fden.assign(sp.hs, 1.0);
        if (sp.fit_den)
            for (int bb = 0; bb < sp.hs; ++bb) fden[bb] = sp.fit_den[bb];
        if (sp.fit_num)
            up(D.fnum, sp.fit_num, 8 * (size_t)sp.hs);
        up(D.fden, fden.data(), 8 * fden.size());
        if (sp.window_len > 0)
            up(D.win, sp.window, 8 * (size_t)sp.window_len);
    }
    if (tab) {
        up(D.Rq, Rqt.data(), 8 * Rqt.size());
        up(D.rfacq, sp.sq_rfac, 8 * (size_t)sp.hs);
        up(D.sqexp, sp.sq_experimental, 8 * (size_t)sp.nq);
    }
    if (!rc) {
        cudaError_t ce = cudaMemsetAsync(D.moves, 0, sizeof(EMove) * sp.move_cap, s->stream);
        if (ce == cudaSuccess)
            ce = cudaMemsetAsync(D.dP, 0, 4 * (size_t)sp.npairs * sp.hs, s->stream);
        if (ce == cudaSuccess)
            ce = cudaMemsetAsync(D.results, 0, sizeof(EResult) * sp.move_cap, s->stream);
        if (ce == cudaSuccess && D.groups)
            ce = cudaMemsetAsync(D.groups, 0, sizeof(EGroup) * sp.move_cap, s->stream);
        if (ce == cudaSuccess)
            ce = cudaStreamSynchronize(s->stream);
        if (ce != cudaSuccess)
            rc = cuda_fail(ce, "engine upload");
    }
    if (rc) {
        cudaFree(sl.blob);
        return rc;
    }
    // reuse a free slot id if any
    int id = -1;
    for (int k = 0; k < (int)s->slots.size(); ++k)
        if (!s->slots[k].live && !s->slots[k].blob) {
            id = k;
            break;
        }
    if (id < 0) {
        id = (int)s->slots.size();
        s->slots.push_back(Slot());
    }
    sl.live = true;
    sl.sq_table = sp.sq_table;
    sl.cost = (cg.nc > 0 ? 4 * (long long)std::ceil(cg.sweep) : (long long)sp.n) * spec_group(sp);
    s->slots[id] = sl;
    s->live.push_back(id);
    std::sort(s->live.begin(), s->live.end());
    s->dirty = true;
    *out_id = id;
    return FRMC_OK;
}

static void free_set(EngineSet *s)
{
    if (s->stream)
        cudaStreamSynchronize(s->stream);
    drop_graphs(s);
    for (auto &sl : s->slots)
        if (sl.blob) cudaFree(sl.blob);
    for (auto &t : s->tables) {
        if (t.blob) cudaFree(t.blob);
        if (t.TD) cudaFree(t.TD);
        if (t.X) cudaFree(t.X);
        if (t.Zf) cudaFree(t.Zf);
        if (t.Zi) cudaFree(t.Zi);
        if (t.cmode) cudaFree(t.cmode);
        if (t.maps) cudaFree(t.maps);
    }
    void *ptrs[] = {s->ddesc, s->fdesc,    s->fpos,      s->items,    s->dlive,
                    s->sched, s->sq_items, s->sq_blocks, s->sq_engs,  s->place_dev};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (int k = 0; k < 2; ++k) {
        if (s->dstage_m[k]) cudaFree(s->dstage_m[k]);
        if (s->dstage_r[k]) cudaFree(s->dstage_r[k]);
        if (s->hstage_m[k]) cudaFreeHost(s->hstage_m[k]);
        if (s->hstage_r[k]) cudaFreeHost(s->hstage_r[k]);
        if (s->stage_ev[k]) cudaEventDestroy(s->stage_ev[k]);
    }
    if (s->stream)
        cudaStreamDestroy(s->stream);
    delete s;
}

static EngineSet *as_set(void *h) { return (EngineSet *)h; }

static bool valid_id(EngineSet *s, int e) { return e >= 0 && e < (int)s->slots.size() && s->slots[e].live; }

}  // namespace frmc

using namespace frmc;

extern "C" {

int frmc_engine_footprint(const frmc_engine_spec *spec, int64_t *bytes)
{
    if (!spec || !bytes)
        return set_error(FRMC_E_ARG, "engine_footprint: null argument");
    int64_t b = (int64_t)blob_layout(*spec).total;
    if (spec->sq_table >= 0) {
        // the engine's columns of its table's fp16 deltas, fp32 digit
        // products and exact products (counted twice: the shared buffers grow
        // by doubling)
        const int64_t hsp = (spec->hs + kSqRows - 1) / kSqRows * kSqRows;
        b += 2 * (int64_t)spec->npairs *
             (hsp * (int64_t)(sizeof(__half) + kSqLimbs * sizeof(float) + sizeof(long long)) + 4);
    }
    *bytes = b;
    return FRMC_OK;
}

int frmc_engines_new(void **handle)
{
    if (!handle)
        return set_error(FRMC_E_ARG, "engines_new: null handle");
    Context *c;
    FRMC_TRY(get_context(&c));
    EngineSet *s = new EngineSet();
    cudaError_t ce = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess)
        ce = cudaMalloc(&s->sched, 2 * sizeof(Sched));
    if (ce == cudaSuccess)
        ce = cudaMemset(s->sched, 0, 2 * sizeof(Sched));
    if (ce != cudaSuccess) {
        free_set(s);
        return cuda_fail(ce, "engine set");
    }
    *handle = s;
    return FRMC_OK;
}

int frmc_engines_create(const frmc_engine_spec *specs, int32_t E, void **handle)
{
    if (!specs || E <= 0 || !handle)
        return set_error(FRMC_E_ARG, "engines_create: need at least one spec");
    for (int e = 0; e < E; ++e) FRMC_TRY(check_spec(specs[e]));
    void *h = nullptr;
    FRMC_TRY(frmc_engines_new(&h));
    EngineSet *s = as_set(h);
    for (int e = 0; e < E; ++e) {
        int id;
        int rc = add_engine(s, specs[e], &id);
        if (rc) {
            free_set(s);
            return rc;
        }
    }
    *handle = s;
    return FRMC_OK;
}

int frmc_engines_add(void *handle, const frmc_engine_spec *spec, int32_t *id)
{
    EngineSet *s = as_set(handle);
    if (!s || !spec || !id)
        return set_error(FRMC_E_ARG, "engines_add: null argument");
    if (s->stage_busy[0] || s->stage_busy[1])
        return set_error(FRMC_E_STATE, "engines_add: a host step is in flight; collect it first");
    int k;
    FRMC_TRY(add_engine(s, *spec, &k));
    int rc = init_engine(s, k);
    if (rc) {
        frmc_engines_remove(handle, k);
        return rc;
    }
    *id = k;
    return FRMC_OK;
}

int frmc_engines_remove(void *handle, int32_t id)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, id))
        return set_error(FRMC_E_ARG, "engines_remove: invalid engine %d", id);
    if (s->stage_busy[0] || s->stage_busy[1])
        return set_error(FRMC_E_STATE, "engines_remove: a host step is in flight; collect it first");
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    FRMC_CUDA(cudaDeviceSynchronize());
    cudaFree(s->slots[id].blob);
    s->slots[id] = Slot();
    s->live.erase(std::remove(s->live.begin(), s->live.end(), id), s->live.end());
    s->dirty = true;
    return FRMC_OK;
}

int frmc_engines_live(void *handle, int32_t *ids, int32_t cap, int32_t *count)
{
    EngineSet *s = as_set(handle);
    if (!s || !count)
        return set_error(FRMC_E_ARG, "engines_live: null argument");
    *count = (int32_t)s->live.size();
    for (int k = 0; k < (int)s->live.size() && k < cap; ++k) ids[k] = s->live[k];
    return FRMC_OK;
}

int frmc_engines_destroy(void *handle)
{
    if (handle)
        free_set(as_set(handle));
    return FRMC_OK;
}

int frmc_engines_set_tune(void *handle, int tile, int threads, int ctas_per_sm)
{
    EngineSet *s = as_set(handle);
    if (!s || tile < 32 || threads < 32 || threads > kMaxEngineThreads || threads % 32 || ctas_per_sm < 1 ||
        ctas_per_sm > 32)
        return set_error(FRMC_E_ARG, "engines_set_tune: threads must be a multiple of 32 in [32, %d]",
                         kMaxEngineThreads);
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    s->tile = tile;
    s->threads = threads;
    s->ctas_per_sm = ctas_per_sm;
    s->dirty = true;
    return refresh(s);
}

int frmc_engines_set_sq_gemm_limit(void *handle, int32_t limit)
{
    EngineSet *s = as_set(handle);
    if (!s || limit < -1 || limit > kSqGemmMaxDelta)
        return set_error(FRMC_E_ARG, "engines_set_sq_gemm_limit: limit must be in [-1, %d]", kSqGemmMaxDelta);
    for (auto &sl : s->slots) sl.d.sq_gemm_max = limit;
    s->dirty = true;
    return FRMC_OK;
}

int frmc_engines_set_sq_splits(void *handle, int32_t max_splits)
{
    EngineSet *s = as_set(handle);
    if (!s || max_splits < 0)
        return set_error(FRMC_E_ARG, "engines_set_sq_splits: need max_splits >= 0");
    s->sq_split_max = max_splits;
    s->dirty = true;
    return FRMC_OK;
}

int frmc_engines_set_cells(void *handle, int32_t on)
{
    EngineSet *s = as_set(handle);
    if (!s)
        return set_error(FRMC_E_ARG, "null handle");
    s->cells = on ? 1 : 0;
    return FRMC_OK;
}

int frmc_engines_cells(void *handle, int32_t e, int32_t *ncells, int64_t *swept)
{
    EngineSet *s = as_set(handle);
    if (!s || !ncells)
        return set_error(FRMC_E_ARG, "null argument");
    if (e < 0 || e >= (int)s->slots.size() || !s->slots[e].live)
        return set_error(FRMC_E_ARG, "engines_cells: no engine %d", e);
    *ncells = s->slots[e].d.nc;
    if (swept) {
        FRMC_CUDA(cudaStreamSynchronize(s->stream));
        EState S;
        FRMC_CUDA(cudaMemcpy(&S, s->slots[e].d.st, sizeof(EState), cudaMemcpyDeviceToHost));
        *swept = (int64_t)S.swept;
    }
    return FRMC_OK;
}

int frmc_engines_set_mode(void *handle, int fused)
{
    EngineSet *s = as_set(handle);
    if (!s)
        return set_error(FRMC_E_ARG, "null handle");
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    s->fused = fused ? 1 : 0;
    s->dirty = true;
    return refresh(s);
}

int frmc_engines_get_tune(void *handle, int *tile, int *threads, int *ctas_per_sm, int *nitems)
{
    EngineSet *s = as_set(handle);
    if (!s)
        return set_error(FRMC_E_ARG, "null handle");
    FRMC_TRY(refresh(s));
    if (tile) *tile = s->tile;
    if (threads) *threads = s->threads;
    if (ctas_per_sm) *ctas_per_sm = s->ctas_per_sm;
    if (nitems) *nitems = s->nbatch;
    return FRMC_OK;
}

int frmc_engines_init(void *handle)
{
    EngineSet *s = as_set(handle);
    if (!s)
        return set_error(FRMC_E_ARG, "null handle");
    for (int id : std::vector<int>(s->live))
        if (!s->slots[id].initialized)
            FRMC_TRY(init_engine(s, id));
    return FRMC_OK;
}

int frmc_engines_push_moves(void *handle, int32_t e, const int32_t *atoms, const float *vecs, const float *u,
                            int32_t count, int64_t first_step, int from_device)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, e) || count < 0 || first_step < 0 || from_device)
        return set_error(FRMC_E_ARG, "push_moves: invalid arguments");
    const EDesc &D = s->slots[e].d;
    if (D.group > 1)
        return set_error(FRMC_E_ARG, "push_moves: engine %d moves groups of %d atoms (frmc_engines_push_group_moves)",
                         e, D.group);
    if (count > D.move_cap)
        return set_error(FRMC_E_ARG, "push_moves: %d moves exceed the ring of %d", count, D.move_cap);
    for (int k = 0; k < count; ++k)
        if (atoms[k] < 0 || atoms[k] >= D.n)
            return set_error(FRMC_E_INDEX, "push_moves: atom %d out of range", atoms[k]);
    std::vector<EMove> mv(count);
    for (int k = 0; k < count; ++k) {
        mv[k].atom = atoms[k];
        mv[k].v[0] = vecs[3 * k];
        mv[k].v[1] = vecs[3 * k + 1];
        mv[k].v[2] = vecs[3 * k + 2];
        mv[k].u = u ? u[k] : 1.0f;
    }
    long long pos = first_step % D.move_cap;
    int done = 0;
    while (done < count) {
        int chunk = (int)std::min<long long>(count - done, D.move_cap - pos);
        FRMC_CUDA(cudaMemcpyAsync(D.moves + pos, mv.data() + done, sizeof(EMove) * chunk, cudaMemcpyHostToDevice,
                                  s->stream));
        done += chunk;
        pos = 0;
    }
    k_bump_gen<<<1, 1, 0, s->stream>>>(D.st);  // after the copies: staged moves are stale
    FRMC_CUDA(cudaGetLastError());
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    return FRMC_OK;
}

int frmc_engines_push_group_moves(void *handle, int32_t e, const int32_t *atoms, const int32_t *kinds,
                                  const float *params, const float *u, int32_t count, int64_t first_step)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, e) || count < 0 || first_step < 0 || (count && (!atoms || !kinds || !params)))
        return set_error(FRMC_E_ARG, "push_group_moves: invalid arguments");
    const EDesc &D = s->slots[e].d;
    const int G = D.group;
    if (count > D.move_cap)
        return set_error(FRMC_E_ARG, "push_group_moves: %d moves exceed the ring of %d", count, D.move_cap);
    std::vector<EMove> mv(count);
    std::vector<EGroup> gv(G > 1 ? count : 0);
    for (int k = 0; k < count; ++k) {
        const int32_t *a = atoms + (size_t)k * G;
        for (int t = 0; t < G; ++t) {
            if (a[t] < 0 || a[t] >= D.n)
                return set_error(FRMC_E_INDEX, "push_group_moves: atom %d out of range", a[t]);
            for (int r = 0; r < t; ++r)
                if (a[r] == a[t])
                    return set_error(FRMC_E_ARG, "push_group_moves: atom %d twice in one group", a[t]);
        }
        if (kinds[k] != 0 && kinds[k] != 1)
            return set_error(FRMC_E_ARG, "push_group_moves: move kind %d (0 translation, 1 rotation)", kinds[k]);
        if (kinds[k] == 1 && G == 1)
            return set_error(FRMC_E_ARG, "push_group_moves: a rotation needs a group of at least two atoms");
        const float *pr = params + (size_t)k * 9;
        mv[k].atom = a[0];
        mv[k].v[0] = kinds[k] == 0 ? pr[0] : 0.f;
        mv[k].v[1] = kinds[k] == 0 ? pr[1] : 0.f;
        mv[k].v[2] = kinds[k] == 0 ? pr[2] : 0.f;
        mv[k].u = u ? u[k] : 1.0f;
        if (G > 1) {
            EGroup &g = gv[k];
            memset(&g, 0, sizeof(g));
            g.kind = kinds[k];
            if (g.kind == 1)
                for (int q = 0; q < 9; ++q) g.rot[q] = pr[q];
            for (int t = 1; t < G; ++t) g.atoms[t - 1] = a[t];
        }
    }
    long long pos = first_step % D.move_cap;
    int done = 0;
    while (done < count) {
        int chunk = (int)std::min<long long>(count - done, D.move_cap - pos);
        FRMC_CUDA(cudaMemcpyAsync(D.moves + pos, mv.data() + done, sizeof(EMove) * chunk, cudaMemcpyHostToDevice,
                                  s->stream));
        if (G > 1)
            FRMC_CUDA(cudaMemcpyAsync(D.groups + pos, gv.data() + done, sizeof(EGroup) * chunk,
                                      cudaMemcpyHostToDevice, s->stream));
        done += chunk;
        pos = 0;
    }
    k_bump_gen<<<1, 1, 0, s->stream>>>(D.st);  // after the copies: staged moves are stale
    FRMC_CUDA(cudaGetLastError());
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    return FRMC_OK;
}

int frmc_engines_step(void *handle, int32_t engine, int32_t steps, int use_graph, void *stream)
{
    EngineSet *s = as_set(handle);
    if (!s || steps < 0 || (engine != -1 && !valid_id(s, engine)))
        return set_error(FRMC_E_ARG, "engines_step: invalid arguments");
    FRMC_TRY(refresh(s));
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    const int count = engine < 0 ? s->nbatch : s->item_count[engine];
    if (count == 0 || steps == 0)
        return FRMC_OK;
    auto one = [&](cudaStream_t sx) {
        if (engine < 0)
            return launch_batched(s, sx);
        const int fi = s->fused_item[engine];
        if (fi >= 0 && s->slots[engine].cost <= kSoloFusedCost)  // one CTA beats tiles plus a finisher
            // one engine alone: the largest CTA (its layout fits by the fused check)
            FRMC_TRY(launch_items(s, s->items + fi, 1, 0, sx,
                                  (int)fused_dyn_bytes(s->fused_dp_ints, s->fused_bins, kMaxEngineThreads), true,
                                  nullptr, nullptr, kMaxEngineThreads));
        else
            FRMC_TRY(launch_items(s, s->items + s->item_first[engine], count, 0, sx, 0, false, nullptr, nullptr,
                                  kMaxEngineThreads));
        return launch_sq(s, s->sq_first[engine], s->sq_count[engine], sx);
    };
    if (!use_graph) {
        for (int k = 0; k < steps; ++k) FRMC_TRY(one(st));
        return FRMC_OK;
    }
    auto key = std::make_pair(engine, steps);
    auto it = s->graphs.find(key);
    if (it == s->graphs.end()) {
        cudaStream_t cap;
        FRMC_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t g;
        cudaError_t ce = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        int rc = FRMC_OK;
        if (ce == cudaSuccess) {
            for (int k = 0; k < steps && !rc; ++k) rc = one(cap);
            ce = cudaStreamEndCapture(cap, &g);
        }
        cudaStreamDestroy(cap);
        if (rc)
            return rc;
        if (ce != cudaSuccess)
            return cuda_fail(ce, "graph capture");
        cudaGraphExec_t ex;
        ce = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess)
            return cuda_fail(ce, "cudaGraphInstantiate");
        it = s->graphs.emplace(key, ex).first;
    }
    FRMC_CUDA(cudaGraphLaunch(it->second, st));
    return FRMC_OK;
}

// One batched step from host arrays into staging slot `slot` (0 or 1): the
// moves are written to the slot's pinned buffer, and one CUDA graph copies
// them in, scatters them into the rings, steps, gathers the results and
// copies them back; the slot's event marks its completion.
static int step_host_submit(EngineSet *s, const int32_t *atoms, const float *vecs, const float *u, int slot)
{
    if (slot < 0 || slot > 1)
        return set_error(FRMC_E_ARG, "step_host: slot must be 0 or 1");
    if (s->stage_busy[slot])
        return set_error(FRMC_E_STATE, "step_host: slot %d holds a step whose results were not collected", slot);
    const bool other_busy = s->stage_busy[1 - slot];
    if (s->dirty && other_busy)
        return set_error(FRMC_E_STATE, "step_host: the engine set changed while a step is in flight");
    FRMC_TRY(refresh(s));
    const int E = (int)s->live.size();
    if (E == 0)
        return FRMC_OK;
    for (int k = 0; k < E; ++k)
        if (s->slots[s->live[k]].d.group > 1)
            return set_error(FRMC_E_ARG, "step_host: engine %d moves groups; push its moves instead", s->live[k]);
    for (int k = 0; k < E; ++k)
        if (atoms[k] < 0 || atoms[k] >= s->slots[s->live[k]].d.n)
            return set_error(FRMC_E_INDEX, "step_host: atom %d out of range for engine %d", atoms[k], s->live[k]);
    if (E > s->stage_cap) {
        if (other_busy)
            return set_error(FRMC_E_STATE, "step_host: the staging must grow while a step is in flight");
        FRMC_CUDA(cudaStreamSynchronize(s->stream));
        drop_graphs(s);  // the captured copies name the staging buffers
        const int cap = std::max(E, 2 * s->stage_cap);
        for (int k = 0; k < 2; ++k) {
            if (s->hstage_m[k]) cudaFreeHost(s->hstage_m[k]);
            if (s->hstage_r[k]) cudaFreeHost(s->hstage_r[k]);
            if (s->dstage_m[k]) cudaFree(s->dstage_m[k]);
            if (s->dstage_r[k]) cudaFree(s->dstage_r[k]);
            s->hstage_m[k] = nullptr;
            s->hstage_r[k] = nullptr;
            s->dstage_m[k] = nullptr;
            s->dstage_r[k] = nullptr;
            // mapped: a step of fused engines reads its moves and writes its
            // results here directly
            FRMC_CUDA(cudaHostAlloc((void **)&s->hstage_m[k], sizeof(EMove) * cap, cudaHostAllocMapped));
            FRMC_CUDA(cudaHostAlloc((void **)&s->hstage_r[k], sizeof(EResult) * cap, cudaHostAllocMapped));
            FRMC_CUDA(cudaMalloc(&s->dstage_m[k], sizeof(EMove) * cap));
            FRMC_CUDA(cudaMalloc(&s->dstage_r[k], sizeof(EResult) * cap));
            if (!s->stage_ev[k])
                FRMC_CUDA(cudaEventCreateWithFlags(&s->stage_ev[k], cudaEventDisableTiming));
        }
        s->stage_cap = cap;
    }
    EMove *hm = s->hstage_m[slot];
    for (int k = 0; k < E; ++k) {
        EMove &m = hm[k];
        m.atom = atoms[k];
        m.v[0] = vecs[3 * k];
        m.v[1] = vecs[3 * k + 1];
        m.v[2] = vecs[3 * k + 2];
        m.u = u ? u[k] : 1.0f;
    }
    cudaStream_t st = s->stream;
    // every live engine fused and none with an S(Q) term: one kernel reads
    // the moves from the mapped staging buffer and writes the results there
    const bool direct = s->nfused == s->nbatch && s->sq_host.empty() && s->nfused == E;
    auto body = [&](cudaStream_t sx) -> int {
        if (direct) {
            EMove *dm = nullptr;
            EResult *dr = nullptr;
            FRMC_CUDA(cudaHostGetDevicePointer((void **)&dm, s->hstage_m[slot], 0));
            FRMC_CUDA(cudaHostGetDevicePointer((void **)&dr, s->hstage_r[slot], 0));
            return launch_items(s, s->items + s->nsolo, s->nfused, 0, sx, fused_dyn_smem(s), true, dm, dr);
        }
        FRMC_CUDA(cudaMemcpyAsync(s->dstage_m[slot], hm, sizeof(EMove) * E, cudaMemcpyHostToDevice, sx));
        k_scatter_moves<<<(E + 127) / 128, 128, 0, sx>>>(s->ddesc, s->dlive, s->dstage_m[slot], E);
        FRMC_CUDA(cudaGetLastError());
        FRMC_TRY(launch_batched(s, sx));
        k_gather_results<<<(E + 127) / 128, 128, 0, sx>>>(s->ddesc, s->dlive, s->dstage_r[slot], E);
        FRMC_CUDA(cudaGetLastError());
        FRMC_CUDA(cudaMemcpyAsync(s->hstage_r[slot], s->dstage_r[slot], sizeof(EResult) * E, cudaMemcpyDeviceToHost,
                                  sx));
        return FRMC_OK;
    };
    if (!s->host_graph[slot] || s->host_graph_E[slot] != E) {
        if (s->host_graph[slot])
            cudaGraphExecDestroy(s->host_graph[slot]);
        s->host_graph[slot] = nullptr;
        cudaStream_t cap;
        FRMC_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t g;
        cudaError_t ce = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        int rc = FRMC_OK;
        if (ce == cudaSuccess) {
            rc = body(cap);
            ce = cudaStreamEndCapture(cap, &g);
        }
        cudaStreamDestroy(cap);
        if (rc)
            return rc;
        if (ce != cudaSuccess)
            return cuda_fail(ce, "step_host graph capture");
        ce = cudaGraphInstantiate(&s->host_graph[slot], g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
            s->host_graph[slot] = nullptr;
            return cuda_fail(ce, "step_host graph instantiate");
        }
        s->host_graph_E[slot] = E;
    }
    FRMC_CUDA(cudaGraphLaunch(s->host_graph[slot], st));
    FRMC_CUDA(cudaEventRecord(s->stage_ev[slot], st));
    s->stage_busy[slot] = true;
    s->stage_E[slot] = E;
    return FRMC_OK;
}

static int step_host_collect(EngineSet *s, int slot, double *chi2_new, int32_t *accepted)
{
    if (slot < 0 || slot > 1 || !s->stage_busy[slot])
        return set_error(FRMC_E_STATE, "step_host: slot %d holds no submitted step", slot);
    FRMC_CUDA(cudaEventSynchronize(s->stage_ev[slot]));
    s->stage_busy[slot] = false;
    // the engines of the submitted step (add and remove are refused while a
    // slot is busy, so this is also the live count)
    const int E = s->stage_E[slot];
    const EResult *hr = s->hstage_r[slot];
    for (int k = 0; k < E; ++k) {
        if (chi2_new) chi2_new[k] = hr[k].chi2_new;
        if (accepted) accepted[k] = hr[k].accepted;
    }
    return FRMC_OK;
}

int frmc_engines_step_host(void *handle, const int32_t *atoms, const float *vecs, const float *u, double *chi2_new,
                           int32_t *accepted)
{
    EngineSet *s = as_set(handle);
    if (!s)
        return set_error(FRMC_E_ARG, "null handle");
    if (s->live.empty())
        return FRMC_OK;
    FRMC_TRY(step_host_submit(s, atoms, vecs, u, 0));
    return s->stage_busy[0] ? step_host_collect(s, 0, chi2_new, accepted) : FRMC_OK;
}

int frmc_engines_step_host_submit(void *handle, const int32_t *atoms, const float *vecs, const float *u,
                                  int32_t slot)
{
    EngineSet *s = as_set(handle);
    if (!s)
        return set_error(FRMC_E_ARG, "null handle");
    return step_host_submit(s, atoms, vecs, u, slot);
}

int frmc_engines_step_host_collect(void *handle, int32_t slot, double *chi2_new, int32_t *accepted)
{
    EngineSet *s = as_set(handle);
    if (!s)
        return set_error(FRMC_E_ARG, "null handle");
    return step_host_collect(s, slot, chi2_new, accepted);
}

int frmc_engines_place_positions(int32_t n, const int32_t *sm, const double *t, int32_t *pos)
{
    if (n < 0 || (n > 0 && (!sm || !t || !pos)))
        return set_error(FRMC_E_ARG, "place_positions: invalid arguments");
    std::vector<int> smi(sm, sm + n), p(n);
    place_positions(n, smi.data(), t, p.data());
    for (int b = 0; b < n; ++b) pos[b] = p[b];
    return FRMC_OK;
}

int frmc_engines_place(void *handle, int32_t steps)
{
    EngineSet *s = as_set(handle);
    if (!s || steps < 1)
        return set_error(FRMC_E_ARG, "engines_place: steps must be at least 1");
    if (s->stage_busy[0] || s->stage_busy[1])
        return set_error(FRMC_E_STATE, "engines_place: a host-buffer step is in flight");
    // steps launched on other streams finish first (a set-up call)
    FRMC_CUDA(cudaDeviceSynchronize());
    FRMC_TRY(refresh(s));
    Context *c;
    FRMC_TRY(get_context(&c));
    const int n = s->nfused;
    if (n < 2 || n > c->sms * s->ctas_per_sm)
        return FRMC_OK;  // no one-CTA launch with one item per CTA: nothing to place
    if (s->place_cap < n) {
        if (s->place_dev)
            cudaFree(s->place_dev);
        s->place_dev = nullptr;
        s->place_cap = 0;
        FRMC_CUDA(cudaMalloc(&s->place_dev, sizeof(unsigned long long) * n));
        s->place_cap = n;
    }
    // engine id per fused item (fused_item holds the item's index in the
    // whole list, whose first nsolo items are the one-engine tiles)
    std::vector<int> ids(n, -1);
    for (int id : s->live) {
        const int k = s->fused_item[id] - s->nsolo;
        if (s->fused_item[id] >= 0 && k >= 0 && k < n)
            ids[k] = id;
    }
    for (int k = 0; k < n; ++k)
        if (ids[k] < 0)
            return set_error(FRMC_E_STATE, "engines_place: the work list is inconsistent");
    std::vector<unsigned long long> rec(n);
    std::vector<double> took(s->slots.size(), 0.0);
    std::vector<int> sm0(n, -1);
    bool repeat = true;
    s->place_rec = true;
    int rc = FRMC_OK;
    for (int k = 0; k < steps && !rc; ++k) {
        rc = launch_batched(s, s->stream);
        if (!rc) {
            cudaError_t ce = cudaMemcpyAsync(rec.data(), s->place_dev, sizeof(unsigned long long) * n,
                                             cudaMemcpyDeviceToHost, s->stream);
            if (ce == cudaSuccess)
                ce = cudaStreamSynchronize(s->stream);
            if (ce != cudaSuccess)
                rc = cuda_fail(ce, "engines_place");
        }
        for (int b = 0; b < n && !rc; ++b) {
            const int sm = (int)(rec[b] >> 48);
            took[ids[b]] += (double)(rec[b] & 0xffffffffffffull);
            if (k == 0)
                sm0[b] = sm;
            else if (sm0[b] != sm)
                repeat = false;
        }
    }
    s->place_rec = false;
    if (rc)
        return rc;
    if (!repeat) {
        // the SMs did not repeat from step to step: keep the cost order
        s->place_order.clear();
        return FRMC_OK;
    }
    std::vector<double> t(n);
    for (int b = 0; b < n; ++b) t[b] = took[ids[b]];
    std::vector<int> pos(n);
    place_positions(n, sm0.data(), t.data(), pos.data());
    std::vector<int> order(n, -1);
    for (int b = 0; b < n; ++b) order[b] = ids[pos[b]];
    s->place_order = order;
    s->place_key = place_key(s, n);
    s->dirty = true;
    drop_graphs(s);
    return refresh(s);  // the new work list now, not at the next step
}

int frmc_engines_sync(void *handle)
{
    EngineSet *s = as_set(handle);
    if (!s)
        return set_error(FRMC_E_ARG, "null handle");
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    unsigned status = 0;
    FRMC_CUDA(cudaMemcpy(&status, &s->sched[0].status, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (status)
        return set_error(FRMC_E_TIMEOUT, "engine step: a bounded device wait gave up (status 0x%x)", status);
    return FRMC_OK;
}

int frmc_engines_state(void *handle, int32_t e, double *chi2, int64_t *step, int64_t *accepted)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, e))
        return set_error(FRMC_E_ARG, "engines_state: invalid engine");
    EState S;
    FRMC_CUDA(cudaMemcpy(&S, s->slots[e].d.st, sizeof(EState), cudaMemcpyDeviceToHost));
    if (chi2) *chi2 = S.chi2;
    if (step) *step = S.step;
    if (accepted) *accepted = S.accepted;
    return FRMC_OK;
}

int frmc_engines_results(void *handle, int32_t e, int64_t first_step, int32_t count, double *chi2_new,
                         int32_t *accepted, int32_t *atoms)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, e) || count < 0 || first_step < 0)
        return set_error(FRMC_E_ARG, "engines_results: invalid arguments");
    const EDesc &D = s->slots[e].d;
    if (count > D.move_cap)
        return set_error(FRMC_E_ARG, "engines_results: more results than the ring holds");
    std::vector<EResult> r(count);
    long long pos = first_step % D.move_cap;
    int done = 0;
    while (done < count) {
        int chunk = (int)std::min<long long>(count - done, D.move_cap - pos);
        FRMC_CUDA(cudaMemcpy(r.data() + done, D.results + pos, sizeof(EResult) * chunk, cudaMemcpyDeviceToHost));
        done += chunk;
        pos = 0;
    }
    for (int k = 0; k < count; ++k) {
        if (chi2_new) chi2_new[k] = r[k].chi2_new;
        if (accepted) accepted[k] = r[k].accepted;
        if (atoms) atoms[k] = r[k].atom;
    }
    return FRMC_OK;
}

int frmc_engines_counts(void *handle, int32_t e, int32_t *counts)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, e))
        return set_error(FRMC_E_ARG, "engines_counts: invalid engine");
    const EDesc &D = s->slots[e].d;
    FRMC_CUDA(cudaMemcpy(counts, D.counts, sizeof(int) * 2 * D.total, cudaMemcpyDeviceToHost));
    return FRMC_OK;
}

int frmc_engines_coords(void *handle, int32_t e, float *box_coords, float *real_coords)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, e))
        return set_error(FRMC_E_ARG, "engines_coords: invalid engine");
    const EDesc &D = s->slots[e].d;
    std::vector<float4> b(D.n), r(D.n);
    FRMC_CUDA(cudaMemcpy(b.data(), D.box, sizeof(float4) * D.n, cudaMemcpyDeviceToHost));
    FRMC_CUDA(cudaMemcpy(r.data(), D.real, sizeof(float4) * D.n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < D.n; ++i) {
        if (box_coords) {
            box_coords[3 * i] = b[i].x;
            box_coords[3 * i + 1] = b[i].y;
            box_coords[3 * i + 2] = b[i].z;
        }
        if (real_coords) {
            real_coords[3 * i] = r[i].x;
            real_coords[3 * i + 1] = r[i].y;
            real_coords[3 * i + 2] = r[i].z;
        }
    }
    return FRMC_OK;
}

int frmc_cell_metric(const float *basis, int32_t isPBC, double *w, double *lam, int32_t *mode)
{
    if (!basis || !w || !lam || !mode)
        return set_error(FRMC_E_ARG, "cell_metric: null argument");
    int m = 0;
    if (!cell_metric(basis, isPBC ? basis_mode(basis, 1) : BM_IBC, w, lam, &m))
        return set_error(FRMC_E_ARG, "cell_metric: singular basis");
    *mode = m;
    return FRMC_OK;
}

int frmc_engines_regrid(void *handle, int32_t e)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, e))
        return set_error(FRMC_E_ARG, "engines_regrid: invalid engine");
    Slot &sl = s->slots[e];
    EDesc &D = sl.d;
    if (!s->cells)
        return FRMC_OK;
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    std::vector<float4> b(D.n);
    std::vector<int> mol(D.n), el(D.n);
    std::vector<float> box(3 * (size_t)D.n);
    FRMC_CUDA(cudaMemcpy(b.data(), D.box, sizeof(float4) * D.n, cudaMemcpyDeviceToHost));
    FRMC_CUDA(cudaMemcpy(mol.data(), D.mol, sizeof(int) * D.n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < D.n; ++i) {
        box[3 * (size_t)i] = b[i].x;
        box[3 * (size_t)i + 1] = b[i].y;
        box[3 * (size_t)i + 2] = b[i].z;
        int v;
        std::memcpy(&v, &b[i].w, 4);
        el[i] = v;
    }
    frmc_engine_spec sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.n = D.n;
    sp.isPBC = D.bm != BM_IBC;
    sp.box_coords = box.data();
    sp.el = el.data();
    sp.mol = mol.data();
    sp.basis = D.B.b;
    sp.maxDistance = D.maxD;
    sp.group_size = D.group;
    CellGrid cg;
    build_cells(sp, D.bm, cg);
    if (cg.nc > 0) {
        FRMC_CUDA(cudaMemcpy(D.cbox, cg.cbox.data(), 16 * cg.cbox.size(), cudaMemcpyHostToDevice));
        FRMC_CUDA(cudaMemcpy(D.cmol, cg.cmol.data(), 4 * cg.cmol.size(), cudaMemcpyHostToDevice));
        FRMC_CUDA(cudaMemcpy(D.csl, cg.csl.data(), 8 * cg.csl.size(), cudaMemcpyHostToDevice));
        FRMC_CUDA(cudaMemcpy(D.cstart, cg.cstart.data(), 4 * cg.cstart.size(), cudaMemcpyHostToDevice));
        FRMC_CUDA(cudaMemcpy(D.clo, cg.clo.data(), 16 * cg.clo.size(), cudaMemcpyHostToDevice));
        FRMC_CUDA(cudaMemcpy(D.chi, cg.chi.data(), 16 * cg.chi.size(), cudaMemcpyHostToDevice));
    }
    D.nc = cg.nc;
    D.cmode = cg.cmode;
    D.cpbc = cg.cpbc;
    for (int k = 0; k < 3; ++k) D.cw[k] = cg.cw[k];
    D.clam2 = cg.clam2;
    D.cthr2 = cg.cthr2;
    sl.cost = (cg.nc > 0 ? 4 * (long long)std::ceil(cg.sweep) : (long long)D.n) * D.group;
    // a staged next move holds the moved atom's old cell-order slot and cell
    k_bump_gen<<<1, 1, 0, s->stream>>>(D.st);
    FRMC_CUDA(cudaGetLastError());
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    s->dirty = true;  // descriptors and the work list are rebuilt before the next step
    return FRMC_OK;
}

int frmc_engines_sq_table(void *handle, int32_t hs, int32_t nq, const double *M, const double *weights,
                          const double *r0fac, int32_t *table)
{
    EngineSet *s = as_set(handle);
    if (!s || !M || !r0fac || !table || hs < 1 || hs > kSqMaxBins || nq < 1)
        return set_error(FRMC_E_ARG, "engines_sq_table: need 1 <= hs <= %d, nq >= 1, M, r0fac and a table",
                         kSqMaxBins);
    Context *c;
    FRMC_TRY(get_context(&c));
    SqTable t;
    t.hs = hs;
    t.nq = nq;
    const size_t nm = (size_t)hs * nq, nk = (size_t)hs * hs;
    t.bytes = 8 * (nm + nk + hs + (weights ? (size_t)nq : 0) + 1);
    FRMC_CUDA(cudaMalloc(&t.blob, t.bytes));
    t.M = (double *)t.blob;
    double *K = t.M + nm;
    t.R0 = K + nk;
    unsigned long long *dmax = (unsigned long long *)(t.R0 + hs);
    t.w = weights ? (double *)(dmax + 1) : nullptr;
    t.T = (long long *)K;
    unsigned long long mx = 0;
    cudaError_t ce = cudaMemcpyAsync(t.M, M, 8 * nm, cudaMemcpyHostToDevice, s->stream);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(t.R0, r0fac, 8 * (size_t)hs, cudaMemcpyHostToDevice, s->stream);
    if (ce == cudaSuccess && weights)
        ce = cudaMemcpyAsync(t.w, weights, 8 * (size_t)nq, cudaMemcpyHostToDevice, s->stream);
    if (ce == cudaSuccess)
        ce = cudaMemsetAsync(dmax, 0, 8, s->stream);
    if (ce == cudaSuccess) {
        dim3 grid((hs + 63) / 64, (hs + 63) / 64);
        k_sq_gram<<<grid, 256, 0, s->stream>>>(t.M, t.w, hs, nq, K);
        k_sq_absmax<<<c->sms * 2, 256, 0, s->stream>>>(K, t.R0, hs, dmax);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(&mx, dmax, 8, cudaMemcpyDeviceToHost, s->stream);
    if (ce == cudaSuccess)
        ce = cudaStreamSynchronize(s->stream);
    if (ce == cudaSuccess) {
        const double m = reinterpret_cast<const double &>(mx);
        int ex = 0;
        if (m > 0.0 && std::isfinite(m))
            std::frexp(m, &ex);
        t.s = m > 0.0 ? kSqBits - ex : 0;  // max |K R0| 2^s < 2^kSqBits
        if (!std::isfinite(m)) {
            cudaFree(t.blob);
            return set_error(FRMC_E_ARG, "engines_sq_table: the table has non-finite entries");
        }
        k_sq_quantize<<<c->sms * 2, 256, 0, s->stream>>>(K, t.R0, hs, t.s);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) {
        t.hsp = (hs + kSqRows - 1) / kSqRows * kSqRows;
        ce = cudaMalloc(&t.TD, sizeof(__half) * (size_t)kSqLimbs * t.hsp * t.hsp);
    }
    if (ce == cudaSuccess) {
        k_sq_digits<<<c->sms * 4, 256, 0, s->stream>>>(t.T, hs, t.hsp, t.TD);
        ce = cudaGetLastError();
        t.bytes += sizeof(__half) * (size_t)kSqLimbs * t.hsp * t.hsp;
    }
    if (ce == cudaSuccess)
        ce = cudaStreamSynchronize(s->stream);
    if (ce != cudaSuccess) {
        cudaFree(t.blob);
        if (t.TD) cudaFree(t.TD);
        return cuda_fail(ce, "S(Q) table");
    }
    if (const int rc = sq_encode_maps(t)) {
        cudaFree(t.blob);
        cudaFree(t.TD);
        if (t.maps) cudaFree(t.maps);
        return rc;
    }
    s->tables.push_back(t);
    *table = (int32_t)s->tables.size() - 1;
    return FRMC_OK;
}

int frmc_engines_sq(void *handle, int32_t e, double *sq)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, e) || !sq || !s->slots[e].d.sq)
        return set_error(FRMC_E_ARG, "engines_sq: engine %d has no S(Q) term", e);
    FRMC_TRY(refresh(s));
    const EDesc &D = s->slots[e].d;
    FRMC_TRY(launch_sq_eval(s, e, 0, s->stream));
    FRMC_CUDA(cudaMemcpyAsync(sq, D.sqv, 8 * (size_t)D.nq, cudaMemcpyDeviceToHost, s->stream));
    FRMC_CUDA(cudaStreamSynchronize(s->stream));
    return FRMC_OK;
}

int frmc_engines_terms(void *handle, int32_t e, double *sd, double *sd_sq)
{
    EngineSet *s = as_set(handle);
    if (!s || !valid_id(s, e))
        return set_error(FRMC_E_ARG, "engines_terms: invalid engine");
    EState S;
    FRMC_CUDA(cudaMemcpy(&S, s->slots[e].d.st, sizeof(EState), cudaMemcpyDeviceToHost));
    if (sd) *sd = S.sd;
    if (sd_sq) *sd_sq = S.sd_sq;
    return FRMC_OK;
}

int frmc_engines_info(void *handle, int32_t *E, int64_t *total_atoms, int64_t *device_bytes)
{
    EngineSet *s = as_set(handle);
    if (!s)
        return set_error(FRMC_E_ARG, "null handle");
    long long atoms = 0, bytes = 0;
    for (int id : s->live) {
        atoms += s->slots[id].d.n;
        bytes += (long long)s->slots[id].bytes;
    }
    for (const auto &t : s->tables) bytes += (long long)t.bytes;
    if (E) *E = (int32_t)s->live.size();
    if (total_atoms) *total_atoms = atoms;
    if (device_bytes) *device_bytes = bytes;
    return FRMC_OK;
}

}  // extern "C"
