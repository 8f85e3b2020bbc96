// Host runtime shared by the library's translation units: per-device context
// (stream, SM count, grow-only device buffers), error reporting and the
// host-side helpers that prepare kernel parameters.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "frmc_gpu.h"
#include "frmc_math.cuh"

namespace frmc {

// Thread-local last error message; returns `code` for convenience.
int set_error(int code, const char *fmt, ...);
const char *last_error();
int cuda_fail(cudaError_t e, const char *what);

#define FRMC_CUDA(call)                                  \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return ::frmc::cuda_fail(_e, #call); \
    } while (0)

#define FRMC_TRY(x)              \
    do {                         \
        int _rc = (x);           \
        if (_rc) return _rc;     \
    } while (0)
#define TRY_RC FRMC_TRY

inline float int_bits_as_float(int v)
{
    float f;
    static_assert(sizeof(f) == sizeof(v), "int/float size");
    __builtin_memcpy(&f, &v, sizeof(f));
    return f;
}

// A device allocation that only grows.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    template <class T>
    T *as() const { return static_cast<T *>(p); }
};

// Roles of the drop-in path's device buffers.
enum BufRole {
    BUF_COORDS = 0,
    BUF_EL,
    BUF_MOL,
    BUF_ATOMS4,
    BUF_ROWS,
    BUF_COUNTS,
    BUF_OUT,
    BUF_AUX0,
    BUF_AUX1,
    BUF_AUX2,
    BUF_STATUS,
    BUF_ATOMIC_COUNTS,
    BUF_ATOMIC_TOTALS,
    BUF_ATOMIC_LIST_B,
    BUF_ATOMIC_LIST_V,
    BUF_ATOMIC_ACC,
    BUF_ATOMIC_LIMITS,
    BUF_COORD_LISTS,
    BUF_COORD_META,
    BUF_COUNT_
};

struct Context {
    int device = -1;
    int sms = 0;
    int max_smem_optin = 0;
    // the device reads and writes pageable host memory coherently
    // (cudaDevAttrPageableMemoryAccess, e.g. through NVLink-C2C on Grace):
    // small host-buffer calls then pass the caller's arrays to the kernels
    // instead of copying them (FRMC_HOST_DIRECT=0 turns this off)
    int pageable = 0;
    size_t counts_clean = 0;  // leading bytes of BUF_COUNTS known to be zero
    cudaStream_t stream = nullptr;
    std::mutex mu;  // serialises host-buffer entry points on this device
    DevBuf buf[BUF_COUNT_];
};

// Context of the current device (created on first use).
int get_context(Context **out);

// Basis shape from the exact zero pattern of B (row-major, rows = vectors).
int basis_mode(const float *B, int isPBC);
Basis make_basis(const float *B);

// Squared-distance limits: for d = sqrtf(s) (IEEE),
//   d >= minD  <=>  s >= s_lo      and      d < maxD  <=>  s < s_hi.
void sq_limits(float minD, float maxD, float *s_lo, float *s_hi);

// ---------------------------------------------------------------- launchers
struct FullTune {
    int threads = 512;  // CTA size
    int rows = 2;       // row atoms per thread (tile = threads * rows)
    int queued = -1;    // -1: choose from the expected acceptance
    int qcap = 16;      // queue slots per thread
    int ctas_per_sm = 1;
    double min_pairs_tiled = 8.0e6;
    int aggregate = 0;  // 1: queued pairs binned with warp-aggregated atomics (__match_any_sync)
};

// All-pairs (i < j) histogram of `n` packed atoms (x, y, z, el bits) into
// uint32 counts intra[total], inter[total] (total = ne*ne*hs), which must be
// zeroed by the caller.
int launch_full_hist(const float4 *atoms, const int *mol, int n, int bm, const Basis &B, float minD, float maxD,
                     float binw, int ne, int hs, unsigned *intra, unsigned *inter, uint32_t *status,
                     double accept_fraction, const FullTune *tune, cudaStream_t st, long long item_begin = 0,
                     long long item_end = -1);
// The same with the device's SM count and opt-in shared-memory limit given
// (touches no library context).
int launch_full_hist_on(int sms, int max_smem_optin, const float4 *atoms, const int *mol, int n, int bm,
                        const Basis &B, float minD, float maxD, float binw, int ne, int hs, unsigned *intra,
                        unsigned *inter, uint32_t *status, double accept_fraction, const FullTune *tune,
                        cudaStream_t st, long long item_begin = 0, long long item_end = -1);
// Tile configuration currently set by frmc_set_full_tune.
FullTune current_tune();
// Expected fraction of pairs inside [minD, maxD) for uniform density
// (chooses queued or direct binning).
double accept_fraction(const float *basis, int isPBC, float minD, float maxD);
// Number of work items of the all-pairs kernel for n atoms under `tune`.
long long full_hist_items(int n, const FullTune *tune);

// Rows (explicit atom indexes, or explicit coordinates) against every column
// atom j in [start, n), j != row atom.  Counts are added with global atomics.
int launch_rows_hist(const float *coords, const int *el, const int *mol, int n, const int *rows, int K,
                     int allAtoms, int bm, const Basis &B, float minD, float maxD, float binw, int ne, int hs,
                     unsigned *intra, unsigned *inter, cudaStream_t st);

// A group move's change of fullrmc's before/after-move data (M - F after
// minus M - F before) into signed counts; rows in group order, sorted = the
// rows in increasing order followed by their group positions (2K ints).
int launch_group_delta(const float *coords, const float *newc, const int *el, const int *mol, int n, const int *rows,
                       const int *sorted, int K, int bm, const Basis &B, float minD, float maxD, float binw, int ne,
                       int hs, int *intra, int *inter, cudaStream_t st);

// Histogram of given distances: dists is (n, K) row-major, column k holds the
// distances of atom rows[k].
int launch_dists_hist(const float *dists, int n, int K, const int *rows, const int *el, const int *mol,
                      int allAtoms, float minD, float maxD, float binw, int ne, int hs, unsigned *intra,
                      unsigned *inter, cudaStream_t st);

// out[k] = h0[k] + 1.0f added counts[k] times in float32 (h0 may be null = 0).
int launch_counts_pair_to_f32_zero(unsigned *counts, int64_t total, float *out0, float *out1, cudaStream_t st);
int launch_counts_to_f32(const unsigned *counts, const float *h0, float *out, int64_t total, cudaStream_t st);

// Atomic distance constraint sums (atomic_kernels.cu): rows (device, K atom
// indexes) against every column j of n atoms (j >= row atom unless allAtoms,
// j != row atom), from box coordinates (device (n, 3)) or given distances
// (device (n, K)); flags: 1 inter, 2 intra, 4 count within limits, 8 / 16 / 32
// reduce to upper / lower / nearest limit.  dsum / nsum (device, [2][ne][ne],
// intra then inter) hold the starting values and receive the sums.
int atomic_distances_run(Context *c, const float *coords, const float *dists, const int *rows, int K, int n,
                         int allAtoms, int flags, int ne, const float *basis_host, int isPBC, const int *mol,
                         const int *el, const float *lower, const float *upper, float *dsum, int *nsum,
                         cudaStream_t st);
// pair_elements_stats counts ([2][ne][ne] int, zeroed by the caller).
int launch_pair_stats(const int *el, const int *mol, int n, int ne, int *nintra, int *ninter, cudaStream_t st);

// Pack AoS coordinates and element indexes into float4 (x, y, z, el bits).
int launch_pack_atoms(const float *coords, const int *el, int n, float4 *out, cudaStream_t st);
// The inverse: float4 (x, y, z, el bits) -> AoS coordinates and elements.
int launch_unpack_atoms(const float4 *atoms, int n, float *coords, int *el, cudaStream_t st);

// Coordination-number terms (coord_kernels.cu).  A term adds to data[def]
// the number of entries j of one index list (terms[t].begin, terms[t].len in
// `lists`; negative j counts from the end of the row) with
// lower[def] <= d(row, j) <= upper[def].
struct CoordTerm {
    int row;           // core atom (coordinates) or distance row
    int def;           // definition: window and accumulator
    long long begin;   // first entry of the term's list in `lists`
    int len;           // entries in the list
    int pad;
};
struct CoordLaunch {
    const float *coords = nullptr;  // device (n, 3) box coordinates, or null
    const float *basis = nullptr;   // host 3x3 basis (coordinates only)
    int isPBC = 0;
    int n = 0;
    const float *dists = nullptr;   // device distance rows (when coords is null)
    const long long *dist_off = nullptr;
    const int *dist_len = nullptr;
    const int *lists = nullptr;
    const CoordTerm *terms = nullptr;
    const int2 *items = nullptr;    // (term, first entry) per CTA
    long long nitems = 0;
    const float *lower = nullptr, *upper = nullptr;
    int *counts = nullptr;          // per term, zeroed
    const int *def_ids = nullptr, *def_off = nullptr, *def_terms = nullptr;
    int ndefs = 0;                  // definitions touched
    float *data = nullptr;          // device accumulators, updated in place
};
int coordination_run(const CoordLaunch &L, cudaStream_t st);
// List entries handled by one CTA of the counting kernel.
int coordination_chunk();

// ShapeFunction in FP64 (fp64_kernels.cu): G on the shells from the oriented
// uint32 counts, S on q, and the shape function on rv; w1 (hs) and w2 (nq)
// are scratch.  Every array is on the device.
int launch_shape_function(const unsigned *counts, int ne, int hs, int npairs, const int *pi, const int *pj,
                          const double *pc, const double *r, const double *vol, double rho0, double dr,
                          const double *q, int nq, double dq, const double *rv, int nr, double *G, double *S,
                          double *Gs, double *w1, double *w2, cudaStream_t st);

}  // namespace frmc
