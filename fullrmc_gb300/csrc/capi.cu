// extern "C" entry points (declared in include/frmc_gpu.h).
//
// Host-buffer entry points copy their inputs to the current device on the
// context's stream, run the kernels, copy the results back and synchronise;
// they keep no host data between calls (fullrmc mutates its coordinate array
// between calls, PairDistributionConstraints.py:1092-1122).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "frmc_gpu.h"
#include "frmc_runtime.h"

namespace frmc {
int launch_distances(const float *coords, int n, const float *pts, long long ps, const int *idx, int K,
                     int fromIndex, int isPBC, const float *basis, float *out, cudaStream_t st);
int launch_differences(const float *coords, int n, const float *pts, long long ps, const int *idx, int K,
                       int fromIndex, int isPBC, const float *basis, float *out, cudaStream_t st);
int launch_from_to(const float *from, const float *to, int n, int isPBC, const float *basis, float *out,
                   cudaStream_t st);
int launch_transform(const float *M, const float *coords, int n, float *out, cudaStream_t st);
int launch_sine(int kind, const float *xs, int nx, const float *ys, const float *f, int ny, double rho, double *out,
                double *scratch, cudaStream_t st);

static FullTune g_full_tune;
static std::mutex g_tune_mu;

FullTune current_tune()
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_full_tune;
}

static const float kIdentity[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};

static int check_n(int64_t n, const char *what)
{
    if (n < 0 || n > INT_MAX / 4)
        return set_error(FRMC_E_ARG, "%s: size %lld out of range", what, (long long)n);
    return FRMC_OK;
}

static int check_hist(int32_t ne, int32_t hs, int64_t *total)
{
    if (ne < 0 || hs < 0)
        return set_error(FRMC_E_ARG, "negative histogram shape (%d, %d)", ne, hs);
    int64_t t = (int64_t)ne * ne * hs;
    if (t > (int64_t)INT_MAX / 8)
        return set_error(FRMC_E_ARG, "histogram too large (%lld bins)", (long long)t);
    *total = t;
    return FRMC_OK;
}

static int check_indexes(const int32_t *idx, int64_t K, int64_t n)
{
    for (int64_t k = 0; k < K; ++k)
        if (idx[k] < 0 || idx[k] >= n)
            return set_error(FRMC_E_INDEX, "index %d out of range for %lld atoms", idx[k], (long long)n);
    return FRMC_OK;
}

double accept_fraction(const float *basis, int isPBC, float minD, float maxD)
{
    if (!isPBC)
        return 1.0;
    const float *B = basis;
    double det = (double)B[0] * ((double)B[4] * B[8] - (double)B[5] * B[7]) -
                 (double)B[1] * ((double)B[3] * B[8] - (double)B[5] * B[6]) +
                 (double)B[2] * ((double)B[3] * B[7] - (double)B[4] * B[6]);
    double V = std::fabs(det);
    if (!(V > 0))
        return 1.0;
    double lo = minD > 0 ? (double)minD : 0.0;
    double hi = (double)maxD;
    if (!(hi > lo))
        return 0.0;
    double f = 4.0 / 3.0 * M_PI * (hi * hi * hi - lo * lo * lo) / V;
    return f > 1.0 ? 1.0 : f;
}

#define LOCKED_CTX(c)                      \
    Context *c = nullptr;                  \
    {                                      \
        int _rc = get_context(&c);         \
        if (_rc) return _rc;               \
    }                                      \
    std::lock_guard<std::mutex> _lk(c->mu)

#define TRY(x)                   \
    do {                         \
        int _rc = (x);           \
        if (_rc) return _rc;     \
    } while (0)

static int h2d(void *dst, const void *src, size_t bytes, cudaStream_t st)
{
    if (!bytes)
        return FRMC_OK;
    FRMC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    return FRMC_OK;
}

static int d2h(void *dst, const void *src, size_t bytes, cudaStream_t st)
{
    if (!bytes)
        return FRMC_OK;
    FRMC_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    return FRMC_OK;
}

static int finish(Context *c)
{
    FRMC_CUDA(cudaStreamSynchronize(c->stream));
    return FRMC_OK;
}

// Upload coordinates, element and molecule indexes of n atoms.
static int upload_atoms(Context *c, const float *coords, const int32_t *mol, const int32_t *el, int64_t n)
{
    TRY(c->buf[BUF_COORDS].ensure(n * 12 + 16));
    TRY(h2d(c->buf[BUF_COORDS].p, coords, n * 12, c->stream));
    if (el) {
        TRY(c->buf[BUF_EL].ensure(n * 4 + 16));
        TRY(h2d(c->buf[BUF_EL].p, el, n * 4, c->stream));
    }
    if (mol) {
        TRY(c->buf[BUF_MOL].ensure(n * 4 + 16));
        TRY(h2d(c->buf[BUF_MOL].p, mol, n * 4, c->stream));
    }
    return FRMC_OK;
}

// Full histogram counts of the atoms already uploaded by upload_atoms.
static int full_counts(Context *c, int64_t n, const float *basis, int isPBC, int32_t ne, float minD, float maxD,
                       float bin, int32_t hs, int64_t total, unsigned *counts)
{
    const float *B = isPBC ? basis : kIdentity;
    const int bm = basis_mode(B, isPBC);
    Basis Bs = make_basis(B);
    const double pairs = 0.5 * (double)n * (double)(n - 1);
    FullTune tn = current_tune();
    if (pairs < tn.min_pairs_tiled) {
        return launch_rows_hist(c->buf[BUF_COORDS].as<float>(), c->buf[BUF_EL].as<int>(), c->buf[BUF_MOL].as<int>(),
                                (int)n, nullptr, (int)n, 0, bm, Bs, minD, maxD, bin, ne, hs, counts, counts + total,
                                c->stream);
    }
    TRY(c->buf[BUF_ATOMS4].ensure(n * 16 + 16));
    float4 *a4 = c->buf[BUF_ATOMS4].as<float4>();
    TRY(launch_pack_atoms(c->buf[BUF_COORDS].as<float>(), c->buf[BUF_EL].as<int>(), (int)n, a4, c->stream));
    return launch_full_hist(a4, c->buf[BUF_MOL].as<int>(), (int)n, bm, Bs, minD, maxD, bin, ne, hs, counts,
                            counts + total, c->buf[BUF_STATUS].as<uint32_t>(), accept_fraction(B, isPBC, minD, maxD),
                            &tn, c->stream);
}

// Zeroed counts for a call (skipping the memset where the previous call's
// conversion left them zero) and, unless the call's kernels never set it, a
// zero device status word.
static int prepare_counts(Context *c, int64_t total, bool status = true)
{
    const size_t need = 2 * (size_t)total * 4;
    const void *before = c->buf[BUF_COUNTS].p;
    TRY(c->buf[BUF_COUNTS].ensure(need + 16));
    if (c->buf[BUF_COUNTS].p != before)
        c->counts_clean = 0;
    TRY(c->buf[BUF_OUT].ensure(need + 16));
    TRY(c->buf[BUF_STATUS].ensure(16));
    if (c->counts_clean < need)
        FRMC_CUDA(cudaMemsetAsync(c->buf[BUF_COUNTS].p, 0, need, c->stream));
    c->counts_clean = 0;  // in use until a conversion resets them
    if (status)
        FRMC_CUDA(cudaMemsetAsync(c->buf[BUF_STATUS].p, 0, 4, c->stream));
    return FRMC_OK;
}

// Convert counts to float32 and copy both histograms back; checks the status.
static int counts_out(Context *c, int64_t total, const float *h0intra, const float *h0inter, float *hintra,
                      float *hinter)
{
    unsigned *cnt = c->buf[BUF_COUNTS].as<unsigned>();
    float *out = c->buf[BUF_OUT].as<float>();
    const float *d0i = nullptr, *d0e = nullptr;
    if (h0intra) {
        TRY(c->buf[BUF_AUX2].ensure(2 * total * 4 + 16));
        float *h0 = c->buf[BUF_AUX2].as<float>();
        TRY(h2d(h0, h0intra, total * 4, c->stream));
        TRY(h2d(h0 + total, h0inter, total * 4, c->stream));
        d0i = h0;
        d0e = h0 + total;
    }
    TRY(launch_counts_to_f32(cnt, d0i, out, total, c->stream));
    TRY(launch_counts_to_f32(cnt + total, d0e, out + total, total, c->stream));
    TRY(d2h(hintra, out, total * 4, c->stream));
    TRY(d2h(hinter, out + total, total * 4, c->stream));
    uint32_t status = 0;
    TRY(d2h(&status, c->buf[BUF_STATUS].p, 4, c->stream));
    TRY(finish(c));
    if (status)
        return set_error(FRMC_E_TIMEOUT, "device wait gave up (status 0x%x)", status);
    return FRMC_OK;
}

// Host-buffer calls with at most this many rows read the caller's arrays
// directly where the device accesses pageable memory: the row kernel reads
// every column once per 64 rows, so up to 64 rows read no more than a copy.
constexpr int64_t kDirectRows = 64;

// counts_out for pageable-access devices after kernels without device waits
// (no status to read): one conversion kernel writes the caller's float32
// histograms directly and leaves the counts zero for the next call.
static int counts_out_direct(Context *c, int64_t total, float *hintra, float *hinter)
{
    unsigned *cnt = c->buf[BUF_COUNTS].as<unsigned>();
    TRY(launch_counts_pair_to_f32_zero(cnt, total, hintra, hinter, c->stream));
    c->counts_clean = 2 * (size_t)total * 4;
    return finish(c);
}

}  // namespace frmc


using namespace frmc;

extern "C" {

int frmc_version(void) { return 10000; }

const char *frmc_last_error(void) { return last_error(); }

int frmc_set_device(int device)
{
    FRMC_CUDA(cudaSetDevice(device));
    return FRMC_OK;
}

int frmc_device_info(int *sms, int *max_smem_optin, int *cc_major, int *cc_minor)
{
    Context *c;
    TRY(get_context(&c));
    if (sms) *sms = c->sms;
    if (max_smem_optin) *max_smem_optin = c->max_smem_optin;
    int dev = c->device;
    if (cc_major) FRMC_CUDA(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev));
    if (cc_minor) FRMC_CUDA(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
    return FRMC_OK;
}

int frmc_set_full_tune(int threads, int rows, int queued, int qcap, int ctas_per_sm, double min_pairs_tiled)
{
    if (threads % 32 || threads < 64 || threads > 1024 || (rows != 1 && rows != 2) || qcap < 0 || ctas_per_sm < 1 ||
        !(min_pairs_tiled >= 0))
        return set_error(FRMC_E_ARG, "invalid tile configuration");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_full_tune.threads = threads;
    g_full_tune.rows = rows;
    g_full_tune.queued = queued;
    g_full_tune.qcap = qcap;
    g_full_tune.ctas_per_sm = ctas_per_sm;
    g_full_tune.min_pairs_tiled = min_pairs_tiled;
    return FRMC_OK;
}

int frmc_set_full_aggregate(int on)
{
    if (on != 0 && on != 1)
        return set_error(FRMC_E_ARG, "aggregate must be 0 or 1");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_full_tune.aggregate = on;
    return FRMC_OK;
}

int frmc_sq_limits(float minDistance, float maxDistance, float *s_lo, float *s_hi)
{
    sq_limits(minDistance, maxDistance, s_lo, s_hi);
    return FRMC_OK;
}

int frmc_basis_mode(const float *basis, int isPBC) { return basis_mode(isPBC ? basis : kIdentity, isPBC); }

int frmc_full_items(int64_t n, int64_t *nitems)
{
    TRY(check_n(n, "atoms"));
    FullTune tn = current_tune();
    *nitems = n < 2 ? 0 : full_hist_items((int)n, &tn);
    return FRMC_OK;
}

// ----------------------------------------------------------- distances (host)
static int distances_common(int diff, int32_t atomIndex, const int32_t *indexes, int64_t K, const float *points,
                            int64_t ps, const float *coords, int64_t n, const float *basis, int isPBC, int allAtoms,
                            float *out)
{
    TRY(check_n(n, "coords"));
    if (K < 0 || K > 65535)
        return set_error(FRMC_E_ARG, "number of points %lld out of range", (long long)K);
    int single_index = indexes == nullptr && points == nullptr;
    if (single_index && (atomIndex < 0 || atomIndex >= n))
        return set_error(FRMC_E_INDEX, "atomIndex %d out of range for %lld atoms", atomIndex, (long long)n);
    if (indexes)
        TRY(check_indexes(indexes, K, n));
    if (n == 0 || K == 0)
        return FRMC_OK;
    const float *B = isPBC ? basis : kIdentity;
    LOCKED_CTX(c);
    TRY(upload_atoms(c, coords, nullptr, nullptr, n));
    const int width = diff ? 3 : 1;
    const int64_t out_elems = n * width * K;
    TRY(c->buf[BUF_OUT].ensure(out_elems * 4 + 16));
    const int *didx = nullptr;
    const float *dpts = nullptr;
    if (single_index || indexes) {
        TRY(c->buf[BUF_ROWS].ensure(K * 4 + 16));
        TRY(h2d(c->buf[BUF_ROWS].p, single_index ? &atomIndex : indexes, K * 4, c->stream));
        didx = c->buf[BUF_ROWS].as<int>();
    } else {
        TRY(c->buf[BUF_AUX0].ensure(3 * ps * 4 + 16));
        TRY(h2d(c->buf[BUF_AUX0].p, points, 3 * ps * 4, c->stream));
        dpts = c->buf[BUF_AUX0].as<float>();
    }
    const int fromIndex = (didx && !allAtoms) ? 1 : 0;
    float *dout = c->buf[BUF_OUT].as<float>();
    // Multi-index rows below their start keep the caller's values.
    if (fromIndex && !single_index)
        TRY(h2d(dout, out, out_elems * 4, c->stream));
    if (diff)
        TRY(launch_differences(c->buf[BUF_COORDS].as<float>(), (int)n, dpts, ps, didx, (int)K, fromIndex, isPBC, B,
                               dout, c->stream));
    else
        TRY(launch_distances(c->buf[BUF_COORDS].as<float>(), (int)n, dpts, ps, didx, (int)K, fromIndex, isPBC, B,
                             dout, c->stream));
    if (fromIndex && single_index) {
        const int64_t off = (int64_t)atomIndex * width;
        TRY(d2h(out + off, dout + off, (out_elems - off) * 4, c->stream));
    } else {
        TRY(d2h(out, dout, out_elems * 4, c->stream));
    }
    return finish(c);
}

int frmc_pairs_distances_to_indexcoords(int32_t atomIndex, const float *coords, int64_t n, const float *basis,
                                        int isPBC, int allAtoms, float *distances)
{
    return distances_common(0, atomIndex, nullptr, 1, nullptr, 0, coords, n, basis, isPBC, allAtoms, distances);
}

int frmc_pairs_distances_to_point(const float *point, const float *coords, int64_t n, const float *basis, int isPBC,
                                  float *distances)
{
    return distances_common(0, 0, nullptr, 1, point, 1, coords, n, basis, isPBC, 1, distances);
}

int frmc_pairs_distances_to_multi_points(const float *points, int64_t ps, int64_t K, const float *coords, int64_t n,
                                         const float *basis, int isPBC, float *distances)
{
    return distances_common(0, 0, nullptr, K, points, ps, coords, n, basis, isPBC, 1, distances);
}

int frmc_pairs_distances_to_multi_indexcoords(const int32_t *indexes, int64_t K, const float *coords, int64_t n,
                                              const float *basis, int isPBC, int allAtoms, float *distances)
{
    if (K == 0)
        return FRMC_OK;
    return distances_common(0, 0, indexes, K, nullptr, 0, coords, n, basis, isPBC, allAtoms, distances);
}

int frmc_point_to_point_distance(const float *point1, const float *point2, const float *basis, int isPBC,
                                 float *distance)
{
    return distances_common(0, 0, nullptr, 1, point1, 1, point2, 1, basis, isPBC, 1, distance);
}

int frmc_pairs_differences_to_point(const float *point, const float *coords, int64_t n, const float *basis,
                                    int isPBC, float *differences)
{
    return distances_common(1, 0, nullptr, 1, point, 1, coords, n, basis, isPBC, 1, differences);
}

int frmc_pairs_differences_to_indexcoords(int32_t atomIndex, const float *coords, int64_t n, const float *basis,
                                          int isPBC, int allAtoms, float *differences)
{
    return distances_common(1, atomIndex, nullptr, 1, nullptr, 0, coords, n, basis, isPBC, allAtoms, differences);
}

int frmc_pairs_differences_to_multi_points(const float *points, int64_t ps, int64_t K, const float *coords,
                                           int64_t n, const float *basis, int isPBC, float *differences)
{
    return distances_common(1, 0, nullptr, K, points, ps, coords, n, basis, isPBC, 1, differences);
}

int frmc_pairs_differences_to_multi_indexcoords(const int32_t *indexes, int64_t K, const float *coords, int64_t n,
                                                const float *basis, int isPBC, int allAtoms, float *differences)
{
    if (K == 0)
        return FRMC_OK;
    return distances_common(1, 0, indexes, K, nullptr, 0, coords, n, basis, isPBC, allAtoms, differences);
}

int frmc_pair_difference_to_point(const float *point1, const float *point2, const float *basis, int isPBC,
                                  float *difference)
{
    // bc(point2 - point1): the "point" is point2, the single coordinate point1.
    return distances_common(1, 0, nullptr, 1, point2, 1, point1, 1, basis, isPBC, 1, difference);
}

int frmc_from_to_points_differences(const float *pointsFrom, const float *pointsTo, int64_t n, const float *basis,
                                    int isPBC, float *differences)
{
    TRY(check_n(n, "points"));
    if (n == 0)
        return FRMC_OK;
    const float *B = isPBC ? basis : kIdentity;
    LOCKED_CTX(c);
    TRY(c->buf[BUF_COORDS].ensure(n * 12 + 16));
    TRY(c->buf[BUF_AUX0].ensure(n * 12 + 16));
    TRY(c->buf[BUF_OUT].ensure(n * 12 + 16));
    TRY(h2d(c->buf[BUF_COORDS].p, pointsFrom, n * 12, c->stream));
    TRY(h2d(c->buf[BUF_AUX0].p, pointsTo, n * 12, c->stream));
    TRY(launch_from_to(c->buf[BUF_COORDS].as<float>(), c->buf[BUF_AUX0].as<float>(), (int)n, isPBC, B,
                       c->buf[BUF_OUT].as<float>(), c->stream));
    TRY(d2h(differences, c->buf[BUF_OUT].p, n * 12, c->stream));
    return finish(c);
}

int frmc_transform_coordinates(const float *transMatrix, const float *coords, int64_t n, float *out)
{
    TRY(check_n(n, "coords"));
    if (n == 0)
        return FRMC_OK;
    LOCKED_CTX(c);
    TRY(c->buf[BUF_COORDS].ensure(n * 12 + 16));
    TRY(c->buf[BUF_OUT].ensure(n * 12 + 16));
    TRY(h2d(c->buf[BUF_COORDS].p, coords, n * 12, c->stream));
    TRY(launch_transform(transMatrix, c->buf[BUF_COORDS].as<float>(), (int)n, c->buf[BUF_OUT].as<float>(),
                         c->stream));
    TRY(d2h(out, c->buf[BUF_OUT].p, n * 12, c->stream));
    return finish(c);
}

// ---------------------------------------------------------- histograms (host)
int frmc_full_pairs_histograms_coords(const float *boxCoords, int64_t n, const float *basis, int isPBC,
                                      const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                      float minDistance, float maxDistance, float bin, int32_t hs, float *hintra,
                                      float *hinter)
{
    int64_t total;
    TRY(check_n(n, "boxCoords"));
    TRY(check_hist(ne, hs, &total));
    if (total == 0)
        return FRMC_OK;
    if (n < 2) {
        memset(hintra, 0, total * 4);
        memset(hinter, 0, total * 4);
        return FRMC_OK;
    }
    LOCKED_CTX(c);
    TRY(upload_atoms(c, boxCoords, moleculeIndex, elementIndex, n));
    TRY(prepare_counts(c, total));
    TRY(full_counts(c, n, basis, isPBC, ne, minDistance, maxDistance, bin, hs, total,
                    c->buf[BUF_COUNTS].as<unsigned>()));
    return counts_out(c, total, nullptr, nullptr, hintra, hinter);
}

int frmc_shape_function(const float *boxCoords, int64_t n, const float *basis, int isPBC,
                        const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne, float minDistance,
                        float maxDistance, float bin, int32_t hs, int32_t npairs, const int32_t *pair_i,
                        const int32_t *pair_j, const double *pair_coef, const double *shellCenters,
                        const double *shellVolumes, double rho0, const double *qValues, int32_t nq,
                        const double *rValues, int32_t nr, double *Gr, double *Sq, double *Gshape)
{
    int64_t total;
    TRY(check_n(n, "boxCoords"));
    TRY(check_hist(ne, hs, &total));
    if (hs < 2 || nq < 2 || nr < 0 || npairs < 0)
        return set_error(FRMC_E_ARG, "shape function: needs at least two shells and two q values");
    for (int32_t p = 0; p < npairs; ++p)
        if (pair_i[p] < 0 || pair_i[p] >= ne || pair_j[p] < 0 || pair_j[p] >= ne)
            return set_error(FRMC_E_INDEX, "shape function: element pair %d out of range", p);
    for (int64_t i = 0; i < n; ++i)
        if (elementIndex[i] < 0 || elementIndex[i] >= ne)
            return set_error(FRMC_E_INDEX, "element index %d out of range for %d elements", elementIndex[i], ne);
    LOCKED_CTX(c);
    TRY(prepare_counts(c, total));
    if (n >= 2) {
        TRY(upload_atoms(c, boxCoords, moleculeIndex, elementIndex, n));
        TRY(full_counts(c, n, basis, isPBC, ne, minDistance, maxDistance, bin, hs, total,
                        c->buf[BUF_COUNTS].as<unsigned>()));
    }
    // FP64 block: pc, r, vol, q, rv, G, S, Gs, w1, w2 (doubles), then pair_i, pair_j (ints)
    const size_t nd = (size_t)npairs + 2 * (size_t)hs + (size_t)nq + (size_t)nr + (size_t)hs + (size_t)nq +
                      (size_t)nr + (size_t)hs + (size_t)nq;
    TRY(c->buf[BUF_AUX1].ensure(8 * nd + 8 * (size_t)npairs + 64));
    double *d = c->buf[BUF_AUX1].as<double>();
    double *pc = d, *r = pc + npairs, *vol = r + hs, *q = vol + hs, *rv = q + nq, *G = rv + nr, *S = G + hs,
           *Gs = S + nq, *w1 = Gs + nr, *w2 = w1 + hs;
    int *pij = reinterpret_cast<int *>(w2 + nq);
    TRY(h2d(pc, pair_coef, 8 * (size_t)npairs, c->stream));
    TRY(h2d(r, shellCenters, 8 * (size_t)hs, c->stream));
    TRY(h2d(vol, shellVolumes, 8 * (size_t)hs, c->stream));
    TRY(h2d(q, qValues, 8 * (size_t)nq, c->stream));
    TRY(h2d(rv, rValues, 8 * (size_t)nr, c->stream));
    TRY(h2d(pij, pair_i, 4 * (size_t)npairs, c->stream));
    TRY(h2d(pij + npairs, pair_j, 4 * (size_t)npairs, c->stream));
    TRY(launch_shape_function(c->buf[BUF_COUNTS].as<unsigned>(), ne, hs, npairs, pij, pij + npairs, pc, r, vol, rho0,
                              shellCenters[1] - shellCenters[0], q, nq, qValues[1] - qValues[0], rv, nr, G, S, Gs,
                              w1, w2, c->stream));
    if (Gr)
        TRY(d2h(Gr, G, 8 * (size_t)hs, c->stream));
    if (Sq)
        TRY(d2h(Sq, S, 8 * (size_t)nq, c->stream));
    if (Gshape)
        TRY(d2h(Gshape, Gs, 8 * (size_t)nr, c->stream));
    uint32_t status = 0;
    TRY(d2h(&status, c->buf[BUF_STATUS].p, 4, c->stream));
    TRY(finish(c));
    if (status)
        return set_error(FRMC_E_TIMEOUT, "device wait gave up (status 0x%x)", status);
    return FRMC_OK;
}

int frmc_multiple_pairs_histograms_coords(const int32_t *indexes, int64_t K, const float *boxCoords, int64_t n,
                                          const float *basis, int isPBC, const int32_t *moleculeIndex,
                                          const int32_t *elementIndex, int32_t ne, float minDistance,
                                          float maxDistance, float bin, int32_t hs, int allAtoms, float *hintra,
                                          float *hinter)
{
    int64_t total;
    TRY(check_n(n, "boxCoords"));
    TRY(check_hist(ne, hs, &total));
    if (K < 0 || K > (int64_t)65535 * 64)
        return set_error(FRMC_E_ARG, "number of indexes %lld out of range", (long long)K);
    TRY(check_indexes(indexes, K, n));
    if (total == 0)
        return FRMC_OK;
    if (K == 0 || n == 0) {
        memset(hintra, 0, total * 4);
        memset(hinter, 0, total * 4);
        return FRMC_OK;
    }
    const float *B = isPBC ? basis : kIdentity;
    LOCKED_CTX(c);
    const bool direct = c->pageable && K <= kDirectRows;
    TRY(prepare_counts(c, total, !direct));  // the row kernels have no device waits
    unsigned *cnt = c->buf[BUF_COUNTS].as<unsigned>();
    if (direct) {
        // the per-move call (fullrmc's moved atoms, PairDistributionConstraints.py:1016-1026):
        // the kernels read the caller's arrays and write its histograms in place
        TRY(launch_rows_hist(boxCoords, elementIndex, moleculeIndex, (int)n, indexes, (int)K, allAtoms,
                             basis_mode(B, isPBC), make_basis(B), minDistance, maxDistance, bin, ne, hs, cnt,
                             cnt + total, c->stream));
        return counts_out_direct(c, total, hintra, hinter);
    }
    TRY(upload_atoms(c, boxCoords, moleculeIndex, elementIndex, n));
    TRY(c->buf[BUF_ROWS].ensure(K * 4 + 16));
    TRY(h2d(c->buf[BUF_ROWS].p, indexes, K * 4, c->stream));
    TRY(launch_rows_hist(c->buf[BUF_COORDS].as<float>(), c->buf[BUF_EL].as<int>(), c->buf[BUF_MOL].as<int>(), (int)n,
                         c->buf[BUF_ROWS].as<int>(), (int)K, allAtoms, basis_mode(B, isPBC), make_basis(B),
                         minDistance, maxDistance, bin, ne, hs, cnt, cnt + total, c->stream));
    return counts_out(c, total, nullptr, nullptr, hintra, hinter);
}

int frmc_group_move_delta_histograms(const int32_t *indexes, int64_t K, const float *boxCoords, int64_t n,
                                     const float *newBoxCoords, const float *basis, int isPBC,
                                     const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                     float minDistance, float maxDistance, float bin, int32_t hs, int32_t *dintra,
                                     int32_t *dinter)
{
    int64_t total;
    TRY(check_n(n, "boxCoords"));
    TRY(check_hist(ne, hs, &total));
    if (K < 0 || K > 1024)
        return set_error(FRMC_E_ARG, "group_move_delta_histograms: %lld moved atoms (at most 1024)", (long long)K);
    TRY(check_indexes(indexes, K, n));
    if (total == 0)
        return FRMC_OK;
    memset(dintra, 0, total * 4);
    memset(dinter, 0, total * 4);
    if (K == 0 || n == 0)
        return FRMC_OK;
    const float *B = isPBC ? basis : kIdentity;
    // the group in group order, then its atoms sorted with their positions
    std::vector<int32_t> rows(3 * (size_t)K);
    std::vector<std::pair<int32_t, int32_t>> order((size_t)K);
    for (int64_t k = 0; k < K; ++k) {
        rows[k] = indexes[k];
        order[k] = std::make_pair(indexes[k], (int32_t)k);
    }
    std::sort(order.begin(), order.end());
    for (int64_t k = 0; k < K; ++k) {
        rows[K + k] = order[k].first;
        rows[2 * K + k] = order[k].second;
    }
    LOCKED_CTX(c);
    TRY(upload_atoms(c, boxCoords, moleculeIndex, elementIndex, n));
    TRY(c->buf[BUF_ROWS].ensure(K * 12 + 16));
    TRY(h2d(c->buf[BUF_ROWS].p, rows.data(), K * 12, c->stream));
    TRY(c->buf[BUF_AUX0].ensure(K * 12 + 16));
    TRY(h2d(c->buf[BUF_AUX0].p, newBoxCoords, K * 12, c->stream));
    TRY(c->buf[BUF_AUX1].ensure(total * 8 + 16));
    int *d = c->buf[BUF_AUX1].as<int>();
    FRMC_CUDA(cudaMemsetAsync(d, 0, total * 8, c->stream));
    const int *rw = c->buf[BUF_ROWS].as<int>();
    TRY(launch_group_delta(c->buf[BUF_COORDS].as<float>(), c->buf[BUF_AUX0].as<float>(), c->buf[BUF_EL].as<int>(),
                           c->buf[BUF_MOL].as<int>(), (int)n, rw, rw + K, (int)K, basis_mode(B, isPBC), make_basis(B),
                           minDistance, maxDistance, bin, ne, hs, d, d + total, c->stream));
    TRY(d2h(dintra, d, total * 4, c->stream));
    TRY(d2h(dinter, d + total, total * 4, c->stream));
    return finish(c);
}

int frmc_multiple_pairs_histograms_dists(const int32_t *indexes, int64_t K, const float *distances, int64_t n,
                                         const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                         float minDistance, float maxDistance, float bin, int32_t hs, int allAtoms,
                                         float *hintra, float *hinter)
{
    int64_t total;
    TRY(check_n(n, "distances"));
    TRY(check_hist(ne, hs, &total));
    if (K < 0 || K > 65535)
        return set_error(FRMC_E_ARG, "number of indexes %lld out of range", (long long)K);
    TRY(check_indexes(indexes, K, n));
    if (total == 0)
        return FRMC_OK;
    if (K == 0 || n == 0) {
        memset(hintra, 0, total * 4);
        memset(hinter, 0, total * 4);
        return FRMC_OK;
    }
    LOCKED_CTX(c);
    TRY(c->buf[BUF_AUX0].ensure(n * K * 4 + 16));
    TRY(h2d(c->buf[BUF_AUX0].p, distances, n * K * 4, c->stream));
    TRY(c->buf[BUF_EL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_EL].p, elementIndex, n * 4, c->stream));
    TRY(c->buf[BUF_MOL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_MOL].p, moleculeIndex, n * 4, c->stream));
    TRY(c->buf[BUF_ROWS].ensure(K * 4 + 16));
    TRY(h2d(c->buf[BUF_ROWS].p, indexes, K * 4, c->stream));
    TRY(prepare_counts(c, total));
    unsigned *cnt = c->buf[BUF_COUNTS].as<unsigned>();
    TRY(launch_dists_hist(c->buf[BUF_AUX0].as<float>(), (int)n, (int)K, c->buf[BUF_ROWS].as<int>(),
                          c->buf[BUF_EL].as<int>(), c->buf[BUF_MOL].as<int>(), allAtoms, minDistance, maxDistance, bin,
                          ne, hs, cnt, cnt + total, c->stream));
    return counts_out(c, total, nullptr, nullptr, hintra, hinter);
}

int frmc_single_pairs_histograms(int32_t atomIndex, const float *distances, int64_t n, const int32_t *moleculeIndex,
                                 const int32_t *elementIndex, int32_t ne, int32_t hs, float *hintra, float *hinter,
                                 float minDistance, float maxDistance, float bin, int allAtoms)
{
    int64_t total;
    TRY(check_n(n, "distances"));
    TRY(check_hist(ne, hs, &total));
    if (atomIndex < 0 || atomIndex >= n)
        return set_error(FRMC_E_INDEX, "atomIndex %d out of range for %lld atoms", atomIndex, (long long)n);
    if (total == 0)
        return FRMC_OK;
    LOCKED_CTX(c);
    TRY(c->buf[BUF_AUX0].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_AUX0].p, distances, n * 4, c->stream));
    TRY(c->buf[BUF_EL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_EL].p, elementIndex, n * 4, c->stream));
    TRY(c->buf[BUF_MOL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_MOL].p, moleculeIndex, n * 4, c->stream));
    TRY(c->buf[BUF_ROWS].ensure(16));
    TRY(h2d(c->buf[BUF_ROWS].p, &atomIndex, 4, c->stream));
    TRY(prepare_counts(c, total));
    unsigned *cnt = c->buf[BUF_COUNTS].as<unsigned>();
    TRY(launch_dists_hist(c->buf[BUF_AUX0].as<float>(), (int)n, 1, c->buf[BUF_ROWS].as<int>(), c->buf[BUF_EL].as<int>(),
                          c->buf[BUF_MOL].as<int>(), allAtoms, minDistance, maxDistance, bin, ne, hs, cnt, cnt + total,
                          c->stream));
    return counts_out(c, total, hintra, hinter, hintra, hinter);
}

// ------------------------------------------------------------ FP64 transforms
static int sine_common(int kind, const float *xs, int64_t nx, const float *ys, const float *f, int64_t ny, double rho,
                       double *out)
{
    TRY(check_n(nx, "output grid"));
    TRY(check_n(ny, "input grid"));
    if (nx == 0)
        return FRMC_OK;
    if (ny < 2)
        return set_error(FRMC_E_ARG, "the summation grid needs at least two points");
    LOCKED_CTX(c);
    TRY(c->buf[BUF_AUX0].ensure(nx * 4 + 16));
    TRY(c->buf[BUF_AUX1].ensure(ny * 8 + 16));
    TRY(c->buf[BUF_OUT].ensure(nx * 8 + 16));
    float *dxs = c->buf[BUF_AUX0].as<float>();
    float *dys = c->buf[BUF_AUX1].as<float>();
    float *df = dys + ny;
    TRY(h2d(dxs, xs, nx * 4, c->stream));
    TRY(h2d(dys, ys, ny * 4, c->stream));
    TRY(h2d(df, f, ny * 4, c->stream));
    TRY(c->buf[BUF_AUX2].ensure(8 * (size_t)(nx + 2 * ny) + 16));
    TRY(launch_sine(kind, dxs, (int)nx, dys, df, (int)ny, rho, c->buf[BUF_OUT].as<double>(),
                    c->buf[BUF_AUX2].as<double>(), c->stream));
    TRY(d2h(out, c->buf[BUF_OUT].p, nx * 8, c->stream));
    return finish(c);
}

// ----------------------------------------------- atomic distances (host)
// atomic_distances.pyx: counts and float32 sums of the pairs inside (or
// outside) per-element-pair limits; see atomic_kernels.cu.

static int atomic_checks(int64_t n, int64_t K, int32_t ne, const int32_t *el, int64_t nel)
{
    TRY(check_n(n, "coordinates"));
    if (K < 0 || K > INT_MAX / 4)
        return set_error(FRMC_E_ARG, "number of indexes %lld out of range", (long long)K);
    if (ne < 1 || ne > 16)
        return set_error(FRMC_E_ARG, "numberOfElements %d out of range (1..16)", ne);
    for (int64_t i = 0; i < nel; ++i)
        if (el[i] < 0 || el[i] >= ne)
            return set_error(FRMC_E_INDEX, "element index %d out of range for %d elements", el[i], ne);
    return FRMC_OK;
}

// Device accumulators [dsum 2 ne^2 floats][nsum 2 ne^2 ints], limits
// [lower ne^2][upper ne^2]; starting values from the given arrays (or 0).
static int atomic_prepare(Context *c, int32_t ne, const float *lower, const float *upper, const int32_t *nintra0,
                          const float *dintra0, const int32_t *ninter0, const float *dinter0)
{
    const size_t m = (size_t)ne * ne;
    TRY(c->buf[BUF_ATOMIC_LIMITS].ensure(8 * m + 16));
    TRY(c->buf[BUF_ATOMIC_ACC].ensure(16 * m + 16));
    float *lim = c->buf[BUF_ATOMIC_LIMITS].as<float>();
    TRY(h2d(lim, lower, 4 * m, c->stream));
    TRY(h2d(lim + m, upper, 4 * m, c->stream));
    float *acc = c->buf[BUF_ATOMIC_ACC].as<float>();
    if (dintra0) {
        TRY(h2d(acc, dintra0, 4 * m, c->stream));
        TRY(h2d(acc + m, dinter0, 4 * m, c->stream));
        TRY(h2d(acc + 2 * m, nintra0, 4 * m, c->stream));
        TRY(h2d(acc + 3 * m, ninter0, 4 * m, c->stream));
    } else {
        FRMC_CUDA(cudaMemsetAsync(acc, 0, 16 * m, c->stream));
    }
    return FRMC_OK;
}

static int atomic_finish(Context *c, int32_t ne, int32_t *nintra, float *dintra, int32_t *ninter, float *dinter)
{
    const size_t m = (size_t)ne * ne;
    const float *acc = c->buf[BUF_ATOMIC_ACC].as<float>();
    TRY(d2h(dintra, acc, 4 * m, c->stream));
    TRY(d2h(dinter, acc + m, 4 * m, c->stream));
    TRY(d2h(nintra, acc + 2 * m, 4 * m, c->stream));
    TRY(d2h(ninter, acc + 3 * m, 4 * m, c->stream));
    return finish(c);
}

static int atomic_run(Context *c, const float *dists_dev, int K, int n, int allAtoms, int flags, int ne,
                      const float *basis, int isPBC)
{
    const size_t m = (size_t)ne * ne;
    float *lim = c->buf[BUF_ATOMIC_LIMITS].as<float>();
    float *acc = c->buf[BUF_ATOMIC_ACC].as<float>();
    return atomic_distances_run(c, dists_dev ? nullptr : c->buf[BUF_COORDS].as<float>(), dists_dev,
                                c->buf[BUF_ROWS].as<int>(), K, n, allAtoms, flags, ne, basis, isPBC,
                                c->buf[BUF_MOL].as<int>(), c->buf[BUF_EL].as<int>(), lim, lim + m, acc,
                                reinterpret_cast<int *>(acc + 2 * m), c->stream);
}

int frmc_multiple_atomic_distances_coords(const int32_t *indexes, int64_t K, const float *boxCoords, int64_t n,
                                          const float *basis, int isPBC, const int32_t *moleculeIndex,
                                          const int32_t *elementIndex, int32_t ne, const float *lowerLimit,
                                          const float *upperLimit, int flags, int allAtoms, int32_t *nintra,
                                          float *dintra, int32_t *ninter, float *dinter)
{
    TRY(atomic_checks(n, K, ne, elementIndex, n));
    TRY(check_indexes(indexes, K, n));
    LOCKED_CTX(c);
    TRY(upload_atoms(c, boxCoords, moleculeIndex, elementIndex, n));
    TRY(c->buf[BUF_ROWS].ensure(K * 4 + 16));
    TRY(h2d(c->buf[BUF_ROWS].p, indexes, K * 4, c->stream));
    TRY(atomic_prepare(c, ne, lowerLimit, upperLimit, nullptr, nullptr, nullptr, nullptr));
    TRY(atomic_run(c, nullptr, (int)K, (int)n, allAtoms, flags, ne, basis, isPBC));
    return atomic_finish(c, ne, nintra, dintra, ninter, dinter);
}

int frmc_multiple_atomic_distances_dists(const int32_t *indexes, int64_t K, const float *distances, int64_t n,
                                         const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                         const float *lowerLimit, const float *upperLimit, int flags, int allAtoms,
                                         int32_t *nintra, float *dintra, int32_t *ninter, float *dinter)
{
    TRY(atomic_checks(n, K, ne, elementIndex, n));
    TRY(check_indexes(indexes, K, n));
    LOCKED_CTX(c);
    TRY(c->buf[BUF_EL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_EL].p, elementIndex, n * 4, c->stream));
    TRY(c->buf[BUF_MOL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_MOL].p, moleculeIndex, n * 4, c->stream));
    TRY(c->buf[BUF_AUX0].ensure((size_t)n * K * 4 + 16));
    TRY(h2d(c->buf[BUF_AUX0].p, distances, (size_t)n * K * 4, c->stream));
    TRY(c->buf[BUF_ROWS].ensure(K * 4 + 16));
    TRY(h2d(c->buf[BUF_ROWS].p, indexes, K * 4, c->stream));
    TRY(atomic_prepare(c, ne, lowerLimit, upperLimit, nullptr, nullptr, nullptr, nullptr));
    TRY(atomic_run(c, c->buf[BUF_AUX0].as<float>(), (int)K, (int)n, allAtoms, flags, ne, nullptr, 0));
    return atomic_finish(c, ne, nintra, dintra, ninter, dinter);
}

int frmc_single_atomic_distances_dists(int32_t atomIndex, const float *distances, int64_t n,
                                       const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                       float *dintra, float *dinter, int32_t *nintra, int32_t *ninter,
                                       const float *lowerLimit, const float *upperLimit, int flags, int allAtoms)
{
    TRY(atomic_checks(n, 1, ne, elementIndex, n));
    if (atomIndex < 0 || atomIndex >= n)
        return set_error(FRMC_E_INDEX, "atomIndex %d out of range for %lld atoms", atomIndex, (long long)n);
    LOCKED_CTX(c);
    TRY(c->buf[BUF_EL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_EL].p, elementIndex, n * 4, c->stream));
    TRY(c->buf[BUF_MOL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_MOL].p, moleculeIndex, n * 4, c->stream));
    TRY(c->buf[BUF_AUX0].ensure((size_t)n * 4 + 16));
    TRY(h2d(c->buf[BUF_AUX0].p, distances, (size_t)n * 4, c->stream));
    TRY(c->buf[BUF_ROWS].ensure(16));
    TRY(h2d(c->buf[BUF_ROWS].p, &atomIndex, 4, c->stream));
    TRY(atomic_prepare(c, ne, lowerLimit, upperLimit, nintra, dintra, ninter, dinter));
    TRY(atomic_run(c, c->buf[BUF_AUX0].as<float>(), 1, (int)n, allAtoms, flags, ne, nullptr, 0));
    return atomic_finish(c, ne, nintra, dintra, ninter, dinter);
}

int frmc_pair_elements_stats(const int32_t *elementIndex, const int32_t *moleculeIndex, int64_t n, int32_t ne,
                             int32_t *nintra, int32_t *ninter)
{
    TRY(atomic_checks(n, 0, ne, elementIndex, n));
    const size_t m = (size_t)ne * ne;
    LOCKED_CTX(c);
    TRY(c->buf[BUF_EL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_EL].p, elementIndex, n * 4, c->stream));
    TRY(c->buf[BUF_MOL].ensure(n * 4 + 16));
    TRY(h2d(c->buf[BUF_MOL].p, moleculeIndex, n * 4, c->stream));
    TRY(c->buf[BUF_ATOMIC_ACC].ensure(8 * m + 16));
    int *acc = c->buf[BUF_ATOMIC_ACC].as<int>();
    FRMC_CUDA(cudaMemsetAsync(acc, 0, 8 * m, c->stream));
    TRY(launch_pair_stats(c->buf[BUF_EL].as<int>(), c->buf[BUF_MOL].as<int>(), (int)n, ne, acc, acc + m, c->stream));
    TRY(d2h(nintra, acc, 4 * m, c->stream));
    TRY(d2h(ninter, acc + m, 4 * m, c->stream));
    return finish(c);
}

// ----------------------------------------------- coordination numbers (host)
// atomic_coordination.pyx: every entry point is a sequence of terms (a row,
// an index list, a definition); see coord_kernels.cu.  Everything is checked
// before anything runs, so an index error leaves coordNumData unchanged.

static int coord_index_error(const int32_t *list, int64_t len, int64_t rowlen)
{
    for (int64_t e = 0; e < len; ++e)
        if (list[e] < -rowlen || list[e] >= rowlen)
            return set_error(FRMC_E_INDEX, "index %d is out of bounds for axis 0 with size %lld", list[e],
                             (long long)rowlen);
    return FRMC_OK;
}

static size_t align16(size_t x)
{
    return (x + 15) & ~(size_t)15;
}

int frmc_coordination_terms(const float *boxCoords, int64_t n, const float *basis, int isPBC, const float *distances,
                            const int64_t *dist_off, const int32_t *dist_len, int32_t nrows, const int32_t *lists,
                            const int64_t *list_off, int32_t nlists, const int32_t *term_row,
                            const int32_t *term_list, const int32_t *term_def, int64_t nterms,
                            const float *lowerShells, const float *upperShells, float *coordNumData, int32_t ndata)
{
    const bool coords = boxCoords != nullptr;
    TRY(check_n(coords ? n : 0, "coordinates"));
    if (nterms < 0 || nterms > INT_MAX / 2 || nlists < 0 || ndata < 0 || nrows < 0)
        return set_error(FRMC_E_ARG, "coordination: negative or too many terms, lists or definitions");
    if (nterms == 0)
        return FRMC_OK;
    if (!coords && !distances)
        return set_error(FRMC_E_ARG, "coordination: neither coordinates nor distances given");
    const int64_t npool = nlists ? list_off[nlists] : 0;
    for (int32_t l = 0; l < nlists; ++l)
        if (list_off[l] < 0 || list_off[l] > list_off[l + 1] || list_off[l + 1] - list_off[l] > INT_MAX)
            return set_error(FRMC_E_ARG, "coordination: bad list offsets");
    int64_t dpool = 0;
    if (!coords)
        for (int32_t r = 0; r < nrows; ++r) {
            if (dist_off[r] < 0 || dist_len[r] < 0)
                return set_error(FRMC_E_ARG, "coordination: bad distance row offsets");
            dpool = std::max<int64_t>(dpool, dist_off[r] + dist_len[r]);
        }
    // per-list extremes, computed for the lists the terms use
    std::vector<int32_t> lmin(nlists, INT_MAX), lmax(nlists, INT_MIN);
    std::vector<char> seen(nlists, 0);
    std::vector<int> def_count((size_t)ndata + 1, 0);
    long long nitems = 0;
    const int chunk = coordination_chunk();
    for (int64_t t = 0; t < nterms; ++t) {
        const int32_t l = term_list[t], d = term_def[t], r = term_row[t];
        if (l < 0 || l >= nlists)
            return set_error(FRMC_E_ARG, "coordination: term %lld names list %d of %d", (long long)t, l, nlists);
        if (d < 0 || d >= ndata)
            return set_error(FRMC_E_INDEX, "definition index %d out of range for %d definitions", d, ndata);
        const int64_t rows = coords ? n : nrows;
        if (r < 0 || r >= rows)
            return set_error(FRMC_E_INDEX, "index %d is out of bounds for axis 0 with size %lld", r,
                             (long long)rows);
        const int32_t *lp = lists + list_off[l];
        const int64_t len = list_off[l + 1] - list_off[l];
        if (!seen[l]) {
            seen[l] = 1;
            for (int64_t e = 0; e < len; ++e) {
                lmin[l] = std::min(lmin[l], lp[e]);
                lmax[l] = std::max(lmax[l], lp[e]);
            }
        }
        const int64_t rowlen = coords ? n : dist_len[r];
        if (len && (lmin[l] < -rowlen || lmax[l] >= rowlen))
            return coord_index_error(lp, len, rowlen);
        nitems += (len + chunk - 1) / chunk;
        def_count[d] += 1;
    }
    if (nitems > INT_MAX)
        return set_error(FRMC_E_ARG, "coordination: too many list entries");
    int ndefs = 0;
    for (int32_t d = 0; d < ndata; ++d) ndefs += def_count[d] > 0;
    // one staging block: terms, items, distance rows, definitions, windows,
    // accumulators and the zeroed per-term counts
    const size_t o_terms = 0;
    const size_t o_items = align16(o_terms + sizeof(CoordTerm) * (size_t)nterms);
    const size_t o_doff = align16(o_items + sizeof(int2) * (size_t)nitems);
    const size_t o_dlen = align16(o_doff + 8 * (size_t)(coords ? 0 : nrows));
    const size_t o_ids = align16(o_dlen + 4 * (size_t)(coords ? 0 : nrows));
    const size_t o_off = align16(o_ids + 4 * (size_t)ndefs);
    const size_t o_dterms = align16(o_off + 4 * (size_t)(ndefs + 1));
    const size_t o_lower = align16(o_dterms + 4 * (size_t)nterms);
    const size_t o_upper = align16(o_lower + 4 * (size_t)ndata);
    const size_t o_data = align16(o_upper + 4 * (size_t)ndata);
    const size_t o_counts = align16(o_data + 4 * (size_t)ndata);
    const size_t total = align16(o_counts + 4 * (size_t)nterms);
    std::vector<unsigned char> stage(total, 0);
    CoordTerm *T = reinterpret_cast<CoordTerm *>(stage.data() + o_terms);
    int2 *I = reinterpret_cast<int2 *>(stage.data() + o_items);
    long long k = 0;
    for (int64_t t = 0; t < nterms; ++t) {
        const int32_t l = term_list[t];
        const int64_t len = list_off[l + 1] - list_off[l];
        T[t] = CoordTerm{term_row[t], term_def[t], (long long)list_off[l], (int)len, 0};
        for (int64_t e = 0; e < len; e += chunk) I[k++] = make_int2((int)t, (int)e);
    }
    if (!coords) {
        std::memcpy(stage.data() + o_doff, dist_off, 8 * (size_t)nrows);
        std::memcpy(stage.data() + o_dlen, dist_len, 4 * (size_t)nrows);
    }
    int *ids = reinterpret_cast<int *>(stage.data() + o_ids);
    int *off = reinterpret_cast<int *>(stage.data() + o_off);
    int *dterms = reinterpret_cast<int *>(stage.data() + o_dterms);
    std::vector<int> slot((size_t)ndata, -1);
    int u = 0, acc = 0;
    for (int32_t d = 0; d < ndata; ++d)
        if (def_count[d]) {
            ids[u] = d;
            off[u] = acc;
            slot[d] = acc;
            acc += def_count[d];
            ++u;
        }
    off[ndefs] = acc;
    for (int64_t t = 0; t < nterms; ++t) dterms[slot[term_def[t]]++] = (int)t;  // stable: call order
    std::memcpy(stage.data() + o_lower, lowerShells, 4 * (size_t)ndata);
    std::memcpy(stage.data() + o_upper, upperShells, 4 * (size_t)ndata);
    std::memcpy(stage.data() + o_data, coordNumData, 4 * (size_t)ndata);

    LOCKED_CTX(c);
    TRY(c->buf[BUF_COORD_META].ensure(total));
    unsigned char *meta = c->buf[BUF_COORD_META].as<unsigned char>();
    TRY(h2d(meta, stage.data(), total, c->stream));
    TRY(c->buf[BUF_COORD_LISTS].ensure(4 * (size_t)npool + 16));
    TRY(h2d(c->buf[BUF_COORD_LISTS].p, lists, 4 * (size_t)npool, c->stream));
    CoordLaunch L;
    if (coords) {
        TRY(c->buf[BUF_COORDS].ensure(12 * (size_t)n + 16));
        TRY(h2d(c->buf[BUF_COORDS].p, boxCoords, 12 * (size_t)n, c->stream));
        L.coords = c->buf[BUF_COORDS].as<float>();
        L.basis = basis ? basis : kIdentity;
        L.isPBC = isPBC;
        L.n = (int)n;
    } else {
        TRY(c->buf[BUF_AUX0].ensure(4 * (size_t)dpool + 16));
        TRY(h2d(c->buf[BUF_AUX0].p, distances, 4 * (size_t)dpool, c->stream));
        L.dists = c->buf[BUF_AUX0].as<float>();
        L.dist_off = reinterpret_cast<const long long *>(meta + o_doff);
        L.dist_len = reinterpret_cast<const int *>(meta + o_dlen);
    }
    L.lists = c->buf[BUF_COORD_LISTS].as<int>();
    L.terms = reinterpret_cast<const CoordTerm *>(meta + o_terms);
    L.items = reinterpret_cast<const int2 *>(meta + o_items);
    L.nitems = nitems;
    L.lower = reinterpret_cast<const float *>(meta + o_lower);
    L.upper = reinterpret_cast<const float *>(meta + o_upper);
    L.counts = reinterpret_cast<int *>(meta + o_counts);
    L.def_ids = reinterpret_cast<const int *>(meta + o_ids);
    L.def_off = reinterpret_cast<const int *>(meta + o_off);
    L.def_terms = reinterpret_cast<const int *>(meta + o_dterms);
    L.ndefs = ndefs;
    L.data = reinterpret_cast<float *>(meta + o_data);
    TRY(coordination_run(L, c->stream));
    TRY(d2h(coordNumData, meta + o_data, 4 * (size_t)ndata, c->stream));
    return finish(c);
}

int frmc_gr_to_sq(const float *distances, const float *gr, int64_t nr, const float *qrange, int64_t nq, double rho,
                  double *sq)
{
    return sine_common(0, qrange, nq, distances, gr, nr, rho, sq);
}

int frmc_Gr_to_sq(const float *distances, const float *Gr, int64_t nr, const float *qrange, int64_t nq, double *sq)
{
    return sine_common(1, qrange, nq, distances, Gr, nr, 0.0, sq);
}

int frmc_sq_to_Gr(const float *qValues, int64_t nq, const float *rValues, int64_t nr, const float *sq, double *Gr)
{
    return sine_common(2, rValues, nr, qValues, sq, nq, 0.0, Gr);
}

// ------------------------------------------------------------ device entry points
static int dev_full(const void *atoms4, const int32_t *moleculeIndex, int64_t n, const float *basis_host, int isPBC,
                    int32_t ne, float minDistance, float maxDistance, float bin, int32_t hs, int64_t item_begin,
                    int64_t item_end, uint32_t *counts, void *stream)
{
    int64_t total;
    TRY(check_n(n, "atoms"));
    TRY(check_hist(ne, hs, &total));
    Context *c;
    TRY(get_context(&c));
    cudaStream_t st = (cudaStream_t)stream;
    FRMC_CUDA(cudaMemsetAsync(counts, 0, 2 * total * 4, st));
    if (n < 2 || total == 0)
        return FRMC_OK;
    if (((uintptr_t)atoms4 & 15u) || ((uintptr_t)moleculeIndex & 15u))
        return set_error(FRMC_E_ARG, "atoms4 and moleculeIndex must be 16-byte aligned");
    {
        std::lock_guard<std::mutex> lk(c->mu);
        TRY(c->buf[BUF_STATUS].ensure(16));
    }
    const float *B = isPBC ? basis_host : kIdentity;
    FullTune tn = current_tune();
    return launch_full_hist((const float4 *)atoms4, moleculeIndex, (int)n, basis_mode(B, isPBC), make_basis(B),
                            minDistance, maxDistance, bin, ne, hs, counts, counts + total,
                            c->buf[BUF_STATUS].as<uint32_t>(), accept_fraction(B, isPBC, minDistance, maxDistance),
                            &tn, st, item_begin, item_end);
}

int frmc_dev_full_hist_counts(const void *atoms4, const int32_t *moleculeIndex, int64_t n, const float *basis_host,
                              int isPBC, int32_t ne, float minDistance, float maxDistance, float bin, int32_t hs,
                              uint32_t *counts, void *stream)
{
    return dev_full(atoms4, moleculeIndex, n, basis_host, isPBC, ne, minDistance, maxDistance, bin, hs, 0, -1, counts,
                    stream);
}

int frmc_dev_full_hist_counts_range(const void *atoms4, const int32_t *moleculeIndex, int64_t n,
                                    const float *basis_host, int isPBC, int32_t ne, float minDistance,
                                    float maxDistance, float bin, int32_t hs, int64_t item_begin, int64_t item_end,
                                    uint32_t *counts, void *stream)
{
    if (item_begin < 0 || item_end < item_begin)
        return set_error(FRMC_E_ARG, "invalid item range [%lld, %lld)", (long long)item_begin, (long long)item_end);
    return dev_full(atoms4, moleculeIndex, n, basis_host, isPBC, ne, minDistance, maxDistance, bin, hs, item_begin,
                    item_end, counts, stream);
}

int frmc_dev_multiple_hist_counts(const int32_t *indexes, int64_t K, const float *boxCoords, int64_t n,
                                  const float *basis_host, int isPBC, const int32_t *moleculeIndex,
                                  const int32_t *elementIndex, int32_t ne, float minDistance, float maxDistance,
                                  float bin, int32_t hs, int allAtoms, uint32_t *counts, void *stream)
{
    int64_t total;
    TRY(check_n(n, "boxCoords"));
    TRY(check_hist(ne, hs, &total));
    if (K < 0 || K > (int64_t)65535 * 64)
        return set_error(FRMC_E_ARG, "number of indexes %lld out of range", (long long)K);
    Context *c;
    TRY(get_context(&c));
    cudaStream_t st = (cudaStream_t)stream;
    FRMC_CUDA(cudaMemsetAsync(counts, 0, 2 * total * 4, st));
    const float *B = isPBC ? basis_host : kIdentity;
    return launch_rows_hist(boxCoords, elementIndex, moleculeIndex, (int)n, indexes, (int)K, allAtoms,
                            basis_mode(B, isPBC), make_basis(B), minDistance, maxDistance, bin, ne, hs, counts,
                            counts + total, st);
}

int frmc_dev_pack_atoms(const float *coords, const int32_t *elementIndex, int64_t n, void *atoms4, void *stream)
{
    TRY(check_n(n, "coords"));
    Context *c;
    TRY(get_context(&c));
    return launch_pack_atoms(coords, elementIndex, (int)n, (float4 *)atoms4, (cudaStream_t)stream);
}

int frmc_dev_counts_to_f32(const uint32_t *counts, int64_t total, float *out, void *stream)
{
    Context *c;
    TRY(get_context(&c));
    return launch_counts_to_f32(counts, nullptr, out, total, (cudaStream_t)stream);
}

}  // extern "C"
