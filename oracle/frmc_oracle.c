/*
 * CPU oracle for fullrmc's pair-distance and histogram path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the float32
 * arithmetic of the reference Cython modules so that the CUDA library can be
 * checked against it on machines where the reference itself is not present.
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark load
 * it; the product never does.
 *
 * Build: gcc -O2 -fPIC -shared -ffp-contract=off (see oracle/oracle.py).
 * -ffp-contract=off keeps a*b+c as a rounded multiply followed by a rounded
 * add, which is what the reference's C does on x86-64.
 *
 * Reference operation order (all float32, FLT_EVAL_METHOD == 0):
 *   round(x)  = x > 0 ? floor(x + 0.5) : ceil(x - 0.5)
 *                                         Extensions/pairs_distances.pyx:31-32
 *   diff      = a - b;  box = diff - round(diff)
 *   real_k    = (box_x*B[0][k] + box_y*B[1][k]) + box_z*B[2][k]
 *   d         = (float) sqrt((rx*rx + ry*ry) + rz*rz)
 *                                         Extensions/pairs_distances.pyx:375-386
 *   IBC:  d   = (float) sqrt((dx*dx + dy*dy) + dz*dz), dx = a - b
 *                                         Extensions/pairs_distances.pyx:443-471
 *   histogram: skip i == atom; reject d < min and d >= max;
 *              bin = (int)((d - min) / bin); intra if mol[i] == mol[atom]
 *                                         Extensions/pairs_histograms.pyx:53-68
 *
 * `floor`, `ceil` and `sqrt` are libm double functions in the reference; the
 * float argument is promoted and the result rounded back to float.  For floor
 * and ceil that is exact; for sqrt, double rounding of a float operand is
 * innocuous (53 >= 2*24+2), so sqrtf gives the same bits.
 *
 * The reference indexes hintra/hinter[ne][ne][hs] with boundscheck off, so a
 * bin index equal to hs (possible after float rounding of d just below max)
 * lands in bin 0 of the next [a][b+1] row of the C-contiguous array.  The
 * oracle reproduces that by flat indexing and drops a write whose flat index
 * falls outside the array (the reference would write out of bounds there).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

static inline float ref_round(float x)
{
    return x > 0.0f ? floorf(x + 0.5f) : ceilf(x - 0.5f);
}

/* pairs_distances.pyx:375-386 (PBC) and :443-471 (IBC); a - b order. */
static inline float pair_distance(const float *a, const float *b,
                                  const float *B, int isPBC)
{
    float dx = a[0] - b[0];
    float dy = a[1] - b[1];
    float dz = a[2] - b[2];
    if (isPBC) {
        float bx = dx - ref_round(dx);
        float by = dy - ref_round(dy);
        float bz = dz - ref_round(dz);
        float rx = bx * B[0] + by * B[3] + bz * B[6];
        float ry = bx * B[1] + by * B[4] + bz * B[7];
        float rz = bx * B[2] + by * B[5] + bz * B[8];
        return (float)sqrt((double)(rx * rx + ry * ry + rz * rz));
    }
    return (float)sqrt((double)(dx * dx + dy * dy + dz * dz));
}

/* pairs_distances.pyx:53-63 and the *_differences_* loops: a - b order. */
static inline void pair_difference(const float *a, const float *b,
                                   const float *B, int isPBC, float *out)
{
    float dx = a[0] - b[0];
    float dy = a[1] - b[1];
    float dz = a[2] - b[2];
    if (isPBC) {
        float bx = dx - ref_round(dx);
        float by = dy - ref_round(dy);
        float bz = dz - ref_round(dz);
        out[0] = bx * B[0] + by * B[3] + bz * B[6];
        out[1] = bx * B[1] + by * B[4] + bz * B[7];
        out[2] = bx * B[2] + by * B[5] + bz * B[8];
    } else {
        out[0] = dx;
        out[1] = dy;
        out[2] = dz;
    }
}

/* ---------------------------------------------------------------- distances */

/* pairs_distances.pyx:874-916 -> :348-386 / :443-471.
 * distances[i] = d(coords[atom], coords[i]) for i in [start, n). */
void oracle_distances_to_indexcoords(int32_t atomIndex, const float *coords,
                                     int64_t n, const float *basis, int isPBC,
                                     int allAtoms, float *distances)
{
    int64_t start = allAtoms ? 0 : atomIndex;
    const float *a = coords + 3 * (int64_t)atomIndex;
    float p[3] = {a[0], a[1], a[2]};
    for (int64_t i = start; i < n; ++i)
        distances[i] = pair_distance(p, coords + 3 * i, basis, isPBC);
}

/* pairs_distances.pyx:827-866 -> :311-340 (PBC, point - coords[i]) and
 * :424-437 (IBC, coords[i] - point; same bits after squaring). */
void oracle_distances_to_point(const float *point, const float *coords,
                               int64_t n, const float *basis, int isPBC,
                               float *distances)
{
    float p[3] = {point[0], point[1], point[2]};
    for (int64_t i = 0; i < n; ++i) {
        if (isPBC) {
            distances[i] = pair_distance(p, coords + 3 * i, basis, 1);
        } else {
            const float *c = coords + 3 * i;
            float dx = c[0] - p[0], dy = c[1] - p[1], dz = c[2] - p[2];
            distances[i] = (float)sqrt((double)(dx * dx + dy * dy + dz * dz));
        }
    }
}

/* pairs_distances.pyx:924-966: points is indexed as points[:, k] (so its
 * shape is (3, K) in practice); output (n, K) row-major. */
void oracle_distances_to_multi_points(const float *points, int64_t pstride0,
                                      int64_t K, const float *coords,
                                      int64_t n, const float *basis, int isPBC,
                                      float *distances)
{
    for (int64_t k = 0; k < K; ++k) {
        float p[3] = {points[k], points[pstride0 + k], points[2 * pstride0 + k]};
        for (int64_t i = 0; i < n; ++i) {
            float d;
            if (isPBC) {
                d = pair_distance(p, coords + 3 * i, basis, 1);
            } else {
                const float *c = coords + 3 * i;
                float dx = c[0] - p[0], dy = c[1] - p[1], dz = c[2] - p[2];
                d = (float)sqrt((double)(dx * dx + dy * dy + dz * dz));
            }
            distances[i * K + k] = d;
        }
    }
}

/* pairs_distances.pyx:975-1021; output (n, K), rows < indexes[k] untouched
 * when allAtoms is false. */
void oracle_distances_to_multi_indexcoords(const int32_t *indexes, int64_t K,
                                           const float *coords, int64_t n,
                                           const float *basis, int isPBC,
                                           int allAtoms, float *distances)
{
    for (int64_t k = 0; k < K; ++k) {
        int64_t atom = indexes[k];
        int64_t start = allAtoms ? 0 : atom;
        const float *a = coords + 3 * atom;
        float p[3] = {a[0], a[1], a[2]};
        for (int64_t i = start; i < n; ++i)
            distances[i * K + k] = pair_distance(p, coords + 3 * i, basis, isPBC);
    }
}

/* pairs_distances.pyx:786-819 -> :271-295 / :398-410. */
float oracle_point_to_point_distance(const float *p1, const float *p2,
                                     const float *basis, int isPBC)
{
    return pair_distance(p1, p2, basis, isPBC);
}

/* -------------------------------------------------------------- differences */

/* pairs_distances.pyx:483-521 -> :71-93 (PBC: to - from) / :113-126. */
void oracle_from_to_points_differences(const float *from, const float *to,
                                       int64_t n, const float *basis,
                                       int isPBC, float *out)
{
    for (int64_t i = 0; i < n; ++i)
        pair_difference(to + 3 * i, from + 3 * i, basis, isPBC, out + 3 * i);
}

/* pairs_distances.pyx:529-561 -> :45-63 (PBC: to - from) / :100-108. */
void oracle_pair_difference_to_point(const float *p1, const float *p2,
                                     const float *basis, int isPBC, float *out)
{
    pair_difference(p2, p1, basis, isPBC, out);
}

/* pairs_distances.pyx:569-607 -> :135-160 (point - coords[i]) / :168-188. */
void oracle_differences_to_point(const float *point, const float *coords,
                                 int64_t n, const float *basis, int isPBC,
                                 float *out)
{
    float p[3] = {point[0], point[1], point[2]};
    for (int64_t i = 0; i < n; ++i)
        pair_difference(p, coords + 3 * i, basis, isPBC, out + 3 * i);
}

/* pairs_distances.pyx:615-654 -> :198-236 / :244-265; rows before atomIndex
 * untouched when allAtoms is false. */
void oracle_differences_to_indexcoords(int32_t atomIndex, const float *coords,
                                       int64_t n, const float *basis,
                                       int isPBC, int allAtoms, float *out)
{
    int64_t start = allAtoms ? 0 : atomIndex;
    const float *a = coords + 3 * (int64_t)atomIndex;
    float p[3] = {a[0], a[1], a[2]};
    for (int64_t i = start; i < n; ++i)
        pair_difference(p, coords + 3 * i, basis, isPBC, out + 3 * i);
}

/* pairs_distances.pyx:662-711: output (n, 3, K), point k = points[:, k]. */
void oracle_differences_to_multi_points(const float *points, int64_t pstride0,
                                        int64_t K, const float *coords,
                                        int64_t n, const float *basis,
                                        int isPBC, float *out)
{
    for (int64_t k = 0; k < K; ++k) {
        float p[3] = {points[k], points[pstride0 + k], points[2 * pstride0 + k]};
        for (int64_t i = 0; i < n; ++i) {
            float d[3];
            pair_difference(p, coords + 3 * i, basis, isPBC, d);
            out[(i * 3 + 0) * K + k] = d[0];
            out[(i * 3 + 1) * K + k] = d[1];
            out[(i * 3 + 2) * K + k] = d[2];
        }
    }
}

/* pairs_distances.pyx:719-774: output (n, 3, K). */
void oracle_differences_to_multi_indexcoords(const int32_t *indexes, int64_t K,
                                             const float *coords, int64_t n,
                                             const float *basis, int isPBC,
                                             int allAtoms, float *out)
{
    for (int64_t k = 0; k < K; ++k) {
        int64_t atom = indexes[k];
        int64_t start = allAtoms ? 0 : atom;
        const float *a = coords + 3 * atom;
        float p[3] = {a[0], a[1], a[2]};
        for (int64_t i = start; i < n; ++i) {
            float d[3];
            pair_difference(p, coords + 3 * i, basis, isPBC, d);
            out[(i * 3 + 0) * K + k] = d[0];
            out[(i * 3 + 1) * K + k] = d[1];
            out[(i * 3 + 2) * K + k] = d[2];
        }
    }
}

/* ---------------------------------------------------------------- histograms */

/* pairs_histograms.pyx:36-68 with the wrapper of :77-141.  hintra/hinter are
 * C-contiguous (ne, ne, hs) float32, updated in place by float additions of
 * 1.0 in increasing i order, as the ncores=1 reference does. */
void oracle_single_pairs_histograms(int32_t atomIndex, const float *distances,
                                    int64_t n, const int32_t *mol,
                                    const int32_t *el, int32_t ne, int32_t hs,
                                    float *hintra, float *hinter,
                                    float minD, float maxD, float bin,
                                    int allAtoms)
{
    int64_t total = (int64_t)ne * ne * hs;
    int32_t amol = mol[atomIndex];
    int64_t row = (int64_t)el[atomIndex] * ne;
    int64_t start = allAtoms ? 0 : atomIndex;
    for (int64_t i = start; i < n; ++i) {
        if (i == atomIndex)
            continue;
        float d = distances[i];
        if (d < minD)
            continue;
        if (d >= maxD)
            continue;
        float q = (d - minD) / bin;
        if (!(q < 2147483648.0f))
            continue;
        int64_t flat = (row + el[i]) * hs + (int32_t)q;
        if (flat < 0 || flat >= total)
            continue;
        if (mol[i] == amol)
            hintra[flat] += 1.0f;
        else
            hinter[flat] += 1.0f;
    }
}

/* pairs_histograms.pyx:150-217: zeroed histograms, then for each index the
 * distances of :874-916 followed by :77-141.  The per-atom distance row is
 * computed on the fly instead of being stored (same values). */
void oracle_multiple_pairs_histograms_coords(
    const int32_t *indexes, int64_t K, const float *coords, int64_t n,
    const float *basis, int isPBC, const int32_t *mol, const int32_t *el,
    int32_t ne, float minD, float maxD, float bin, int32_t hs, int allAtoms,
    float *hintra, float *hinter)
{
    int64_t total = (int64_t)ne * ne * hs;
    memset(hintra, 0, sizeof(float) * total);
    memset(hinter, 0, sizeof(float) * total);
    for (int64_t k = 0; k < K; ++k) {
        int64_t atom = indexes[k];
        int64_t start = allAtoms ? 0 : atom;
        int32_t amol = mol[atom];
        int64_t row = (int64_t)el[atom] * ne;
        const float *a = coords + 3 * atom;
        float p[3] = {a[0], a[1], a[2]};
        for (int64_t i = start; i < n; ++i) {
            if (i == atom)
                continue;
            float d = pair_distance(p, coords + 3 * i, basis, isPBC);
            if (d < minD)
                continue;
            if (d >= maxD)
                continue;
            float q = (d - minD) / bin;
            if (!(q < 2147483648.0f))
                continue;
            int64_t flat = (row + el[i]) * hs + (int32_t)q;
            if (flat < 0 || flat >= total)
                continue;
            if (mol[i] == amol)
                hintra[flat] += 1.0f;
            else
                hinter[flat] += 1.0f;
        }
    }
}

/* pairs_histograms.pyx:289-335: indexes = arange(n), allAtoms = False. */
void oracle_full_pairs_histograms_coords(
    const float *coords, int64_t n, const float *basis, int isPBC,
    const int32_t *mol, const int32_t *el, int32_t ne, float minD, float maxD,
    float bin, int32_t hs, float *hintra, float *hinter)
{
    int64_t total = (int64_t)ne * ne * hs;
    memset(hintra, 0, sizeof(float) * total);
    memset(hinter, 0, sizeof(float) * total);
    for (int64_t atom = 0; atom < n; ++atom) {
        int32_t amol = mol[atom];
        int64_t row = (int64_t)el[atom] * ne;
        const float *a = coords + 3 * atom;
        float p[3] = {a[0], a[1], a[2]};
        for (int64_t i = atom + 1; i < n; ++i) {
            float d = pair_distance(p, coords + 3 * i, basis, isPBC);
            if (d < minD)
                continue;
            if (d >= maxD)
                continue;
            float q = (d - minD) / bin;
            if (!(q < 2147483648.0f))
                continue;
            int64_t flat = (row + el[i]) * hs + (int32_t)q;
            if (flat < 0 || flat >= total)
                continue;
            if (mol[i] == amol)
                hintra[flat] += 1.0f;
            else
                hinter[flat] += 1.0f;
        }
    }
}

/* pairs_histograms.pyx:225-281: column k of a (n, K) distance matrix is the
 * distance row of atom indexes[k]. */
void oracle_multiple_pairs_histograms_dists(
    const int32_t *indexes, int64_t K, const float *distances, int64_t n,
    const int32_t *mol, const int32_t *el, int32_t ne, float minD, float maxD,
    float bin, int32_t hs, int allAtoms, float *hintra, float *hinter)
{
    int64_t total = (int64_t)ne * ne * hs;
    memset(hintra, 0, sizeof(float) * total);
    memset(hinter, 0, sizeof(float) * total);
    for (int64_t k = 0; k < K; ++k) {
        int64_t atom = indexes[k];
        int64_t start = allAtoms ? 0 : atom;
        int32_t amol = mol[atom];
        int64_t row = (int64_t)el[atom] * ne;
        for (int64_t i = start; i < n; ++i) {
            if (i == atom)
                continue;
            float d = distances[i * K + k];
            if (d < minD)
                continue;
            if (d >= maxD)
                continue;
            float q = (d - minD) / bin;
            if (!(q < 2147483648.0f))
                continue;
            int64_t flat = (row + el[i]) * hs + (int32_t)q;
            if (flat < 0 || flat >= total)
                continue;
            if (mol[i] == amol)
                hintra[flat] += 1.0f;
            else
                hinter[flat] += 1.0f;
        }
    }
}

/* boundary_conditions_collection.pyx:88-110: row-vector transform. */
void oracle_transform_coordinates(const float *M, const float *coords,
                                  int64_t n, float *out)
{
    for (int64_t i = 0; i < n; ++i) {
        const float *c = coords + 3 * i;
        out[3 * i + 0] = c[0] * M[0] + c[1] * M[3] + c[2] * M[6];
        out[3 * i + 1] = c[0] * M[1] + c[1] * M[4] + c[2] * M[7];
        out[3 * i + 2] = c[0] * M[2] + c[1] * M[5] + c[2] * M[8];
    }
}

/* -------------------------------------------------------- atomic distances */

/* atomic_distances.pyx:42-126 (one row atom) as called by :326-417 and
 * :419-498: rows indexes[k] in order, columns i from start (0 if allAtoms,
 * else the row atom) to n - 1 in order, float32 sums in that order.  The
 * distance of column i is d(coords[row], coords[i]) (pairs_distances, row
 * atom first) or dists[i * K + k].  flags: 1 inter, 2 intra, 4 count within
 * limits, 8 / 16 / 32 reduce to upper / lower / nearest limit.  Outputs
 * (ne, ne), added to. */
void oracle_atomic_distances(const int32_t *indexes, int64_t K, const float *coords, const float *dists,
                             int64_t n, const float *basis, int isPBC, const int32_t *mol, const int32_t *el,
                             int32_t ne, const float *lower, const float *upper, int flags, int allAtoms,
                             float *dintra, float *dinter, int32_t *nintra, int32_t *ninter)
{
    for (int64_t k = 0; k < K; ++k) {
        const int32_t a = indexes[k];
        const int64_t start = allAtoms ? 0 : a;
        const int32_t ea = el[a], ma = mol[a];
        float p[3] = {0.f, 0.f, 0.f};
        if (!dists) {
            p[0] = coords[3 * (int64_t)a];
            p[1] = coords[3 * (int64_t)a + 1];
            p[2] = coords[3 * (int64_t)a + 2];
        }
        for (int64_t i = start; i < n; ++i) {
            if (i == a)
                continue;
            const int32_t mi = mol[i];
            if (!(flags & 2) && mi == ma)
                continue;
            if (!(flags & 1) && mi != ma)
                continue;
            float d = dists ? dists[i * K + k] : pair_distance(p, coords + 3 * i, basis, isPBC);
            const int32_t ei = el[i];
            const float lo = lower[ei * ne + ea];
            const float up = upper[ei * ne + ea];
            if (flags & 4) {
                if (d < lo)
                    continue;
                if (d >= up)
                    continue;
            } else if (d >= lo && d < up) {
                continue;
            }
            if (flags & 8)
                d = fabsf(up - d);
            else if (flags & 16)
                d = fabsf(lo - d);
            else if (flags & 32)
                d = d > (lo + up) / 2.0f ? fabsf(up - d) : fabsf(lo - d);
            if (mi == ma) {
                dintra[ea * ne + ei] += d;
                nintra[ea * ne + ei] += 1;
            } else {
                dinter[ea * ne + ei] += d;
                ninter[ea * ne + ei] += 1;
            }
        }
    }
}

/* atomic_distances.pyx:632-657: pairs i < j at [el(i)][el(j)]. */
void oracle_pair_elements_stats(const int32_t *el, const int32_t *mol, int64_t n, int32_t ne, int32_t *nintra,
                                int32_t *ninter)
{
    for (int64_t i = 0; i + 1 < n; ++i)
        for (int64_t j = i + 1; j < n; ++j) {
            if (mol[j] == mol[i])
                nintra[el[i] * ne + el[j]] += 1;
            else
                ninter[el[i] * ne + el[j]] += 1;
        }
}
