/*
 * frmc_gpu.h -- C ABI of the GB300 (sm_103a) pair-distance / histogram library.
 *
 * The library replaces fullrmc's Cython modules fullrmc.Core.pairs_distances,
 * fullrmc.Core.pairs_histograms and fullrmc.Core.reciprocal_space.  Every
 * entry point below names the reference function it stands in for
 * (path:line inside the fullrmc source tree).  A thin ctypes layer
 * (fullrmc_gb300/pairs_*.py) gives them the reference's Python signatures.
 *
 * Conventions
 *   - Plain pointers and sizes; no framework types.  int return: 0 on
 *     success, a negative FRMC_E_* code otherwise; frmc_last_error() returns
 *     the thread's last message.
 *   - "Host" entry points take host memory, copy to the current CUDA device,
 *     compute and copy back before returning (the drop-in path).  They keep no
 *     host data between calls.
 *   - "frmc_dev_*" entry points take device pointers and a cudaStream_t
 *     (passed as void*; NULL is the CUDA legacy default stream) and return
 *     without synchronising.
 *   - Coordinates are float32 (n, 3) row-major; basis is float32 (3, 3)
 *     row-major with the box vectors as rows (real = box . basis).
 *   - Histograms are float32 C-contiguous (ne, ne, hs); counts are uint32.
 *   - Arithmetic is bit-identical to the reference's float32 order; where the
 *     reference's behaviour is undefined (indexes outside [0, n), arrays
 *     shorter than n) these functions return FRMC_E_ARG instead.
 */
#ifndef FRMC_GPU_H
#define FRMC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#define FRMC_OK 0
#define FRMC_E_ARG (-1)     /* invalid argument (maps to ValueError)      */
#define FRMC_E_CUDA (-2)    /* CUDA runtime error                         */
#define FRMC_E_NOMEM (-3)   /* device allocation failed (MemoryError)     */
#define FRMC_E_NODEV (-4)   /* no CUDA device                             */
#define FRMC_E_TIMEOUT (-5) /* a bounded device wait gave up              */
#define FRMC_E_STATE (-6)   /* object in the wrong state for this call    */
#define FRMC_E_INDEX (-7)   /* index out of range (maps to IndexError)    */

/* ---------------------------------------------------------------- runtime */
int frmc_version(void);
const char *frmc_last_error(void);
/* Select the CUDA device used by later calls from this thread. */
int frmc_set_device(int device);
/* Number of SMs and the opt-in shared-memory limit of the current device. */
int frmc_device_info(int *sms, int *max_smem_optin, int *cc_major, int *cc_minor);

/* Host-only helpers (no device needed).  Exact squared-distance limits: for
 * d = sqrtf(s) correctly rounded, d >= minDistance <=> s >= *s_lo and
 * d < maxDistance <=> s < *s_hi (the kernels test s, and take the IEEE sqrt
 * and division of pairs_histograms.pyx:63 only for accepted pairs). */
int frmc_sq_limits(float minDistance, float maxDistance, float *s_lo, float *s_hi);
/* Basis shape used to drop exactly-zero basis terms: 0 infinite boundary
 * conditions, 1 diagonal, 2 (a||x, b in xy, c||z), 3 lower triangular,
 * 4 general. */
int frmc_basis_mode(const float *basis, int isPBC);

/* --------------------------------------------------- pairs_distances (host)
 * Extensions/pairs_distances.pyx:874-916 pairs_distances_to_indexcoords:
 * distances[i] = d(coords[atomIndex], coords[i]) for i in [start, n), start =
 * allAtoms ? 0 : atomIndex; entries below start are left untouched. */
int frmc_pairs_distances_to_indexcoords(int32_t atomIndex, const float *coords, int64_t n, const float *basis,
                                        int isPBC, int allAtoms, float *distances);
/* pairs_distances.pyx:827-866 pairs_distances_to_point. */
int frmc_pairs_distances_to_point(const float *point, const float *coords, int64_t n, const float *basis, int isPBC,
                                  float *distances);
/* pairs_distances.pyx:924-966 pairs_distances_to_multi_points: point k is
 * (points[0*ps+k], points[1*ps+k], points[2*ps+k]) -- the reference reads
 * points[:, k]; distances is (n, K) row-major. */
int frmc_pairs_distances_to_multi_points(const float *points, int64_t ps, int64_t K, const float *coords, int64_t n,
                                         const float *basis, int isPBC, float *distances);
/* pairs_distances.pyx:975-1021 pairs_distances_to_multi_indexcoords:
 * distances (n, K); rows below indexes[k] untouched when !allAtoms. */
int frmc_pairs_distances_to_multi_indexcoords(const int32_t *indexes, int64_t K, const float *coords, int64_t n,
                                              const float *basis, int isPBC, int allAtoms, float *distances);
/* pairs_distances.pyx:786-819 point_to_point_distance. */
int frmc_point_to_point_distance(const float *point1, const float *point2, const float *basis, int isPBC,
                                 float *distance);
/* pairs_distances.pyx:483-521 from_to_points_differences: out[i] = bc(to[i] - from[i]). */
int frmc_from_to_points_differences(const float *pointsFrom, const float *pointsTo, int64_t n, const float *basis,
                                    int isPBC, float *differences);
/* pairs_distances.pyx:529-561 pair_difference_to_point: out = bc(point2 - point1). */
int frmc_pair_difference_to_point(const float *point1, const float *point2, const float *basis, int isPBC,
                                  float *difference);
/* pairs_distances.pyx:569-607 pairs_differences_to_point: out[i] = bc(point - coords[i]). */
int frmc_pairs_differences_to_point(const float *point, const float *coords, int64_t n, const float *basis,
                                    int isPBC, float *differences);
/* pairs_distances.pyx:615-654 pairs_differences_to_indexcoords. */
int frmc_pairs_differences_to_indexcoords(int32_t atomIndex, const float *coords, int64_t n, const float *basis,
                                          int isPBC, int allAtoms, float *differences);
/* pairs_distances.pyx:662-711 pairs_differences_to_multi_points: out (n, 3, K). */
int frmc_pairs_differences_to_multi_points(const float *points, int64_t ps, int64_t K, const float *coords,
                                           int64_t n, const float *basis, int isPBC, float *differences);
/* pairs_distances.pyx:719-774 pairs_differences_to_multi_indexcoords: out (n, 3, K). */
int frmc_pairs_differences_to_multi_indexcoords(const int32_t *indexes, int64_t K, const float *coords, int64_t n,
                                                const float *basis, int isPBC, int allAtoms, float *differences);

/* -------------------------------------------------- pairs_histograms (host)
 * Extensions/pairs_histograms.pyx:77-141 single_pairs_histograms: adds the
 * counts of atom atomIndex's distance row to hintra/hinter (ne, ne, hs) in
 * place, with float32 additions of 1.0 (saturating at 2^24 like the
 * reference). */
int frmc_single_pairs_histograms(int32_t atomIndex, const float *distances, int64_t n, const int32_t *moleculeIndex,
                                 const int32_t *elementIndex, int32_t ne, int32_t hs, float *hintra, float *hinter,
                                 float minDistance, float maxDistance, float bin, int allAtoms);
/* pairs_histograms.pyx:150-217 multiple_pairs_histograms_coords: hintra and
 * hinter (ne, ne, hs) are overwritten. */
int frmc_multiple_pairs_histograms_coords(const int32_t *indexes, int64_t K, const float *boxCoords, int64_t n,
                                          const float *basis, int isPBC, const int32_t *moleculeIndex,
                                          const int32_t *elementIndex, int32_t ne, float minDistance,
                                          float maxDistance, float bin, int32_t hs, int allAtoms, float *hintra,
                                          float *hinter);
/* pairs_histograms.pyx:289-335 full_pairs_histograms_coords (all i < j). */
int frmc_full_pairs_histograms_coords(const float *boxCoords, int64_t n, const float *basis, int isPBC,
                                      const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                      float minDistance, float maxDistance, float bin, int32_t hs, float *hintra,
                                      float *hinter);
/* ShapeFunction (Constraints/Collection.py:15-160) in FP64: the all-pairs
 * counts of a StructureFactorConstraint's histogram (minDistance, maxDistance,
 * bin, hs), its total G on the shells
 *   G(b) = 4 pi r_b rho0 (sum_p pair_coef[p] n_p(b) / shellVolumes[b] - 1)
 * (n_p: intra + inter counts of element pair (pair_i, pair_j), both
 * orientations for unlike elements; pair_coef = w_ij V / N_ij;
 * StructureFactorConstraints.py:836-896), S(q) = 1 + sum_b G(b) dr sin(q r_b) / q
 * (:302-312, 772-773; dr = r_1 - r_0) and the shape function
 *   Gshape(r) = 2/pi sum_q dq q (S(q) - 1) sin(q r)   (Collection.py:131-139).
 * The counts are exact (the reference's float32 histogram stops at 2^24 per
 * bin).  Gr (hs), Sq (nq) and Gshape (nr) may each be NULL. */
int frmc_shape_function(const float *boxCoords, int64_t n, const float *basis, int isPBC,
                        const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne, float minDistance,
                        float maxDistance, float bin, int32_t hs, int32_t npairs, const int32_t *pair_i,
                        const int32_t *pair_j, const double *pair_coef, const double *shellCenters,
                        const double *shellVolumes, double rho0, const double *qValues, int32_t nq,
                        const double *rValues, int32_t nr, double *Gr, double *Sq, double *Gshape);
/* pairs_histograms.pyx:225-281 multiple_pairs_histograms_dists: distances is
 * (n, K) row-major, column k belongs to atom indexes[k]. */
/* The change of fullrmc's before/after-move data for one group move, in one
 * launch: (M - F) after minus (M - F) before, where M is
 * multiple_pairs_histograms_coords(indexes, ..., allAtoms=True) and F is
 * full_pairs_histograms_coords on the group's own coordinates
 * (PairDistributionConstraints.py:1044-1129, compute_before_move and
 * compute_after_move).  boxCoords (n, 3) are all atoms before the move,
 * newBoxCoords (K, 3) the group's atoms after it, in the order of indexes
 * (at most 1024).  dintra / dinter (ne, ne, hs) int32 receive signed counts;
 * every pair takes the reference's float32 order, so the counts equal the
 * differences of the four reference histograms exactly.  An extension of the
 * module, not a reference export. */
int frmc_group_move_delta_histograms(const int32_t *indexes, int64_t K, const float *boxCoords, int64_t n,
                                     const float *newBoxCoords, const float *basis, int isPBC,
                                     const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                     float minDistance, float maxDistance, float bin, int32_t hs, int32_t *dintra,
                                     int32_t *dinter);
int frmc_multiple_pairs_histograms_dists(const int32_t *indexes, int64_t K, const float *distances, int64_t n,
                                         const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                         float minDistance, float maxDistance, float bin, int32_t hs, int allAtoms,
                                         float *hintra, float *hinter);

/* Extensions/atomic_distances.pyx (InterMolecularDistanceConstraint,
 * Constraints/DistanceConstraints.py:569-697).  For every row atom (indexes,
 * in order) and every other atom j (j >= the row atom unless allAtoms), pairs
 * whose distance d passes the limits lowerLimit/upperLimit[el(j)][el(row)]
 * (flags & 4: lower <= d < upper; otherwise outside) are counted and their
 * value summed in float32, in the reference's loop order, into
 * [el(row)][el(j)] of the intra- (same molecule) or inter-molecular arrays.
 * flags: 1 interMolecular, 2 intraMolecular, 4 countWithinLimits, 8
 * reduceDistanceToUpper (value |upper - d|), 16 reduceDistanceToLower
 * (|lower - d|), 32 reduceDistance (the nearer limit).  Outputs are (ne, ne)
 * (the reference's (ne, ne, 1)).  multiple_atomic_distances_coords
 * (atomic_distances.pyx:326-417); full_atomic_distances_coords (:500-567) is
 * the same with indexes = 0..n-1 and allAtoms = 0. */
int frmc_multiple_atomic_distances_coords(const int32_t *indexes, int64_t K, const float *boxCoords, int64_t n,
                                          const float *basis, int isPBC, const int32_t *moleculeIndex,
                                          const int32_t *elementIndex, int32_t ne, const float *lowerLimit,
                                          const float *upperLimit, int flags, int allAtoms, int32_t *nintra,
                                          float *dintra, int32_t *ninter, float *dinter);
/* multiple_atomic_distances_dists (atomic_distances.pyx:419-498): distances
 * (n, K), column k the distances of atom indexes[k]; full_* (:569-630) with
 * indexes = 0..K-1, allAtoms = 0. */
int frmc_multiple_atomic_distances_dists(const int32_t *indexes, int64_t K, const float *distances, int64_t n,
                                         const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                         const float *lowerLimit, const float *upperLimit, int flags, int allAtoms,
                                         int32_t *nintra, float *dintra, int32_t *ninter, float *dinter);
/* single_atomic_distances_dists (atomic_distances.pyx:128-324): adds into the
 * given arrays in place. */
int frmc_single_atomic_distances_dists(int32_t atomIndex, const float *distances, int64_t n,
                                       const int32_t *moleculeIndex, const int32_t *elementIndex, int32_t ne,
                                       float *dintra, float *dinter, int32_t *nintra, int32_t *ninter,
                                       const float *lowerLimit, const float *upperLimit, int flags, int allAtoms);
/* pair_elements_stats (atomic_distances.pyx:632-672): pairs i < j counted at
 * [el(i)][el(j)], intra or inter. */
int frmc_pair_elements_stats(const int32_t *elementIndex, const int32_t *moleculeIndex, int64_t n, int32_t ne,
                             int32_t *nintra, int32_t *ninter);

/* Extensions/atomic_coordination.pyx (AtomicCoordinationNumberConstraint,
 * Constraints/AtomicCoordinationConstraints.py:476-580).  Every function of
 * that module is a sequence of terms; this entry point runs any sequence:
 * for t = 0 .. nterms-1, in order,
 *   coordNumData[term_def[t]] += (float) min(2^24, count of entries j of list
 *       term_list[t] with lowerShells[def] <= d(term_row[t], j) <= upperShells[def])
 * in float32 (atomic_coordination.pyx:31-44 counts, :184-198 and :220-240 add).
 * List l is lists[list_off[l] .. list_off[l+1]); a negative entry j counts
 * from the end of the row (numpy indexing, :77, :99).
 * With boxCoords (n, 3), the row is a core atom and d the minimum-image
 * distance |bc(box[row] - box[j])| (pairs_distances_to_point, :98-102);
 * with boxCoords null, the row r is distances[dist_off[r] .. + dist_len[r])
 * and d its entry j (single_atom_single_shell_totdists, :71-80).
 * lowerShells, upperShells and coordNumData have ndata entries; coordNumData
 * is updated in place.  Out-of-range indexes return FRMC_E_INDEX before
 * anything changes. */
int frmc_coordination_terms(const float *boxCoords, int64_t n, const float *basis, int isPBC, const float *distances,
                            const int64_t *dist_off, const int32_t *dist_len, int32_t nrows, const int32_t *lists,
                            const int64_t *list_off, int32_t nlists, const int32_t *term_row,
                            const int32_t *term_list, const int32_t *term_def, int64_t nterms,
                            const float *lowerShells, const float *upperShells, float *coordNumData, int32_t ndata);

/* ---------------------------------------------- reciprocal space (host, FP64)
 * Extensions/reciprocal_space.pyx:42-73 gr_to_sq:
 *   sq[q] = 1 + 4 pi rho sum_r dr r sin(q r)/q (gr[r] - 1), dr = r[1] - r[0]. */
int frmc_gr_to_sq(const float *distances, const float *gr, int64_t nr, const float *qrange, int64_t nq, double rho,
                  double *sq);
/* reciprocal_space.pyx:82-109 Gr_to_sq: sq[q] = 1 + sum_r dr sin(q r)/q Gr[r]. */
int frmc_Gr_to_sq(const float *distances, const float *Gr, int64_t nr, const float *qrange, int64_t nq, double *sq);
/* reciprocal_space.pyx:118-145 sq_to_Gr (the formula the reference intends;
 * its own body raises TypeError):  Gr[r] = 2/pi sum_q q (sq[q] - 1) sin(q r) dq. */
int frmc_sq_to_Gr(const float *qValues, int64_t nq, const float *rValues, int64_t nr, const float *sq, double *Gr);

/* ------------------------------------- boundary_conditions_collection (host)
 * Extensions/boundary_conditions_collection.pyx:88-110 transform_coordinates:
 * out[i] = coords[i] . M (float32, reference order). */
int frmc_transform_coordinates(const float *transMatrix, const float *coords, int64_t n, float *out);

/* ------------------------------------------------ device-resident entry points
 * Same computations on device buffers; counts are uint32 [2][ne][ne][hs]
 * (index 0 = intra, 1 = inter) and are zeroed by the call.
 *
 * All-pairs histogram (full_pairs_histograms_coords, pairs_histograms.pyx:289-335)
 * of atoms packed as float4 (x, y, z, element index bits). */
int frmc_dev_full_hist_counts(const void *atoms4, const int32_t *moleculeIndex, int64_t n, const float *basis_host,
                              int isPBC, int32_t ne, float minDistance, float maxDistance, float bin, int32_t hs,
                              uint32_t *counts, void *stream);
/* Tile configuration of the all-pairs kernel: threads per CTA, row atoms
 * per thread (1 or 2), queued binning (-1 auto, 0 off, 1 on), queue slots per
 * thread, CTAs per SM, and the pair count from which the host entry point
 * frmc_full_pairs_histograms_coords uses it (below: the row kernel).  Applies
 * to later calls from every thread. */
int frmc_set_full_tune(int threads, int rows, int queued, int qcap, int ctas_per_sm, double min_pairs_tiled);
/* Binning of the tiled kernel's queued pairs: 0 (default) plain shared-memory
 * atomics, 1 warp-aggregated atomics (lanes whose pairs fall in the same
 * counter are grouped with __match_any_sync and add once).  Counts are the
 * same either way; the switch exists to measure both. */
int frmc_set_full_aggregate(int on);
/* The same all-pairs histogram restricted to work items [item_begin, item_end)
 * of the kernel's (row tile, column tile) triangle, for sharding one system
 * across devices; the per-item partial counts of disjoint ranges sum to the
 * full counts.  frmc_full_items() gives the item count for n atoms. */
int frmc_full_items(int64_t n, int64_t *nitems);
int frmc_dev_full_hist_counts_range(const void *atoms4, const int32_t *moleculeIndex, int64_t n,
                                    const float *basis_host, int isPBC, int32_t ne, float minDistance,
                                    float maxDistance, float bin, int32_t hs, int64_t item_begin, int64_t item_end,
                                    uint32_t *counts, void *stream);
/* multiple_pairs_histograms_coords on device buffers (boxCoords (n, 3)). */
int frmc_dev_multiple_hist_counts(const int32_t *indexes, int64_t K, const float *boxCoords, int64_t n,
                                  const float *basis_host, int isPBC, const int32_t *moleculeIndex,
                                  const int32_t *elementIndex, int32_t ne, float minDistance, float maxDistance,
                                  float bin, int32_t hs, int allAtoms, uint32_t *counts, void *stream);
/* All-pairs histograms into caller-owned float32 device buffers hintra and
 * hinter (ne, ne, hs) without allocating device memory -- for callers that
 * cannot let a library call cudaMalloc (a framework that owns all device
 * memory through its own pool, or a loop that must not stall on an
 * allocation).  There is no counterpart of this entry point in fullrmc; the
 * histograms equal those of full_pairs_histograms_coords.  The uint32
 * counts live in one fixed device array of 2^20 counts (4 MiB) that every GPU
 * loading the library holds until exit: 2*ne*ne*hs above 1048576 returns
 * FRMC_E_ARG, and so does n above INT_MAX / 4 (the limit of
 * frmc_dev_full_hist_counts).  The first call on a device is its set-up: it
 * resolves that array's device address.  All calls share the array, so calls
 * that overlap on the GPU (other streams, other threads) race.  Every call
 * copies its status word back and synchronises `stream` before returning, so
 * the call is synchronous and cannot be recorded into a CUDA graph. */
int frmc_dev_full_pairs_histograms_noalloc(const void *atoms4, const int32_t *moleculeIndex, int64_t n,
                                           const float *basis_host, int isPBC, int32_t ne, float minDistance,
                                           float maxDistance, float bin, int32_t hs, float *hintra, float *hinter,
                                           void *stream);
/* Pack (n, 3) coordinates and element indexes into float4 (x, y, z, el bits). */
int frmc_dev_pack_atoms(const float *coords, const int32_t *elementIndex, int64_t n, void *atoms4, void *stream);
/* float32 histogram values of uint32 counts (sequential additions of 1.0f). */
int frmc_dev_counts_to_f32(const uint32_t *counts, int64_t total, float *out, void *stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* FRMC_GPU_H */
