/*
 * frmc_gpu_engine.h -- device-resident RMC engines (batched and served).
 *
 * Each engine is one fullrmc Metropolis chain with a PairDistributionConstraint
 * and optionally a StructureFactorConstraint on the same histograms, stepped
 * entirely on the GPU:
 *   - the step is fullrmc's Engine.run step (Engine.py:3278-3344) with
 *     single-atom translation moves (Generators/Translations.py:171-190),
 *   - the histogram update is the M term of compute_before_move /
 *     compute_after_move (Constraints/PairDistributionConstraints.py:1044-1129),
 *     kept as oriented int32 counts equal to the constraint's running data,
 *   - G(r) (PairDistributionConstraints.py:847-895), S(Q)
 *     (StructureFactorConstraints.py:780-822) and chi2 are FP64.
 * Moves (atom, displacement vector, uniform number for the tolerance test)
 * are generated by the caller and pushed into a per-engine ring, so the
 * chains stay strictly sequential and reproducible: an engine gives the same
 * accept sequence and bit-identical counts alone or in any batch.
 *
 * There is no counterpart of these entry points in fullrmc itself; they are
 * the batched engines and the serving loop built around the histogram path.
 * Conventions as in frmc_gpu.h (int status, frmc_last_error()).
 */
#ifndef FRMC_GPU_ENGINE_H
#define FRMC_GPU_ENGINE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef struct {
    int32_t n;            /* atoms                                              */
    int32_t ne;           /* elements                                           */
    int32_t hs;           /* histogram bins                                     */
    int32_t isPBC;
    const float *box_coords;   /* (n, 3) box (fractional) coordinates           */
    const float *real_coords;  /* (n, 3) real coordinates                       */
    const int32_t *el;         /* (n,) element index in [0, ne)                 */
    const int32_t *mol;        /* (n,) molecule index                           */
    const float *basis;        /* (3, 3) rows = box vectors                     */
    const float *rbasis;       /* (3, 3) inverse of basis (real -> box)         */
    float minDistance, maxDistance, bin;
    int32_t npairs;            /* unordered element pairs (i <= j)              */
    const int32_t *pair_i;
    const int32_t *pair_j;
    const double *pair_coef;   /* w_ij / (N_ij / V)                             */
    const double *rfac;        /* (hs,) 4 pi r rho0                             */
    const double *inv_shell_volume; /* (hs,) 1 / shell volume                   */
    const double *experimental;     /* (hs,) experimental G(r)                  */
    const double *data_weights;     /* (hs,) or NULL                            */
    double variance_squared;
    double tolerance;          /* Engine tolerance (reject iff chi2 rises and u > tolerance) */
    int32_t move_cap;          /* ring size for moves and step results          */
    /* Optional StructureFactorConstraint on the same histograms (its rmin, dr
     * and rmax equal to minDistance, bin and maxDistance above):
     * S(Q) = 1 + sum_r G_S(r) M[r][Q], G_S = 4 pi r rho0 (g(r) - 1) with the
     * S(Q) shells' own r and volumes, chi2 term sum_Q w (S_exp - S)^2 /
     * sq_variance_squared (StructureFactorConstraints.py:742-822).  sq_table
     * is an id from frmc_engines_sq_table (-1: no S(Q) term); nq its Q points. */
    int32_t sq_table;
    int32_t nq;
    const double *sq_rfac;             /* (hs,) 4 pi r rho0 on the S(Q) shells  */
    const double *sq_inv_shell_volume; /* (hs,) 1 / S(Q) shell volume           */
    const double *sq_experimental;     /* (nq,) experimental S(Q)               */
    double sq_variance_squared;
    double sq_rho0;                    /* number density: sq_rfac = sq_rho0 r0fac of the table */
    /* Atoms per move (0 or 1: single-atom moves; up to 16: moves of atom
     * groups such as molecules, pushed with frmc_engines_push_group_moves). */
    int32_t group_size;
    /* Scale factor and window function of the G(r) term
     * (PairDistributionConstraints.py:884-893, Core/Constraint.py:1363-1424;
     * PairCorrelationConstraints.py:155-184 for g(r)).  The model compared
     * with `experimental` is window * (s G) (numpy.convolve 'same') with
     * G(b) = R(b) sum_p pair_coef_p n_p(b) - rfac(b).  s is scale_factor, or,
     * when fit_frequency > 0 and the engine's accepted count is a multiple of
     * it, clamp(sum fit_num G / sum fit_den G^2, fit_min, fit_max) of the
     * proposed G (fit_den NULL = 1); an accepted move keeps its s.  A
     * scale_factor of 0 is taken as 1 (a spec zeroed past group_size).
     * Engines with s != 1, fit_frequency > 0 or a window evaluate every bin
     * at every step (they take the tile-split path). */
    double scale_factor;
    int32_t fit_frequency;
    double fit_min, fit_max;
    const double *fit_num;     /* (hs,) fit numerator weights times the fit target */
    const double *fit_den;     /* (hs,) fit denominator weights, or NULL        */
    int32_t window_len;        /* 0: no window; at most 255 and at most hs      */
    const double *window;      /* (window_len,) the window, already normalized  */
} frmc_engine_spec;

/* A G(r) -> S(Q) table shared by the set's engines that use the same r shells
 * (hs) and Q points (nq): M (hs, nq) row-major, M[r][Q] = dr sin(Q r) / Q
 * (StructureFactorConstraints.py:302-312), optional per-Q data weights w
 * (NULL = 1) and r0fac (hs,) = 4 pi r / shell volume of those shells.  The
 * set keeps M, w and the fixed-point table round(K r0fac 2^s), K = M diag(w)
 * M^T (hs x hs, built on the device), until it is destroyed; *table receives
 * the id to put in a spec's sq_table.  Device bytes: 8 (hs nq + hs hs + hs +
 * nq + 1).  hs <= 4096. */
int frmc_engines_sq_table(void *handle, int32_t hs, int32_t nq, const double *M, const double *weights,
                          const double *r0fac, int32_t *table);
/* Current S(Q) of engine e recomputed from its counts (FP64, nq values). */
int frmc_engines_sq(void *handle, int32_t e, double *sq);
/* The two chi2 terms of engine e: sd = sum w (G_exp - G)^2 of the G(r) term and
 * sd_sq of the S(Q) term (0 without one); chi2 = sd / variance_squared +
 * sd_sq / sq_variance_squared. */
int frmc_engines_terms(void *handle, int32_t e, double *sd, double *sd_sq);
/* Device bytes one engine of this spec occupies (its state, tables, rings and
 * column grid, and with an S(Q) term its share of the table's fp16 delta
 * columns; the shared S(Q) table itself is not included). */
int frmc_engine_footprint(const frmc_engine_spec *spec, int64_t *bytes);
/* An empty engine set on the current device. */
int frmc_engines_new(void **handle);
/* Create E engines on the current device (all state resident in HBM); engine
 * ids are 0..E-1.  frmc_engines_init computes their initial histograms. */
int frmc_engines_create(const frmc_engine_spec *specs, int32_t E, void **handle);
/* Add one engine (allocated, uploaded and initialised; *id receives its id)
 * or remove one; ids of removed engines are reused.  Used by the serving loop. */
int frmc_engines_add(void *handle, const frmc_engine_spec *spec, int32_t *id);
int frmc_engines_remove(void *handle, int32_t id);
/* Live engine ids in stepping order (ascending); *count receives the number. */
int frmc_engines_live(void *handle, int32_t *ids, int32_t cap, int32_t *count);
int frmc_engines_destroy(void *handle);
/* Work-list configuration: atoms per item, threads per CTA (multiple of 32,
 * at most 512), CTAs per SM. */
int frmc_engines_set_tune(void *handle, int tile, int threads, int ctas_per_sm);
int frmc_engines_get_tune(void *handle, int *tile, int *threads, int *ctas_per_sm, int *nitems);
/* Batched steps run one CTA per engine where the engine's element-pair deltas
 * fit in shared memory (fused = 1, the default), else every engine is split
 * over atom tiles (fused = 0).  Results are identical either way. */
int frmc_engines_set_mode(void *handle, int fused);
/* Column grids (on = 1, the default): an engine added afterwards gets its
 * atoms sorted into at most 512 cells where that pays, and the one-CTA step
 * sweeps only the cells whose bounding box may come within maxDistance of a
 * moved atom (a lower bound of the minimum-image distance with a margin far
 * above float32 rounding, so every skipped pair is out of range before and
 * after the move).  Results are identical with and without grids.
 * frmc_engines_cells reports an engine's number of cells (0: no grid) and,
 * when swept is not null, the columns its one-CTA steps swept since init. */
int frmc_engines_set_cells(void *handle, int32_t on);
/* Rebuild engine e's column grid from its current coordinates (cell bounds
 * only grow as atoms move; a long run with large moves can re-tighten them).
 * Results are unchanged. */
int frmc_engines_regrid(void *handle, int32_t e);
/* The column grids' distance bound for a basis (host only, no device use):
 * w[k] and lam such that the reference's minimum-image distance of box
 * difference g satisfies |g B| >= |g_k| w[k] and |g B|^2 >= lam |g|^2
 * (mode 1), or |g B|^2 >= sum (g_k w[k])^2 (mode 0: orthorhombic box, or free
 * boundaries with w = 1). */
int frmc_cell_metric(const float *basis, int32_t isPBC, double *w, double *lam, int32_t *mode);
int frmc_engines_cells(void *handle, int32_t e, int32_t *ncells, int64_t *swept);
/* The S(Q) term's product y = T x runs on the tensor cores (the library's own
 * tcgen05 kernel: fp16 base-4096 digit planes of T times fp16 deltas, fp32
 * accumulators in tensor memory) for an element-pair delta column whose
 * entries are at most `limit` in magnitude (default and maximum 2048) and
 * whose absolute sum is at most 2^13, where every product sum is an exact
 * integer; other columns take an exact integer sum over the step's list of
 * deltas; -1 takes the dense integer loop.  All three give the same
 * integers; the lower limits exist to test that. */
int frmc_engines_set_sq_gemm_limit(void *handle, int32_t limit);
/* At most `max_splits` K splits per 128-row block of the S(Q) product (0, the
 * default: as many as let one step's tiles fill the SMs).  The products are
 * exact integers, so the split changes the time of a step, not its result. */
int frmc_engines_set_sq_splits(void *handle, int32_t max_splits);
/* All-pairs histograms of the initial coordinates and the initial chi2. */
int frmc_engines_init(void *handle);
/* Moves for steps [first_step, first_step + count) of engine e: atoms (count,),
 * vecs (count, 3) real-space displacements, u (count,) uniforms (NULL = 1). */
int frmc_engines_push_moves(void *handle, int32_t e, const int32_t *atoms, const float *vecs, const float *u,
                            int32_t count, int64_t first_step, int from_device);
/* Group moves for steps [first_step, first_step + count) of an engine with
 * group_size G: atoms (count, G) distinct per move, kinds (count,) 0 =
 * translation of every atom by params[0..2], 1 = rotation of the group about
 * its centroid c (float32 mean of the atoms' real coordinates in the order
 * given): x -> (x - c) R + c with R = params (3 x 3 row-major, row-vector
 * convention); params (count, 9); u (count,) uniforms (NULL = 1).  The moves
 * of fullrmc's TranslationGenerator / RotationGenerator on molecule groups
 * (Generators/Translations.py, Generators/Rotations.py). */
int frmc_engines_push_group_moves(void *handle, int32_t e, const int32_t *atoms, const int32_t *kinds,
                                  const float *params, const float *u, int32_t count, int64_t first_step);
/* Advance `steps` steps: engine == -1 steps every engine in one launch per
 * step (the batched path); engine >= 0 steps that engine alone.  use_graph
 * captures the launches in a CUDA graph (cached per engine/steps).  Returns
 * without synchronising; stream NULL = the set's own stream. */
int frmc_engines_step(void *handle, int32_t engine, int32_t steps, int use_graph, void *stream);
/* Measured placement of the batched one-CTA launch (no counterpart in
 * fullrmc).  Runs `steps` batched steps (they advance every chain like
 * frmc_engines_step, on the set's own stream, synchronously) recording for
 * each engine its CTA's SM and time.  Where one item per CTA is launched and
 * the CTAs landed on the same SMs in every recorded step, the work list is
 * reordered for this set of engines and launch shape: the CTAs that hold an
 * SM alone get the engines that took longest, and on shared SMs the longest
 * remaining engine goes with the shortest.  Results do not depend on the
 * order; adding or removing engines or changing the tuning falls back to the
 * cost order.  Waits for all work on the device first.  Returns
 * FRMC_E_STATE while a host-buffer step is in flight. */
int frmc_engines_place(void *handle, int32_t steps);
/* The ordering frmc_engines_place applies, on the host (no GPU): CTA b of a
 * launch of n one-CTA items ran on SM sm[b] and its item took t[b]; pos[b]
 * receives the item CTA b gets.  CTAs alone on their SM take the longest
 * items; on a shared SM the first CTA takes the longest remaining item and
 * the others the shortest. */
int frmc_engines_place_positions(int32_t n, const int32_t *sm, const double *t, int32_t *pos);
/* One batched step of every live engine from host buffers: atoms (E,), vecs
 * (E, 3), u (E,) in live-id order are uploaded in one copy, the step runs,
 * and each engine's new chi2 and decision come back in one copy (chi2_new,
 * accepted may be NULL).  Synchronous. */
int frmc_engines_step_host(void *handle, const int32_t *atoms, const float *vecs, const float *u, double *chi2_new,
                           int32_t *accepted);
/* The same in two halves, so that a host can submit step k + 1 before it
 * reads step k: submit writes the moves into staging slot `slot` (0 or 1)
 * and enqueues the copy in, the step and the copy of the results out;
 * collect waits for that slot's step and returns its results.  A slot takes
 * one step at a time, steps run in submission order, and the engine set must
 * not change while a step is in flight. */
int frmc_engines_step_host_submit(void *handle, const int32_t *atoms, const float *vecs, const float *u,
                                  int32_t slot);
int frmc_engines_step_host_collect(void *handle, int32_t slot, double *chi2_new, int32_t *accepted);
int frmc_engines_sync(void *handle);
int frmc_engines_state(void *handle, int32_t e, double *chi2, int64_t *step, int64_t *accepted);
/* Per-step results of steps [first_step, first_step + count). */
int frmc_engines_results(void *handle, int32_t e, int64_t first_step, int32_t count, double *chi2_new,
                         int32_t *accepted, int32_t *atoms);
/* Oriented int32 counts [2][ne][ne][hs] (0 = intra, 1 = inter). */
int frmc_engines_counts(void *handle, int32_t e, int32_t *counts);
int frmc_engines_coords(void *handle, int32_t e, float *box_coords, float *real_coords);
int frmc_engines_info(void *handle, int32_t *E, int64_t *total_atoms, int64_t *device_bytes);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* FRMC_GPU_ENGINE_H */
