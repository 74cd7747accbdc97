/* CPU oracle for the periodic REPEAT fit — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithm (pyREPEAT repeat.py and
 * repeat_cpu_omp.cpp), used by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py, to check results.  Nothing in the product links or
 * calls it.  All arithmetic is IEEE FP64 with floating-point contraction
 * disabled (-ffp-contract=off), so the filter mask is reproducible bit for bit.
 *
 * Parity of this restatement is pinned against the reference itself: golden
 * fixtures under tests/golden/ were produced by running repeat.py
 * (--fp64 --no-jit path) and the compiled repeat_cpu_omp.cpp on the same cubes.
 */
#ifndef REPEAT_ORACLE_H
#define REPEAT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* k vectors / coefficients, repeat.py:1127-1143. Returns K (or -needed if cap too small). */
int orc_kspace(const double box[9], double cutoff, int kmax, double *kvecs, double *kcoefs, int cap);
/* full real-space shift list, repeat.py:1101-1104 and 815-822. Returns S. */
int orc_realspace_shifts(const double box[9], double cutoff, double *shifts, int cap);
/* AABB pruning of shifts, repeat.py:1031-1069. Returns kept count, zero_idx via pointer. */
int orc_prune_shifts(const double *shifts, int S, const double *grid, int64_t M, const double *atoms,
                     int N, double cutoff, double *out, int *zero_idx);

/* vdW filter, repeat.py:1922-2113 with the squared-distance rule of repeat.py:508-516.
 * mask[flat] = 1 for kept points; flat = i + j*nx + k*nx*ny. Returns kept count. */
int64_t orc_filter(int nx, int ny, int nz, const double axis[9], int N, const double *atoms,
                   const int *Z, double vdw_factor, double vdw_max, uint8_t *mask, int threads);
/* same mask from sqrt distances (the cdist form, repeat.py:2176-2177), for the tie report */
int64_t orc_filter_sqrt(int nx, int ny, int nz, const double axis[9], int N, const double *atoms,
                        const int *Z, double vdw_factor, double vdw_max, uint8_t *mask, int threads);

/* kept positions and mean-removed V over kept points (repeat.py:2081-2113). */
void orc_compact(int nx, int ny, int nz, const double axis[9], const uint8_t *mask, const double *V,
                 int64_t *kept_flat, double *grid, double *Vc, int64_t M);

/* one Phi row block: phi[m*N + a] = real + recip, repeat.py:944-998 (no self term). */
void orc_phi(int64_t M, const double *grid, int N, const double *atoms, int K, const double *kvecs,
             const double *kcoefs, int S, const double *shifts, int zero_idx, double cutoff,
             double sqrt_alpha, double *phi, int threads);

/* streamed normal equations over M points (repeat.py:2184-2276): A (N*N, mean removed),
 * b (N), sum_phi (N), sum_V.  Phi rows are computed in blocks, never stored in full. */
int orc_normal_equations(int64_t M, const double *grid, const double *V, int N, const double *atoms,
                         int K, const double *kvecs, const double *kcoefs, int S, const double *shifts,
                         int zero_idx, double cutoff, double *A, double *b, double *sum_phi,
                         double *sum_V, int threads);

/* constraints + bordered solve, repeat.py:2278-2313, 2445-2520.
 * groups: flattened lists; group_ptr[g]..group_ptr[g+1], first entry = base (0-based).
 * resp_s/resp_t: per-atom restraint strength/target (0 for none), indexed by ORIGINAL atom.
 * A and b are modified in place. charges: N outputs. Returns 0, or 1 if the pivot was tiny. */
int orc_solve(int N, double *A, double *b, int n_groups, const int *group_ptr, const int *group_idx,
              const double *resp_s, const double *resp_t, double qtot, double *charges);

/* dense LU with partial pivoting (GE as repeat_cpu_omp.cpp:466-495 / LAPACK gesv). */
int orc_lu_solve(int n, double *A, double *b, double *x);

#ifdef __cplusplus
}
#endif
#endif
