/* repeat_gb300 — C ABI of the GB300 (sm_103a) periodic REPEAT charge fit.
 *
 * The reference has no C ABI: its fit path is Python (pyREPEAT repeat.py) and
 * its native programs are executables.  Each entry point below replaces one
 * step of repeat.py's fit path; the step is cited beside it.  A Python host
 * (pyrepeat_gb300, via ctypes) and any other FFI bind these symbols.
 *
 * Conventions
 *  - Every function returns RP_OK (0) or a negative RP_E* status and never
 *    aborts; rp_last_error() gives the message of the last failure on a ctx.
 *  - Pointers named *_dev are device pointers on the ctx's device; all other
 *    pointers are host memory.  Device buffers passed in are owned by the
 *    caller; scratch a call needs is owned by the ctx and counted against its
 *    HBM budget.
 *  - Grid values use the reference's flat order flat = i + j*nx + k*nx*ny
 *    (repeat.py:2086), grid point (i,j,k) = i*axis[0] + j*axis[1] + k*axis[2]
 *    (origin ignored, repeat.py:2097-2110).
 *  - A ctx is used by one host thread at a time.  `stream` may be 0 (the
 *    legacy default stream).
 */
#ifndef REPEAT_GB300_H
#define REPEAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RP_OK 0
#define RP_E_ARG -1       /* invalid argument / size */
#define RP_E_CUDA -2      /* CUDA runtime or driver error */
#define RP_E_NOMEM -3     /* over the ctx's HBM budget or allocation failed */
#define RP_E_SINGULAR -4  /* bordered system singular (pivot below threshold) */
#define RP_E_TIMEOUT -5   /* a bounded device-side wait ran out */
#define RP_E_STATE -6     /* call out of order (e.g. gram before filter) */
#define RP_E_UNSUPPORTED -7

/* Arithmetic of the Phi -> normal-equations stage. */
#define RP_PREC_FP64 0  /* plain FP64: FP64 tables, FP64 real space, FP64 Gram (cuBLAS DGEMM / DSYRK) */
#define RP_PREC_MIXED 1 /* FP32 real space from double-float coordinates, separable FP32 reciprocal
                           sum, exact fixed-point Gram on the tensor cores (tcgen05), FP64 solve.
                           In rp_fit / rp_fit_batch a cube whose kappa / (n+1) exceeds the ctx's
                           limit (rp_set_kappa_limit) is refitted in FP64 and flagged
                           RP_FIT_ESCALATED. */

/* Words per system of rp_solve's and rp_solve_noalloc's info: [0] residual inf-norm after
 * refinement, [1] min |pivot|, [2] max |pivot|, [3] kappa = ||A||_1 ||K^-1||_1 with A the
 * folded normal matrix (RESP included) and K the bordered matrix (||K^-1||_1 by Hager's
 * estimator on the factors that solved it).  A relative perturbation e of A moves the
 * charges by at most about e * kappa * max|q|. */
#define RP_SOLVE_INFO_WORDS 4
/* Words per cube of rp_fit_batch's (and rp_batch_submit's) info_out: [0] residual,
 * [1] min |pivot|, [2] max |pivot|, [3] singular flag, [4] kappa (as above), [5] the
 * factorisation that solved it (0 FP32 LU in one CTA, 1 FP32 LU across the GPU, 2 FP64 LU in
 * one CTA, 3 FP64 LU across the GPU; FP32 factors are refined with FP64 residuals),
 * [6] the precision that produced the charges (RP_PREC_*), [7] RP_FIT_* flags. */
#define RP_FIT_INFO_WORDS 8
#define RP_FIT_ESCALATED 1 /* mixed-precision cube refitted in FP64: kappa/(n+1) above the limit */
#define RP_FIT_TWO_PASS 2  /* mixed-precision cube refitted in two passes after a fixed-point clamp */

typedef void *rp_stream_t; /* a cudaStream_t */
typedef struct rp_ctx rp_ctx;
typedef struct rp_ewald rp_ewald;

/* Cube geometry: grid counts and grid step vectors (rows, Bohr). */
typedef struct {
    int n_grid[3];
    double axis[9];
} rp_grid;

/* Library version, major*10000 + minor*100 + patch (2.0.0: the info words above). */
int rp_version(void);

/* Create a context on `device`.  hbm_budget: bytes of scratch the ctx may hold
 * (0 = 90% of free memory at creation). */
int rp_ctx_create(int device, size_t hbm_budget, rp_ctx **out);
int rp_ctx_destroy(rp_ctx *ctx);
/* Copies the last error message (NUL-terminated, truncated to cap). */
int rp_last_error(const rp_ctx *ctx, char *buf, size_t cap);

/* vdW grid filter + compaction + centring.
 * Replaces ChargeCalculator._filter_grid (repeat.py:1922-2113) including its GPU
 * kernel filter_bins (repeat.py:445-518) and the CPU cdist path
 * (repeat.py:2115-2180).  Keep rule: every image (27 per atom) has
 * |g-e|^2 > (vdw_factor*r)^2 and some image has |g-e|^2 <= (vdw_max*r)^2, in FP64
 * (bit-exact mask).  Outputs kept flat indices in increasing order, the ESP at
 * kept points minus its mean, and the kept count.
 *   V_dev        [nx*ny*nz] f64   ESP on the full grid
 *   atoms        [N*3] f64 (host) atom positions; Z [N] int32 atomic numbers (host)
 *   kept_idx_dev [capacity] int32 out; Vc_dev [capacity] f64 out
 *   mask_dev     [nx*ny*nz] u8 out, or NULL
 *   M_out        kept count (host); RP_E_ARG if it exceeds capacity (M_out still set) */
int rp_filter(rp_ctx *ctx, const rp_grid *grid, const double *atoms, const int *Z, int N,
              const double *V_dev, double vdw_factor, double vdw_max, int32_t *kept_idx_dev,
              double *Vc_dev, int64_t capacity, int64_t *M_out, uint8_t *mask_dev,
              rp_stream_t stream);

/* Ewald setup: alpha = (pi/Rc)^2, the integer-index k-set 0<=kx<=KMAX,
 * |ky|,|kz|<=KMAX, 0<k^2<KMAX^2 with kcoef = 4pi/V exp(-k^2/4alpha)/k^2, and the
 * real-space shifts |n_i| <= floor(Rc/|a_i|)+1 pruned by AABB distance.
 * Replaces EwaldCalculator.__init__/_setup_kspace/prepare_pruned_shifts
 * (repeat.py:1077-1143, 1708-1731, 1031-1069).  kmax = 7 is the reference.
 * kmax = 0 selects the non-periodic basis of --fit-type 0 (repeat.py:991-994,
 * 1263-1270): Phi = 1/|g - r_a| for the atom itself (0 at r <= 1e-10), no k-set and
 * no images; the cutoff is ignored.  Every consumer (rp_gram, rp_potential, rp_fit
 * and rp_fit_batch through rp_fit_desc.kmax) then fits or evaluates that basis. */
int rp_ewald_setup(rp_ctx *ctx, const rp_grid *grid, double cutoff, int kmax, rp_ewald **out);
int rp_ewald_destroy(rp_ewald *ew);
/* K (k vectors), S (shifts before pruning), alpha. Any out pointer may be NULL. */
int rp_ewald_info(const rp_ewald *ew, int *K, int *S, double *alpha);

/* Mean-removed normal equations of the Ewald basis over the kept points.
 * Replaces the streaming loop of ChargeCalculator.fit_charges
 * (repeat.py:2184-2276: Phi via EwaldCalculator._compute_gpu*, repeat.py:1199-1435,
 * then ATA += Phi^T Phi, ATb += Phi^T V, mean correction).  Phi is produced
 * tile by tile on the device and never returned.
 *   A_dev [N*N] f64 out (row-major), b_dev [N] f64 out: A = Phi^T (I - 11^T/M) Phi,
 *   b = Phi^T (I - 11^T/M) Vc;  sum_phi_dev [N] out: column sums of Phi (may be NULL);
 *   precision: RP_PREC_FP64 or RP_PREC_MIXED. */
int rp_gram(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
            const double *Vc_dev, int64_t M, int precision, double *A_dev, double *b_dev,
            double *sum_phi_dev, rp_stream_t stream);

/* Constraints and bordered solve on the device, FP64.
 * Replaces repeat.py:2278-2313 with _apply_symmetry/_expand_charges
 * (repeat.py:2445-2489) and _apply_resp (repeat.py:2511-2520):
 * symmetry groups fold columns then rows into the base atom, RESP adds
 * resp_s[i] to A_ii and resp_s[i]*resp_t[i] to b_i (per original atom, 0 = none),
 * the (n+1) bordered system [[A, w],[w^T, 0]] [q; l] = [b; qtot] is solved by LU
 * with partial pivoting plus one step of FP64 iterative refinement, and charges
 * are expanded back to all N atoms.
 *   A_dev, b_dev   inputs (not modified)
 *   group_ptr [n_groups+1], group_idx [group_ptr[n_groups]] (host, 0-based, first = base)
 *   resp_s, resp_t [N] (host, may be NULL)
 *   q_dev [N] f64 out;  info [RP_SOLVE_INFO_WORDS] (host, may be NULL).
 *   No escalation happens here: a caller of rp_gram + rp_solve reads kappa and may run
 *   rp_gram again with RP_PREC_FP64. */
int rp_solve(rp_ctx *ctx, const double *A_dev, const double *b_dev, int N, int n_groups,
             const int *group_ptr, const int *group_idx, const double *resp_s, const double *resp_t,
             double qtot, double *q_dev, double *info, rp_stream_t stream);

/* Ewald potential of point charges q at grid points (no Phi matrix):
 * out[m] = sum_a q_a phi_a(g_m) with the same k-set, weights and real-space
 * images as the fit.  Replaces the V_coul = Phi q pass of compute_stats
 * (repeat.py:2326-2441) used by --stats and --output.
 *   atoms [N*3], q [N] host; idx_dev [npts] int32 flat grid indices, or NULL for
 *   every grid point (npts = nx*ny*nz); out_dev [npts] f64. */
int rp_potential(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, const double *q, int N,
                 const int32_t *idx_dev, int64_t npts, double *out_dev, rp_stream_t stream);

/* QEq charges: replaces ChargeCalculator.compute_qeq_charges (repeat.py:2539-2634)
 * below its per-element parameter lookup, i.e. the Coulomb matrix
 *   J_ii = j_self[i],  J_ij = sum over every shift (|n_i| <= floor(Rc/|a_i|)+1, no cutoff)
 *   with r > 1e-10 of erfc(sqrt(alpha) r)/r + sum_k kcoef_k cos(k.(r_i - r_j))
 * (repeat.py:2575-2595, 2615-2634; with an ewald object of kmax 0, J_ij = 1/r_ij as in
 * the non-periodic branch) and the equalisation system of repeat.py:2597-2613: sum q =
 * qtot and (J q)_i + chi_i equal for every atom, solved in its bordered form
 * [[J, 1],[1^T, 0]] [q; mu] = [-chi; qtot] by the same solve as rp_solve.
 *   atoms [3N] host (Bohr, as in the cube), chi [N] host (electronegativity, Hartree),
 *   j_self [N] host (J_ii = 2 x hardness); q [N] host out; J [N*N] host out
 *   (row-major, may be NULL); info as rp_solve's (may be NULL).
 *   RP_E_SINGULAR where the reference falls back to least squares. */
int rp_qeq(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const double *chi,
           const double *j_self, double qtot, double *q, double *J, double *info, rp_stream_t stream);

/* rp_solve without any device allocation, for callers that cannot allocate
 * device memory while they run (a serving loop that must not stall on the
 * device-wide synchronisation cudaMalloc/cudaFree may cause, or an embedder whose
 * device memory is owned by its own allocator).  Same arguments and results as
 * rp_solve, but no ctx: its scratch is a static 4.5 MiB device array inside the
 * library, so N is limited to 512 atoms (RP_E_ARG beyond that).  No counterpart in
 * the reference.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make it before any stream
 * capture.  Under lazy module loading that first call may also load the library's
 * device code and, with it, the array.  The address is kept for the life of the
 * process, so a cudaDeviceReset voids this entry point.  A call is synchronous: it
 * returns once its solve on `stream` has finished.  Every call shares the array:
 * calls that overlap on the GPU race, so serialise them.  Returns RP_E_SINGULAR
 * for a singular bordered system. */
int rp_solve_noalloc(const double *A_dev, const double *b_dev, int N, int n_groups, const int *group_ptr,
                     const int *group_idx, const double *resp_s, const double *resp_t, double qtot, double *q_dev,
                     double *info, rp_stream_t stream);

/* One whole fit from host memory, as repeat.py's main() runs it for
 * `--fit-type 1 [--gpu]`: H2D of V, filter, Ewald setup, normal equations,
 * constraints, solve, D2H of the charges.  q_out [N] host. M_out may be NULL. */
typedef struct {
    rp_grid grid;
    const double *V;        /* [nx*ny*nz] host */
    const double *atoms;    /* [N*3] host */
    const int *Z;           /* [N] host */
    int N;
    double vdw_factor, vdw_max, cutoff, qtot;
    int kmax;               /* 7 = the reference; 0 = the non-periodic fit (--fit-type 0) */
    int n_groups;
    const int *group_ptr, *group_idx;
    const double *resp_s, *resp_t;
    int precision;
} rp_fit_desc;
int rp_fit(rp_ctx *ctx, const rp_fit_desc *desc, double *q_out, int64_t *M_out, rp_stream_t stream);

/* Many independent fits in one call (the batched workload).  The cubes run as a
 * pipeline of up to four groups: each group's filters (their host halves on the
 * ctx's host workers, one pinned upload), then, as its kept counts arrive, its
 * normal equations on four worker streams and its folds and bordered solves (one
 * launch, one CTA per system) on `stream`, while the next group's filters run.  The
 * call returns when every charge is on the host.  No reference counterpart:
 * repeat.py fits one cube per process.
 *   descs[n]     as for rp_fit (each with its own precision)
 *   V_dev        NULL, or n device pointers (an entry may be NULL: use descs[i].V on the host)
 *   q_out        host, the charges of all cubes concatenated (sum of N_i doubles)
 *   M_out[n]     host kept counts (may be NULL); info_out[RP_FIT_INFO_WORDS * n] host
 *                (may be NULL), per cube as described at RP_FIT_INFO_WORDS */
int rp_fit_batch(rp_ctx *ctx, int n, const rp_fit_desc *descs, const double *const *V_dev, double *q_out,
                 int64_t *M_out, double *info_out, rp_stream_t stream);

/* Asynchronous batches, the serving interface (no reference counterpart: repeat.py
 * is a one-shot program).  rp_batch_submit queues a batch for the ctx's worker
 * thread, which runs queued batches in order as rp_fit_batch does (on a stream of
 * its own), and returns a ticket.  The descriptor array is copied; the arrays it
 * points to, V_dev and the outputs must stay valid until the ticket is retired.
 * While tickets are outstanding the ctx belongs to the worker: only submit, poll,
 * wait and rp_last_error may be called on it.  rp_batch_poll sets *done (and, when
 * done, *status = the batch's rp_fit_batch status, its message in rp_last_error)
 * without blocking; rp_batch_wait blocks.  A finished ticket is retired by the poll
 * or wait that reports it; rp_ctx_destroy lets the running batch finish and drops
 * the queued ones. */
int rp_batch_submit(rp_ctx *ctx, int n, const rp_fit_desc *descs, const double *const *V_dev, double *q_out,
                    int64_t *M_out, double *info_out, long long *ticket);
int rp_batch_poll(rp_ctx *ctx, long long ticket, int *done, int *status);
int rp_batch_wait(rp_ctx *ctx, long long ticket, int *status);

/* Limit on kappa / (n+1) (kappa as in RP_SOLVE_INFO_WORDS, n+1 the unknowns of the
 * bordered system after symmetry folding) above which rp_fit / rp_fit_batch refit a
 * mixed-precision cube in FP64; 0 = never refit.  On seeded cubes of 9 to 2000 atoms the
 * mixed charges differed from FP64 by about 2e-11 kappa/(n+1) e, so the default, 2e5, keeps
 * that near 4e-6 e; cubes beyond it (hundreds of densely packed atoms leaving few ESP
 * points) are fitted in FP64.  No reference counterpart: repeat.py fits in the precision
 * it is asked for. */
int rp_set_kappa_limit(rp_ctx *ctx, double kappa_max);

/* Autotuner of the mixed-precision path's tile shapes (no reference counterpart): for every
 * bucket of (atoms, kept points, KMAX) that the given cubes fall in and the ctx has no entry
 * for, the first such cube's normal equations are timed (CUDA events) with each tile shape
 * (Phi atoms per CTA 8/16/32 x Gram points per CTA 256/512/1024) and the fastest is kept
 * for the bucket; rp_fit / rp_fit_batch use the ctx's table.  Tile shapes change no result
 * (every Phi value and exact digit sum is the same whatever the tiling).  cache_path (may
 * be NULL): the whole table is written there as text lines "key phi_atoms gram_split
 * [best_ms default_ms N M]"; rp_load_tiles reads such a file into a ctx. */
int rp_autotune(rp_ctx *ctx, int n, const rp_fit_desc *descs, const double *const *V_dev, const char *cache_path);
int rp_load_tiles(rp_ctx *ctx, const char *cache_path);

/* Profiling hooks (no reference counterpart).  With timing on, every stage
 * records CUDA events on the stream it runs on; rp_stage_times synchronises,
 * returns per stage name the summed milliseconds and launch count
 * (ms[2k], ms[2k+1]), names '\n'-separated, and clears the record.
 * *count_inout: capacity in, stages written out. */
int rp_set_timing(rp_ctx *ctx, int enable);
/* Total kernel launches the library has issued in this process. */
int rp_launch_count(long long *out);
int rp_stage_times(rp_ctx *ctx, char *names, size_t names_cap, double *ms, int *count_inout);

#ifdef __cplusplus
}
#endif
#endif
