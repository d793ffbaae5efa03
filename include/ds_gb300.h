/*
 * dachshund-gb300 C ABI: the Wiener-filter hot path of Dachshund on one
 * GB300 (sm_103a), behind plain pointers and sizes.
 *
 * The path: the Gaussian signal covariance S (table or exact exp), the
 * operator A = S + N (SN form) or A = w S w + I (W form), Jacobi-PCG on
 * A x = b, and the map projection m = S_mp x.  Most functions here replace
 * one call of the reference library (caseywstark/dachshund, the headers in
 * lib/); each declaration names the reference interface it stands in for,
 * or says that it has no counterpart there.
 *
 * Conventions
 *  - Host arrays are caller-owned; nothing here keeps a host pointer after
 *    the call returns (lib/wf_vector.h:35,70 hold non-owning pointers; the
 *    operator here copies the records into device memory instead).
 *  - Pixel records are 5 doubles each, in the reference layouts
 *    (lib/pixel.h:16-50): Pixel {x,y,z,n,d}, NPixel {x,y,z,N=n^2,d},
 *    WPixel {x,y,z,w=1/n,wd=d/n}.  Points are 3 doubles {x,y,z}.
 *  - Vectors passed to and from an operator are in the caller's record
 *    order.  ``*_dev`` variants take device pointers (same order) and run on
 *    the context's stream without a host synchronisation at the end.
 *  - Every function returns a ds_status.  The reference reports errors by
 *    exit(1) (I/O) or PCGResult.success (solver); here the caller decides.
 *  - One context = one device + one CUDA stream.  Calls on one context are
 *    sequential; distinct contexts may be used from distinct threads.
 */
#ifndef DS_GB300_H
#define DS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
typedef enum {
  DS_OK = 0,
  DS_ERR_ARG = 1,           /* bad argument (null pointer, n <= 0, bad form) */
  DS_ERR_CUDA = 2,          /* a CUDA runtime call failed */
  DS_ERR_NOT_CONVERGED = 3, /* PCG hit max_iter (lib/pcg.h:151-155) */
  DS_ERR_NORM_B = 4,        /* |b| <= 0: early return (lib/pcg.h:79-86) */
  DS_ERR_OOM = 5,           /* device allocation failed */
  DS_ERR_NO_DEVICE = 6,     /* no CUDA device or wrong architecture */
  DS_ERR_STATE = 7,         /* object used after a fatal error */
  DS_ERR_TIMEOUT = 8        /* a bounded wait inside a tensor-core kernel ran out; the
                               kernel released its tensor memory and returned, and the
                               context stays usable */
} ds_status;

const char* ds_status_string(int status);

/* ---- kernel (signal covariance) parameters ----------------------------- */
typedef enum { DS_FORM_SN = 0, DS_FORM_W = 1 } ds_form;

typedef enum {
  DS_EVAL_TABLE = 0, /* 200-knot exp table + linear interpolation, zero for
                        c_perp*dperp^2 + c_para*dz^2 at or beyond the last
                        interval (lib/signal_covar.h:53-77) */
  DS_EVAL_EXACT = 1  /* var_s * exp(-arg) (lib/signal_covar.h:79-86), zero for
                        arg >= exact_cutoff */
} ds_eval;

#define DS_TABLE_N 200                /* default_gaussian_table_n */
#define DS_DEFAULT_EXACT_CUTOFF 40.0  /* exp(-40) = 4.2e-18 */
/* Cutoff of the FP32 inner operator of the mixed-precision solvers: terms
 * below exp(-12) = 6e-6 var_s are dropped from the inner products only (the
 * FP64-accurate residual keeps the operator's own cutoff, so the solution and
 * its stopping test are unchanged).  On the 262,144-pixel workload cutoffs
 * 24 down to 10 all take 162 iterations and 2 reliable updates; 9 takes 3
 * updates; 12 keeps a margin and evaluates half the pairs of 24. */
#define DS_DEFAULT_INNER_CUTOFF 12.0
/* The same cutoff for the structured FP32 inner operator
 * (ds_operator_set_skewer_grid), which drops every term beyond it (the pair
 * kernel keeps whole 32 x 32 sub-tiles that reach the cutoff, i.e. more
 * terms): on the 262,144-pixel workload with the cluster preconditioner, 12
 * takes 101 iterations and 3 reliable updates, 14 to 24 take 90 and 2, and 14
 * is the fastest. */
#define DS_DEFAULT_STRUCTURED_INNER_CUTOFF 14.0

typedef struct {
  double var_s;          /* SignalCovarParams::var_s */
  double l_perp;         /* -> gaussian_const_perp = 1/(2 l_perp^2) */
  double l_para;         /* -> gaussian_const_para = 1/(2 l_para^2) */
  int eval;              /* ds_eval */
  double exact_cutoff;   /* exponent cutoff for DS_EVAL_EXACT; <= 0: default */
  const double* table;   /* optional DS_TABLE_N host-built knots f_i (e.g.
                            SignalCovarParams::func_table); NULL: built here */
} ds_kernel_params;

/* SignalCovarParams ctor (lib/signal_covar.h:19-41): fills the 200-knot
 * table f_i = exp(-i dx), dx = 8/199, and the index scale 1/dx. */
void ds_table_init(double* table, double* dx_inv);

/* signal_covar / signal_covar_exact (lib/signal_covar.h:67-86) evaluated on
 * the device for n (perp^2, para^2) pairs; host arrays. */
int ds_signal_covar(const ds_kernel_params* kp, int n, const double* perp2,
                    const double* para2, double* out);

/* ---- context ------------------------------------------------------------ */
/* No reference counterpart: the reference keeps no device state.  A context
 * owns one device, one CUDA stream (every call of its objects is ordered on
 * it, and their device buffers are allocated and freed stream-ordered on it)
 * and the message of the last failed call.  Not thread-safe; sequential
 * calls from one thread, as the reference's single caller thread makes them. */
typedef struct ds_context ds_context;

int ds_context_create(int device, ds_context** out);
void ds_context_destroy(ds_context* ctx);
/* The context's CUDA stream (a cudaStream_t) for event timing and for
 * ordering caller work against the *_dev entry points. */
void* ds_context_stream(ds_context* ctx);
int ds_context_synchronize(ds_context* ctx);
/* Message of the last failed call on this context ("" when none). */
const char* ds_context_last_error(ds_context* ctx);

/* Instrumentation (no reference counterpart; the reference only has wall
 * clocks, lib/timer.h:13-26).  When enabled, every launch of a pair kernel
 * (the matvec / residual / map kernels) on this context is bracketed by CUDA
 * events on the context's stream; the profile accumulates their device time,
 * their count and the tile-evaluated pairs they covered (for the batched
 * kernels of ds_batch_*: pair x right-hand-side products, and a profiled
 * batched solve runs its iterations without the CUDA graph so that each
 * launch can be timed).  Disabling keeps the totals until the next enable. */
typedef struct {
  long long pair_launches;   /* pair-kernel launches timed (FP64 + FP32) */
  double pair_ms;            /* their summed device time */
  double pair_evaluated;     /* pairs evaluated (tile pairs x tile^2) */
  long long kernel_launches; /* every kernel this library launched (process-wide) */
  long long f64_launches;    /* the FP64 pair kernels alone */
  double f64_ms;
  double f64_evaluated;
  long long f32_launches;    /* the FP32 pair kernels alone (products) */
  double f32_ms;
  double f32_evaluated;
  long long map_launches;    /* map products (FP64 or FP32) */
  double map_ms;
  double map_evaluated;
  long long dense_launches;  /* dense-operator matvecs (ds_operator_set_dense) */
  double dense_ms;
  double dense_entries;      /* matrix entries read (n_pad^2 per matvec) */
} ds_profile;
int ds_context_set_profiling(ds_context* ctx, int enable);
int ds_context_get_profile(ds_context* ctx, ds_profile* out);

/* Bound, in SM clock cycles, of every mbarrier wait of the batched
 * tensor-core matvec (ds_batch_set_variant DS_BATCH_TENSOR) launched on this
 * context; 0 restores the default of 4e9 cycles (about 2 s).  A wait that
 * runs out records its code, the kernel waits (with the default bound) for
 * its own MMAs and copies in flight, frees its tensor memory and returns, and
 * the call returns DS_ERR_TIMEOUT.  The same bound applies to each grid
 * barrier wait of the persistent mixed solve (ds_operator_set_iteration_form;
 * checked before each poll, so a bound of 1 gives up at once): a CTA that
 * runs out records the phase, every CTA leaves when it finds the record (in
 * that wait or at its next barrier), and the call returns DS_ERR_TIMEOUT.  No reference counterpart
 * (the reference has no device code). */
int ds_context_set_wait_limit(ds_context* ctx, long long cycles);

/* ---- the operator A over one pixel set --------------------------------- */
typedef struct ds_operator ds_operator;

/* WFVectorSN / WFVectorW ctor (lib/wf_vector.h:37-46, 72-81).  ``records``:
 * n NPixel (form SN) or WPixel (form W) records.  Copies them to the device
 * in a spatially sorted, tiled layout and builds the culled tile-pair list. */
int ds_operator_create(ds_context* ctx, int form, int n, const double* records,
                       const ds_kernel_params* kp, ds_operator** out);
void ds_operator_destroy(ds_operator* op);

/* Statistics of the tiling (no reference counterpart; the reference visits
 * every pair): tiles, interacting tile pairs, evaluated pairs per matvec
 * (tile pairs x tile^2), and the tile size. */
typedef struct {
  int n;
  int n_pad;
  int tile;
  int n_tiles;
  long long n_tile_pairs;
  long long evaluated_pairs;
} ds_operator_info;
int ds_operator_get_info(ds_operator* op, ds_operator_info* info);

/* WFVector{SN,W}::A_product, b = A a (lib/wf_vector.cc:51-74, 196-220). */
int ds_A_product(ds_operator* op, const double* a, double* b);
int ds_A_product_dev(ds_operator* op, const double* a, double* b);

/* WFVector{SN,W}::A_residual, r = b - A x (lib/wf_vector.cc:76-103,
 * 222-251), b = d (SN) or wd (W) from the records. */
int ds_A_residual(ds_operator* op, const double* x, double* r);
int ds_A_residual_dev(ds_operator* op, const double* x, double* r);

/* WFVector{SN,W}::preconditioner_solve, x = M^-1 b (lib/wf_vector.cc:42-49,
 * 185-194). */
int ds_preconditioner_solve(ds_operator* op, const double* b, double* x);

/* WFVector{SN,W}::norm_b (lib/wf_vector.cc:105-112, 253-260). */
int ds_norm_b(ds_operator* op, double* norm_b);

/* WFVector{SN,W}::A(i, j, exact) (lib/wf_vector.cc:16-40, 157-183) for m
 * index pairs, evaluated on the device.  ``eval``: DS_EVAL_TABLE,
 * DS_EVAL_EXACT (the reference's ``exact`` flag), or -1 for the operator's
 * own mode. */
int ds_A_entries(ds_operator* op, int eval, int m, const int* ii,
                 const int* jj, double* out);

/* Dense S_pp in HBM (no reference counterpart; the reference builds the
 * dense matrix only inside solve_cf, lib/wf_vector.cc:127-133, and its
 * A_product, lib/wf_vector.cc:51-74 and 196-220, visits every pair).
 * enable = 1 builds the n_pad x n_pad FP64 operator in device memory
 * (8 n_pad^2 bytes, n_pad = n rounded up to 128; DS_ERR_OOM when it does not
 * fit) and makes A_product, A_residual and solve_pcg use the dense matvec;
 * enable = 0 frees it and returns to the matrix-free kernels. */
int ds_operator_set_dense(ds_operator* op, int enable);

/* Arithmetic of the dense matvec (no reference counterpart).  The matrix is
 * FP64 in either case.  DS_DENSE_FLOAT_PAIR splits each entry into two
 * floats (47 significant bits, 2^-46 relative) and accumulates in
 * float-float on the FP32 pipe, which keeps the product at the HBM rate;
 * DS_DENSE_FP64 uses FP64 FMAs (GB300 issues 2 per clock per SM, which caps
 * the product below the HBM rate).  DS_DENSE_AUTO (default) takes float
 * pairs when every nonzero |A_ij| lies in [2^-100, 2^100] (checked when the
 * matrix is built), else FP64; products agree to about 1e-14 relative.
 * ds_operator_get_dense_arith reports the one in use (dense operator
 * built). */
enum { DS_DENSE_AUTO = 0, DS_DENSE_FLOAT_PAIR = 1, DS_DENSE_FP64 = 2 };
int ds_operator_set_dense_arith(ds_operator* op, int arith);
int ds_operator_get_dense_arith(ds_operator* op, int* arith);

/* Inner matvec of the mixed-precision form (no reference counterpart; the
 * reference has no FP32 path).  DS_INNER_CUDA_CORE uses the CUDA-core pair
 * kernel (4 FMA lanes + 1 ex2 per pair); DS_INNER_TENSOR the tensor-core
 * pair kernel (pair exponents by tcgen05 TF32 MMAs, one ex2 per pair) where
 * the operator's tiles allow the expanded exponent form, else the CUDA-core
 * one; DS_INNER_STRUCTURED the FP32 structured operator (perpendicular factor
 * per skewer pair x Toeplitz z taps) of ds_operator_set_skewer_grid, else the
 * CUDA-core one.  DS_INNER_AUTO: the structured operator when a skewer grid
 * is installed, else the CUDA-core pair kernel. */
enum { DS_INNER_AUTO = 0, DS_INNER_CUDA_CORE = 1, DS_INNER_TENSOR = 2,
       DS_INNER_STRUCTURED = 3 };
int ds_operator_set_inner_matvec(ds_operator* op, int variant);

/* How the mixed-precision form launches its iterations (no reference
 * counterpart).  DS_ITER_AUTO (default): with the structured inner operator
 * and a band preconditioner (cluster or learned), the whole iteration loop
 * is one cooperative launch whose CTAs stay resident and meet at bounded
 * grid barriers (the call returns DS_ERR_TIMEOUT if a barrier wait runs out,
 * see ds_context_set_wait_limit); otherwise, and with DS_ITER_GRAPH, eight
 * iterations are one CUDA graph replayed until the solve ends.  Both run the
 * same recurrence; sums are taken in a different order, so iteration counts
 * can differ by rounding. */
enum { DS_ITER_AUTO = 0, DS_ITER_GRAPH = 1 };
int ds_operator_set_iteration_form(ds_operator* op, int form);

/* Phase timers of the persistent launches (%globaltimer on the device,
 * accumulated since the last reset).  out[0] launches, out[1] their total
 * device time (ms), out[2] CTAs, out[3] one empty grid barrier (us, from the
 * calibration barriers each launch starts with); then for each phase
 * c = 1..5 (1 levels of the first direction, 2 product, 3 step, 4 FP64
 * levels of an update, 5 the update's residual and preconditioner) four
 * values at out[4 + 4 (c - 1)]: us per visit (exit of the previous barrier
 * to exit of this one, CTA 0), the CTAs' mean work per visit (us, to their
 * arrival), the slowest CTA's work per visit (us) and the visits; out[24]
 * the neighbour values one product loads (resident form: each distinct
 * (neighbour skewer, level) row a cluster uses, once; 0 for the general
 * form) and out[25] those rows.  Writes min(n, 26) values; *written (may be
 * null) gets that count, 0 before the first persistent launch.  reset != 0
 * clears the timers after reading. */
int ds_operator_get_persistent_profile(ds_operator* op, double* out, int n, int reset,
                                       int* written);

/* ---- PCG ---------------------------------------------------------------- */
/* PCGParams (lib/pcg.h:13-19); n is the operator's. */
typedef struct {
  int max_iter;
  int step_r;
  double tol;
  int verbose;  /* print the reference's per-iteration trace to stdout */
} ds_pcg_params;

/* PCGResult (lib/pcg.h:21-25) minus the history vector, which is written
 * to the caller's buffer. */
typedef struct {
  int success;        /* PCGResult::success */
  int num_iters;      /* PCGResult::num_iters */
  double norm_b;      /* |b| */
  double final_norm;  /* last |r| */
  int n_outer;        /* FP64 true-residual evaluations (mixed form) */
  int n_inner;        /* FP32 iterations (mixed form) */
  double seconds;     /* device time of the solve */
} ds_pcg_result;

/* WFVector{SN,W}::solve_pcg (lib/wf_vector.cc:114-121, 263-274) driving
 * pcg_solve (lib/pcg.h:67-160): x holds the initial guess on entry and the
 * solution (multiplied by w in the W form) on return.  ``residual_norms``
 * may be NULL or hold max_iter + 1 doubles; it receives |r| per iteration as
 * PCGResult::residual_norms does.  Returns DS_OK, DS_ERR_NOT_CONVERGED or
 * DS_ERR_NORM_B (with the result filled in each case). */
int ds_solve_pcg(ds_operator* op, const ds_pcg_params* pp, double* x,
                 ds_pcg_result* res, double* residual_norms);
int ds_solve_pcg_dev(ds_operator* op, const ds_pcg_params* pp, double* x,
                     ds_pcg_result* res, double* residual_norms);

/* Jacobi-PCG that allocates no device memory.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc: a host application
 * that hands out all device memory from its own pool or arena and keeps the
 * rest of the GPU for other work, or a solver loop that must not stop the
 * device (cudaMalloc can synchronise the device and can fail under memory
 * pressure in the middle of a run).  The caller supplies every buffer:
 * ``records`` (n NPixel / WPixel records) and ``x`` (initial guess in,
 * solution out, times w in the W form) are DEVICE pointers in the caller's
 * order; ``residual_norms`` is an optional HOST buffer of max_iter + 1
 * doubles (at most the first 8192 norms are recorded).  The work space is
 * one fixed device array in the library (about 3.3 MB, held on every GPU
 * that loads the library until the process exits), so n is limited to
 * 32,768 pixels; larger n returns DS_ERR_ARG with a message.  There is no
 * spatial tiling (it needs temporary memory): every pixel pair is evaluated,
 * so this entry point suits small and medium problems.
 *  - The first call on a device looks up the work space's device address
 *    (once per device).  CUDA loads device code lazily by default, so that
 *    first call is also when the work space is reserved on the device and
 *    the library's code is loaded there (unless the process sets
 *    CUDA_MODULE_LOADING=EAGER): it can then allocate, synchronise or fail
 *    for lack of memory.  Make the first call on each device during set-up,
 *    before any stream capture; later calls allocate nothing.
 *  - All calls share the one work space and each call re-initialises it:
 *    calls that overlap on the GPU (other streams or threads) race.
 *  - ``stream`` is a cudaStream_t (NULL: the legacy default stream); the call
 *    returns after the solve has finished on it. */
int ds_solve_pcg_noalloc(int form, int n, const double* records,
                         const ds_kernel_params* kp, const ds_pcg_params* pp,
                         double* x, ds_pcg_result* res,
                         double* residual_norms, void* stream);

/* WFVector{SN,W}::solve_cf (lib/wf_vector.cc:123-155, 276-319): the dense
 * system built on the device (table or exact kernel per kp->eval, as the
 * reference's ``exact`` flag) and solved by an FP64 Cholesky factorisation
 * (the reference uses Eigen's LDL^T; A is SPD, so the solutions agree to
 * round-off).  ``records``: n NPixel / WPixel host records; ``x`` receives the
 * solution (times w in the W form).  Needs 8 n^2 bytes of device memory. */
int ds_solve_cf(ds_context* ctx, int form, int n, const double* records,
                const ds_kernel_params* kp, double* x);

/* MapCovarDiag::solve_pcg (lib/map_covar.cc:73-113): for every map point i,
 * the SN-form PCG solve of (S + N) x = S_pm[:, i] from x = 0, then
 * sigma_m[i] = S_mp[i, :] . x when the solve succeeded (else 0).  Writes the
 * per-point iteration counts and success flags.  Table kernel (the
 * reference's): one FP64 Jacobi-PCG per point, as the reference.  Exact
 * kernel (DS_EVAL_EXACT, no reference counterpart): groups of 64 map points
 * are the right-hand sides of one batched mixed-precision solve (ds_batch_*;
 * FP32 iterations reported, stopping test on the FP64-accurate residual). */
int ds_map_covar_diag(ds_context* ctx, int n_pix, const double* npixels, int n_map,
                      const double* map_points, const ds_kernel_params* kp,
                      const ds_pcg_params* pp, double* sigma_m, int* iters,
                      int* success);

/* ---- mixed-precision form (no reference counterpart) --------------------
 * Solves the same system as ds_solve_pcg with the exact kernel
 * (DS_EVAL_EXACT): FP32 Jacobi-PCG on an FP32 matrix-free operator (MUFU
 * ex2) inside FP64 reliable updates, which recompute the true residual
 * b - A x with the FP64 operator and stop on |r| <= tol |b| in FP64.  It is
 * the fast path that stands in for WFVector{SN,W}::solve_pcg
 * (lib/wf_vector.cc:114-121, 263-274) when the exact kernel is wanted. */
typedef struct {
  int max_iter;          /* cap on FP32 iterations */
  double tol;            /* FP64 stopping test |b - A x| <= tol |b| */
  double reliable_delta; /* update when the FP32 residual fell by this factor
                            since the last update; <= 0: 1e-4 */
  double inner_cutoff;   /* exponent cutoff of the FP32 operator;
                            <= 0: DS_DEFAULT_INNER_CUTOFF (pair kernels) or
                            DS_DEFAULT_STRUCTURED_INNER_CUTOFF (structured) */
  int verbose;
} ds_mixed_params;

/* The mixed form's outer residual r = b - A x on its own: the exact kernel
 * evaluated in float-float arithmetic (unevaluated pairs of FP32 numbers,
 * about 48 significant bits) on the FP32 pipe, agreeing with ds_A_residual
 * (FP64, DS_EVAL_EXACT) to about 1e-13 relative.  Needs DS_EVAL_EXACT with an
 * exponent cutoff of at most 60 (the mixed form falls back to the FP64
 * residual otherwise).  x, r in caller order (host). */
int ds_A_residual_ff(ds_operator* op, const double* x, double* r);

/* x: initial guess in, solution out (times w in the W form), caller order.
 * ``residual_norms`` (optional, max_iter + 1 doubles) receives the FP32
 * recurrence norms, replaced by the FP64 true norm at update iterations.
 * res->num_iters = FP32 iterations, res->n_outer = FP64 residual updates. */
int ds_solve_mixed(ds_operator* op, const ds_mixed_params* mp, double* x,
                   ds_pcg_result* res, double* residual_norms);
int ds_solve_mixed_dev(ds_operator* op, const ds_mixed_params* mp, double* x,
                       ds_pcg_result* res, double* residual_norms);

/* ---- batched chunks with several right-hand sides (no reference
 * counterpart) -------------------------------------------------------------
 * Many independent operators ("chunks", each the operator of
 * ds_operator_create over its own records) with n_rhs right-hand sides each
 * (e.g. noise realisations of the data), solved together by the
 * mixed-precision method of ds_solve_mixed with per-(chunk, RHS) CG scalars
 * and convergence.  Each (chunk, RHS) solve stands in for one
 * WFVector{SN,W}::solve_pcg call (lib/wf_vector.cc:114-121, 263-274) on that
 * chunk's pixels with that right-hand side, x0 = 0.  Exact kernel only. */
typedef struct ds_batch ds_batch;

typedef enum {
  DS_BATCH_AUTO = -1,       /* autotuner's choice (timed on first solve) */
  DS_BATCH_CUDA_CORE = 0,   /* FP32 FMA/MUFU matvec */
  DS_BATCH_TENSOR = 1       /* BF16 hi/lo tensor-core S-tile x RHS matvec */
} ds_batch_variant;

typedef struct {
  int n_chunks;
  int n_rhs;
  int n_total;             /* pixels over all chunks */
  int n_pad;               /* padded (tiled) pixels */
  int n_tiles;
  long long inner_tile_pairs;   /* FP32 operator (inner cutoff) */
  long long outer_tile_pairs;   /* FP64 residual operator (exact cutoff) */
  long long inner_evaluated;    /* (i, j) pairs per product, after sub-tile
                                   culling, FP32 operator */
  long long outer_evaluated;    /* the same, FP64 residual operator */
  int variant;             /* ds_batch_variant in use */
  int rhs_block;           /* RHS per work item of the CUDA-core matvec */
  int graph_replays;       /* iterations replayed by the last solve */
} ds_batch_info;

/* records: the chunks' records back to back (chunk c holds chunk_sizes[c]
 * records, 5 doubles each, layout by form as for ds_operator_create);
 * inner_cutoff as ds_mixed_params.inner_cutoff (<= 0: DS_DEFAULT_INNER_CUTOFF). */
int ds_batch_create(ds_context* ctx, int form, int n_chunks,
                    const int* chunk_sizes, const double* records,
                    const ds_kernel_params* kp, int n_rhs, double inner_cutoff,
                    ds_batch** out);
void ds_batch_destroy(ds_batch* batch);
int ds_batch_get_info(ds_batch* batch, ds_batch_info* info);

/* Selects the matvec variant (ds_batch_variant) and, for the CUDA-core
 * variant, the RHS block (1, 2, 4, 8, 16 or 32 dividing n_rhs; <= 0 keeps
 * the current one).  DS_BATCH_AUTO re-runs the autotuner now. */
int ds_batch_set_variant(ds_batch* batch, int variant, int rhs_block);

/* rhs: n_total x n_rhs doubles (record-major, RHS fastest: the value for
 * record k and right-hand side r at rhs[k * n_rhs + r]), in the form's
 * convention (d for SN, w d for W).  x: same shape, solution out (times w in
 * the W form).  Optional per-(chunk, RHS) outputs, n_chunks x n_rhs each
 * (index c * n_rhs + r): FP32 iterations, converged flags, FP64 residual
 * updates and the final FP64 relative residual |b - A x| / |b|.  *seconds:
 * device time of the iteration.  Returns DS_ERR_NOT_CONVERGED when any
 * (chunk, RHS) hit max_iter. */
int ds_batch_solve_mixed(ds_batch* batch, const ds_mixed_params* mp,
                         const double* rhs, double* x, int* iters,
                         int* converged, int* n_updates, double* rel_resid,
                         double* seconds);
/* The same with rhs and x in device memory. */
int ds_batch_solve_mixed_dev(ds_batch* batch, const ds_mixed_params* mp,
                             const double* rhs, double* x, int* iters,
                             int* converged, int* n_updates,
                             double* rel_resid, double* seconds);

/* One FP32 batched product q = A32 p over every chunk and RHS with the
 * current variant (p, q: n_total x n_rhs, caller order, device memory); for
 * testing the variants against each other and against the FP64 operator. */
int ds_batch_product_f32_dev(ds_batch* batch, const double* p, double* q);

/* ---- learned warm start + skewer-band preconditioner (no reference
 * counterpart) ------------------------------------------------------------
 * For skewer-structured pixel sets (n_skewers skewers of n_per pixels that
 * share one z grid; records skewer-contiguous, record s n_per + k is pixel
 * k of skewer s): a 4-layer message-passing network over each skewer and its
 * 8 nearest neighbour skewers (inputs z, noise, w d and the perpendicular
 * distances; hidden width `hidden`, BF16 weights with FP32 arithmetic)
 * predicts a warm start y0 of the W-form system (I + w S w) y = w d and per
 * skewer a lower-triangular band factor L (bandwidth `band` = 2; diagonal =
 * the Jacobi factor 1/sqrt(1 + w^2 var_s) times a learned factor in
 * [1/e, e]; sub-diagonals from row polynomials inside the stability
 * triangle) whose M^-1 = L L^T preconditions that skewer's block.  Trained
 * by its own forward / backward / Adam kernels on solutions of the solver;
 * the mixed-precision PCG then runs to the same tolerance from y0 with
 * M^-1 (Jacobi-PCG stays the fallback and the yardstick for its error). */
typedef struct ds_learned ds_learned;

/* kp: the kernel parameters of the systems it is trained for (exact). */
int ds_learned_create(ds_context* ctx, const ds_kernel_params* kp, int hidden,
                      int band, unsigned seed, ds_learned** out);
void ds_learned_destroy(ds_learned* net);
int ds_learned_num_params(ds_learned* net, long long* n);
/* Flat FP32 parameter vector (W_in, b_in, W_1, b_1, .., W_4, b_4, W_o, b_o;
 * W row-major [inputs x outputs]); host arrays of ds_learned_num_params. */
int ds_learned_get_params(ds_learned* net, float* params);
int ds_learned_set_params(ds_learned* net, const float* params);
/* Gradients of the last ds_learned_train_step_dev, same layout. */
int ds_learned_get_grads(ds_learned* net, float* grads);
/* Weight file: "DSLN", int32 version 1, hidden, band, int64 n, n FP32. */
int ds_learned_save(ds_learned* net, const char* path);
int ds_learned_load(ds_learned* net, const char* path);
/* records: device WPixel records (x, y, z, w, w d), n = n_skewers n_per.
 * y0 (device, n doubles, may be NULL): warm start in the operator's unscaled
 * variable y; L_rows (device, n x (band + 1) floats): row k of skewer s
 * holds L[k][k - m] at m = 0..band (zero outside the skewer). */
int ds_learned_forward_dev(ds_learned* net, int n_skewers, int n_per,
                           const double* records, double* y0, float* L_rows);
/* Inference GEMMs of ds_learned_forward_dev: 1 (default) runs the
 * message-passing layers on the tensor cores (TF32 activations, a ~1e-3
 * relative perturbation), 0 on the CUDA cores in FP32 like training. */
int ds_learned_set_inference(ds_learned* net, int tensor_cores);

/* One training step on one system: y_star (device) its solution y, probe
 * (device, n floats) the probe vector of the preconditioner loss.  losses[0]
 * = w_x sum (y0 - y*)^2 / sum y*^2, losses[1] = w_p sum |L L^T A_bb v - v|^2
 * / n over the skewers' own blocks A_bb.  update != 0 applies an Adam step
 * with learning rate lr. */
int ds_learned_train_step_dev(ds_learned* net, int n_skewers, int n_per,
                              const double* records, const double* y_star,
                              const float* probe, float lr, float w_x,
                              float w_p, int update, double* losses);
/* Installs (L_rows != NULL, host or device, copied) or removes (NULL) the
 * skewer-band preconditioner M^-1 = L L^T of the operator's mixed-precision
 * solves (ds_solve_mixed*); n_skewers n_per must equal the operator's n. */
int ds_operator_set_skewer_preconditioner(ds_operator* op, int n_skewers,
                                          int n_per, int band,
                                          const float* L_rows);

/* Installs (cluster > 0) or removes (cluster = 0) a cluster preconditioner
 * M^-1 = G G^T of the operator's mixed-precision solves (ds_solve_mixed*),
 * in place of Jacobi.  No reference counterpart (the reference's PCG is
 * Jacobi, lib/wf_vector.cc:42-49,185-194).  For skewer-structured pixel
 * sets (records skewer-contiguous, record s n_per + k is pixel k of skewer
 * s): the skewers are grouped into clusters of `cluster` neighbours
 * (cluster n_per <= 1024), a cluster's pixels are ordered by z, then by
 * skewer, and G is the factorized sparse approximate inverse of each
 * cluster's block of A with `band` sub-diagonals (0..24): column j of G
 * solves the (band + 1)-point system A[J, J] g = e_1, J = j .. j + band.
 * Built on the device in FP32 from the operator's coefficients; a column
 * whose small system is not positive definite in FP32 falls back to Jacobi,
 * and *n_fallback (may be NULL) counts them. */
int ds_operator_set_cluster_preconditioner(ds_operator* op, int n_skewers,
                                           int n_per, int cluster, int band,
                                           int* n_fallback);

/* Structured form of the exact-kernel operator (no reference counterpart;
 * the operator of lib/wf_vector.cc:196-251 evaluated in another order), for
 * skewer-structured pixel sets whose skewers all sample the same uniform z
 * grid (record s n_per + k = pixel k of skewer s; every skewer at one (x, y);
 * the same z values in every skewer).  The exact kernel then factorises into
 * a perpendicular factor per skewer pair times a Toeplitz z factor, so a
 * product costs one short z convolution per skewer and one FP64 FMA per
 * (skewer pair, pixel) instead of an exponential per pixel pair.  Installs
 * (n_skewers > 0) or removes (0) it; while installed the FP64-accurate outer
 * residual of the mixed-precision solves (ds_solve_mixed*) uses it.
 * DS_ERR_ARG when the records do not have that structure or the kernel is
 * the table kernel. */
int ds_operator_set_skewer_grid(ds_operator* op, int n_skewers, int n_per);
/* out = A v (residual = 0) or b - A v (residual != 0) with the structured
 * operator; v, out: n doubles in the caller's record order, device memory. */
int ds_operator_skewer_product_dev(ds_operator* op, int residual,
                                   const double* v, double* out);

/* ---- map projection ----------------------------------------------------- */
typedef struct ds_map ds_map;

/* A map grid or point set (init_uniform_map_coords output or any Point
 * array, lib/util.h:16, lib/map.h:41-44), copied to the device (DS_ERR_ARG
 * for a non-finite coordinate); sorted and tiled there by the first product
 * that needs it (the structured column-grid map does not) and reused by
 * every product with it. */
int ds_map_create(ds_context* ctx, int n_map, const double* map_points,
                  ds_map** out);
void ds_map_destroy(ds_map* map);

/* smp_product (lib/map.cc:20-43): m_i = sum_j S(map_i, pix_j) x_j with the
 * operator's pixels and kernel; x in the operator's record order. */
int ds_map_product(ds_map* map, ds_operator* op, const double* x, double* m);
int ds_map_product_dev(ds_map* map, ds_operator* op, const double* x,
                       double* m);

/* smp_product (lib/map.cc:20-43) of the mixed-precision form (no reference
 * counterpart for the FP32 evaluation): FP32 evaluation of the exact
 * kernel (MUFU ex2), FP32 sums per column tile, FP64 accumulation across
 * tiles; pairs beyond ``cutoff`` (exponent; <= 0: 30) are skipped.  Map
 * error against the FP64 product is about 1e-7 relative.  When the map was
 * declared a column grid (ds_map_set_column_grid) and the operator has a
 * skewer grid (ds_operator_set_skewer_grid), the product is instead the
 * structured FP64 one (per map column and skewer: perpendicular factor x
 * z-convolved solution), exact to rounding within the same cutoff. */
int ds_map_product_f32(ds_map* map, ds_operator* op, double cutoff,
                       const double* x, double* m);
int ds_map_product_f32_dev(ds_map* map, ds_operator* op, double cutoff,
                           const double* x, double* m);

/* Declares the map points a column grid (no reference counterpart; the
 * layout of init_uniform_map_coords, lib/util.cc:25-46): point c nz + j at
 * column c's (x, y) and at the j-th z value of column 0, for n_columns
 * columns of nz points.  0 columns removes the declaration.  DS_ERR_ARG when
 * the points do not have that layout.  Used by ds_map_product_f32* with an
 * operator that has a skewer grid; the z values of the map and of the
 * pixels must give at most 32 distinct distances within the cutoff. */
int ds_map_set_column_grid(ds_map* map, int n_columns, int nz);

/* One-shot smp_product with the reference's argument list (lib/map.h:41-44):
 * pixel and map points as Point arrays, x in pixel order; host arrays. */
int ds_smp_product(ds_context* ctx, int n_pix, const double* pixel_points,
                   int n_map, const double* map_points,
                   const ds_kernel_params* kp, const double* x, double* m);

/* sigma_m_noise_dom (lib/map_covar.cc:11-38): sigma_m_i = sum_j S_ij^2 / N_j
 * over NPixel records. */
int ds_sigma_m_noise_dom(ds_context* ctx, int n_pix, const double* npixels,
                         int n_map, const double* map_points,
                         const ds_kernel_params* kp, double* sigma_m);

#ifdef __cplusplus
}
#endif
#endif /* DS_GB300_H */
