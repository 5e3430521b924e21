/*
 * libjurassic_gb300 -- C ABI of the GB300 JURASSIC forward model.
 *
 * Plain C: opaque context handle, plain pointers and sizes, int status
 * codes (JGB_OK == 0) instead of the reference's exit() on error
 * (ERRMSG, jurassic.h:237-241).  All array arguments are host pointers
 * unless a function name ends in _dev (device pointers, inputs already
 * resident in GPU memory).
 *
 * Array layouts follow the reference structs with runtime sizes:
 *   channel-major results rad/tau [nd][nray] (obs_t, jurassic.h:766-772),
 *   emitter-major volume mixing ratios q [ng][nlev] (atm_t, jurassic.h:518).
 *
 * Threading: a context owns one CUDA stream, and every entry point that takes
 * a context (or an engine of it) holds the context's lock while it runs, so
 * host threads may share a context: their calls run one after another, as
 * the reference's kernel() calls formod from OpenMP threads
 * (jurassic.c:4036).  Contexts are independent; one context per thread runs
 * calls side by side.  jgb_last_error gives the message of the last failed
 * call on the context, from whichever thread.
 */
#ifndef JURASSIC_GB300_H
#define JURASSIC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define JGB_OK 0
#define JGB_ERR_ARG 1          /* invalid argument or size */
#define JGB_ERR_CUDA 2         /* CUDA runtime failure */
#define JGB_ERR_STATE 3        /* tables or source function not set */
#define JGB_ERR_LOS 4          /* too many LOS points (jurassic.c:4335) */
#define JGB_ERR_SURFACE 5      /* observer below surface (jurassic.c:4238) */
#define JGB_ERR_UNSUPPORTED 6  /* option outside the device path (e.g. RFM) */
#define JGB_ERR_IO 7           /* file could not be read */
#define JGB_ERR_NUMERIC 8      /* matrix not positive definite */

#define JGB_FP64 0   /* plain FP64: rounding-level agreement with the reference */
#define JGB_MIXED 1  /* FP32 path loop with compensated sums (<= 10 mK BT) */

typedef struct jgb_ctx jgb_ctx;

/* Forward-model control parameters: the fields of ctl_t (jurassic.h:541-675)
   that the forward model, Jacobian and retrieval read. */
typedef struct {
  int ng;                        /* emitters */
  const char *const *emitter;    /* [ng] names; "CO2"/"H2O" enable continua */
  int nd;                        /* channels */
  const double *nu;              /* [nd] centroid wavenumbers [cm^-1] */
  int nw;                        /* spectral windows */
  const int *window;             /* [nd] window of each channel */
  int ncl;                       /* cloud spectral grid points */
  const double *clnu;            /* [ncl] */
  int nsf;                       /* surface spectral grid points */
  const double *sfnu;            /* [nsf] */
  int sftype;                    /* 0 none, 1 emission, 2 +downward, 3 +solar */
  double sfsza;                  /* solar zenith angle, <0 = computed */
  double hydz;                   /* hydrostatic reference height, <0 = off */
  int ctm_co2, ctm_h2o, ctm_n2, ctm_o2;  /* continua switches */
  int refrac;                    /* refraction on/off */
  double rayds, raydz;           /* ray-tracing step controls [km] */
  int formod;                    /* 0 = CGA, 1 = EGA */
  int write_bbt;                 /* 1 = results as brightness temperature */
  double retp_zmin, retp_zmax;   /* state-vector windows (atm2x) */
  double rett_zmin, rett_zmax;
  const double *retq_zmin, *retq_zmax;  /* [ng] */
  const double *retk_zmin, *retk_zmax;  /* [nw] */
  int ret_clz, ret_cldz, ret_clk, ret_sfz, ret_sfp, ret_sft, ret_sfeps;
  int nlos_max;                  /* LOS points per ray (reference NLOS); 0 = 4096 */
} jgb_ctl;

/* A batch of independent observations, each with its own atmosphere
   (levels lev_off[i]..lev_off[i+1]-1) and rays (ray_off[i]..ray_off[i+1]-1).
   One observation is the reference's (atm_t, obs_t) pair of formod(). */
typedef struct {
  int nobs;
  const int *lev_off;            /* [nobs+1] */
  const double *time, *z, *lon, *lat;  /* [nlev] */
  double *p;                     /* [nlev]; rewritten when hydz >= 0 */
  const double *t;               /* [nlev] */
  const double *q;               /* [ng][nlev] */
  const double *k;               /* [nw][nlev] */
  const double *scal;            /* [nobs][5+ncl+nsf]: clz cldz clk[] sfz sfp sft sfeps[] */
  const int *ray_off;            /* [nobs+1] */
  const double *geo;             /* [7][nray]: time obsz obslon obslat vpz vplon vplat */
  double *rad;                   /* [nd][nray] in: NaN = masked channel; out: radiance/BT */
  double *tau;                   /* [nd][nray] out: path transmittance */
  double *tp;                    /* [3][nray] out: tangent point z lon lat */
} jgb_batch;

/* Device times [ms] of the last forward call, measured with CUDA events on
   the context stream. */
typedef struct {
  double h2d_ms, hydro_ms, trace_ms, pack_ms, path_ms, d2h_ms, total_ms;
  long long los_points;          /* LOS points of the batch */
  int path_launches;             /* kernels launched by the last call */
  int path_variant;              /* mixed path kernel variant chosen by the autotuner:
                                    0-13: register cap (path_variant % 7) and block
                                    shape (path_variant / 7: 0 = 4 channels of one
                                    tile, 1 = one channel of 4 tiles); 14, 15: one
                                    channel of 8 tiles (256 threads), at most 64 or
                                    51 registers */
  float tune_ms[16];             /* autotuner timings of the variants [ms] */
  int trace_passes;              /* ray-tracing passes over the batch: 1 = one
                                    pass, 2 = count + fill, 3 = a capacity
                                    bound was exceeded and the rays were
                                    counted */
  double resume_skip;            /* share of the perturbed rays' LOS points
                                    taken from their bases (resumed
                                    Jacobian chunks; 0 otherwise) */
} jgb_stats;

/* Context: replaces the process-global table state initialised by the first
   formod_pencil call (jurassic.c:3202-3217). */
int jgb_create(const jgb_ctl *ctl, int device, jgb_ctx **out);
/* Frees the context's device memory, and that of the engines made from it
   and still open: their handles then accept only jgb_engine_destroy (every
   other engine call returns JGB_ERR_STATE). */
void jgb_destroy(jgb_ctx *ctx);
const char *jgb_last_error(const jgb_ctx *ctx);

/* Emissivity tables (tbl_t, jurassic.h:778-807; read_tbl, jurassic.c:4949).
   jgb_tables_init fixes the capacities; jgb_set_table uploads one
   (channel, emitter) table whose arrays have the layout of tbl_t rows:
   p[np], nt[np], t[np][tt_cap], nu[np][tt_cap], u/eps[np][tt_cap][tu_cap]. */
int jgb_tables_init(jgb_ctx *ctx, int tp, int tt, int tu);
int jgb_set_table(jgb_ctx *ctx, int id, int ig, int np, const double *p, const int *nt,
                  const double *t, const int *nu, const float *u, const float *eps,
                  int tt_cap, int tu_cap);

/* Table files of the reference (read_tbl, jurassic.c:4949-5110; write_tbl,
   jurassic.c:5810-5892): tblfmt 1 = ASCII lines "p T u eps", 2 = binary.
   jgb_read_tables reads, for every channel id and emitter ig of the context,
   the file "<tblbase>_<nu[id] as %.4f>_<emitter[ig]>.tab" (.bin for tblfmt
   2) on the host and uploads it with jgb_set_table; jgb_tables_init must
   have set capacities that hold the tables (JGB_ERR_ARG otherwise).  A
   missing file leaves that table empty, as the reference does (it warns);
   an unreadable or truncated one returns JGB_ERR_IO.
   jgb_read_table_file / jgb_write_table_file read or write one file into or
   from caller arrays with the row layout of jgb_set_table (capacities tp or
   np, tt, tu); no device work.  Reading one format and writing the other
   converts a table (the reference's tblfmt tool). */
int jgb_read_tables(jgb_ctx *ctx, const char *tblbase, int tblfmt);
int jgb_read_table_file(const char *path, int tblfmt, int tp, int tt, int tu, int *np_out,
                        double *p, int *nt, double *t, int *nu, float *u, float *eps);
int jgb_write_table_file(const char *path, int tblfmt, int np, const double *p, const int *nt,
                         const double *t, const int *nu, const float *u, const float *eps,
                         int tt_cap, int tu_cap);

/* Field of view (formod_fov, jurassic.c:3121-3192; FOV control parameter,
   read_shape of the FOV file): n samples of altitude offset dz [km] and
   weight w.  Every forward model of the context then convolves the pencil
   beams of the rays within +-5 of each ray (same observation, same time)
   over view-point altitude before BT conversion and masking.  n = 0 turns it
   off.  Not available in jgb_formod_batch_dev_noalloc. */
int jgb_set_fov(jgb_ctx *ctx, int n, const double *dz, const double *w);

/* Mixed-precision ray tracing of a batch larger than 2^23 / NLOS rays runs
   in one pass into per-ray capacities from a geometric bound of the LOS
   points (a ray that outgrows its capacity makes the batch count its rays
   first, as FP64 always does).  scale multiplies the bound (memory against
   the chance of a second pass); 0 always counts first.  Default 1.  The
   results do not depend on it. */
int jgb_set_los_bound_scale(jgb_ctx *ctx, double scale);

/* Mixed-precision path loop of a batch too small to fill the device (at most
   32 x SMs warps of tile x channel x emitter): split over the emitters, one
   warp per (tile, channel, emitter) for the emitters' path states, then one
   per (tile, channel) for their combination and the radiance.  mode -1 (the
   default) decides by that size, 0 never splits, 1 always does.  The results
   do not depend on it. */
int jgb_set_path_split(jgb_ctx *ctx, int mode);

/* Mixed-precision finite-difference Jacobians: a perturbation of a level
   value leaves the line of sight and the path state unchanged until the ray
   comes within half a step of the neighbouring levels, so the perturbed
   path restarts from its unperturbed base's saved state there (exact; not
   with hydrostatic pressures, a field of view or surface reflection).  The
   bases run first and the lanes of a warp walk the union of their ranges,
   so it pays on large batches: mode 1 (default) resumes a Jacobian chunk
   when the estimated schedule of its tiles is shorter, 2 always, 0 never.
   A perturbation of one emitter's mixing ratio (or of an extinction) also
   leaves the other emitters' path states equal to the base's: resumed
   chunks then take those emitters' segment emissivities from the base's
   walk and compute only the perturbed one, where at least 30 % of the
   perturbed lookups can be shared (mode 3: always resume and always share).
   In EGA, modes 2 and 3 also trace the perturbed rays from their bases'
   walks (a perturbed mixing ratio or extinction takes the base's geometry,
   a perturbed temperature walks on from the base's state); mode 1 does so
   only for chunks of at least four waves of the trace kernel.
   The results do not depend on it. */
int jgb_set_fd_resume(jgb_ctx *ctx, int mode);

/* Source function of channel id from its filter function
   (init_srcfunc, jurassic.c:3631-3681), computed on the device. */
int jgb_set_filter(jgb_ctx *ctx, int id, int n, const double *fnu, const double *f);
/* Upload / read back a source-function table sr[1200][nd]. */
int jgb_set_srcfunc(jgb_ctx *ctx, const double *sr);
int jgb_get_srcfunc(jgb_ctx *ctx, double *st, double *sr);

/* Forward model of one observation (formod, jurassic.c:3026-3071):
   atmosphere arrays of np levels, nr rays; same layouts as jgb_batch. */
int jgb_formod(jgb_ctx *ctx, int np, const double *time, const double *z, const double *lon,
               const double *lat, double *p, const double *t, const double *q,
               const double *k, const double *scal, int nr, const double *geo, double *rad,
               double *tau, double *tp, int precision);

/* Batched forward model of many observations: the seam of the reference's
   external GPU library, jur_unified_formod_multiple_packages (formod.c:72-73).
   Host buffers; copies are part of the call. */
int jgb_formod_batch(jgb_ctx *ctx, const jgb_batch *b, int precision);
/* Same with every jgb_batch pointer a device pointer. */
int jgb_formod_batch_dev(jgb_ctx *ctx, const jgb_batch *b, int precision);

/* Finite-difference Jacobian of every observation of a batch (kernel,
   jurassic.c:4004-4099).  jgb_kernel_sizes gives per observation the
   measurement size m (finite rad entries, obs2y order: ray-major, then
   channel) and the state size n (atm2x order, jurassic.c:29-83, from the
   RET* windows of the control set).  jgb_kernel_batch writes K_i (m_i x n_i,
   row-major) of observation i at kmat + sum_{j<i} m_j n_j, and returns the
   unperturbed forward model in b->rad/tau/tp (and the hydrostatic p) like
   jgb_formod_batch.  All n_i perturbed forward models of a chunk of
   observations run as one batched launch sequence.  Host buffers. */
int jgb_kernel_sizes(jgb_ctx *ctx, const jgb_batch *b, int *m, int *n);
int jgb_kernel_batch(jgb_ctx *ctx, const jgb_batch *b, double *kmat, int precision);

/* Normal-equation products of the retrieval for nret retrievals of sizes
   m[i] x n[i] (matrix_product, retrieval.c:403-444, and the gradient
   K^T W dy of retrieval.c:573-577):  A_i = K_i^T W_i K_i (n_i x n_i) and
   b_i = K_i^T W_i dy_i with W_i = diag(w_i^2), w = 1/sigma_eps.
   K, w, dy, A, b are concatenations of the per-retrieval arrays (K_i
   row-major).  JGB_MIXED: 3xTF32 on the tensor cores (FP32-level
   accuracy); JGB_FP64: FP64 in the reference's operation order. */
int jgb_normal_equations(jgb_ctx *ctx, int nret, const int *m, const int *n, const double *K,
                         const double *w, const double *dy, double *A, double *b,
                         int precision);

/* jgb_normal_equations on device buffers (K, w, dy, A, b device pointers;
   m, n host arrays; at most 65535 problems).  Returns when done; with
   kernel_ms != NULL the products are computed twice and *kernel_ms is the
   CUDA-event time of the second launch (descriptor upload excluded). */
int jgb_normal_equations_dev(jgb_ctx *ctx, int nret, const int *m, const int *n,
                             const double *K, const double *w, const double *dy, double *A,
                             double *b, int precision, float *kernel_ms);

/* Inverse of nret symmetric positive-definite matrices in place
   (matrix_invert, retrieval.c:373-399), FP64: a matrix with every element
   right of the diagonal equal to 0 by its reciprocal diagonal, any other by
   Cholesky decomposition and inverse (gsl_linalg_cholesky_decomp /
   gsl_linalg_cholesky_invert), symmetrised.  A holds the concatenated
   n[i] x n[i] row-major matrices.  status (host, nret entries, may be NULL)
   gets 1 for a matrix that is not positive definite, which is then left as
   it was (the reference aborts there), else 0.  At most 65535 matrices. */
int jgb_matrix_invert(jgb_ctx *ctx, int nret, const int *n, double *A, int *status);
/* The same on a device buffer A; with kernel_ms != NULL, *kernel_ms is the
   CUDA-event time of the kernels (descriptor upload excluded). */
int jgb_matrix_invert_dev(jgb_ctx *ctx, int nret, const int *n, double *A, int *status,
                          float *kernel_ms);

/* Emitter contributions (TASK c, formod.c:200-249) of every observation of a
   host batch: continua off; variant g < ng keeps only emitter g (all other
   mixing ratios and all extinction zero), variant ng ("EXTINCT") has all
   mixing ratios zero and the extinction kept.  The batch holds the
   atmosphere as after formod (pressures after hydrostatic equilibrium) and
   in rad the mask (NaN = not computed).
   Out: rad[ng+1][nd][nray], tau[ng+1][nd][nray] (tau may be NULL). */
int jgb_formod_contrib(jgb_ctx *ctx, const jgb_batch *b, double *rad, double *tau,
                       int precision);

/* Retrieval settings (ret_t, retrieval.c:32-112; read_ret, 753-804). */
typedef struct {
  int kernel_recomp, conv_itmax, err_ana;
  double conv_dmin;
  const double *err_formod, *err_noise;       /* [nd]: percent, radiance units */
  double err_press, err_press_cz, err_press_ch;
  double err_temp, err_temp_cz, err_temp_ch;
  const double *err_q, *err_q_cz, *err_q_ch;  /* [ng] */
  const double *err_k, *err_k_cz, *err_k_ch;  /* [nw] */
  double err_clz, err_cldz;
  const double *err_clk;                      /* [ncl] */
  double err_sfz, err_sfp, err_sft;
  const double *err_sfeps;                    /* [nsf] */
} jgb_ret;

/* Optimal-estimation retrievals (optimal_estimation, retrieval.c:448-749)
   of every observation of a batch (all submitted at once to a retrieval
   engine and stepped until done).
   In:  b holds the a-priori atmospheres and in b->rad the measurement
        (NaN = channel not used).
   Out: x: final state vectors (atm2x of the final atmosphere, sizes n_i of
        jgb_kernel_sizes, concatenated); b->rad/tau/tp: forward model of the
        final iterate, b->p its pressure; cov (optional, err_ana): retrieval
        covariances n_i x n_i concatenated; costs (optional):
        [nobs][conv_itmax+1] chi^2/m after each iteration (NaN after
        convergence); iters (optional): iterations done.
   JGB_MIXED: FP32 forward model and Jacobian, 3xTF32 normal equations;
   FP64 Cholesky, LM step, cost and convergence test in both modes. */
int jgb_retrieve_batch(jgb_ctx *ctx, const jgb_ret *ret, const jgb_batch *b, double *x,
                       double *cov, double *costs, int *iters, int precision);

/* ---------------------------------------------------------------------------
   Retrieval engine (continuous batching).  Replaces the reference's
   one-retrieval-per-process driver (retrieval.c:148-245 main loop over
   directories calling optimal_estimation, 448-749) by a queue of independent
   requests served on one device: requests are admitted while at most
   max_active are in flight and their working set fits mem_budget bytes
   (0 = unlimited; a request larger than the budget is admitted alone when
   nothing else runs); every admitted request keeps its atmosphere, Jacobian
   and LM state resident on the device.  jgb_engine_step advances every
   admitted request by one LM iteration (newly admitted ones are first
   initialised: a-priori forward model, S_a^-1, cost, Jacobian).  A request's
   results do not depend on which other requests share its steps.  Peak
   device memory is about twice the working set (it is rebuilt into a
   second buffer when requests join or leave) plus the forward-model scratch
   of the context.  The engine uses its context's stream, and its calls hold
   the context's lock like every other call on the context. */
typedef struct jgb_engine jgb_engine;

typedef struct {
  unsigned long long submitted, finished, failed, steps, rebuilds, forward_calls, lm_trials,
      jacobians;
  double step_ms;              /* host wall time spent in jgb_engine_step */
  /* of which (stream synchronised at each phase end): working-set rebuilds,
     initialisation forward models + S_a, Jacobians, normal equations +
     gradient, damped trials (Cholesky + forward model + cost), results */
  double rebuild_ms, init_ms, jacobian_ms, normal_ms, trial_ms, finish_ms;
  /* of trial_ms: forward-model calls (host wall time), and their ray-tracing
     and path-kernel device times (CUDA events) */
  double trial_fwd_ms, trial_trace_ms, trial_path_ms;
  int active, queued, done;    /* requests in flight, waiting, finished and not yet collected */
  unsigned long long used_bytes;  /* working-set bytes of the active requests */
} jgb_engine_stats;

/* Results of one request; every pointer may be NULL (not copied).
   Sizes: n state elements, m measurement elements (jgb_engine_sizes).
   x[n] final state (atm2x order); costs[conv_itmax+1] chi^2/m per iteration
   (NaN after convergence); rad/tau[nd][nr], tp[3][nr], p[np] forward model
   and pressures of the final iterate.  With err_ana (has_err_ana = 1):
   cov[n*n] retrieval covariance, avk[n*n] averaging kernel, gain[n*m] (only
   if the engine keeps gains), err_total/err_noise/err_formod[n] standard
   deviations (write_stddev "total", "noise", "formod"), cont[n] and res[n]
   as written to atm_cont.tab and atm_res.tab by analyze_avk
   (retrieval.c:257-336), in state-vector order. */
typedef struct {
  double *x, *cov, *costs, *rad, *tau, *tp, *p;
  double *gain, *avk, *err_total, *err_noise, *err_formod, *cont, *res;
  int iters, status, has_err_ana;
} jgb_ret_out;

int jgb_engine_create(jgb_ctx *ctx, const jgb_ret *ret, int precision,
                      unsigned long long mem_budget, int max_active, int keep_gain,
                      jgb_engine **out);
/* Frees an engine (before or after its context). */
void jgb_engine_destroy(jgb_engine *e);
/* Queue every observation of a host batch (a-priori atmosphere, geometry and
   measurement in b->rad, NaN = not used) as one request; ids[nobs] out.
   Checks of set_cov_apr/set_cov_meas are made here. */
int jgb_engine_submit(jgb_engine *e, const jgb_batch *b, unsigned long long *ids);
/* Admission plus one LM iteration of every admitted request. */
int jgb_engine_step(jgb_engine *e, int *n_active, int *n_queued, int *n_done);
/* Ids of finished requests not collected yet (ascending, up to max). */
int jgb_engine_finished(jgb_engine *e, unsigned long long *ids, int max, int *count);
int jgb_engine_sizes(jgb_engine *e, unsigned long long id, int *n, int *m, int *np, int *nr);
/* Copy the results of a finished request and release it. */
int jgb_engine_result(jgb_engine *e, unsigned long long id, jgb_ret_out *out);
int jgb_engine_get_stats(const jgb_engine *e, jgb_engine_stats *out);

int jgb_get_stats(const jgb_ctx *ctx, jgb_stats *out);

/* State vector of one atmosphere of np levels in the order of the
   context's RET* windows (atm2x, jurassic.c:29-83: p, T, q per emitter, k
   per window on the levels inside each window, then the retrieved cloud and
   surface scalars), and back (x2atm, jurassic.c:5896-5946).  Arrays have
   the layouts of jgb_batch for one observation (q[ng][np], k[nw][np],
   scal[5+ncl+nsf]); an array whose elements are not retrieved may be NULL.
   jgb_atm2x sets *n (and writes x[n] when x is not NULL). */
int jgb_atm2x(jgb_ctx *ctx, int np, const double *z, const double *p, const double *t,
              const double *q, const double *k, const double *scal, double *x, int *n);
int jgb_x2atm(jgb_ctx *ctx, int np, const double *z, const double *x, double *p, double *t,
              double *q, double *k, double *scal);

/* Shape function file (read_shape, jurassic.c:4907-4945): filter functions
   "<tblbase>_<nu %.4f>.filt" and the field of view.  Lines of two numbers
   x y are read, other lines skipped; more than nmax points is JGB_ERR_ARG,
   a missing file or fewer than two points JGB_ERR_IO.  Host only. */
int jgb_read_shape(const char *path, int nmax, double *x, double *y, int *n);

/* Allocation-free FP64 forward model of a device-resident batch.  This entry
   point has no counterpart in the reference.  It is for callers that cannot
   allocate GPU memory while they run (a fixed memory budget handed over at
   start-up, an allocator owned by another runtime, sections where allocation
   is forbidden): all scratch comes from one 64 MiB device array, and no
   cudaMalloc/cudaFree or allocating library routine is called.  Same
   arguments and results as jgb_formod_batch_dev with JGB_FP64.
   - The array is part of the library's device code.  jgb_create loads it,
     with the kernels this entry point launches, onto the context's device
     and resolves its address there, so the calls themselves load and
     allocate nothing; it stays on every device where it was loaded until the
     process exits.
   - A batch whose rays and LOS points need more than 64 MiB of scratch is
     rejected with JGB_ERR_ARG (jgb_last_error names the bytes needed); a
     field of view is not available here (JGB_ERR_UNSUPPORTED).
   - All calls on a device share the array and it keeps the previous call's
     contents: calls on one context run one after another (the context's
     lock), but calls from different contexts on one device that overlap on
     the GPU race and must be serialised by the caller.
   - jgb_get_stats then reports the call's LOS points, kernel launches and
     total device time; its per-stage times are zero. */
int jgb_formod_batch_dev_noalloc(jgb_ctx *ctx, const jgb_batch *b);

/* Page-locked host memory for fast transfers (cudaHostAlloc). */
void *jgb_host_alloc(unsigned long long bytes);
void jgb_host_free(void *p);
/* Device memory for callers that stage inputs themselves. */
void *jgb_dev_alloc(unsigned long long bytes);
void jgb_dev_free(void *p);
int jgb_memcpy_h2d(void *dst, const void *src, unsigned long long bytes);
int jgb_memcpy_d2h(void *dst, const void *src, unsigned long long bytes);

/* Measurement helper (no reference counterpart): L2 read bandwidth of this
   GPU in GB/s, from passes sweeps over a device buffer of the given size
   (small enough to stay in L2) in one launch, loads that skip L1, best of
   5 launches timed with CUDA events.  Roofline denominator for the
   table-lookup loop, whose probes are served by L1 and L2. */
int jgb_measure_l2_read(unsigned long long bytes, int passes, double *gbs);

/* Self-test of the device-side bounded wait (the mbarrier wait of the
   tensor-core kernels, limited to about one second of the global timer):
   one thread waits for a barrier phase that completes at once (arrive = 1)
   or never (arrive = 0).  *timed_out = 1 when the wait gave up, *seconds =
   how long it waited.  The device stays usable either way. */
int jgb_selftest_bounded_wait(int device, int arrive, int *timed_out, double *seconds);

#ifdef __cplusplus
}
#endif
#endif
