/*
 * jrc_oracle: CPU restatement (plain C, FP64) of the reference JURASSIC
 * forward model, finite-difference Jacobian and optimal-estimation retrieval.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA library is
 * compared against (tests, smoke check) and the "port" CPU baseline that the
 * benchmark times; the product never links it.  Every function cites the
 * reference lines (src/jurassic.c, src/retrieval.c) whose behaviour it
 * restates.  It holds no global state: everything lives in a context.
 *
 * Parity pin: oracle/_ref (the reference compiled from its own sources) on
 * identical inputs, plus the reference test fixtures (the limb and nadir rad.org
 * tangent points); see tests/test_oracle_pin.py.
 */
#ifndef JRC_ORACLE_H
#define JRC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct jrc_ctx jrc_ctx;

/* Control parameters (the subset of ctl_t, jurassic.h:541-675, that the
   forward model, Jacobian and retrieval read).  Arrays are copied. */
typedef struct {
  int ng, nd, nw, ncl, nsf;
  const int *emitter_kind;  /* [ng]: 1 = CO2, 2 = H2O, 0 = other */
  const double *nu;         /* [nd] */
  const int *window;        /* [nd] */
  const double *clnu;       /* [ncl] */
  const double *sfnu;       /* [nsf] */
  int sftype;
  double sfsza;
  double hydz;
  int ctm_co2, ctm_h2o, ctm_n2, ctm_o2;
  int refrac;
  double rayds, raydz;
  int formod;               /* 0 = CGA, 1 = EGA */
  int write_bbt;
  double retp_zmin, retp_zmax, rett_zmin, rett_zmax;
  const double *retq_zmin, *retq_zmax; /* [ng] */
  const double *retk_zmin, *retk_zmax; /* [nw] */
  int ret_clz, ret_cldz, ret_clk, ret_sfz, ret_sfp, ret_sft, ret_sfeps;
  int nlos_max;             /* LOS capacity (reference NLOS, jurassic.h:403) */
} jrc_ctl;

/* Table capacities: pressures, temperatures, column densities per row. */
jrc_ctx *jrc_create(const jrc_ctl *ctl, int tbl_np, int tbl_nt, int tbl_nu);
void jrc_destroy(jrc_ctx *c);
const char *jrc_error(const jrc_ctx *c);

/* One (channel, emitter) table in dense form: p[np], nt[np], t[np][tbl_nt],
   nu[np][tbl_nt], u/eps[np][tbl_nt][tbl_nu].  np < 0 marks a missing table. */
int jrc_set_table(jrc_ctx *c, int id, int ig, int np, const double *p,
                  const int *nt, const double *t, const int *nu,
                  const float *u, const float *eps);

/* Source-function table of one channel from its filter function
   (init_srcfunc, jurassic.c:3631-3681). */
int jrc_init_srcfunc(jrc_ctx *c, int id, int n, const double *fnu,
                     const double *f);
/* Copy out the source-function table: st[1200], sr[1200][nd]. */
void jrc_get_srcfunc(const jrc_ctx *c, double *st, double *sr);

/* Continuum coefficient tables, float64 in the order of continua.bin. */
int jrc_set_continua(jrc_ctx *c, const double *blob, long n);

/* Atmosphere: np levels; q[ng][np]; k[nw][np];
   scal = {clz, cldz, clk[ncl], sfz, sfp, sft, sfeps[nsf]}.
   Observation: nr rays; geo[7][nr] = time obsz obslon obslat vpz vplon vplat;
   rad[nd][nr] in = mask (NaN = masked), out = radiance or BT;
   tau[nd][nr] out; tp[3][nr] out = tangent point z lon lat. */
typedef struct {
  int np;
  const double *time, *z, *lon, *lat;
  double *p, *t, *q, *k, *scal;
} jrc_atm;

typedef struct {
  int nr;
  const double *geo;
  double *rad, *tau, *tp;
} jrc_obs;

int jrc_formod(jrc_ctx *c, jrc_atm *atm, jrc_obs *obs);

/* Batched forward model over independent observations with OpenMP
   (nthreads <= 0: all).  lev_off[nobs+1], ray_off[nobs+1] index packed
   level and ray arrays; scal is [nobs][nscal]. */
int jrc_formod_batch(jrc_ctx *c, int nobs, const int *lev_off,
                     const double *time, const double *z, const double *lon,
                     const double *lat, double *p, double *t, double *q,
                     double *k, double *scal, const int *ray_off,
                     const double *geo, double *rad, double *tau, double *tp,
                     int nthreads);

/* LOS of ray ir: rows of 7 + 5*ng + 2*nd doubles (same layout as
   oracle/ref_harness.c jref_raytrace).  Returns number of points or < 0. */
int jrc_raytrace(jrc_ctx *c, const jrc_atm *atm, jrc_obs *obs, int ir,
                 int maxpts, double *out);

/* Sizes of state and measurement vectors (atm2x / obs2y). */
int jrc_sizes(const jrc_ctx *c, const jrc_atm *atm, const jrc_obs *obs,
              int *m, int *n);
int jrc_atm2x(const jrc_ctx *c, const jrc_atm *atm, double *x, int *iqa,
              int *ipa);

/* Field of view (formod_fov, jurassic.c:3121-3192): n samples of (dz, w)
   as read by read_shape from the FOV file; n = 0 switches it off. */
int jrc_set_fov(jrc_ctx *c, int n, const double *dz, const double *w);

/* Finite-difference Jacobian (kernel, jurassic.c:4004-4099): kmat[m][n]. */
int jrc_kernel(jrc_ctx *c, jrc_atm *atm, jrc_obs *obs, double *kmat,
               int nthreads);

/* Retrieval settings (ret_t, retrieval.c:32-112). */
typedef struct {
  int kernel_recomp, conv_itmax, err_ana;
  double conv_dmin;
  const double *err_formod, *err_noise;   /* [nd] */
  double err_press, err_press_cz, err_press_ch;
  double err_temp, err_temp_cz, err_temp_ch;
  const double *err_q, *err_q_cz, *err_q_ch;  /* [ng] */
  const double *err_k, *err_k_cz, *err_k_ch;  /* [nw] */
  double err_clz, err_cldz;
  const double *err_clk;                   /* [ncl] */
  double err_sfz, err_sfp, err_sft;
  const double *err_sfeps;                 /* [nsf] */
} jrc_ret;

/* Optimal estimation (optimal_estimation, retrieval.c:448-749).
   atm_apr is the a-priori (unchanged); obs_meas holds the measurement.
   Outputs: x_final[n], y_final[m], cov[n][n] (if err_ana), costs[] with
   chi^2/m per iteration (incl. iteration 0); info = {n, m, ncost, iters}. */
int jrc_retrieval(jrc_ctx *c, const jrc_ret *ret, const jrc_atm *atm_apr,
                  const jrc_obs *obs_meas, double *x_final, double *y_final,
                  double *cov, double *costs, int maxcost, int *info,
                  int nthreads);

/* Error analysis outputs (retrieval.c:668-726), any pointer may be NULL:
   gain[n][m], avk[n][n], standard deviations err_total/err_noise/err_formod[n]
   and analyze_avk's cont/res[n], all in state-vector order. */
typedef struct {
  double *gain, *avk, *err_total, *err_noise, *err_formod, *cont, *res;
} jrc_ana;

/* jrc_retrieval plus the error analysis (needs err_ana and cov != NULL). */
int jrc_retrieval_ex(jrc_ctx *c, const jrc_ret *ret, const jrc_atm *atm_apr,
                     const jrc_obs *obs_meas, double *x_final, double *y_final,
                     double *cov, double *costs, int maxcost, int *info,
                     int nthreads, jrc_ana *ana);

/* matrix_invert (retrieval.c:373-399) of one n x n row-major matrix in
   place: the reciprocal diagonal if every element right of the diagonal is
   zero, else the Cholesky inverse (symmetrised).  Returns -1 when a is not
   positive definite (a is then partly factored), else 0. */
int jrc_matrix_invert(double *a, int n);

#ifdef __cplusplus
}
#endif
#endif
