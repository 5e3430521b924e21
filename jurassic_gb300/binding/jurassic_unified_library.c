/*
 * jurassic_unified_library.c -- binding of the reference code base to
 * libjurassic_gb300 (declarations and conventions in
 * jurassic_unified_library.h).
 *
 * The reference keeps every observation in fixed-size structs (atm_t,
 * obs_t: arrays of NP levels, ND x NR radiances); the library takes a batch
 * of observations as dense arrays with offsets (jgb_batch).  pack() and the
 * unpack helpers move between the two; every entry point here packs all of
 * its packages into ONE batch, so n packages cost one library call, not n.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "jurassic_unified_library.h"

static ctl_t g_ctl;
static jgb_ctx *g_ctx;
static int g_precision = JGB_MIXED;

#define JUR_CHECK(call)                                   \
  do {                                                    \
    if ((call) != JGB_OK) ERRMSG("%s", jgb_last_error(g_ctx)); \
  } while (0)

/* Dense copy of n packages (the jgb_batch layouts). */
typedef struct {
  jgb_batch b;
  int *lev_off, *ray_off;
  double *time, *z, *lon, *lat, *p, *t, *q, *k, *scal, *geo, *rad, *tau, *tp;
} packed_t;

static void *jur_alloc(size_t n) {
  void *p = calloc(n > 0 ? n : 1, 1);
  if (!p) ERRMSG("Out of memory!");
  return p;
}

static int nscal(void) { return 5 + g_ctl.ncl + g_ctl.nsf; }

/* atm[i] and obs[i] of n packages -> one dense batch; rad carries obs->rad
   (NaN = channel masked, or not measured). */
static void pack(const atm_t *atm, const obs_t *obs, int n, packed_t *P) {
  const int ng = g_ctl.ng, nw = g_ctl.nw, nd = g_ctl.nd, ns = nscal();
  memset(P, 0, sizeof *P);
  P->lev_off = jur_alloc(sizeof(int) * (size_t)(n + 1));
  P->ray_off = jur_alloc(sizeof(int) * (size_t)(n + 1));
  for (int i = 0; i < n; i++) {
    if (atm[i].np < 2 || atm[i].np > NP || obs[i].nr < 1 || obs[i].nr > NR)
      ERRMSG("Package %d: bad level or ray count!", i);
    P->lev_off[i + 1] = P->lev_off[i] + atm[i].np;
    P->ray_off[i + 1] = P->ray_off[i] + obs[i].nr;
  }
  const size_t nl = (size_t)P->lev_off[n], nr = (size_t)P->ray_off[n];
  P->time = jur_alloc(sizeof(double) * nl);
  P->z = jur_alloc(sizeof(double) * nl);
  P->lon = jur_alloc(sizeof(double) * nl);
  P->lat = jur_alloc(sizeof(double) * nl);
  P->p = jur_alloc(sizeof(double) * nl);
  P->t = jur_alloc(sizeof(double) * nl);
  P->q = jur_alloc(sizeof(double) * nl * (size_t)(ng > 0 ? ng : 1));
  P->k = jur_alloc(sizeof(double) * nl * (size_t)(nw > 0 ? nw : 1));
  P->scal = jur_alloc(sizeof(double) * (size_t)n * (size_t)ns);
  P->geo = jur_alloc(sizeof(double) * 7 * nr);
  P->rad = jur_alloc(sizeof(double) * (size_t)nd * nr);
  P->tau = jur_alloc(sizeof(double) * (size_t)nd * nr);
  P->tp = jur_alloc(sizeof(double) * 3 * nr);
  for (int i = 0; i < n; i++) {
    const atm_t *a = &atm[i];
    const obs_t *o = &obs[i];
    const size_t l0 = (size_t)P->lev_off[i], r0 = (size_t)P->ray_off[i];
    const size_t np = (size_t)a->np, nri = (size_t)o->nr;
    memcpy(P->time + l0, a->time, sizeof(double) * np);
    memcpy(P->z + l0, a->z, sizeof(double) * np);
    memcpy(P->lon + l0, a->lon, sizeof(double) * np);
    memcpy(P->lat + l0, a->lat, sizeof(double) * np);
    memcpy(P->p + l0, a->p, sizeof(double) * np);
    memcpy(P->t + l0, a->t, sizeof(double) * np);
    for (int ig = 0; ig < ng; ig++) memcpy(P->q + ig * nl + l0, a->q[ig], sizeof(double) * np);
    for (int iw = 0; iw < nw; iw++) memcpy(P->k + iw * nl + l0, a->k[iw], sizeof(double) * np);
    double *s = P->scal + (size_t)i * (size_t)ns;
    int j = 0;
    s[j++] = a->clz;
    s[j++] = a->cldz;
    for (int icl = 0; icl < g_ctl.ncl; icl++) s[j++] = a->clk[icl];
    s[j++] = a->sfz;
    s[j++] = a->sfp;
    s[j++] = a->sft;
    for (int isf = 0; isf < g_ctl.nsf; isf++) s[j++] = a->sfeps[isf];
    const double *rows[7] = {o->time, o->obsz, o->obslon, o->obslat, o->vpz, o->vplon, o->vplat};
    for (int g = 0; g < 7; g++) memcpy(P->geo + g * nr + r0, rows[g], sizeof(double) * nri);
    for (int id = 0; id < nd; id++) memcpy(P->rad + id * nr + r0, o->rad[id], sizeof(double) * nri);
  }
  jgb_batch *b = &P->b;
  b->nobs = n;
  b->lev_off = P->lev_off;
  b->time = P->time;
  b->z = P->z;
  b->lon = P->lon;
  b->lat = P->lat;
  b->p = P->p;
  b->t = P->t;
  b->q = P->q;
  b->k = P->k;
  b->scal = P->scal;
  b->ray_off = P->ray_off;
  b->geo = P->geo;
  b->rad = P->rad;
  b->tau = P->tau;
  b->tp = P->tp;
}

static void unpack_free(packed_t *P) {
  void *ptrs[] = {P->lev_off, P->ray_off, P->time, P->z, P->lon, P->lat, P->p, P->t, P->q,
                  P->k, P->scal, P->geo, P->rad, P->tau, P->tp};
  for (size_t i = 0; i < sizeof ptrs / sizeof ptrs[0]; i++) free(ptrs[i]);
  memset(P, 0, sizeof *P);
}

/* Forward-model results of package i back into obs (rad, tau, tangent
   points) and atm (pressures). */
static void unpack_forward(const packed_t *P, int i, atm_t *atm, obs_t *obs) {
  const size_t nr = (size_t)P->ray_off[P->b.nobs];
  const size_t r0 = (size_t)P->ray_off[i], nri = (size_t)obs->nr;
  for (int id = 0; id < g_ctl.nd; id++) {
    memcpy(obs->rad[id], P->rad + id * nr + r0, sizeof(double) * nri);
    memcpy(obs->tau[id], P->tau + id * nr + r0, sizeof(double) * nri);
  }
  memcpy(obs->tpz, P->tp + r0, sizeof(double) * nri);
  memcpy(obs->tplon, P->tp + nr + r0, sizeof(double) * nri);
  memcpy(obs->tplat, P->tp + 2 * nr + r0, sizeof(double) * nri);
  if (atm) memcpy(atm->p, P->p + P->lev_off[i], sizeof(double) * (size_t)atm->np);
}

void jur_unified_init_ctl(const ctl_t *ctl, int device, int precision) {
  static const char *names[NG];
  static double fx[NSHAPE], fy[NSHAPE];
  char fn[2 * LEN];
  int n;
  if (g_ctx) jur_unified_finalize();
  memcpy(&g_ctl, ctl, sizeof g_ctl);
  g_precision = precision == JGB_FP64 ? JGB_FP64 : JGB_MIXED;
  for (int ig = 0; ig < g_ctl.ng; ig++) names[ig] = g_ctl.emitter[ig];
  jgb_ctl c;
  memset(&c, 0, sizeof c);
  c.ng = g_ctl.ng;
  c.emitter = names;
  c.nd = g_ctl.nd;
  c.nu = g_ctl.nu;
  c.nw = g_ctl.nw;
  c.window = g_ctl.window;
  c.ncl = g_ctl.ncl;
  c.clnu = g_ctl.clnu;
  c.nsf = g_ctl.nsf;
  c.sfnu = g_ctl.sfnu;
  c.sftype = g_ctl.sftype;
  c.sfsza = g_ctl.sfsza;
  c.hydz = g_ctl.hydz;
  c.ctm_co2 = g_ctl.ctm_co2;
  c.ctm_h2o = g_ctl.ctm_h2o;
  c.ctm_n2 = g_ctl.ctm_n2;
  c.ctm_o2 = g_ctl.ctm_o2;
  c.refrac = g_ctl.refrac;
  c.rayds = g_ctl.rayds;
  c.raydz = g_ctl.raydz;
  c.formod = g_ctl.formod;
  c.write_bbt = g_ctl.write_bbt;
  c.retp_zmin = g_ctl.retp_zmin;
  c.retp_zmax = g_ctl.retp_zmax;
  c.rett_zmin = g_ctl.rett_zmin;
  c.rett_zmax = g_ctl.rett_zmax;
  c.retq_zmin = g_ctl.retq_zmin;
  c.retq_zmax = g_ctl.retq_zmax;
  c.retk_zmin = g_ctl.retk_zmin;
  c.retk_zmax = g_ctl.retk_zmax;
  c.ret_clz = g_ctl.ret_clz;
  c.ret_cldz = g_ctl.ret_cldz;
  c.ret_clk = g_ctl.ret_clk;
  c.ret_sfz = g_ctl.ret_sfz;
  c.ret_sfp = g_ctl.ret_sfp;
  c.ret_sft = g_ctl.ret_sft;
  c.ret_sfeps = g_ctl.ret_sfeps;
  c.nlos_max = NLOS;
  if (jgb_create(&c, device, &g_ctx) != JGB_OK) ERRMSG("Cannot create the GPU context!");
  /* tables: the library reads read_tbl's files itself */
  JUR_CHECK(jgb_tables_init(g_ctx, TBLNP, TBLNT, TBLNU));
  JUR_CHECK(jgb_read_tables(g_ctx, g_ctl.tblbase, g_ctl.tblfmt));
  /* source functions from the filter functions (init_srcfunc) */
  for (int id = 0; id < g_ctl.nd; id++) {
    snprintf(fn, sizeof fn, "%s_%.4f.filt", g_ctl.tblbase, g_ctl.nu[id]);
    if (jgb_read_shape(fn, NSHAPE, fx, fy, &n) != JGB_OK) ERRMSG("Cannot read filter %s!", fn);
    JUR_CHECK(jgb_set_filter(g_ctx, id, n, fx, fy));
  }
  /* field of view (read_shape of the FOV file, formod_fov) */
  if (g_ctl.fov[0] != '-') {
    if (jgb_read_shape(g_ctl.fov, NSHAPE, fx, fy, &n) != JGB_OK)
      ERRMSG("Cannot read FOV %s!", g_ctl.fov);
    JUR_CHECK(jgb_set_fov(g_ctx, n, fx, fy));
  }
}

void jur_unified_init(int argc, char *argv[]) {
  ctl_t *ctl = jur_alloc(sizeof(ctl_t));
  read_ctl(argc, argv, ctl);
  const int precision = (int) scan_ctl(argc, argv, "JGB_PRECISION", -1, "1", NULL);
  const int device = (int) scan_ctl(argc, argv, "JGB_DEVICE", -1, "0", NULL);
  jur_unified_init_ctl(ctl, device, precision);
  free(ctl);
}

jgb_ctx *jur_unified_context(void) { return g_ctx; }

void jur_unified_finalize(void) {
  if (g_ctx) jgb_destroy(g_ctx);
  g_ctx = NULL;
}

void jur_unified_formod_multiple_packages(atm_t *atm, obs_t *obs, int n, void *unused) {
  if (!g_ctx) ERRMSG("Call jur_unified_init first!");
  if (unused != NULL || n < 0) ERRMSG("Bad arguments!");
  if (n == 0) return;
  packed_t P;
  pack(atm, obs, n, &P);
  JUR_CHECK(jgb_formod_batch(g_ctx, &P.b, g_precision));
  for (int i = 0; i < n; i++) unpack_forward(&P, i, &atm[i], &obs[i]);
  unpack_free(&P);
}

void jur_unified_kernel_multiple_packages(atm_t *atm, obs_t *obs, int n, gsl_matrix **k) {
  if (!g_ctx) ERRMSG("Call jur_unified_init first!");
  if (n <= 0) return;
  packed_t P;
  pack(atm, obs, n, &P);
  int *m = jur_alloc(sizeof(int) * (size_t)n), *nn = jur_alloc(sizeof(int) * (size_t)n);
  JUR_CHECK(jgb_kernel_sizes(g_ctx, &P.b, m, nn));
  size_t tot = 0;
  for (int i = 0; i < n; i++) {
    if ((size_t)m[i] != k[i]->size1 || (size_t)nn[i] != k[i]->size2)
      ERRMSG("Package %d: kernel matrix is %zu x %zu, expected %d x %d!", i, k[i]->size1,
             k[i]->size2, m[i], nn[i]);
    tot += (size_t)m[i] * (size_t)nn[i];
  }
  double *K = jur_alloc(sizeof(double) * tot);
  JUR_CHECK(jgb_kernel_batch(g_ctx, &P.b, K, g_precision));
  size_t off = 0;
  for (int i = 0; i < n; i++) {
    for (int r = 0; r < m[i]; r++)   /* row-major with the caller's tda */
      memcpy(k[i]->data + (size_t)r * k[i]->tda, K + off + (size_t)r * (size_t)nn[i],
             sizeof(double) * (size_t)nn[i]);
    off += (size_t)m[i] * (size_t)nn[i];
    unpack_forward(&P, i, &atm[i], &obs[i]);
  }
  free(K);
  free(m);
  free(nn);
  unpack_free(&P);
}

void jur_unified_kernel(ctl_t *ctl, atm_t *atm, obs_t *obs, gsl_matrix *k) {
  if (ctl && (ctl->nd != g_ctl.nd || ctl->ng != g_ctl.ng))
    ERRMSG("Control set differs from the one given to jur_unified_init!");
  jur_unified_kernel_multiple_packages(atm, obs, 1, &k);
}

/* x2atm of x onto one atmosphere (the library restates the reference's
   element order from the context's RET* windows). */
static void state_to_atm(const double *x, atm_t *a) {
  const int np = a->np, ng = g_ctl.ng, nw = g_ctl.nw;
  double *q = jur_alloc(sizeof(double) * (size_t)np * (size_t)(ng > 0 ? ng : 1));
  double *k = jur_alloc(sizeof(double) * (size_t)np * (size_t)(nw > 0 ? nw : 1));
  double scal[5 + NCL + NSF];
  for (int ig = 0; ig < ng; ig++) memcpy(q + (size_t)ig * np, a->q[ig], sizeof(double) * np);
  for (int iw = 0; iw < nw; iw++) memcpy(k + (size_t)iw * np, a->k[iw], sizeof(double) * np);
  int j = 0;
  scal[j++] = a->clz;
  scal[j++] = a->cldz;
  for (int icl = 0; icl < g_ctl.ncl; icl++) scal[j++] = a->clk[icl];
  scal[j++] = a->sfz;
  scal[j++] = a->sfp;
  scal[j++] = a->sft;
  for (int isf = 0; isf < g_ctl.nsf; isf++) scal[j++] = a->sfeps[isf];
  JUR_CHECK(jgb_x2atm(g_ctx, np, a->z, x, a->p, a->t, q, k, scal));
  for (int ig = 0; ig < ng; ig++) memcpy(a->q[ig], q + (size_t)ig * np, sizeof(double) * np);
  for (int iw = 0; iw < nw; iw++) memcpy(a->k[iw], k + (size_t)iw * np, sizeof(double) * np);
  j = 0;
  a->clz = scal[j++];
  a->cldz = scal[j++];
  for (int icl = 0; icl < g_ctl.ncl; icl++) a->clk[icl] = scal[j++];
  a->sfz = scal[j++];
  a->sfp = scal[j++];
  a->sft = scal[j++];
  for (int isf = 0; isf < g_ctl.nsf; isf++) a->sfeps[isf] = scal[j++];
  free(q);
  free(k);
}

void jur_unified_optimal_estimation_multiple_packages(const jgb_ret *ret, obs_t *obs_meas,
                                                      obs_t *obs_i, atm_t *atm_apr,
                                                      atm_t *atm_i, int n, gsl_matrix **cov) {
  if (!g_ctx) ERRMSG("Call jur_unified_init first!");
  if (!ret || n <= 0) return;
  packed_t P;
  pack(atm_apr, obs_meas, n, &P);
  int *m = jur_alloc(sizeof(int) * (size_t)n), *nn = jur_alloc(sizeof(int) * (size_t)n);
  JUR_CHECK(jgb_kernel_sizes(g_ctx, &P.b, m, nn));
  size_t nx = 0, ncov = 0;
  for (int i = 0; i < n; i++) {
    nx += (size_t)nn[i];
    ncov += (size_t)nn[i] * (size_t)nn[i];
  }
  double *x = jur_alloc(sizeof(double) * nx);
  double *c = ret->err_ana ? jur_alloc(sizeof(double) * ncov) : NULL;
  JUR_CHECK(jgb_retrieve_batch(g_ctx, ret, &P.b, x, c, NULL, NULL, g_precision));
  size_t ox = 0, oc = 0;
  for (int i = 0; i < n; i++) {
    memcpy(&atm_i[i], &atm_apr[i], sizeof(atm_t));
    state_to_atm(x + ox, &atm_i[i]);
    memcpy(&obs_i[i], &obs_meas[i], sizeof(obs_t));
    unpack_forward(&P, i, &atm_i[i], &obs_i[i]);
    if (c && cov && cov[i]) {
      if (cov[i]->size1 != (size_t)nn[i] || cov[i]->size2 != (size_t)nn[i])
        ERRMSG("Package %d: covariance matrix is not %d x %d!", i, nn[i], nn[i]);
      for (int r = 0; r < nn[i]; r++)
        memcpy(cov[i]->data + (size_t)r * cov[i]->tda, c + oc + (size_t)r * (size_t)nn[i],
               sizeof(double) * (size_t)nn[i]);
    }
    ox += (size_t)nn[i];
    oc += (size_t)nn[i] * (size_t)nn[i];
  }
  free(x);
  free(c);
  free(m);
  free(nn);
  unpack_free(&P);
}

void jur_unified_optimal_estimation(const jgb_ret *ret, obs_t *obs_meas, obs_t *obs_i,
                                    atm_t *atm_apr, atm_t *atm_i, gsl_matrix *cov) {
  jur_unified_optimal_estimation_multiple_packages(ret, obs_meas, obs_i, atm_apr, atm_i, 1, &cov);
}
