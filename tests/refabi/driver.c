/*
 * Test driver of the reference binding (TEST INFRASTRUCTURE ONLY): holds
 * reference-layout packages (atm_t, obs_t of tests/refabi/jurassic.h),
 * fills them from flat arrays given by the Python tests, calls the
 * binding's entry points and hands the results back as flat arrays.
 * drv_fill_ctl is generated by the test from its control set.
 */
#include "jurassic.h"
#include "jurassic_unified_library.h"

void drv_fill_ctl(ctl_t *ctl);

static ctl_t g_ctl;
static atm_t *g_atm[2];   /* [0]: inputs (a priori), [1]: retrieval results */
static obs_t *g_obs[2];
static int g_cap;

/* the binding's jur_unified_init reads a control file with the reference's
   parser, which this driver does not have; the tests call
   jur_unified_init_ctl instead */
void read_ctl(int argc, char *argv[], ctl_t *ctl) {
  (void)argc;
  (void)argv;
  (void)ctl;
  ERRMSG("read_ctl is not available in the test driver");
}

double scan_ctl(int argc, char *argv[], const char *varname, int arridx, const char *defvalue,
                char *value) {
  (void)argc;
  (void)argv;
  (void)varname;
  (void)arridx;
  (void)defvalue;
  (void)value;
  ERRMSG("scan_ctl is not available in the test driver");
  return 0;
}

int drv_sizeof_atm(void) { return (int)sizeof(atm_t); }
int drv_sizeof_obs(void) { return (int)sizeof(obs_t); }

int drv_init(int npack, int device, int precision) {
  memset(&g_ctl, 0, sizeof g_ctl);
  drv_fill_ctl(&g_ctl);
  for (int w = 0; w < 2; w++) {
    free(g_atm[w]);
    free(g_obs[w]);
    g_atm[w] = calloc((size_t)npack, sizeof(atm_t));
    g_obs[w] = calloc((size_t)npack, sizeof(obs_t));
    if (!g_atm[w] || !g_obs[w]) return 1;
  }
  g_cap = npack;
  jur_unified_init_ctl(&g_ctl, device, precision);
  return 0;
}

void drv_finalize(void) { jur_unified_finalize(); }

/* q[ng][np], k[nw][np], scal = clz cldz clk[ncl] sfz sfp sft sfeps[nsf] */
void drv_set_atm(int i, int np, const double *time, const double *z, const double *lon,
                 const double *lat, const double *p, const double *t, const double *q,
                 const double *k, const double *scal) {
  atm_t *a = &g_atm[0][i];
  memset(a, 0, sizeof *a);
  a->np = np;
  memcpy(a->time, time, sizeof(double) * np);
  memcpy(a->z, z, sizeof(double) * np);
  memcpy(a->lon, lon, sizeof(double) * np);
  memcpy(a->lat, lat, sizeof(double) * np);
  memcpy(a->p, p, sizeof(double) * np);
  memcpy(a->t, t, sizeof(double) * np);
  for (int ig = 0; ig < g_ctl.ng; ig++) memcpy(a->q[ig], q + ig * np, sizeof(double) * np);
  for (int iw = 0; iw < g_ctl.nw; iw++) memcpy(a->k[iw], k + iw * np, sizeof(double) * np);
  int j = 0;
  a->clz = scal[j++];
  a->cldz = scal[j++];
  for (int icl = 0; icl < g_ctl.ncl; icl++) a->clk[icl] = scal[j++];
  a->sfz = scal[j++];
  a->sfp = scal[j++];
  a->sft = scal[j++];
  for (int isf = 0; isf < g_ctl.nsf; isf++) a->sfeps[isf] = scal[j++];
}

/* geo[7][nr] = time obsz obslon obslat vpz vplon vplat, rad[nd][nr] */
void drv_set_obs(int i, int nr, const double *geo, const double *rad) {
  obs_t *o = &g_obs[0][i];
  memset(o, 0, sizeof *o);
  o->nr = nr;
  double *rows[7] = {o->time, o->obsz, o->obslon, o->obslat, o->vpz, o->vplon, o->vplat};
  for (int g = 0; g < 7; g++) memcpy(rows[g], geo + g * nr, sizeof(double) * nr);
  for (int id = 0; id < g_ctl.nd; id++) memcpy(o->rad[id], rad + id * nr, sizeof(double) * nr);
}

/* which 0: the input packages (after a forward model or Jacobian), 1: the
   retrieval results; rad/tau [nd][nr], tp [3][nr], p/t [np], q [ng][np] */
void drv_get(int which, int i, double *rad, double *tau, double *tp, double *p, double *t,
             double *q) {
  const obs_t *o = &g_obs[which][i];
  const atm_t *a = &g_atm[which][i];
  const int nr = o->nr, np = a->np;
  for (int id = 0; id < g_ctl.nd; id++) {
    memcpy(rad + id * nr, o->rad[id], sizeof(double) * nr);
    memcpy(tau + id * nr, o->tau[id], sizeof(double) * nr);
  }
  memcpy(tp, o->tpz, sizeof(double) * nr);
  memcpy(tp + nr, o->tplon, sizeof(double) * nr);
  memcpy(tp + 2 * nr, o->tplat, sizeof(double) * nr);
  memcpy(p, a->p, sizeof(double) * np);
  memcpy(t, a->t, sizeof(double) * np);
  for (int ig = 0; ig < g_ctl.ng; ig++) memcpy(q + ig * np, a->q[ig], sizeof(double) * np);
}

void drv_formod(int n) { jur_unified_formod_multiple_packages(g_atm[0], g_obs[0], n, NULL); }

/* Matrices of m[i] x nn[i] with a row pitch of nn[i] + pad (the caller's tda
   need not equal the row length); kout gets them densely, concatenated.
   n == 1 goes through the single-package kernel() drop-in. */
void drv_kernel(int n, const int *m, const int *nn, int pad, double *kout) {
  gsl_matrix **k = calloc((size_t)n, sizeof(gsl_matrix *));
  for (int i = 0; i < n; i++) {
    k[i] = calloc(1, sizeof(gsl_matrix));
    k[i]->size1 = (size_t)m[i];
    k[i]->size2 = (size_t)nn[i];
    k[i]->tda = (size_t)(nn[i] + pad);
    k[i]->data = calloc((size_t)m[i] * (size_t)(nn[i] + pad) + 1, sizeof(double));
  }
  if (n == 1)
    jur_unified_kernel(&g_ctl, g_atm[0], g_obs[0], k[0]);
  else
    jur_unified_kernel_multiple_packages(g_atm[0], g_obs[0], n, k);
  size_t off = 0;
  for (int i = 0; i < n; i++) {
    for (int r = 0; r < m[i]; r++)
      for (int c = 0; c < nn[i]; c++) kout[off++] = k[i]->data[(size_t)r * k[i]->tda + c];
    free(k[i]->data);
    free(k[i]);
  }
  free(k);
}

/* optimal_estimation of n packages; cov_out (may be NULL) gets the
   covariances nn[i] x nn[i] concatenated. n == 1 goes through the
   single-package drop-in. */
void drv_retrieve(const jgb_ret *ret, int n, const int *nn, double *cov_out) {
  gsl_matrix **cov = calloc((size_t)n, sizeof(gsl_matrix *));
  for (int i = 0; cov_out && i < n; i++) cov[i] = gsl_matrix_alloc((size_t)nn[i], (size_t)nn[i]);
  if (n == 1)
    jur_unified_optimal_estimation(ret, g_obs[0], g_obs[1], g_atm[0], g_atm[1], cov[0]);
  else
    jur_unified_optimal_estimation_multiple_packages(ret, g_obs[0], g_obs[1], g_atm[0], g_atm[1],
                                                     n, cov);
  size_t off = 0;
  for (int i = 0; cov_out && i < n; i++) {
    for (int r = 0; r < nn[i]; r++)
      for (int c = 0; c < nn[i]; c++) cov_out[off++] = cov[i]->data[(size_t)r * cov[i]->tda + c];
    gsl_matrix_free(cov[i]);
  }
  free(cov);
}
