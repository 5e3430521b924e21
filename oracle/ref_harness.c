/*
 * Flat C entry points around the UNMODIFIED reference sources
 * (src/jurassic.c, src/retrieval.c), compiled together by oracle/build_ref.sh
 * into oracle/_ref/libjref.so.  TEST INFRASTRUCTURE ONLY: this library is the
 * reference itself, used to pin the CPU restatement (oracle/jrc_oracle.c) and
 * as the timed CPU baseline; nothing in the product links it.
 *
 * The reference keeps process-global state (static tables in formod_pencil,
 * jurassic.c:3202-3217), so one loaded copy of this library serves one
 * control file.  Callers load it in a fresh process per configuration.
 *
 * retrieval.c is compiled with its writers renamed (write_atm, write_obs,
 * write_matrix -> jref_hook_*), so that the retrieval's results are captured
 * here at full double precision instead of being printed with %g.
 */
#include "jurassic.h"

static ctl_t g_ctl;
static atm_t g_atm;
static obs_t g_obs;

/* Retrieval control (ret_t, retrieval.c:32-112) is file-local to
   retrieval.c.  Its first member is the working directory (char[LEN]); the
   rest is filled by read_ret() (retrieval.c:753).  It is held here in an
   opaque, generously sized and aligned buffer so that no layout is mirrored. */
static union {
  char dir[LEN];
  double align;
  char pad[1 << 20];
} g_ret;

void read_ret(int argc, char *argv[], ctl_t * ctl, void *ret);
void optimal_estimation(void *ret, ctl_t * ctl, obs_t * obs_meas,
                        obs_t * obs_i, atm_t * atm_apr, atm_t * atm_i);

int jref_init(int argc, char **argv);
int jref_dims(int *out);
void jref_set_atm(int np, const double *time, const double *z,
                  const double *lon, const double *lat, const double *p,
                  const double *t, const double *q, const double *k,
                  const double *scal);
void jref_get_atm(double *p, double *t, double *q, double *k,
                  double *scal);
void jref_set_obs(int nr, const double *geo, const double *rad);
void jref_get_obs(double *tp, double *rad, double *tau);
int jref_formod(void);
int jref_kernel(double *kmat, int maxm, int maxn, int *mn);
int jref_raytrace(int ir, int maxpts, double *out, double *tp);
int jref_retrieval(const char *dir, double *x_final, int maxn,
                   double *cov, double *costs, int maxcost, int *info);
void jref_hook_write_atm(const char *dirname, const char *filename,
                         const ctl_t * ctl, const atm_t * atm);
void jref_hook_write_obs(const char *dirname, const char *filename,
                         const ctl_t * ctl, const obs_t * obs);
void jref_hook_write_matrix(const char *dirname, const char *filename,
                            const ctl_t * ctl, const gsl_matrix * matrix,
                            const atm_t * atm, const obs_t * obs,
                            const char *rowspace, const char *colspace,
                            const char *sort);

int jref_init(int argc, char **argv) {
  read_ctl(argc, argv, &g_ctl);
  read_ret(argc, argv, &g_ctl, &g_ret);
  return 0;
}

/* Compile-time capacities of this build: ND NG NP NR NW NLOS NCL NSF. */
int jref_dims(int *out) {
  out[0] = ND;
  out[1] = NG;
  out[2] = NP;
  out[3] = NR;
  out[4] = NW;
  out[5] = NLOS;
  out[6] = NCL;
  out[7] = NSF;
  return 0;
}

/* scal = {clz, cldz, clk[ncl], sfz, sfp, sft, sfeps[nsf]} */
void jref_set_atm(int np, const double *time, const double *z,
                  const double *lon, const double *lat, const double *p,
                  const double *t, const double *q, const double *k,
                  const double *scal) {
  g_atm.np = np;
  for (int i = 0; i < np; i++) {
    g_atm.time[i] = time[i];
    g_atm.z[i] = z[i];
    g_atm.lon[i] = lon[i];
    g_atm.lat[i] = lat[i];
    g_atm.p[i] = p[i];
    g_atm.t[i] = t[i];
    for (int ig = 0; ig < g_ctl.ng; ig++)
      g_atm.q[ig][i] = q[ig * np + i];
    for (int iw = 0; iw < g_ctl.nw; iw++)
      g_atm.k[iw][i] = k[iw * np + i];
  }
  int s = 0;
  g_atm.clz = scal[s++];
  g_atm.cldz = scal[s++];
  for (int icl = 0; icl < g_ctl.ncl; icl++)
    g_atm.clk[icl] = scal[s++];
  g_atm.sfz = scal[s++];
  g_atm.sfp = scal[s++];
  g_atm.sft = scal[s++];
  for (int isf = 0; isf < g_ctl.nsf; isf++)
    g_atm.sfeps[isf] = scal[s++];
}

void jref_get_atm(double *p, double *t, double *q, double *k, double *scal) {
  const int np = g_atm.np;
  for (int i = 0; i < np; i++) {
    p[i] = g_atm.p[i];
    t[i] = g_atm.t[i];
    for (int ig = 0; ig < g_ctl.ng; ig++)
      q[ig * np + i] = g_atm.q[ig][i];
    for (int iw = 0; iw < g_ctl.nw; iw++)
      k[iw * np + i] = g_atm.k[iw][i];
  }
  int s = 0;
  scal[s++] = g_atm.clz;
  scal[s++] = g_atm.cldz;
  for (int icl = 0; icl < g_ctl.ncl; icl++)
    scal[s++] = g_atm.clk[icl];
  scal[s++] = g_atm.sfz;
  scal[s++] = g_atm.sfp;
  scal[s++] = g_atm.sft;
  for (int isf = 0; isf < g_ctl.nsf; isf++)
    scal[s++] = g_atm.sfeps[isf];
}

/* geo = [7][nr]: time, obsz, obslon, obslat, vpz, vplon, vplat.
   rad = [nd][nr]: NaN entries mark masked channels (jurassic.c:3037-3040). */
void jref_set_obs(int nr, const double *geo, const double *rad) {
  g_obs.nr = nr;
  for (int ir = 0; ir < nr; ir++) {
    g_obs.time[ir] = geo[0 * nr + ir];
    g_obs.obsz[ir] = geo[1 * nr + ir];
    g_obs.obslon[ir] = geo[2 * nr + ir];
    g_obs.obslat[ir] = geo[3 * nr + ir];
    g_obs.vpz[ir] = geo[4 * nr + ir];
    g_obs.vplon[ir] = geo[5 * nr + ir];
    g_obs.vplat[ir] = geo[6 * nr + ir];
    g_obs.tpz[ir] = g_obs.tplon[ir] = g_obs.tplat[ir] = 0;
    for (int id = 0; id < g_ctl.nd; id++) {
      g_obs.rad[id][ir] = rad ? rad[id * nr + ir] : 0.0;
      g_obs.tau[id][ir] = 0.0;
    }
  }
}

/* tp = [3][nr], rad/tau = [nd][nr] */
void jref_get_obs(double *tp, double *rad, double *tau) {
  const int nr = g_obs.nr;
  for (int ir = 0; ir < nr; ir++) {
    tp[0 * nr + ir] = g_obs.tpz[ir];
    tp[1 * nr + ir] = g_obs.tplon[ir];
    tp[2 * nr + ir] = g_obs.tplat[ir];
    for (int id = 0; id < g_ctl.nd; id++) {
      rad[id * nr + ir] = g_obs.rad[id][ir];
      tau[id * nr + ir] = g_obs.tau[id][ir];
    }
  }
}

int jref_formod(void) {
  formod(&g_ctl, &g_atm, &g_obs);
  return 0;
}

/* Jacobian through the reference kernel() (jurassic.c:4004), row-major. */
int jref_kernel(double *kmat, int maxm, int maxn, int *mn) {
  const size_t m = obs2y(&g_ctl, &g_obs, NULL, NULL, NULL);
  const size_t n = atm2x(&g_ctl, &g_atm, NULL, NULL, NULL);
  mn[0] = (int) m;
  mn[1] = (int) n;
  if ((int) m > maxm || (int) n > maxn || m == 0 || n == 0)
    return -1;
  gsl_matrix *k = gsl_matrix_alloc(m, n);
  kernel(&g_ctl, &g_atm, &g_obs, k);
  for (size_t i = 0; i < m; i++)
    for (size_t j = 0; j < n; j++)
      kmat[i * n + j] = gsl_matrix_get(k, i, j);
  gsl_matrix_free(k);
  return 0;
}

/* One LOS through the reference raytrace() (jurassic.c:4201).
   Each LOS point is one row of 7 + 5*ng + 2*nd doubles:
   z lon lat p t ds sft | q[ng] | u[ng] | cgp[ng] | cgt[ng] | cgu[ng] |
   k[nd] | sfeps[nd].  Returns the number of points. */
int jref_raytrace(int ir, int maxpts, double *out, double *tp) {
  los_t *los = (los_t *) malloc(sizeof(los_t));
  raytrace(&g_ctl, &g_atm, &g_obs, los, ir);
  const int ng = g_ctl.ng, nd = g_ctl.nd;
  const int w = 7 + 5 * ng + 2 * nd;
  const int np = los->np;
  if (np > maxpts) {
    free(los);
    return -1;
  }
  for (int ip = 0; ip < np; ip++) {
    double *r = out + (size_t) ip * w;
    int c = 0;
    r[c++] = los->z[ip];
    r[c++] = los->lon[ip];
    r[c++] = los->lat[ip];
    r[c++] = los->p[ip];
    r[c++] = los->t[ip];
    r[c++] = los->ds[ip];
    r[c++] = los->sft;
    for (int ig = 0; ig < ng; ig++)
      r[c++] = los->q[ip][ig];
    for (int ig = 0; ig < ng; ig++)
      r[c++] = los->u[ip][ig];
    for (int ig = 0; ig < ng; ig++)
      r[c++] = los->cgp[ip][ig];
    for (int ig = 0; ig < ng; ig++)
      r[c++] = los->cgt[ip][ig];
    for (int ig = 0; ig < ng; ig++)
      r[c++] = los->cgu[ip][ig];
    for (int id = 0; id < nd; id++)
      r[c++] = los->k[ip][id];
    for (int id = 0; id < nd; id++)
      r[c++] = los->sfeps[id];
  }
  tp[0] = g_obs.tpz[ir];
  tp[1] = g_obs.tplon[ir];
  tp[2] = g_obs.tplat[ir];
  free(los);
  return np;
}

/* ---- captured retrieval outputs ---- */

static atm_t g_cap_atm_final;
static int g_cap_have_atm;
static double *g_cap_cov;
static size_t g_cap_cov_n;

/* error analysis (retrieval.c:668-726): gain [n][m], averaging kernel
   [n][n] and the state-vector form (atm2x) of the atm_err_{total,noise,
   formod}.tab, atm_cont.tab and atm_res.tab files */
static double *g_cap_gain, *g_cap_avk;
static size_t g_cap_gain_n, g_cap_gain_m, g_cap_avk_n;
static const char *g_ana_files[5] = {"atm_err_total.tab", "atm_err_noise.tab",
                                     "atm_err_formod.tab", "atm_cont.tab", "atm_res.tab"};
static double *g_cap_ana[5];
static size_t g_cap_ana_n[5];

static void cap_matrix(const gsl_matrix *m, double **dst, size_t *n1, size_t *n2) {
  free(*dst);
  *n1 = m->size1;
  if (n2) *n2 = m->size2;
  *dst = (double *) malloc(m->size1 * m->size2 * sizeof(double));
  for (size_t i = 0; i < m->size1; i++)
    for (size_t j = 0; j < m->size2; j++)
      (*dst)[i * m->size2 + j] = gsl_matrix_get(m, i, j);
}

void jref_hook_write_atm(const char *dirname, const char *filename,
                         const ctl_t * ctl, const atm_t * atm) {
  if (strcmp(filename, "atm_final.tab") == 0) {
    copy_atm(ctl, &g_cap_atm_final, atm, 0);
    g_cap_have_atm = 1;
  }
  for (int k = 0; k < 5; k++)
    if (strcmp(filename, g_ana_files[k]) == 0) {
      const size_t n = atm2x(ctl, atm, NULL, NULL, NULL);
      gsl_vector *v = gsl_vector_alloc(n);
      atm2x(ctl, atm, v, NULL, NULL);
      free(g_cap_ana[k]);
      g_cap_ana[k] = (double *) malloc(n * sizeof(double));
      for (size_t i = 0; i < n; i++)
        g_cap_ana[k][i] = gsl_vector_get(v, i);
      g_cap_ana_n[k] = n;
      gsl_vector_free(v);
    }
  write_atm(dirname, filename, ctl, atm);
}

void jref_hook_write_obs(const char *dirname, const char *filename,
                         const ctl_t * ctl, const obs_t * obs) {
  write_obs(dirname, filename, ctl, obs);
}

void jref_hook_write_matrix(const char *dirname, const char *filename,
                            const ctl_t * ctl, const gsl_matrix * matrix,
                            const atm_t * atm, const obs_t * obs,
                            const char *rowspace, const char *colspace,
                            const char *sort) {
  (void) dirname;
  (void) ctl;
  (void) atm;
  (void) obs;
  (void) rowspace;
  (void) colspace;
  (void) sort;
  if (strcmp(filename, "matrix_gain.tab") == 0)
    cap_matrix(matrix, &g_cap_gain, &g_cap_gain_n, &g_cap_gain_m);
  if (strcmp(filename, "matrix_avk.tab") == 0)
    cap_matrix(matrix, &g_cap_avk, &g_cap_avk_n, NULL);
  if (strcmp(filename, "matrix_cov_ret.tab") == 0) {
    free(g_cap_cov);
    g_cap_cov_n = matrix->size1;
    g_cap_cov = (double *) malloc(g_cap_cov_n * g_cap_cov_n * sizeof(double));
    for (size_t i = 0; i < g_cap_cov_n; i++)
      for (size_t j = 0; j < g_cap_cov_n; j++)
        g_cap_cov[i * g_cap_cov_n + j] = gsl_matrix_get(matrix, i, j);
  }
}

/* Runs optimal_estimation (retrieval.c:448) on the atmosphere/observation
   set with jref_set_atm (a priori) and jref_set_obs (measurement).
   x_final receives atm2x of the final state, cov the retrieval covariance
   (if ERR_ANA), costs the chi^2/m history parsed from costs.tab.
   info = {n, m, number of costs, have_cov}. */
int jref_retrieval(const char *dir, double *x_final, int maxn, double *cov,
                   double *costs, int maxcost, int *info) {
  static atm_t atm_i;
  static obs_t obs_i;
  snprintf(g_ret.dir, LEN, "%s", dir);
  g_cap_have_atm = 0;
  g_cap_cov_n = 0;
  g_cap_gain_n = g_cap_gain_m = g_cap_avk_n = 0;
  for (int k = 0; k < 5; k++)
    g_cap_ana_n[k] = 0;
  optimal_estimation(&g_ret, &g_ctl, &g_obs, &obs_i, &g_atm, &atm_i);
  gsl_vector *x = gsl_vector_alloc((size_t) maxn);
  const size_t n = atm2x(&g_ctl, &atm_i, NULL, NULL, NULL);
  if ((int) n > maxn)
    return -1;
  atm2x(&g_ctl, &atm_i, x, NULL, NULL);
  for (size_t i = 0; i < n; i++)
    x_final[i] = gsl_vector_get(x, i);
  gsl_vector_free(x);
  info[0] = (int) n;
  info[1] = (int) obs2y(&g_ctl, &g_obs, NULL, NULL, NULL);
  info[3] = 0;
  if (g_cap_cov_n == n && cov) {
    memcpy(cov, g_cap_cov, n * n * sizeof(double));
    info[3] = 1;
  }
  /* cost history */
  char file[2 * LEN];
  snprintf(file, sizeof(file), "%s/costs.tab", dir);
  FILE *in = fopen(file, "r");
  int nc = 0;
  if (in) {
    char line[LEN];
    while (fgets(line, LEN, in)) {
      int it, mm, nn;
      double c;
      if (sscanf(line, "%d %lg %d %d", &it, &c, &mm, &nn) == 4 && nc < maxcost)
        costs[nc++] = c;
    }
    fclose(in);
  }
  info[2] = nc;
  return 0;
}

/* Error-analysis outputs of the last jref_retrieval (ERR_ANA): gain[n*m],
   avk[n*n], ana[5*n] = err_total, err_noise, err_formod, cont, res in
   state-vector order.  Returns 0, or -1 if they were not written. */
int jref_retrieval_ana(double *gain, double *avk, double *ana, int maxn, int maxm) {
  const size_t n = g_cap_avk_n;
  if (n == 0 || g_cap_gain_n != n || (int) n > maxn || (int) g_cap_gain_m > maxm)
    return -1;
  for (int k = 0; k < 5; k++)
    if (g_cap_ana_n[k] != n)
      return -1;
  memcpy(gain, g_cap_gain, n * g_cap_gain_m * sizeof(double));
  memcpy(avk, g_cap_avk, n * n * sizeof(double));
  for (int k = 0; k < 5; k++)
    memcpy(ana + k * n, g_cap_ana[k], n * sizeof(double));
  return 0;
}
