/*
 * jrc_oracle.c -- CPU restatement of the reference JURASSIC forward model,
 * Jacobian and retrieval.  TEST INFRASTRUCTURE ONLY (see jrc_oracle.h).
 *
 * Written for this project from the reference's documented behaviour; each
 * routine names the reference lines it restates.  Arithmetic is FP64 and the
 * order of floating-point operations follows the reference expression by
 * expression, so that (compiled with -ffp-contract=off, as the build does)
 * results agree with the reference to the last bit on the same machine
 * apart from libm differences between machines.
 */
#include "jrc_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Physical constants (jurassic.h:254-345). */
#define K_C1 1.19104259e-8
#define K_C2 1.43877506
#define K_G0 9.80665
#define K_KB 1.3806504e-23
#define K_NA 6.02214199e23
#define K_RE 6367.421
#define K_RI 8.3144598
#define K_P0 1013.25
#define K_TMIN 100.
#define K_TMAX 400.
#define K_TSUN 5780.
#define K_NS 1200 /* source-function temperatures, TBLNS jurassic.h:433 */
#define K_PI 3.14159265358979323846

/* Continuum table sizes and offsets inside the continua.bin blob. */
#define CT_N 2001
enum { CT_CO2_296 = 0, CT_CO2_260 = 2001, CT_CO2_230 = 4002,
       CT_H2O_296 = 6003, CT_H2O_260 = 8004, CT_H2O_FRN = 10005,
       CT_XFCREV = 12006, CT_N2_B = 12021, CT_N2_BETA = 12119,
       CT_N2_NU = 12217, CT_O2_B = 12315, CT_O2_BETA = 12405,
       CT_O2_NU = 12495, CT_TOTAL = 12585 };

struct jrc_ctx {
  /* control */
  int ng, nd, nw, ncl, nsf;
  int *kind;
  double *nu, *clnu, *sfnu;
  int *window;
  int sftype;
  double sfsza, hydz;
  int ctm_co2, ctm_h2o, ctm_n2, ctm_o2, refrac, formod, write_bbt;
  double rayds, raydz;
  double retp_zmin, retp_zmax, rett_zmin, rett_zmax;
  double *retq_zmin, *retq_zmax, *retk_zmin, *retk_zmax;
  int ret_clz, ret_cldz, ret_clk, ret_sfz, ret_sfp, ret_sft, ret_sfeps;
  int nlos_max;
  int ig_co2, ig_h2o;
  /* tables */
  int cap_p, cap_t, cap_u;
  int *tnp;          /* [nd][ng] */
  int *tnt;          /* [nd][ng][cap_p] */
  int *tnu;          /* [nd][ng][cap_p][cap_t] */
  double *tp;        /* [nd][ng][cap_p] */
  double *tt;        /* [nd][ng][cap_p][cap_t] */
  float *tu, *teps;  /* [nd][ng][cap_p][cap_t][cap_u] */
  /* source function */
  double st[K_NS];
  double *sr;        /* [K_NS][nd] */
  /* continua */
  double ct[CT_TOTAL];
  int have_ct;
  /* field of view (formod_fov): nfov samples, 0 = off */
  int nfov;
  double *fov_dz, *fov_w;
  char err[256];
};

/* A line of sight (los_t, jurassic.h:678-731) with runtime capacities. */
typedef struct {
  int np, cap, ng, nd;
  double sft;
  double *z, *lon, *lat, *p, *t, *ds;
  double *q, *u, *cgp, *cgt, *cgu;  /* [cap][ng] */
  double *k, *eps, *src;             /* [cap][nd] */
  double *sfeps;                     /* [nd] */
} los_buf;

static void set_err(jrc_ctx *c, const char *msg) {
  snprintf(c->err, sizeof(c->err), "%s", msg);
}

const char *jrc_error(const jrc_ctx *c) { return c->err; }

/* ---------------------------------------------------------------------- */
/* interpolation helpers (LIN, LOGX, LOGY: jurassic.h:164-175)             */

static inline double lin(double x0, double y0, double x1, double y1, double x) {
  return y0 + (y1 - y0) / (x1 - x0) * (x - x0);
}

static inline double logx(double x0, double y0, double x1, double y1, double x) {
  if (x / x0 > 0 && x1 / x0 > 0)
    return y0 + (y1 - y0) * log(x / x0) / log(x1 / x0);
  return lin(x0, y0, x1, y1, x);
}

static inline double logy(double x0, double y0, double x1, double y1, double x) {
  if (y1 / y0 > 0)
    return y0 * exp(log(y1 / y0) / (x1 - x0) * (x - x0));
  return lin(x0, y0, x1, y1, x);
}

static inline double sq(double x) { return x * x; }

/* Bisection on an ascending or descending double grid: the lower bracket
   index in [0, n-2] (locate_irr, jurassic.c:4103-4129). */
static int bracket_irr(const double *g, int n, double x) {
  int lo = 0, hi = n - 1, mid = (lo + hi) >> 1;
  const int up = g[mid] < g[mid + 1];
  while (hi > lo + 1) {
    mid = (lo + hi) >> 1;
    const int go_low = up ? (g[mid] > x) : (g[mid] <= x);
    if (go_low)
      hi = mid;
    else
      lo = mid;
  }
  return lo;
}

/* Direct index on a regular grid, clamped to [0, n-2]
   (locate_reg, jurassic.c:4133-4148). */
static int bracket_reg(const double *g, int n, double x) {
  const int i = (int) ((x - g[0]) / (g[1] - g[0]));
  if (i < 0)
    return 0;
  if (i > n - 2)
    return n - 2;
  return i;
}

/* Bisection on an ascending float row (locate_tbl, jurassic.c:4152-4170). */
static int bracket_row(const float *g, int n, double x) {
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (g[mid] > x)
      hi = mid;
    else
      lo = mid;
  }
  return lo;
}

/* ---------------------------------------------------------------------- */
/* geometry (cart2geo jurassic.c:108-120, geo2cart 3500-3516)             */

static void to_geo(const double *x, double *z, double *lon, double *lat) {
  const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  *lat = asin(x[2] / r) * (180.0 / K_PI);
  *lon = atan2(x[1], x[0]) * (180.0 / K_PI);
  *z = r - K_RE;
}

static void to_cart(double z, double lon, double lat, double *x) {
  const double r = z + K_RE;
  const double la = lat / 180. * K_PI, lo = lon / 180. * K_PI;
  const double cl = cos(la);
  x[0] = r * cl * cos(lo);
  x[1] = r * cl * sin(lo);
  x[2] = r * sin(la);
}

/* Solar zenith angle [deg] (sza, jurassic.c:5183-5219). */
static double solar_zenith(double sec, double lon, double lat) {
  const double d = sec / 86400 - 0.5;
  const double g = (357.529 + 0.98560028 * d) * (K_PI / 180.0);
  const double q = 280.459 + 0.98564736 * d;
  const double l = (q + 1.915 * sin(g) + 0.020 * sin(2 * g)) * (K_PI / 180.0);
  const double e = (23.439 - 0.00000036 * d) * (K_PI / 180.0);
  const double dec = asin(sin(e) * sin(l));
  const double ra = atan2(cos(e) * sin(l), cos(l));
  const double gmst = 18.697374558 + 24.06570982441908 * d;
  const double lst = gmst + lon / 15;
  const double h = lst / 12 * K_PI - ra;
  const double latr = lat * (K_PI / 180.0);
  return acos(sin(latr) * sin(dec) + cos(latr) * cos(dec) * cos(h)) *
         (180.0 / K_PI);
}

/* ---------------------------------------------------------------------- */
/* context                                                                */

static double *dup_d(const double *src, int n) {
  double *d = (double *) calloc((size_t) (n > 0 ? n : 1), sizeof(double));
  if (src && n > 0)
    memcpy(d, src, (size_t) n * sizeof(double));
  return d;
}

jrc_ctx *jrc_create(const jrc_ctl *ctl, int tbl_np, int tbl_nt, int tbl_nu) {
  jrc_ctx *c = (jrc_ctx *) calloc(1, sizeof(jrc_ctx));
  c->ng = ctl->ng;
  c->nd = ctl->nd;
  c->nw = ctl->nw;
  c->ncl = ctl->ncl;
  c->nsf = ctl->nsf;
  c->kind = (int *) calloc((size_t) (c->ng + 1), sizeof(int));
  for (int ig = 0; ig < c->ng; ig++)
    c->kind[ig] = ctl->emitter_kind[ig];
  c->nu = dup_d(ctl->nu, c->nd);
  c->window = (int *) calloc((size_t) (c->nd + 1), sizeof(int));
  for (int id = 0; id < c->nd; id++)
    c->window[id] = ctl->window ? ctl->window[id] : 0;
  c->clnu = dup_d(ctl->clnu, c->ncl);
  c->sfnu = dup_d(ctl->sfnu, c->nsf);
  c->sftype = ctl->sftype;
  c->sfsza = ctl->sfsza;
  c->hydz = ctl->hydz;
  c->ctm_co2 = ctl->ctm_co2;
  c->ctm_h2o = ctl->ctm_h2o;
  c->ctm_n2 = ctl->ctm_n2;
  c->ctm_o2 = ctl->ctm_o2;
  c->refrac = ctl->refrac;
  c->rayds = ctl->rayds;
  c->raydz = ctl->raydz;
  c->formod = ctl->formod;
  c->write_bbt = ctl->write_bbt;
  c->retp_zmin = ctl->retp_zmin;
  c->retp_zmax = ctl->retp_zmax;
  c->rett_zmin = ctl->rett_zmin;
  c->rett_zmax = ctl->rett_zmax;
  c->retq_zmin = dup_d(ctl->retq_zmin, c->ng);
  c->retq_zmax = dup_d(ctl->retq_zmax, c->ng);
  c->retk_zmin = dup_d(ctl->retk_zmin, c->nw);
  c->retk_zmax = dup_d(ctl->retk_zmax, c->nw);
  c->ret_clz = ctl->ret_clz;
  c->ret_cldz = ctl->ret_cldz;
  c->ret_clk = ctl->ret_clk;
  c->ret_sfz = ctl->ret_sfz;
  c->ret_sfp = ctl->ret_sfp;
  c->ret_sft = ctl->ret_sft;
  c->ret_sfeps = ctl->ret_sfeps;
  c->nlos_max = ctl->nlos_max > 0 ? ctl->nlos_max : 4096;
  if (c->ng > 64 || c->nw > 64) {
    set_err(c, "at most 64 emitters and 64 windows");
    c->ng = c->ng > 64 ? 64 : c->ng;
    c->nw = c->nw > 64 ? 64 : c->nw;
  }
  /* emitter indices used by the continua (find_emitter, jurassic.c:3013) */
  c->ig_co2 = c->ig_h2o = -1;
  for (int ig = c->ng - 1; ig >= 0; ig--) {
    if (c->kind[ig] == 1)
      c->ig_co2 = ig;
    if (c->kind[ig] == 2)
      c->ig_h2o = ig;
  }
  c->cap_p = tbl_np;
  c->cap_t = tbl_nt;
  c->cap_u = tbl_nu;
  const size_t ndg = (size_t) c->nd * (size_t) c->ng;
  c->tnp = (int *) malloc(ndg * sizeof(int));
  for (size_t i = 0; i < ndg; i++)
    c->tnp[i] = -1;
  c->tnt = (int *) calloc(ndg * (size_t) tbl_np, sizeof(int));
  c->tnu = (int *) calloc(ndg * (size_t) tbl_np * (size_t) tbl_nt, sizeof(int));
  c->tp = (double *) calloc(ndg * (size_t) tbl_np, sizeof(double));
  c->tt = (double *) calloc(ndg * (size_t) tbl_np * (size_t) tbl_nt, sizeof(double));
  const size_t nrow = ndg * (size_t) tbl_np * (size_t) tbl_nt * (size_t) tbl_nu;
  c->tu = (float *) calloc(nrow, sizeof(float));
  c->teps = (float *) calloc(nrow, sizeof(float));
  c->sr = (double *) calloc((size_t) K_NS * (size_t) (c->nd > 0 ? c->nd : 1), sizeof(double));
  for (int it = 0; it < K_NS; it++)
    c->st[it] = lin(0.0, K_TMIN, K_NS - 1.0, K_TMAX, (double) it);
  return c;
}

void jrc_destroy(jrc_ctx *c) {
  if (!c)
    return;
  free(c->kind); free(c->nu); free(c->window); free(c->clnu); free(c->sfnu);
  free(c->retq_zmin); free(c->retq_zmax); free(c->retk_zmin); free(c->retk_zmax);
  free(c->tnp); free(c->tnt); free(c->tnu); free(c->tp); free(c->tt);
  free(c->tu); free(c->teps); free(c->sr);
  free(c->fov_dz); free(c->fov_w);
  free(c);
}

int jrc_set_fov(jrc_ctx *c, int n, const double *dz, const double *w) {
  free(c->fov_dz);
  free(c->fov_w);
  c->fov_dz = c->fov_w = NULL;
  c->nfov = 0;
  if (n <= 0)
    return 0;
  c->fov_dz = malloc((size_t) n * sizeof(double));
  c->fov_w = malloc((size_t) n * sizeof(double));
  memcpy(c->fov_dz, dz, (size_t) n * sizeof(double));
  memcpy(c->fov_w, w, (size_t) n * sizeof(double));
  c->nfov = n;
  return 0;
}

/* formod_fov (jurassic.c:3121-3192): each ray's radiance and transmittance
   become the FOV-weighted average of the pencil-beam profiles over view-point
   altitude, built from the rays within +-5 indices with the same time. */
#define K_NFOV 5
static int fov_apply(const jrc_ctx *c, jrc_obs *obs) {
  const int nd = c->nd, nr = obs->nr;
  const double *time = obs->geo, *vpz = obs->geo + 4 * (size_t) nr;
  double *rad0 = malloc((size_t) (nd * nr) * sizeof(double));
  double *tau0 = malloc((size_t) (nd * nr) * sizeof(double));
  memcpy(rad0, obs->rad, (size_t) (nd * nr) * sizeof(double));
  memcpy(tau0, obs->tau, (size_t) (nd * nr) * sizeof(double));
  int rc = 0;
  for (int ir = 0; ir < nr && rc == 0; ir++) {
    double zz[2 * K_NFOV + 1];
    int ray[2 * K_NFOV + 1], nz = 0;
    const int lo = ir - K_NFOV > 0 ? ir - K_NFOV : 0;
    const int hi = ir + 1 + K_NFOV < nr ? ir + 1 + K_NFOV : nr;
    for (int ir2 = lo; ir2 < hi; ir2++)
      if (time[ir2] == time[ir]) {
        zz[nz] = vpz[ir2];
        ray[nz++] = ir2;
      }
    if (nz < 2) {
      rc = -4;
      break;
    }
    double wsum = 0;
    for (int id = 0; id < nd; id++) {
      obs->rad[(size_t) id * nr + ir] = 0;
      obs->tau[(size_t) id * nr + ir] = 0;
    }
    for (int i = 0; i < c->nfov; i++) {
      const double zfov = vpz[ir] + c->fov_dz[i];
      const int idx = bracket_irr(zz, nz, zfov);
      for (int id = 0; id < nd; id++) {
        const double *r = rad0 + (size_t) id * nr, *t = tau0 + (size_t) id * nr;
        obs->rad[(size_t) id * nr + ir] +=
          c->fov_w[i] * lin(zz[idx], r[ray[idx]], zz[idx + 1], r[ray[idx + 1]], zfov);
        obs->tau[(size_t) id * nr + ir] +=
          c->fov_w[i] * lin(zz[idx], t[ray[idx]], zz[idx + 1], t[ray[idx + 1]], zfov);
      }
      wsum += c->fov_w[i];
    }
    for (int id = 0; id < nd; id++) {
      obs->rad[(size_t) id * nr + ir] /= wsum;
      obs->tau[(size_t) id * nr + ir] /= wsum;
    }
  }
  free(rad0);
  free(tau0);
  return rc;
}

int jrc_set_table(jrc_ctx *c, int id, int ig, int np, const double *p,
                  const int *nt, const double *t, const int *nu,
                  const float *u, const float *eps) {
  if (id < 0 || id >= c->nd || ig < 0 || ig >= c->ng) {
    set_err(c, "table index out of range");
    return -1;
  }
  if (np > c->cap_p) {
    set_err(c, "too many pressure levels");
    return -1;
  }
  const size_t dg = (size_t) id * (size_t) c->ng + (size_t) ig;
  c->tnp[dg] = np;
  for (int ip = 0; ip < np; ip++) {
    const size_t rp = dg * (size_t) c->cap_p + (size_t) ip;
    c->tp[rp] = p[ip];
    if (nt[ip] > c->cap_t) {
      set_err(c, "too many temperatures");
      return -1;
    }
    c->tnt[rp] = nt[ip];
    for (int it = 0; it < nt[ip]; it++) {
      const size_t src_pt = (size_t) ip * (size_t) c->cap_t + (size_t) it;
      const size_t rt = rp * (size_t) c->cap_t + (size_t) it;
      c->tt[rt] = t[src_pt];
      const int n = nu[src_pt];
      if (n > c->cap_u) {
        set_err(c, "too many column densities");
        return -1;
      }
      c->tnu[rt] = n;
      memcpy(c->tu + rt * (size_t) c->cap_u, u + src_pt * (size_t) c->cap_u,
             (size_t) n * sizeof(float));
      memcpy(c->teps + rt * (size_t) c->cap_u, eps + src_pt * (size_t) c->cap_u,
             (size_t) n * sizeof(float));
    }
  }
  return 0;
}

int jrc_set_continua(jrc_ctx *c, const double *blob, long n) {
  if (n != CT_TOTAL) {
    set_err(c, "continuum blob has the wrong size");
    return -1;
  }
  memcpy(c->ct, blob, sizeof(c->ct));
  c->have_ct = 1;
  return 0;
}

static inline double planck(double t, double nu) {
  return K_C1 * (nu * nu * nu) / expm1(K_C2 * nu / t);
}

/* init_srcfunc, jurassic.c:3631-3681: filter-weighted Planck function on
   1200 temperatures, trapezoid-free sum on the finest filter spacing. */
int jrc_init_srcfunc(jrc_ctx *c, int id, int n, const double *fnu,
                     const double *f) {
  if (n < 2 || id < 0 || id >= c->nd) {
    set_err(c, "bad filter function");
    return -1;
  }
  double dnu = 1.0;
  for (int i = 1; i < n; i++)
    if (fnu[i] - fnu[i - 1] < dnu)
      dnu = fnu[i] - fnu[i - 1];
  for (int it = 0; it < K_NS; it++) {
    const double temp = c->st[it];
    double fsum = 0, acc = 0;
    for (double v = fnu[0]; v <= fnu[n - 1]; v += dnu) {
      const int i = bracket_irr(fnu, n, v);
      const double w = lin(fnu[i], f[i], fnu[i + 1], f[i + 1], v);
      fsum += w;
      acc += w * planck(temp, v);
    }
    c->sr[(size_t) it * (size_t) c->nd + (size_t) id] = acc / fsum;
  }
  return 0;
}

void jrc_get_srcfunc(const jrc_ctx *c, double *st, double *sr) {
  memcpy(st, c->st, sizeof(c->st));
  memcpy(sr, c->sr, (size_t) K_NS * (size_t) c->nd * sizeof(double));
}

/* formod_srcfunc, jurassic.c:3483-3496 */
static void source_at(const jrc_ctx *c, double t, double *src) {
  const int it = bracket_reg(c->st, K_NS, t);
  const double *r0 = c->sr + (size_t) it * (size_t) c->nd;
  const double *r1 = r0 + c->nd;
  for (int id = 0; id < c->nd; id++)
    src[id] = lin(c->st[it], r0[id], c->st[it + 1], r1[id], t);
}

/* ---------------------------------------------------------------------- */
/* continua (ctmco2 886-1743, ctmh2o 1746-2793, ctmn2 2796-2858,           */
/* ctmo2 2861-2917, formod_continua 3075-3117)                             */

static double co2_continuum(const jrc_ctx *c, double nu, double p, double t,
                            double u) {
  const double xw = nu / 2 + 1;
  if (!(xw >= 1 && xw < CT_N))
    return 0;
  const int iw = (int) xw;
  const double dw = xw - iw, ew = 1 - dw;
  const double *t296 = c->ct + CT_CO2_296, *t260 = c->ct + CT_CO2_260,
    *t230 = c->ct + CT_CO2_230;
  const double c296 = ew * t296[iw - 1] + dw * t296[iw];
  const double c260 = ew * t260[iw - 1] + dw * t260[iw];
  const double c230 = ew * t230[iw - 1] + dw * t230[iw];
  const double d230 = t - 230, d260 = t - 260, d296 = t - 296;
  /* quadratic (Lagrange) interpolation in temperature through 230/260/296 K */
  const double ctw = d260 * 5.050505e-4 * d296 * c230 -
    d230 * 9.259259e-4 * d296 * c260 + d230 * 4.208754e-4 * d260 * c296;
  return u / K_NA / 1000 * p / K_P0 * ctw;
}

static double h2o_continuum(const jrc_ctx *c, double nu, double p, double t,
                            double q, double u) {
  const double xw = nu / 10 + 1;
  if (!(xw >= 1 && xw < CT_N))
    return 0;
  const int iw = (int) xw;
  const double dw = xw - iw, ew = 1 - dw;
  const double *s296 = c->ct + CT_H2O_296, *s260 = c->ct + CT_H2O_260,
    *frn = c->ct + CT_H2O_FRN, *xf = c->ct + CT_XFCREV;
  const double c296 = ew * s296[iw - 1] + dw * s296[iw];
  const double c260 = ew * s260[iw - 1] + dw * s260[iw];
  const double cfrn = ew * frn[iw - 1] + dw * frn[iw];
  double sfac = 1;
  if (!(nu <= 820 || nu >= 960)) {
    const double xx = (nu - 820) / 10;
    const int ix = (int) xx;
    const double dx = xx - ix;
    sfac = (1 - dx) * xf[ix] + dx * xf[ix + 1];
  }
  const double self = sfac * c296 * pow(c260 / c296, (296 - t) / (296 - 260));
  const double v2 = sq(nu - 370), v6 = v2 * v2 * v2;
  const double fscal = 36100 / (v2 + v6 * 1e-8 + 36100) * -.25 + 1;
  const double foreign = cfrn * fscal;
  const double a1 = nu * u * tanh(.7193876 / t * nu);
  const double a2 = 296 / t;
  const double a3 = p / K_P0 * (q * self + (1 - q) * foreign) * 1e-20;
  return a1 * a2 * a3;
}

static double cia_continuum(const double *b_tab, const double *beta_tab,
                            const double *nu_tab, int n, double nu, double p,
                            double t, int n2) {
  if (nu < nu_tab[0] || nu > nu_tab[n - 1])
    return 0;
  const int i = bracket_reg(nu_tab, n, nu);
  const double b = lin(nu_tab[i], b_tab[i], nu_tab[i + 1], b_tab[i + 1], nu);
  const double beta =
    lin(nu_tab[i], beta_tab[i], nu_tab[i + 1], beta_tab[i + 1], nu);
  if (n2) {
    const double qn = 0.79, t0 = 273.0, tr = 296.0;
    return 0.1 * sq(p / K_P0 * t0 / t) * exp(beta * (1 / tr - 1 / t)) * qn * b *
      (qn + (1 - qn) * (1.294 - 0.4545 * t / tr));
  }
  const double qo = 0.21, t0 = 273, tr = 296;
  return 0.1 * sq(p / K_P0 * t0 / t) * exp(beta * (1 / tr - 1 / t)) * qo * b;
}

static void continua_at(const jrc_ctx *c, const los_buf *l, int ip,
                        double *beta) {
  for (int id = 0; id < c->nd; id++)
    beta[id] = l->k[(size_t) ip * l->nd + id];
  if (c->ctm_co2 && c->ig_co2 >= 0)
    for (int id = 0; id < c->nd; id++)
      beta[id] += co2_continuum(c, c->nu[id], l->p[ip], l->t[ip],
                                l->u[(size_t) ip * l->ng + c->ig_co2]) / l->ds[ip];
  if (c->ctm_h2o && c->ig_h2o >= 0)
    for (int id = 0; id < c->nd; id++)
      beta[id] += h2o_continuum(c, c->nu[id], l->p[ip], l->t[ip],
                                l->q[(size_t) ip * l->ng + c->ig_h2o],
                                l->u[(size_t) ip * l->ng + c->ig_h2o]) / l->ds[ip];
  if (c->ctm_n2)
    for (int id = 0; id < c->nd; id++)
      beta[id] += cia_continuum(c->ct + CT_N2_B, c->ct + CT_N2_BETA,
                                c->ct + CT_N2_NU, 98, c->nu[id], l->p[ip],
                                l->t[ip], 1);
  if (c->ctm_o2)
    for (int id = 0; id < c->nd; id++)
      beta[id] += cia_continuum(c->ct + CT_O2_B, c->ct + CT_O2_BETA,
                                c->ct + CT_O2_NU, 90, c->nu[id], l->p[ip],
                                l->t[ip], 0);
}

/* ---------------------------------------------------------------------- */
/* emissivity tables                                                      */

typedef struct {
  const float *u, *eps;
  int n;
} tbl_row;

static inline tbl_row row_of(const jrc_ctx *c, int id, int ig, int ip, int it) {
  const size_t r = (((size_t) id * (size_t) c->ng + (size_t) ig) * (size_t) c->cap_p
                    + (size_t) ip) * (size_t) c->cap_t + (size_t) it;
  tbl_row row = { c->tu + r * (size_t) c->cap_u, c->teps + r * (size_t) c->cap_u,
                  c->tnu[r] };
  return row;
}

/* Linear interpolation between two float table entries.  The reference
   applies its LIN macro (jurassic.h:164) to float operands, so by C's usual
   arithmetic conversions the slope (y1-y0)/(x1-x0) is evaluated in single
   precision and only (x-x0) and the final sum in double.  Reproduced here
   exactly; x0 == 0, y0 == 0 gives the below-table branch. */
static inline double lin_f(float x0, float y0, float x1, float y1, double x) {
  const float slope = (y1 - y0) / (x1 - x0);
  return y0 + slope * (x - x0);
}

/* Emissivity at column density u on one row (intpol_tbl_eps,
   jurassic.c:3895-3929): linear from the origin below the first entry,
   Beer-law extrapolation above the last one. */
static double row_eps(tbl_row r, double u) {
  if (u < r.u[0])
    return lin_f(0.0f, 0.0f, r.u[0], r.eps[0], u);
  if (u > r.u[r.n - 1]) {
    const double a = log(1 - r.eps[r.n - 1]) / r.u[r.n - 1];
    return 1 - exp(a * u);
  }
  const int i = bracket_row(r.u, r.n, u);
  return lin_f(r.u[i], r.eps[i], r.u[i + 1], r.eps[i + 1], u);
}

/* Column density at emissivity eps on one row (intpol_tbl_u,
   jurassic.c:3933-3967), the inverse of row_eps. */
static double row_u(tbl_row r, double e) {
  if (e < r.eps[0])
    return lin_f(0.0f, 0.0f, r.eps[0], r.u[0], e);
  if (e > r.eps[r.n - 1]) {
    const double a = log(1 - r.eps[r.n - 1]) / r.u[r.n - 1];
    return log(1 - e) / a;
  }
  const int i = bracket_row(r.eps, r.n, e);
  return lin_f(r.eps[i], r.u[i], r.eps[i + 1], r.u[i + 1], e);
}

/* Segment transmittance per channel for LOS point ip, updating the path
   transmittance per (channel, emitter).  EGA: intpol_tbl_ega,
   jurassic.c:3799-3891; CGA: intpol_tbl_cga, jurassic.c:3710-3795. */
static void gas_transmittance(const jrc_ctx *c, const los_buf *l, int ip,
                              double *tau_path, double *tau_seg) {
  const int ng = c->ng;
  for (int id = 0; id < c->nd; id++) {
    tau_seg[id] = 1;
    for (int ig = 0; ig < ng; ig++) {
      const size_t dg = (size_t) id * (size_t) ng + (size_t) ig;
      double *tp = tau_path + dg;
      double eps;
      if (c->tnp[dg] < 30)
        eps = 0;
      else if (*tp < 1e-9)
        eps = 1;
      else {
        const double *pg = c->tp + dg * (size_t) c->cap_p;
        const int *ntg = c->tnt + dg * (size_t) c->cap_p;
        const double pq = c->formod == 0 ? l->cgp[(size_t) ip * ng + ig] : l->p[ip];
        const double tq = c->formod == 0 ? l->cgt[(size_t) ip * ng + ig] : l->t[ip];
        const int ipr = bracket_irr(pg, c->tnp[dg], pq);
        const double *t0g = c->tt + (dg * (size_t) c->cap_p + (size_t) ipr) * (size_t) c->cap_t;
        const double *t1g = t0g + c->cap_t;
        const int it0 = bracket_reg(t0g, ntg[ipr], tq);
        const int it1 = bracket_reg(t1g, ntg[ipr + 1], tq);
        tbl_row r00 = { 0, 0, 0 }, r01 = r00, r10 = r00, r11 = r00;
        const int rows_ok = ntg[ipr] >= 2 && ntg[ipr + 1] >= 2;
        if (rows_ok) {
          r00 = row_of(c, id, ig, ipr, it0);
          r01 = row_of(c, id, ig, ipr, it0 + 1);
          r10 = row_of(c, id, ig, ipr + 1, it1);
          r11 = row_of(c, id, ig, ipr + 1, it1 + 1);
        }
        if (!rows_ok || r00.n < 2 || r01.n < 2 || r10.n < 2 || r11.n < 2)
          eps = 0;
        else {
          double e00, e01, e10, e11;
          if (c->formod == 0) {
            const double ucg = l->cgu[(size_t) ip * ng + ig];
            e00 = row_eps(r00, ucg);
            e01 = row_eps(r01, ucg);
            e10 = row_eps(r10, ucg);
            e11 = row_eps(r11, ucg);
          } else {
            const double du = l->u[(size_t) ip * ng + ig];
            const double prev = 1 - *tp;
            e00 = row_eps(r00, row_u(r00, prev) + du);
            e01 = row_eps(r01, row_u(r01, prev) + du);
            e10 = row_eps(r10, row_u(r10, prev) + du);
            e11 = row_eps(r11, row_u(r11, prev) + du);
          }
          e00 = lin(t0g[it0], e00, t0g[it0 + 1], e01, tq);
          e11 = lin(t1g[it1], e10, t1g[it1 + 1], e11, tq);
          if (c->formod == 0)
            e00 = logx(pg[ipr], e00, pg[ipr + 1], e11, pq);
          else
            e00 = lin(pg[ipr], e00, pg[ipr + 1], e11, pq);
          e00 = e00 < 1 ? e00 : 1;
          e00 = e00 > 0 ? e00 : 0;
          eps = 1 - (1 - e00) / *tp;
        }
      }
      *tp *= (1 - eps);
      tau_seg[id] *= (1 - eps);
    }
  }
}

/* ---------------------------------------------------------------------- */
/* atmosphere                                                             */

typedef struct {
  int np, ng, nw, ncl, nsf;
  const double *z, *lon, *lat, *time;
  double *p, *t, *q, *k;
  double clz, cldz, sfz, sfp, sft;
  const double *clk, *sfeps;
} atm_view;

static atm_view view_of(const jrc_ctx *c, const jrc_atm *a) {
  atm_view v;
  v.np = a->np;
  v.ng = c->ng;
  v.nw = c->nw;
  v.ncl = c->ncl;
  v.nsf = c->nsf;
  v.z = a->z;
  v.lon = a->lon;
  v.lat = a->lat;
  v.time = a->time;
  v.p = a->p;
  v.t = a->t;
  v.q = a->q;
  v.k = a->k;
  int s = 0;
  v.clz = a->scal[s++];
  v.cldz = a->scal[s++];
  v.clk = a->scal + s;
  s += c->ncl;
  v.sfz = a->scal[s++];
  v.sfp = a->scal[s++];
  v.sft = a->scal[s++];
  v.sfeps = a->scal + s;
  return v;
}

/* intpol_atm, jurassic.c:3685-3706 */
static void atm_at(const atm_view *a, double z, double *p, double *t,
                   double *q, double *k) {
  const int i = bracket_irr(a->z, a->np, z);
  *p = logy(a->z[i], a->p[i], a->z[i + 1], a->p[i + 1], z);
  *t = lin(a->z[i], a->t[i], a->z[i + 1], a->t[i + 1], z);
  for (int ig = 0; ig < a->ng; ig++)
    q[ig] = lin(a->z[i], a->q[ig * a->np + i], a->z[i + 1],
                a->q[ig * a->np + i + 1], z);
  for (int iw = 0; iw < a->nw; iw++)
    k[iw] = lin(a->z[i], a->k[iw * a->np + i], a->z[i + 1],
                a->k[iw * a->np + i + 1], z);
}

/* hydrostatic, jurassic.c:3520-3582: rebuild p(z) from T and H2O,
   integrating upward and downward from the level nearest HYDZ. */
static void hydrostatic_fill(const jrc_ctx *c, atm_view *a) {
  if (c->hydz < 0)
    return;
  const double mmair = 28.96456e-3, mmh2o = 18.0153e-3;
  const int npts = 20;
  double best = 1e99, e = 0;
  int iref = 0;
  for (int ip = 0; ip < a->np; ip++)
    if (fabs(a->z[ip] - c->hydz) < best) {
      best = fabs(a->z[ip] - c->hydz);
      iref = ip;
    }
  const double *qw = c->ig_h2o >= 0 ? a->q + (size_t) c->ig_h2o * a->np : NULL;
  for (int ip = iref + 1; ip < a->np; ip++) {
    double mean = 0;
    for (int i = 0; i < npts; i++) {
      if (qw)
        e = lin(0.0, qw[ip - 1], npts - 1.0, qw[ip], (double) i);
      mean += (e * mmh2o + (1 - e) * mmair) * K_G0 / K_RI /
        lin(0.0, a->t[ip - 1], npts - 1.0, a->t[ip], (double) i) / npts;
    }
    a->p[ip] = exp(log(a->p[ip - 1]) - mean * 1000 * (a->z[ip] - a->z[ip - 1]));
  }
  for (int ip = iref - 1; ip >= 0; ip--) {
    double mean = 0;
    for (int i = 0; i < npts; i++) {
      if (qw)
        e = lin(0.0, qw[ip + 1], npts - 1.0, qw[ip], (double) i);
      mean += (e * mmh2o + (1 - e) * mmair) * K_G0 / K_RI /
        lin(0.0, a->t[ip + 1], npts - 1.0, a->t[ip], (double) i) / npts;
    }
    a->p[ip] = exp(log(a->p[ip + 1]) - mean * 1000 * (a->z[ip] - a->z[ip + 1]));
  }
}

/* ---------------------------------------------------------------------- */
/* line of sight                                                          */

static int los_alloc(los_buf *l, int cap, int ng, int nd) {
  memset(l, 0, sizeof(*l));
  l->cap = cap;
  l->ng = ng;
  l->nd = nd;
  const size_t n = (size_t) cap;
  l->z = malloc(n * sizeof(double));
  l->lon = malloc(n * sizeof(double));
  l->lat = malloc(n * sizeof(double));
  l->p = malloc(n * sizeof(double));
  l->t = malloc(n * sizeof(double));
  l->ds = malloc(n * sizeof(double));
  l->q = malloc(n * (size_t) (ng + 1) * sizeof(double));
  l->u = malloc(n * (size_t) (ng + 1) * sizeof(double));
  l->cgp = malloc(n * (size_t) (ng + 1) * sizeof(double));
  l->cgt = malloc(n * (size_t) (ng + 1) * sizeof(double));
  l->cgu = malloc(n * (size_t) (ng + 1) * sizeof(double));
  l->k = malloc(n * (size_t) (nd + 1) * sizeof(double));
  l->eps = malloc(n * (size_t) (nd + 1) * sizeof(double));
  l->src = malloc(n * (size_t) (nd + 1) * sizeof(double));
  l->sfeps = malloc((size_t) (nd + 1) * sizeof(double));
  return (l->z && l->k && l->eps && l->src) ? 0 : -1;
}

static void los_free(los_buf *l) {
  free(l->z); free(l->lon); free(l->lat); free(l->p); free(l->t); free(l->ds);
  free(l->q); free(l->u); free(l->cgp); free(l->cgt); free(l->cgu);
  free(l->k); free(l->eps); free(l->src); free(l->sfeps);
}

/* Tangent point from a parabola through the lowest LOS point and its two
   neighbours (tangent_point, jurassic.c:5223-5263); nadir/zenith rays take
   the last LOS point.  Uses the raw (pre-trapezoid) step lengths. */
static void tangent_of(const los_buf *l, double *tpz, double *tplon,
                       double *tplat) {
  int imin = 0;
  for (int i = 1; i < l->np; i++)
    if (l->z[i] < l->z[imin])
      imin = i;
  if (imin <= 0 || imin >= l->np - 1) {
    *tpz = l->z[l->np - 1];
    *tplon = l->lon[l->np - 1];
    *tplat = l->lat[l->np - 1];
    return;
  }
  const double y0 = l->z[imin - 1], y1 = l->z[imin], y2 = l->z[imin + 1];
  const double x1 = sqrt(sq(l->ds[imin]) - sq(y1 - y0));
  const double x2 = x1 + sqrt(sq(l->ds[imin + 1]) - sq(y2 - y1));
  const double a = 1 / (x1 - x2) * (-(y0 - y1) / x1 + (y0 - y2) / x2);
  const double b = -(y0 - y1) / x1 - a * x1;
  const double cc = y0;
  const double xt = -b / (2 * a);
  *tpz = a * xt * xt + b * xt + cc;
  double v0[3], v2[3], v[3], dummy;
  to_cart(l->z[imin - 1], l->lon[imin - 1], l->lat[imin - 1], v0);
  to_cart(l->z[imin + 1], l->lon[imin + 1], l->lat[imin + 1], v2);
  for (int i = 0; i < 3; i++)
    v[i] = lin(0.0, v0[i], x2, v2[i], xt);
  to_geo(v, &dummy, tplon, tplat);
}

#define REFRACTIVITY(p, t) (7.753e-05 * (p) / (t)) /* REFRAC, jurassic.h:197 */

/* Ray tracing (raytrace, jurassic.c:4201-4438): entry-point bisection for
   observers above the atmosphere, steps of min(RAYDS, RAYDZ/cos(zenith)),
   refraction below 60 km, clipping at ground/top, trapezoid segment
   lengths, column densities and Curtis-Godson means. */
static int trace(const jrc_ctx *c, const atm_view *a, const double *geo,
                 int nr, int ir, los_buf *l, double *tp3) {
  const double h = 0.02, zrefrac = 60;
  const int ng = c->ng, nd = c->nd, nw = c->nw;
  double ex0[3], ex1[3], x[3], xh[3], xobs[3], xvp[3], ngr[3];
  double q[64], kk[64];
  double z = 1e99, lon, lat, p, t, nref;
  int stop = 0;
  const double obsz = geo[1 * nr + ir], obslon = geo[2 * nr + ir],
    obslat = geo[3 * nr + ir], vpz = geo[4 * nr + ir],
    vplon = geo[5 * nr + ir], vplat = geo[6 * nr + ir];

  l->np = 0;
  l->sft = -999;
  tp3[0] = vpz;
  tp3[1] = vplon;
  tp3[2] = vplat;

  double zmin = a->z[0], zmax = a->z[0];
  for (int i = 0; i < a->np; i++) {
    if (a->z[i] < zmin)
      zmin = a->z[i];
    if (a->z[i] > zmax)
      zmax = a->z[i];
  }
  if (c->nsf > 0) {
    zmin = a->sfz > zmin ? a->sfz : zmin;
    if (a->sfp > 0) {
      const int i = bracket_irr(a->p, a->np, a->sfp);
      const double zs = lin(log(a->p[i]), a->z[i], log(a->p[i + 1]),
                            a->z[i + 1], log(a->sfp));
      zmin = zs > zmin ? zs : zmin;
    }
  }
  if (obsz < zmin)
    return -2; /* observer below surface */
  if (vpz > zmax)
    return 0;

  to_cart(obsz, obslon, obslat, xobs);
  to_cart(vpz, vplon, vplat, xvp);
  for (int i = 0; i < 3; i++)
    ex0[i] = xvp[i] - xobs[i];
  double norm = sqrt(ex0[0] * ex0[0] + ex0[1] * ex0[1] + ex0[2] * ex0[2]);
  for (int i = 0; i < 3; i++)
    ex0[i] /= norm;
  for (int i = 0; i < 3; i++)
    x[i] = xobs[i];

  if (obsz > zmax) {
    double dmax = norm, dmin = 0;
    while (fabs(dmin - dmax) > 0.001) {
      const double d = (dmax + dmin) / 2;
      for (int i = 0; i < 3; i++)
        x[i] = xobs[i] + d * ex0[i];
      to_geo(x, &z, &lon, &lat);
      if (z <= zmax && z > zmax - 0.001)
        break;
      if (z < zmax - 0.0005)
        dmax = d;
      else
        dmin = d;
    }
  }

  for (;;) {
    double ds = c->rayds;
    if (c->raydz > 0) {
      norm = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      for (int i = 0; i < 3; i++)
        xh[i] = x[i] / norm;
      const double cosa = fabs(ex0[0] * xh[0] + ex0[1] * xh[1] + ex0[2] * xh[2]);
      if (cosa != 0)
        ds = c->rayds < c->raydz / cosa ? c->rayds : c->raydz / cosa;
    }
    to_geo(x, &z, &lon, &lat);
    if ((z < zmin || z > zmax) && l->np > 0) {
      stop = (z < zmin ? 2 : 1);
      const int last = l->np - 1;
      const double frac = ((z < zmin ? zmin : zmax) - l->z[last]) / (z - l->z[last]);
      to_cart(l->z[last], l->lon[last], l->lat[last], xh);
      for (int i = 0; i < 3; i++)
        x[i] = xh[i] + frac * (x[i] - xh[i]);
      to_geo(x, &z, &lon, &lat);
      l->ds[last] = ds * frac;
      ds = 0;
    }
    atm_at(a, z, &p, &t, q, kk);
    const int n = l->np;
    if (n >= l->cap)
      return -3; /* too many LOS points */
    l->lon[n] = lon;
    l->lat[n] = lat;
    l->z[n] = z;
    l->p[n] = p;
    l->t[n] = t;
    for (int ig = 0; ig < ng; ig++)
      l->q[(size_t) n * ng + ig] = q[ig];
    for (int id = 0; id < nd; id++)
      l->k[(size_t) n * nd + id] = nw > 0 ? kk[c->window[id]] : 0;
    l->ds[n] = ds;
    if (c->ncl > 0 && a->cldz > 0) {
      const double aux = exp(-0.5 * sq((z - a->clz) / a->cldz));
      for (int id = 0; id < nd; id++) {
        const int icl = bracket_irr(c->clnu, c->ncl, c->nu[id]);
        l->k[(size_t) n * nd + id] += aux * lin(c->clnu[icl], a->clk[icl],
                                                c->clnu[icl + 1], a->clk[icl + 1],
                                                c->nu[id]);
      }
    }
    l->np++;
    if (stop) {
      if (c->nsf > 0 && a->sft > 0)
        t = a->sft;
      l->sft = (stop == 2 ? t : -999);
      for (int id = 0; id < nd; id++) {
        l->sfeps[id] = 1.0;
        if (c->nsf > 0) {
          const int isf = bracket_irr(c->sfnu, c->nsf, c->nu[id]);
          l->sfeps[id] = lin(c->sfnu[isf], a->sfeps[isf], c->sfnu[isf + 1],
                             a->sfeps[isf + 1], c->nu[id]);
        }
      }
      break;
    }
    const int bend = c->refrac && z <= zrefrac;
    nref = bend ? 1 + REFRACTIVITY(p, t) : 1;
    for (int i = 0; i < 3; i++)
      ex1[i] = ex0[i] * nref;
    if (bend) {
      for (int i = 0; i < 3; i++)
        xh[i] = x[i] + 0.5 * ds * ex0[i];
      to_geo(xh, &z, &lon, &lat);
      atm_at(a, z, &p, &t, q, kk);
      nref = REFRACTIVITY(p, t);
      for (int i = 0; i < 3; i++) {
        xh[i] += h;
        to_geo(xh, &z, &lon, &lat);
        atm_at(a, z, &p, &t, q, kk);
        ngr[i] = (REFRACTIVITY(p, t) - nref) / h;
        xh[i] -= h;
      }
    } else
      ngr[0] = ngr[1] = ngr[2] = 0;
    for (int i = 0; i < 3; i++)
      ex1[i] += ds * ngr[i];
    norm = sqrt(ex1[0] * ex1[0] + ex1[1] * ex1[1] + ex1[2] * ex1[2]);
    for (int i = 0; i < 3; i++)
      ex1[i] /= norm;
    for (int i = 0; i < 3; i++)
      x[i] += 0.5 * ds * (ex0[i] + ex1[i]);
    for (int i = 0; i < 3; i++)
      ex0[i] = ex1[i];
  }

  tangent_of(l, &tp3[0], &tp3[1], &tp3[2]);

  for (int ip = l->np - 1; ip >= 1; ip--)
    l->ds[ip] = 0.5 * (l->ds[ip - 1] + l->ds[ip]);
  l->ds[0] *= 0.5;

  for (int ip = 0; ip < l->np; ip++)
    for (int ig = 0; ig < ng; ig++)
      l->u[(size_t) ip * ng + ig] =
        10 * l->q[(size_t) ip * ng + ig] * l->p[ip] / (K_KB * l->t[ip]) * l->ds[ip];

  for (int ig = 0; ig < ng; ig++) {
    l->cgu[ig] = l->u[ig];
    l->cgp[ig] = l->u[ig] * l->p[0];
    l->cgt[ig] = l->u[ig] * l->t[0];
  }
  for (int ip = 1; ip < l->np; ip++)
    for (int ig = 0; ig < ng; ig++) {
      const size_t i = (size_t) ip * ng + ig, j = i - ng;
      l->cgu[i] = l->cgu[j] + l->u[i];
      l->cgp[i] = l->cgp[j] + l->u[i] * l->p[ip];
      l->cgt[i] = l->cgt[j] + l->u[i] * l->t[ip];
    }
  for (int ip = 0; ip < l->np; ip++)
    for (int ig = 0; ig < ng; ig++) {
      const size_t i = (size_t) ip * ng + ig;
      l->cgp[i] /= l->cgu[i];
      l->cgt[i] /= l->cgu[i];
    }
  return l->np;
}

/* ---------------------------------------------------------------------- */
/* forward model                                                          */

/* Radiative transfer along one pencil beam (formod_pencil,
   jurassic.c:3196-3338), including surface emission, reflection of
   down-welling radiance and the solar term. */
static int pencil(const jrc_ctx *c, const atm_view *a, const double *geo,
                  int nr, int ir, los_buf *l, double *work, double *rad_out,
                  double *tau_out, double *tp3) {
  const int nd = c->nd, ng = c->ng;
  double *rad = work, *tau = work + nd, *tau_gas = work + 2 * nd,
    *beta = work + 3 * nd, *tau_path = work + 4 * nd;
  for (int id = 0; id < nd; id++) {
    rad[id] = 0;
    tau[id] = 1;
    for (int ig = 0; ig < ng; ig++)
      tau_path[id * ng + ig] = 1;
  }
  const int rc = trace(c, a, geo, nr, ir, l, tp3);
  if (rc < 0)
    return rc;
  for (int ip = 0; ip < l->np; ip++) {
    gas_transmittance(c, l, ip, tau_path, tau_gas);
    continua_at(c, l, ip, beta);
    double *src = l->src + (size_t) ip * nd;
    double *eps = l->eps + (size_t) ip * nd;
    source_at(c, l->t[ip], src);
    for (int id = 0; id < nd; id++) {
      eps[id] = 0; /* the reference leaves skipped entries unset */
      if (tau_gas[id] > 0) {
        eps[id] = 1 - tau_gas[id] * exp(-beta[id] * l->ds[ip]);
        rad[id] += src[id] * eps[id] * tau[id];
        tau[id] *= (1 - eps[id]);
      }
    }
  }
  if (c->sftype >= 1 && l->sft > 0) {
    double *src_sf = beta; /* reuse */
    source_at(c, l->sft, src_sf);
    for (int id = 0; id < nd; id++)
      rad[id] += l->sfeps[id] * src_sf[id] * tau[id];
    int refl = 0;
    if (c->sftype >= 2)
      for (int id = 0; id < nd; id++)
        if (l->sfeps[id] < 1) {
          refl = 1;
          break;
        }
    if (refl) {
      double *tau_refl = tau_gas; /* reuse */
      for (int id = 0; id < nd; id++)
        tau_refl[id] = 1;
      for (int ip = l->np - 1; ip >= 0; ip--)
        for (int id = 0; id < nd; id++) {
          const double e = l->eps[(size_t) ip * nd + id];
          rad[id] += l->src[(size_t) ip * nd + id] * e * tau_refl[id] * tau[id] *
            (1 - l->sfeps[id]);
          tau_refl[id] *= (1 - e);
        }
      if (c->sftype >= 3) {
        const int last = l->np - 1;
        const double s = c->sfsza < 0 ?
          solar_zenith(geo[ir], l->lon[last], l->lat[last]) : c->sfsza;
        if (s < 89.999) {
          double x0[3], x1[3];
          to_cart(l->z[last], l->lon[last], l->lat[last], x0);
          to_cart(l->z[0], l->lon[0], l->lat[0], x1);
          for (int i = 0; i < 3; i++)
            x1[i] -= x0[i];
          const double cosa = (x0[0] * x1[0] + x0[1] * x1[1] + x0[2] * x1[2]) /
            sqrt(x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2]) /
            sqrt(x1[0] * x1[0] + x1[1] * x1[1] + x1[2] * x1[2]);
          const double rcos = cosa / cos(s * (K_PI / 180.0));
          for (int id = 0; id < nd; id++)
            rad[id] += 6.764e-5 / (2. * K_PI) * planck(K_TSUN, c->nu[id]) *
              tau_refl[id] * (1 - l->sfeps[id]) * tau[id] * rcos;
        }
      }
    }
  }
  for (int id = 0; id < nd; id++) {
    rad_out[(size_t) id * nr + ir] = rad[id];
    tau_out[(size_t) id * nr + ir] = tau[id];
  }
  return 0;
}

/* formod, jurassic.c:3026-3071: mask, hydrostatic, pencil beams, BT, mask. */
static int formod_one(const jrc_ctx *c, const jrc_atm *atm, jrc_obs *obs,
                      los_buf *l, double *work) {
  const int nd = c->nd, nr = obs->nr;
  atm_view a = view_of(c, atm);
  unsigned char *mask = (unsigned char *) malloc((size_t) (nd * nr + 1));
  for (int id = 0; id < nd; id++)
    for (int ir = 0; ir < nr; ir++)
      mask[id * nr + ir] = !isfinite(obs->rad[(size_t) id * nr + ir]);
  hydrostatic_fill(c, &a);
  int rc = 0;
  for (int ir = 0; ir < nr && rc == 0; ir++) {
    double tp3[3];
    rc = pencil(c, &a, obs->geo, nr, ir, l, work, obs->rad, obs->tau, tp3);
    obs->tp[0 * nr + ir] = tp3[0];
    obs->tp[1 * nr + ir] = tp3[1];
    obs->tp[2 * nr + ir] = tp3[2];
  }
  if (rc == 0 && c->nfov > 0)
    rc = fov_apply(c, obs);
  if (c->write_bbt)
    for (int id = 0; id < nd; id++)
      for (int ir = 0; ir < nr; ir++) {
        const double nu = c->nu[id];
        double *r = &obs->rad[(size_t) id * nr + ir];
        *r = K_C2 * nu / log1p(K_C1 * (nu * nu * nu) / *r);
      }
  for (int id = 0; id < nd; id++)
    for (int ir = 0; ir < nr; ir++)
      if (mask[id * nr + ir])
        obs->rad[(size_t) id * nr + ir] = NAN;
  free(mask);
  return rc;
}

static double *work_alloc(const jrc_ctx *c) {
  return (double *) malloc((size_t) (4 * c->nd + c->nd * c->ng + 8) * sizeof(double));
}

int jrc_formod(jrc_ctx *c, jrc_atm *atm, jrc_obs *obs) {
  los_buf l;
  if (los_alloc(&l, c->nlos_max, c->ng, c->nd)) {
    set_err(c, "out of memory");
    return -1;
  }
  double *work = work_alloc(c);
  const int rc = formod_one(c, atm, obs, &l, work);
  free(work);
  los_free(&l);
  if (rc == -2)
    set_err(c, "Observer below surface!");
  if (rc == -3)
    set_err(c, "Too many LOS points!");
  if (rc == -4)
    set_err(c, "Cannot apply FOV convolution!");
  return rc;
}

int jrc_formod_batch(jrc_ctx *c, int nobs, const int *lev_off,
                     const double *time, const double *z, const double *lon,
                     const double *lat, double *p, double *t, double *q,
                     double *k, double *scal, const int *ray_off,
                     const double *geo, double *rad, double *tau, double *tp,
                     int nthreads) {
  const int nlev = lev_off[nobs], nray = ray_off[nobs];
  const int nscal = 5 + c->ncl + c->nsf;
  int fail = 0;
#ifdef _OPENMP
  if (nthreads <= 0)
    nthreads = omp_get_max_threads();
#else
  (void) nthreads;
#endif
#pragma omp parallel num_threads(nthreads)
  {
    los_buf l;
    const int ok = los_alloc(&l, c->nlos_max, c->ng, c->nd) == 0;
    double *work = work_alloc(c);
    /* per-thread staging in the single-observation layout */
    int maxr = 0, maxl = 0;
    for (int i = 0; i < nobs; i++) {
      if (ray_off[i + 1] - ray_off[i] > maxr)
        maxr = ray_off[i + 1] - ray_off[i];
      if (lev_off[i + 1] - lev_off[i] > maxl)
        maxl = lev_off[i + 1] - lev_off[i];
    }
    double *g = malloc((size_t) (7 * maxr + 1) * sizeof(double));
    double *r = malloc((size_t) (c->nd * maxr + 1) * sizeof(double));
    double *ta = malloc((size_t) (c->nd * maxr + 1) * sizeof(double));
    double *tpp = malloc((size_t) (3 * maxr + 1) * sizeof(double));
    double *qq = malloc((size_t) (c->ng * maxl + 1) * sizeof(double));
    double *kk = malloc((size_t) (c->nw * maxl + 1) * sizeof(double));
    double *pp = malloc((size_t) (maxl + 1) * sizeof(double));
#pragma omp for schedule(dynamic, 1)
    for (int i = 0; i < nobs; i++) {
      if (!ok || fail)
        continue;
      const int l0 = lev_off[i], nl = lev_off[i + 1] - lev_off[i];
      const int r0 = ray_off[i], nrr = ray_off[i + 1] - ray_off[i];
      for (int ig = 0; ig < c->ng; ig++)
        memcpy(qq + (size_t) ig * nl, q + (size_t) ig * nlev + l0, (size_t) nl * sizeof(double));
      for (int iw = 0; iw < c->nw; iw++)
        memcpy(kk + (size_t) iw * nl, k + (size_t) iw * nlev + l0, (size_t) nl * sizeof(double));
      memcpy(pp, p + l0, (size_t) nl * sizeof(double));
      for (int j = 0; j < 7; j++)
        memcpy(g + (size_t) j * nrr, geo + (size_t) j * nray + r0, (size_t) nrr * sizeof(double));
      for (int id = 0; id < c->nd; id++)
        memcpy(r + (size_t) id * nrr, rad + (size_t) id * nray + r0, (size_t) nrr * sizeof(double));
      jrc_atm a = { nl, time + l0, z + l0, lon + l0, lat + l0, pp, t + l0, qq, kk,
                    scal + (size_t) i * nscal };
      jrc_obs o = { nrr, g, r, ta, tpp };
      if (formod_one(c, &a, &o, &l, work) != 0) {
        fail = 1;
        continue;
      }
      memcpy(p + l0, pp, (size_t) nl * sizeof(double));
      for (int id = 0; id < c->nd; id++) {
        memcpy(rad + (size_t) id * nray + r0, r + (size_t) id * nrr, (size_t) nrr * sizeof(double));
        memcpy(tau + (size_t) id * nray + r0, ta + (size_t) id * nrr, (size_t) nrr * sizeof(double));
      }
      for (int j = 0; j < 3; j++)
        memcpy(tp + (size_t) j * nray + r0, tpp + (size_t) j * nrr, (size_t) nrr * sizeof(double));
    }
    free(g); free(r); free(ta); free(tpp); free(qq); free(kk); free(pp);
    free(work);
    if (ok)
      los_free(&l);
  }
  if (fail) {
    set_err(c, "forward model failed for an observation");
    return -1;
  }
  return 0;
}

int jrc_raytrace(jrc_ctx *c, const jrc_atm *atm, jrc_obs *obs, int ir,
                 int maxpts, double *out) {
  los_buf l;
  if (los_alloc(&l, c->nlos_max, c->ng, c->nd))
    return -1;
  atm_view a = view_of(c, atm);
  double tp3[3];
  const int nr = obs->nr;
  int np = trace(c, &a, obs->geo, nr, ir, &l, tp3);
  obs->tp[0 * nr + ir] = tp3[0];
  obs->tp[1 * nr + ir] = tp3[1];
  obs->tp[2 * nr + ir] = tp3[2];
  if (np > maxpts)
    np = -4;
  const int ng = c->ng, nd = c->nd, w = 7 + 5 * ng + 2 * nd;
  for (int ip = 0; ip < np; ip++) {
    double *r = out + (size_t) ip * w;
    int col = 0;
    r[col++] = l.z[ip];
    r[col++] = l.lon[ip];
    r[col++] = l.lat[ip];
    r[col++] = l.p[ip];
    r[col++] = l.t[ip];
    r[col++] = l.ds[ip];
    r[col++] = l.sft;
    for (int ig = 0; ig < ng; ig++) r[col++] = l.q[(size_t) ip * ng + ig];
    for (int ig = 0; ig < ng; ig++) r[col++] = l.u[(size_t) ip * ng + ig];
    for (int ig = 0; ig < ng; ig++) r[col++] = l.cgp[(size_t) ip * ng + ig];
    for (int ig = 0; ig < ng; ig++) r[col++] = l.cgt[(size_t) ip * ng + ig];
    for (int ig = 0; ig < ng; ig++) r[col++] = l.cgu[(size_t) ip * ng + ig];
    for (int id = 0; id < nd; id++) r[col++] = l.k[(size_t) ip * nd + id];
    for (int id = 0; id < nd; id++) r[col++] = l.sfeps[id];
  }
  los_free(&l);
  return np;
}

/* ---------------------------------------------------------------------- */
/* state and measurement vectors (atm2x 29-104, x2atm 5896-5958,          */
/* obs2y 4174-4197)                                                        */

/* Quantity indices (jurassic.h:449-485). */
#define Q_P 0
#define Q_T 1
#define Q_Q(ig) (2 + (ig))
#define Q_K(c, iw) (2 + (c)->ng + (iw))
#define Q_CLZ(c) (2 + (c)->ng + (c)->nw)
#define Q_CLDZ(c) (3 + (c)->ng + (c)->nw)
#define Q_CLK(c, icl) (4 + (c)->ng + (c)->nw + (icl))
#define Q_SFZ(c) (4 + (c)->ng + (c)->nw + (c)->ncl)
#define Q_SFP(c) (5 + (c)->ng + (c)->nw + (c)->ncl)
#define Q_SFT(c) (6 + (c)->ng + (c)->nw + (c)->ncl)
#define Q_SFEPS(c, isf) (7 + (c)->ng + (c)->nw + (c)->ncl + (isf))

/* Visits every retrieved state element in atm2x order; op 0 = gather
   (value -> x), op 1 = scatter (x -> value). */
static int state_walk(const jrc_ctx *c, const jrc_atm *atm, double *x,
                      int *iqa, int *ipa, int op) {
  int n = 0;
  const int np = atm->np;
#define VISIT(ptr, q, ip)                          \
  do {                                             \
    if (op == 0 && x) x[n] = *(ptr);               \
    if (op == 1) *(ptr) = x[n];                    \
    if (iqa) iqa[n] = (q);                         \
    if (ipa) ipa[n] = (ip);                        \
    n++;                                           \
  } while (0)
  for (int ip = 0; ip < np; ip++)
    if (atm->z[ip] >= c->retp_zmin && atm->z[ip] <= c->retp_zmax)
      VISIT(&atm->p[ip], Q_P, ip);
  for (int ip = 0; ip < np; ip++)
    if (atm->z[ip] >= c->rett_zmin && atm->z[ip] <= c->rett_zmax)
      VISIT(&atm->t[ip], Q_T, ip);
  for (int ig = 0; ig < c->ng; ig++)
    for (int ip = 0; ip < np; ip++)
      if (atm->z[ip] >= c->retq_zmin[ig] && atm->z[ip] <= c->retq_zmax[ig])
        VISIT(&atm->q[(size_t) ig * np + ip], Q_Q(ig), ip);
  for (int iw = 0; iw < c->nw; iw++)
    for (int ip = 0; ip < np; ip++)
      if (atm->z[ip] >= c->retk_zmin[iw] && atm->z[ip] <= c->retk_zmax[iw])
        VISIT(&atm->k[(size_t) iw * np + ip], Q_K(c, iw), ip);
  double *s = atm->scal;
  if (c->ret_clz) VISIT(&s[0], Q_CLZ(c), 0);
  if (c->ret_cldz) VISIT(&s[1], Q_CLDZ(c), 0);
  if (c->ret_clk)
    for (int icl = 0; icl < c->ncl; icl++) VISIT(&s[2 + icl], Q_CLK(c, icl), 0);
  const int o = 2 + c->ncl;
  if (c->ret_sfz) VISIT(&s[o], Q_SFZ(c), 0);
  if (c->ret_sfp) VISIT(&s[o + 1], Q_SFP(c), 0);
  if (c->ret_sft) VISIT(&s[o + 2], Q_SFT(c), 0);
  if (c->ret_sfeps)
    for (int isf = 0; isf < c->nsf; isf++) VISIT(&s[o + 3 + isf], Q_SFEPS(c, isf), 0);
#undef VISIT
  return n;
}

int jrc_atm2x(const jrc_ctx *c, const jrc_atm *atm, double *x, int *iqa,
              int *ipa) {
  return state_walk(c, atm, x, iqa, ipa, 0);
}

static int meas_gather(const jrc_ctx *c, const jrc_obs *obs, double *y) {
  int m = 0;
  for (int ir = 0; ir < obs->nr; ir++)
    for (int id = 0; id < c->nd; id++) {
      const double v = obs->rad[(size_t) id * obs->nr + ir];
      if (isfinite(v)) {
        if (y)
          y[m] = v;
        m++;
      }
    }
  return m;
}

int jrc_sizes(const jrc_ctx *c, const jrc_atm *atm, const jrc_obs *obs,
              int *m, int *n) {
  *m = meas_gather(c, obs, NULL);
  *n = state_walk(c, atm, NULL, NULL, NULL, 0);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* Jacobian (kernel, jurassic.c:4004-4099)                                */

typedef struct {
  int np, nr, nscal;
  double *p, *t, *q, *k, *scal;
  double *rad, *tau, *tp;
} scratch_state;

static void scratch_init(const jrc_ctx *c, scratch_state *s, int np, int nr) {
  s->np = np;
  s->nr = nr;
  s->nscal = 5 + c->ncl + c->nsf;
  s->p = malloc((size_t) np * sizeof(double));
  s->t = malloc((size_t) np * sizeof(double));
  s->q = malloc((size_t) (c->ng * np + 1) * sizeof(double));
  s->k = malloc((size_t) (c->nw * np + 1) * sizeof(double));
  s->scal = malloc((size_t) s->nscal * sizeof(double));
  s->rad = malloc((size_t) (c->nd * nr + 1) * sizeof(double));
  s->tau = malloc((size_t) (c->nd * nr + 1) * sizeof(double));
  s->tp = malloc((size_t) (3 * nr) * sizeof(double));
}

static void scratch_free(scratch_state *s) {
  free(s->p); free(s->t); free(s->q); free(s->k); free(s->scal);
  free(s->rad); free(s->tau); free(s->tp);
}

static void scratch_load_atm(const jrc_ctx *c, scratch_state *s, const jrc_atm *a) {
  memcpy(s->p, a->p, (size_t) a->np * sizeof(double));
  memcpy(s->t, a->t, (size_t) a->np * sizeof(double));
  memcpy(s->q, a->q, (size_t) (c->ng * a->np) * sizeof(double));
  memcpy(s->k, a->k, (size_t) (c->nw * a->np) * sizeof(double));
  memcpy(s->scal, a->scal, (size_t) s->nscal * sizeof(double));
}

static double fd_step(const jrc_ctx *c, int q, double x) {
  if (q == Q_P) return fmax(fabs(0.01 * x), 1e-7);
  if (q == Q_T) return 1.0;
  if (q >= Q_Q(0) && q < Q_Q(c->ng)) return fmax(fabs(0.01 * x), 1e-15);
  if (q >= Q_K(c, 0) && q < Q_K(c, c->nw)) return 1e-4;
  if (q == Q_CLZ(c) || q == Q_CLDZ(c)) return 1.0;
  if (q >= Q_CLK(c, 0) && q < Q_CLK(c, c->ncl)) return 1e-4;
  if (q == Q_SFZ(c)) return 0.1;
  if (q == Q_SFP(c)) return 10.0;
  if (q == Q_SFT(c)) return 1.0;
  if (q >= Q_SFEPS(c, 0) && q < Q_SFEPS(c, c->nsf)) return 1e-2;
  return NAN;
}

int jrc_kernel(jrc_ctx *c, jrc_atm *atm, jrc_obs *obs, double *kmat,
               int nthreads) {
  int rc = jrc_formod(c, atm, obs);
  if (rc)
    return rc;
  int m, n;
  jrc_sizes(c, atm, obs, &m, &n);
  double *x0 = malloc((size_t) (n + 1) * sizeof(double));
  double *y0 = malloc((size_t) (m + 1) * sizeof(double));
  int *iqa = malloc((size_t) (n + 1) * sizeof(int));
  state_walk(c, atm, x0, iqa, NULL, 0);
  meas_gather(c, obs, y0);
  memset(kmat, 0, (size_t) m * (size_t) n * sizeof(double));
  int fail = 0;
#ifdef _OPENMP
  if (nthreads <= 0)
    nthreads = omp_get_max_threads();
#else
  (void) nthreads;
#endif
#pragma omp parallel num_threads(nthreads)
  {
    los_buf l;
    const int ok = los_alloc(&l, c->nlos_max, c->ng, c->nd) == 0;
    double *work = work_alloc(c);
    scratch_state s;
    scratch_init(c, &s, atm->np, obs->nr);
    double *x1 = malloc((size_t) (n + 1) * sizeof(double));
    double *y1 = malloc((size_t) (m + 1) * sizeof(double));
#pragma omp for schedule(dynamic, 1)
    for (int j = 0; j < n; j++) {
      if (!ok || fail)
        continue;
      const double h = fd_step(c, iqa[j], x0[j]);
      memcpy(x1, x0, (size_t) n * sizeof(double));
      x1[j] = x1[j] + h;
      scratch_load_atm(c, &s, atm);
      memcpy(s.rad, obs->rad, (size_t) (c->nd * obs->nr) * sizeof(double));
      jrc_atm a1 = { atm->np, atm->time, atm->z, atm->lon, atm->lat, s.p, s.t,
                     s.q, s.k, s.scal };
      jrc_obs o1 = { obs->nr, obs->geo, s.rad, s.tau, s.tp };
      state_walk(c, &a1, x1, NULL, NULL, 1);
      if (formod_one(c, &a1, &o1, &l, work)) {
        fail = 1;
        continue;
      }
      meas_gather(c, &o1, y1);
      for (int i = 0; i < m; i++)
        kmat[(size_t) i * n + j] = (y1[i] - y0[i]) / h;
    }
    free(x1); free(y1); free(work);
    scratch_free(&s);
    if (ok)
      los_free(&l);
  }
  free(x0); free(y0); free(iqa);
  return fail ? -1 : 0;
}

/* ---------------------------------------------------------------------- */
/* retrieval (retrieval.c:340-964)                                        */

/* Cholesky factorisation A = L L^T in place (lower triangle). */
static int chol_factor(double *a, int n) {
  for (int j = 0; j < n; j++) {
    double d = a[(size_t) j * n + j];
    for (int k = 0; k < j; k++)
      d -= a[(size_t) j * n + k] * a[(size_t) j * n + k];
    if (d <= 0)
      return -1;
    const double ljj = sqrt(d);
    a[(size_t) j * n + j] = ljj;
    for (int i = j + 1; i < n; i++) {
      double s = a[(size_t) i * n + j];
      for (int k = 0; k < j; k++)
        s -= a[(size_t) i * n + k] * a[(size_t) j * n + k];
      a[(size_t) i * n + j] = s / ljj;
    }
  }
  for (int i = 0; i < n; i++)
    for (int j = i + 1; j < n; j++)
      a[(size_t) i * n + j] = a[(size_t) j * n + i];
  return 0;
}

static void chol_solve(const double *l, int n, const double *b, double *x) {
  for (int i = 0; i < n; i++)
    x[i] = b[i];
  for (int i = 0; i < n; i++) {
    double s = x[i];
    for (int k = 0; k < i; k++)
      s -= l[(size_t) i * n + k] * x[k];
    x[i] = s / l[(size_t) i * n + i];
  }
  for (int i = n - 1; i >= 0; i--) {
    double s = x[i];
    for (int k = i + 1; k < n; k++)
      s -= l[(size_t) k * n + i] * x[k];
    x[i] = s / l[(size_t) i * n + i];
  }
}

/* matrix_invert, retrieval.c:373-399: reciprocal diagonal if the matrix is
   diagonal, else Cholesky inverse (symmetrised). */
static int sym_invert(double *a, int n) {
  int diag = 1;
  for (int i = 0; i < n && diag; i++)
    for (int j = i + 1; j < n; j++)
      if (a[(size_t) i * n + j] != 0) {
        diag = 0;
        break;
      }
  if (diag) {
    for (int i = 0; i < n; i++)
      a[(size_t) i * n + i] = 1 / a[(size_t) i * n + i];
    return 0;
  }
  if (chol_factor(a, n))
    return -1;
  double *inv = malloc((size_t) n * (size_t) n * sizeof(double));
  double *e = malloc((size_t) n * sizeof(double)), *col = malloc((size_t) n * sizeof(double));
  for (int j = 0; j < n; j++) {
    for (int i = 0; i < n; i++)
      e[i] = (i == j);
    chol_solve(a, n, e, col);
    for (int i = 0; i < n; i++)
      inv[(size_t) i * n + j] = col[i];
  }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      a[(size_t) i * n + j] = 0.5 * (inv[(size_t) i * n + j] + inv[(size_t) j * n + i]);
  free(inv); free(e); free(col);
  return 0;
}

int jrc_matrix_invert(double *a, int n) {
  return n > 0 && a ? sym_invert(a, n) : -1;
}

/* K^T diag(w)^2 K (matrix_product, retrieval.c:403-444, transpose == 1). */
static void ktwk(const double *kmat, const double *w, int m, int n, double *out) {
  double *aux = malloc((size_t) m * (size_t) n * sizeof(double));
  for (int i = 0; i < m; i++)
    for (int j = 0; j < n; j++)
      aux[(size_t) i * n + j] = w[i] * kmat[(size_t) i * n + j];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      double s = 0;
      for (int l = 0; l < m; l++)
        s += aux[(size_t) l * n + i] * aux[(size_t) l * n + j];
      out[(size_t) i * n + j] = s;
    }
  free(aux);
}

/* cost_function, retrieval.c:340-369: chi^2/m. */
static double cost_of(const double *dx, const double *dy, const double *sainv,
                      const double *sig_inv, int m, int n) {
  double chim = 0, chia = 0;
  for (int i = 0; i < m; i++)
    chim += sq(dy[i] * sig_inv[i]);
  for (int i = 0; i < n; i++) {
    double s = 0;
    for (int j = 0; j < n; j++)
      s += sainv[(size_t) i * n + j] * dx[j];
    chia += dx[i] * s;
  }
  return (chim + chia) / (double) m;
}

int jrc_retrieval(jrc_ctx *c, const jrc_ret *ret, const jrc_atm *atm_apr,
                  const jrc_obs *obs_meas, double *x_final, double *y_final,
                  double *cov_out, double *costs, int maxcost, int *info,
                  int nthreads) {
  return jrc_retrieval_ex(c, ret, atm_apr, obs_meas, x_final, y_final, cov_out, costs,
                          maxcost, info, nthreads, NULL);
}

/* Error analysis after the covariance (retrieval.c:686-726): gain
   G = cov K^T diag(sig_inv^2) (dgemm in k order), noise and forward-model
   error standard deviations sqrt(diag(G diag(sig^2) G^T)) (matrix_product
   with transpose == 2, write_stddev), averaging kernel A = G K and
   analyze_avk (257-336): per element the row sum over its quantity's block
   on top of copy_atm's init value (1 for surface emissivities, else 0) and
   1/A_ii. */
static void error_analysis(const jrc_ctx *c, const double *cov, const double *kk,
                           const double *sig_inv, const double *sig_noise,
                           const double *sig_fm, const int *iqa, int m, int n,
                           jrc_ana *ana) {
  double *G = malloc((size_t) n * (size_t) m * sizeof(double));
  for (int i = 0; i < n; i++)
    for (int j = 0; j < m; j++) {
      double s = 0;
      for (int k = 0; k < n; k++)
        s += cov[(size_t) i * n + k] * (kk[(size_t) j * n + k] * sq(sig_inv[j]));
      G[(size_t) i * m + j] = s;
    }
  for (int i = 0; i < n; i++) {
    double sn = 0, sf = 0;
    for (int j = 0; j < m; j++) {
      sn += sq(G[(size_t) i * m + j] * sig_noise[j]);
      sf += sq(G[(size_t) i * m + j] * sig_fm[j]);
    }
    if (ana->err_total) ana->err_total[i] = sqrt(cov[(size_t) i * n + i]);
    if (ana->err_noise) ana->err_noise[i] = sqrt(sn);
    if (ana->err_formod) ana->err_formod[i] = sqrt(sf);
  }
  double *A = malloc((size_t) n * (size_t) n * sizeof(double));
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      double s = 0;
      for (int k = 0; k < m; k++)
        s += G[(size_t) i * m + k] * kk[(size_t) k * n + j];
      A[(size_t) i * n + j] = s;
    }
  for (int i = 0; i < n; i++) {
    int n0 = -1, n1 = 0;
    for (int j = 0; j < n; j++)
      if (iqa[j] == iqa[i]) {
        if (n0 < 0) n0 = j;
        n1 = j - n0 + 1;
      }
    double s = iqa[i] >= Q_SFEPS(c, 0) ? 1.0 : 0.0;
    for (int j = 0; j < n1; j++)
      s += A[(size_t) i * n + n0 + j];
    if (ana->cont) ana->cont[i] = s;
    if (ana->res) ana->res[i] = 1 / A[(size_t) i * n + i];
  }
  if (ana->gain) memcpy(ana->gain, G, (size_t) n * (size_t) m * sizeof(double));
  if (ana->avk) memcpy(ana->avk, A, (size_t) n * (size_t) n * sizeof(double));
  free(G);
  free(A);
}

int jrc_retrieval_ex(jrc_ctx *c, const jrc_ret *ret, const jrc_atm *atm_apr,
                     const jrc_obs *obs_meas, double *x_final, double *y_final,
                     double *cov_out, double *costs, int maxcost, int *info,
                     int nthreads, jrc_ana *ana) {
  const int nd = c->nd, np = atm_apr->np, nr = obs_meas->nr;
  int m, n;
  jrc_sizes(c, atm_apr, obs_meas, &m, &n);
  if (m == 0 || n == 0) {
    set_err(c, "Check problem definition!");
    return -1;
  }
  int *iqa = malloc((size_t) n * sizeof(int)), *ipa = malloc((size_t) n * sizeof(int));
  state_walk(c, atm_apr, NULL, iqa, ipa, 0);

  /* working atmosphere/observation (atm_i, obs_i) */
  scratch_state si;
  scratch_init(c, &si, np, nr);
  jrc_atm ai = { np, atm_apr->time, atm_apr->z, atm_apr->lon, atm_apr->lat,
                 si.p, si.t, si.q, si.k, si.scal };
  jrc_obs oi = { nr, obs_meas->geo, si.rad, si.tau, si.tp };
  scratch_load_atm(c, &si, atm_apr);
  memcpy(si.rad, obs_meas->rad, (size_t) (nd * nr) * sizeof(double));
  int rc = jrc_formod(c, &ai, &oi);
  if (rc)
    goto fail_early;

  double *xa = malloc((size_t) n * sizeof(double)), *xi = malloc((size_t) n * sizeof(double));
  double *ym = malloc((size_t) m * sizeof(double)), *yi = malloc((size_t) m * sizeof(double));
  double *dx = malloc((size_t) n * sizeof(double)), *dy = malloc((size_t) m * sizeof(double));
  double *b = calloc((size_t) n, sizeof(double)), *step = malloc((size_t) n * sizeof(double));
  double *yaux = malloc((size_t) m * sizeof(double));
  double *sig_noise = malloc((size_t) m * sizeof(double)), *sig_fm = malloc((size_t) m * sizeof(double));
  double *sig_inv = malloc((size_t) m * sizeof(double));
  double *sainv = malloc((size_t) n * (size_t) n * sizeof(double));
  double *kk = malloc((size_t) m * (size_t) n * sizeof(double));
  double *cov = malloc((size_t) n * (size_t) n * sizeof(double));
  double *a = malloc((size_t) n * (size_t) n * sizeof(double));

  /* the a-priori atmosphere is not modified; copy it for atm2x */
  scratch_state sap;
  scratch_init(c, &sap, np, nr);
  scratch_load_atm(c, &sap, atm_apr);
  jrc_atm aap = { np, atm_apr->time, atm_apr->z, atm_apr->lon, atm_apr->lat,
                  sap.p, sap.t, sap.q, sap.k, sap.scal };
  state_walk(c, &aap, xa, NULL, NULL, 0);
  state_walk(c, &ai, xi, NULL, NULL, 0);
  meas_gather(c, obs_meas, ym);
  meas_gather(c, &oi, yi);

  /* a priori covariance (set_cov_apr, retrieval.c:808-920) */
  {
    double *sig = malloc((size_t) n * sizeof(double));
    state_walk(c, &aap, sig, NULL, NULL, 0);
    for (int i = 0; i < n; i++) {
      const int q = iqa[i];
      if (q == Q_P) sig[i] = ret->err_press / 100 * sig[i];
      if (q == Q_T) sig[i] = ret->err_temp;
      for (int ig = 0; ig < c->ng; ig++)
        if (q == Q_Q(ig)) sig[i] = ret->err_q[ig] / 100 * sig[i];
      for (int iw = 0; iw < c->nw; iw++)
        if (q == Q_K(c, iw)) sig[i] = ret->err_k[iw];
      if (q == Q_CLZ(c)) sig[i] = ret->err_clz;
      if (q == Q_CLDZ(c)) sig[i] = ret->err_cldz;
      for (int icl = 0; icl < c->ncl; icl++)
        if (q == Q_CLK(c, icl)) sig[i] = ret->err_clk[icl];
      if (q == Q_SFZ(c)) sig[i] = ret->err_sfz;
      if (q == Q_SFP(c)) sig[i] = ret->err_sfp;
      if (q == Q_SFT(c)) sig[i] = ret->err_sft;
      for (int isf = 0; isf < c->nsf; isf++)
        if (q == Q_SFEPS(c, isf)) sig[i] = ret->err_sfeps[isf];
    }
    for (int i = 0; i < n; i++)
      if (sq(sig[i]) <= 0) {
        free(sig);
        set_err(c, "Check a priori data (zero standard deviation)!");
        rc = -1;
        goto done;
      }
    memset(sainv, 0, (size_t) n * (size_t) n * sizeof(double));
    for (int i = 0; i < n; i++)
      sainv[(size_t) i * n + i] = sq(sig[i]);
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++)
        if (i != j && iqa[i] == iqa[j]) {
          double cz = 0, ch = 0;
          const int q = iqa[i];
          if (q == Q_P) { cz = ret->err_press_cz; ch = ret->err_press_ch; }
          if (q == Q_T) { cz = ret->err_temp_cz; ch = ret->err_temp_ch; }
          for (int ig = 0; ig < c->ng; ig++)
            if (q == Q_Q(ig)) { cz = ret->err_q_cz[ig]; ch = ret->err_q_ch[ig]; }
          for (int iw = 0; iw < c->nw; iw++)
            if (q == Q_K(c, iw)) { cz = ret->err_k_cz[iw]; ch = ret->err_k_ch[iw]; }
          if (cz > 0 && ch > 0) {
            double x0[3], x1[3];
            to_cart(0, atm_apr->lon[ipa[i]], atm_apr->lat[ipa[i]], x0);
            to_cart(0, atm_apr->lon[ipa[j]], atm_apr->lat[ipa[j]], x1);
            const double dist = sqrt(sq(x0[0] - x1[0]) + sq(x0[1] - x1[1]) + sq(x0[2] - x1[2]));
            const double rho = exp(-dist / ch - fabs(atm_apr->z[ipa[i]] - atm_apr->z[ipa[j]]) / cz);
            sainv[(size_t) i * n + j] = sig[i] * sig[j] * rho;
          }
        }
    free(sig);
    if (sym_invert(sainv, n)) {
      set_err(c, "a priori covariance is not positive definite");
      rc = -1;
      goto done;
    }
  }

  /* measurement errors (set_cov_meas, retrieval.c:924-964) */
  {
    int mm = 0;
    for (int ir = 0; ir < nr; ir++)
      for (int id = 0; id < nd; id++) {
        const double v = obs_meas->rad[(size_t) id * nr + ir];
        if (isfinite(v)) {
          sig_noise[mm] = ret->err_noise[id];
          sig_fm[mm] = fabs(ret->err_formod[id] / 100 * v);
          mm++;
        }
      }
    for (int i = 0; i < m; i++) {
      sig_inv[i] = 1 / sqrt(sq(sig_noise[i]) + sq(sig_fm[i]));
      if (sig_inv[i] <= 0) {
        set_err(c, "Check measurement errors (zero standard deviation)!");
        rc = -1;
        goto done;
      }
    }
  }

  for (int i = 0; i < n; i++) dx[i] = xi[i] - xa[i];
  for (int i = 0; i < m; i++) dy[i] = ym[i] - yi[i];
  double chisq = cost_of(dx, dy, sainv, sig_inv, m, n);
  int ncost = 0;
  if (ncost < maxcost) costs[ncost++] = chisq;

  rc = jrc_kernel(c, &ai, &oi, kk, nthreads);
  if (rc) goto done;

  /* Levenberg-Marquardt (retrieval.c:559-652) */
  double lmpar = 0.001;
  int it;
  for (it = 1; it <= ret->conv_itmax; it++) {
    const double chisq_old = chisq;
    if (it > 1 && it % ret->kernel_recomp == 0) {
      rc = jrc_kernel(c, &ai, &oi, kk, nthreads);
      if (rc) goto done;
    }
    if (it == 1 || it % ret->kernel_recomp == 0)
      ktwk(kk, sig_inv, m, n, cov);
    for (int i = 0; i < m; i++)
      yaux[i] = dy[i] * sq(sig_inv[i]);
    for (int j = 0; j < n; j++) {
      double s = 0;
      for (int i = 0; i < m; i++)
        s += kk[(size_t) i * n + j] * yaux[i];
      b[j] = 1.0 * s + 0.0 * b[j];
    }
    for (int i = 0; i < n; i++) {
      double s = 0;
      for (int j = 0; j < n; j++)
        s += sainv[(size_t) i * n + j] * dx[j];
      b[i] = -1.0 * s + 1.0 * b[i];
    }
    for (int it2 = 0; it2 < 20; it2++) {
      for (size_t i = 0; i < (size_t) n * (size_t) n; i++)
        a[i] = sainv[i] * (1 + lmpar) + cov[i];
      if (chol_factor(a, n)) {
        set_err(c, "normal matrix is not positive definite");
        rc = -1;
        goto done;
      }
      chol_solve(a, n, b, step);
      for (int i = 0; i < n; i++) xi[i] += step[i];
      scratch_load_atm(c, &si, atm_apr);
      memcpy(si.rad, obs_meas->rad, (size_t) (nd * nr) * sizeof(double));
      state_walk(c, &ai, xi, NULL, NULL, 1);
      for (int ip = 0; ip < np; ip++) {
        si.p[ip] = fmin(fmax(si.p[ip], 5e-7), 5e4);
        si.t[ip] = fmin(fmax(si.t[ip], 100), 400);
        for (int ig = 0; ig < c->ng; ig++)
          si.q[(size_t) ig * np + ip] = fmin(fmax(si.q[(size_t) ig * np + ip], 0), 1);
        for (int iw = 0; iw < c->nw; iw++)
          si.k[(size_t) iw * np + ip] = fmax(si.k[(size_t) iw * np + ip], 0);
      }
      si.scal[0] = fmax(si.scal[0], 0);
      si.scal[1] = fmax(si.scal[1], 0.1);
      for (int icl = 0; icl < c->ncl; icl++)
        si.scal[2 + icl] = fmax(si.scal[2 + icl], 0);
      {
        const int o = 2 + c->ncl;
        si.scal[o] = fmax(si.scal[o], 0);
        si.scal[o + 1] = fmax(si.scal[o + 1], 0);
        si.scal[o + 2] = fmin(fmax(si.scal[o + 2], 100), 400);
        for (int isf = 0; isf < c->nsf; isf++)
          si.scal[o + 3 + isf] = fmin(fmax(si.scal[o + 3 + isf], 0), 1);
      }
      rc = jrc_formod(c, &ai, &oi);
      if (rc) goto done;
      meas_gather(c, &oi, yi);
      for (int i = 0; i < n; i++) dx[i] = xi[i] - xa[i];
      for (int i = 0; i < m; i++) dy[i] = ym[i] - yi[i];
      chisq = cost_of(dx, dy, sainv, sig_inv, m, n);
      if (chisq > chisq_old) {
        lmpar *= 10;
        for (int i = 0; i < n; i++) xi[i] -= step[i];
      } else {
        lmpar /= 10;
        break;
      }
    }
    if (ncost < maxcost) costs[ncost++] = chisq;
    double disq = 0;
    for (int i = 0; i < n; i++) disq += step[i] * b[i];
    disq /= (double) n;
    if ((it == 1 || it % ret->kernel_recomp == 0) && disq < ret->conv_dmin)
      break;
  }
  info[3] = it > ret->conv_itmax ? ret->conv_itmax : it;

  state_walk(c, &ai, x_final, NULL, NULL, 0);
  if (y_final) meas_gather(c, &oi, y_final);
  if (ret->err_ana && cov_out) {
    ktwk(kk, sig_inv, m, n, cov);
    for (size_t i = 0; i < (size_t) n * (size_t) n; i++)
      cov[i] += sainv[i];
    if (sym_invert(cov, n)) {
      set_err(c, "retrieval covariance is not positive definite");
      rc = -1;
      goto done;
    }
    memcpy(cov_out, cov, (size_t) n * (size_t) n * sizeof(double));
    if (ana)
      error_analysis(c, cov, kk, sig_inv, sig_noise, sig_fm, iqa, m, n, ana);
  }
  info[0] = n;
  info[1] = m;
  info[2] = ncost;
  rc = 0;
done:
  free(xa); free(xi); free(ym); free(yi); free(dx); free(dy); free(b); free(step);
  free(yaux); free(sig_noise); free(sig_fm); free(sig_inv); free(sainv); free(kk);
  free(cov); free(a);
  scratch_free(&sap);
fail_early:
  scratch_free(&si);
  free(iqa); free(ipa);
  return rc;
}
