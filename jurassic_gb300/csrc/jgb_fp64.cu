// FP64 kernels: ray tracing and the plain FP64 forward model.
//
// This translation unit is compiled with -fmad=false so that every FP64
// expression is rounded like the reference's (no fused multiply-add), which
// keeps the FP64 path within rounding of the reference results.
//
//   k_trace       raytrace (jurassic.c:4201-4438) + tangent_point
//                 (jurassic.c:5223-5263), one thread per ray; a counting pass
//                 sizes the LOS buffer, a filling pass writes it.
//   k_path_fp64   formod_pencil (jurassic.c:3196-3338) with intpol_tbl_ega /
//                 intpol_tbl_cga (3710-3891), formod_continua (3075-3117),
//                 formod_srcfunc (3483-3496), surface/reflection/solar terms,
//                 BT conversion and the observation mask of formod
//                 (3026-3071); one thread per (ray, channel).
//   k_srcfunc     init_srcfunc (jurassic.c:3631-3681) on the device.
//   k_hydrostatic hydrostatic (jurassic.c:3520-3582), one thread per profile.
#include "../../include/jurassic_gb300.h"
#include "jgb_common.cuh"
#include "jgb_internal.h"

namespace jgb {

// ---------------------------------------------------------------------------
// atmosphere access

struct AtmView {
  int np, ng, nw;
  bool asc;           // altitude grid strictly ascending
  long long stride;   // level stride of q/k planes (total levels of the batch)
  const double *z, *p, *t, *q, *k;   // q[ig*stride + i], k[iw*stride + i]
  double clz, cldz, sfz, sfp, sft;
  const double *clk, *sfeps;
};

__device__ inline AtmView atm_view(const CtlDev& c, const BatchDev& b, int o) {
  AtmView a;
  const int l0 = b.lev_off[o];
  a.np = b.lev_off[o + 1] - l0;
  a.ng = c.ng;
  a.nw = c.nw;
  a.stride = b.nlev;
  a.z = b.z + l0;
  a.p = b.p + l0;
  a.t = b.t + l0;
  a.q = b.q + l0;
  a.k = b.k + l0;
  const double* s = b.scal + (long long)o * b.nscal;
  a.clz = s[0];
  a.cldz = s[1];
  a.clk = s + 2;
  a.sfz = s[2 + c.ncl];
  a.sfp = s[3 + c.ncl];
  a.sft = s[4 + c.ncl];
  a.sfeps = s + 5 + c.ncl;
  a.asc = true;
  for (int i = 0; i + 1 < a.np; i++)
    if (!(a.z[i] < a.z[i + 1])) a.asc = false;
  return a;
}

// Altitude of a Cartesian point: the z of cart2geo (jurassic.c:108-120)
// without the latitude/longitude, which the reference computes and discards
// at the refraction sub-points and which the counting pass never needs.
__device__ inline double z_of(const double* x) {
  return sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]) - kRE;
}

// Level bracket with a hint: on a strictly ascending grid the bisection of
// locate_irr returns the unique i with z[i] <= x < z[i+1] (0 below, n-2
// above the grid), so a hint that satisfies this is the bisection result.
__device__ inline int level_of(const AtmView& a, double z, int* hint) {
  const int h = *hint;
  if (a.asc && h >= 0 && h <= a.np - 2) {
    const bool in = a.z[h] <= z && z < a.z[h + 1];
    const bool below = h == 0 && z < a.z[0];
    const bool above = h == a.np - 2 && z >= a.z[a.np - 1];
    if (in || below || above) return h;
  }
  const int i = bracket_irr(a.z, a.np, z);
  *hint = i;
  return i;
}

// intpol_atm (jurassic.c:3685-3706): p (log-linear) and T only.
__device__ inline int atm_pt(const AtmView& a, double z, double* p, double* t, int* hint) {
  const int i = level_of(a, z, hint);
  *p = logy(a.z[i], a.p[i], a.z[i + 1], a.p[i + 1], z);
  *t = lin(a.z[i], a.t[i], a.z[i + 1], a.t[i + 1], z);
  return i;
}

#define JGB_REFRAC(p, t) (7.753e-05 * (p) / (t))

// One ray walk.  STORE=false only counts points; STORE=true writes the LOS
// planes (q of each emitter into the u plane, converted after the walk).
// Returns the number of points, or -1 on error (flag set in *err).
template <bool STORE>
__device__ int walk(const CtlDev& c, const ChanDev& ch, const AtmView& a, const double* g,
                    long long nray, int r, const LosDev& L, long long base, int cap,
                    double* sft_out, unsigned* err) {
  const double h = 0.02, zrefrac = 60;
  double ex0[3], ex1[3], x[3], xh[3], xobs[3], xvp[3], ngr[3];
  double z = 1e99, lon = 0, lat = 0, p, t;
  int stop = 0, n = 0, hint = -1;
  const double obsz = g[1 * nray + r], obslon = g[2 * nray + r], obslat = g[3 * nray + r];
  const double vpz = g[4 * nray + r], vplon = g[5 * nray + r], vplat = g[6 * nray + r];
  double last_z = 0, last_lon = 0, last_lat = 0;
  *sft_out = -999;

  double zmin = a.z[0], zmax = a.z[0];
  for (int i = 0; i < a.np; i++) {
    zmin = a.z[i] < zmin ? a.z[i] : zmin;
    zmax = a.z[i] > zmax ? a.z[i] : zmax;
  }
  if (c.nsf > 0) {
    zmin = a.sfz > zmin ? a.sfz : zmin;
    if (a.sfp > 0) {
      const int i = bracket_irr(a.p, a.np, a.sfp);
      const double zs = lin(log(a.p[i]), a.z[i], log(a.p[i + 1]), a.z[i + 1], log(a.sfp));
      zmin = zs > zmin ? zs : zmin;
    }
  }
  if (obsz < zmin) {
    atomicOr(err, kErrObserverBelowSurface);
    return -1;
  }
  if (vpz > zmax) return 0;

  to_cart(obsz, obslon, obslat, xobs);
  to_cart(vpz, vplon, vplat, xvp);
  for (int i = 0; i < 3; i++) ex0[i] = xvp[i] - xobs[i];
  double norm = sqrt(ex0[0] * ex0[0] + ex0[1] * ex0[1] + ex0[2] * ex0[2]);
  for (int i = 0; i < 3; i++) ex0[i] /= norm;
  for (int i = 0; i < 3; i++) x[i] = xobs[i];

  if (obsz > zmax) {
    double dmax = norm, dmin = 0;
    for (int guard = 0; fabs(dmin - dmax) > 0.001 && guard < 200; guard++) {
      const double d = (dmax + dmin) / 2;
      for (int i = 0; i < 3; i++) x[i] = xobs[i] + d * ex0[i];
      z = z_of(x);
      if (z <= zmax && z > zmax - 0.001) break;
      if (z < zmax - 0.0005) dmax = d; else dmin = d;
    }
  }

  for (;;) {
    double ds = c.rayds;
    if (c.raydz > 0) {
      norm = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      for (int i = 0; i < 3; i++) xh[i] = x[i] / norm;
      const double cosa = fabs(ex0[0] * xh[0] + ex0[1] * xh[1] + ex0[2] * xh[2]);
      if (cosa != 0) ds = c.rayds < c.raydz / cosa ? c.rayds : c.raydz / cosa;
    }
    if (STORE)
      to_geo(x, &z, &lon, &lat);
    else
      z = z_of(x);
    if ((z < zmin || z > zmax) && n > 0) {
      if (!STORE) {  // the clipped last point ends the count
        if (n >= cap) {
          atomicOr(err, kErrLosOverflow);
          return -1;
        }
        return n + 1;
      }
      stop = (z < zmin ? 2 : 1);
      const double frac = ((z < zmin ? zmin : zmax) - last_z) / (z - last_z);
      to_cart(last_z, last_lon, last_lat, xh);
      for (int i = 0; i < 3; i++) x[i] = xh[i] + frac * (x[i] - xh[i]);
      to_geo(x, &z, &lon, &lat);
      if (STORE) L.ds[base + n - 1] = ds * frac;
      ds = 0;
    }
    if (n >= cap) {
      atomicOr(err, kErrLosOverflow);
      return -1;
    }
    const int i = atm_pt(a, z, &p, &t, &hint);
    if (STORE) {
      const long long s = base + n;
      L.z[s] = z;
      L.lon[s] = lon;
      L.lat[s] = lat;
      L.p[s] = p;
      L.t[s] = t;
      L.ds[s] = ds;
      for (int ig = 0; ig < a.ng; ig++)
        L.u[ig * L.cap + s] = lin(a.z[i], a.q[ig * a.stride + i], a.z[i + 1],
                                  a.q[ig * a.stride + i + 1], z);
      if (c.ig_h2o >= 0) L.qh2o[s] = L.u[c.ig_h2o * L.cap + s];
      for (int iw = 0; iw < a.nw; iw++)
        L.kw[iw * L.cap + s] = lin(a.z[i], a.k[iw * a.stride + i], a.z[i + 1],
                                   a.k[iw * a.stride + i + 1], z);
      L.aux[s] = (c.ncl > 0 && a.cldz > 0) ? exp(-0.5 * ((z - a.clz) / a.cldz) * ((z - a.clz) / a.cldz)) : 0.0;
    }
    last_z = z;
    last_lon = lon;
    last_lat = lat;
    n++;
    if (stop) {
      if (c.nsf > 0 && a.sft > 0) t = a.sft;
      *sft_out = (stop == 2 ? t : -999);
      break;
    }
    const bool bend = c.refrac && z <= zrefrac;
    double nref = bend ? 1 + JGB_REFRAC(p, t) : 1;
    for (int k = 0; k < 3; k++) ex1[k] = ex0[k] * nref;
    if (bend) {
      for (int k = 0; k < 3; k++) xh[k] = x[k] + 0.5 * ds * ex0[k];
      z = z_of(xh);
      atm_pt(a, z, &p, &t, &hint);
      nref = JGB_REFRAC(p, t);
      for (int k = 0; k < 3; k++) {
        xh[k] += h;
        z = z_of(xh);
        atm_pt(a, z, &p, &t, &hint);
        ngr[k] = (JGB_REFRAC(p, t) - nref) / h;
        xh[k] -= h;
      }
    } else {
      ngr[0] = ngr[1] = ngr[2] = 0;
    }
    for (int k = 0; k < 3; k++) ex1[k] += ds * ngr[k];
    norm = sqrt(ex1[0] * ex1[0] + ex1[1] * ex1[1] + ex1[2] * ex1[2]);
    for (int k = 0; k < 3; k++) ex1[k] /= norm;
    for (int k = 0; k < 3; k++) x[k] += 0.5 * ds * (ex0[k] + ex1[k]);
    for (int k = 0; k < 3; k++) ex0[k] = ex1[k];
  }
  return n;
}

__global__ void k_trace_count(CtlDev c, ChanDev ch, BatchDev b, LosDev L, unsigned* err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= b.nray) return;
  if (b.obs_skip && b.obs_skip[b.ray_obs[r]]) {
    L.count[r] = 0;
    return;
  }
  const AtmView a = atm_view(c, b, b.ray_obs[r]);
  double sft;
  const int n = walk<false>(c, ch, a, b.geo, b.nray, r, L, 0, c.nlos_max, &sft, err);
  L.count[r] = n < 0 ? 0 : n;
}

__global__ void k_trace_fill(CtlDev c, ChanDev ch, BatchDev b, LosDev L, unsigned* err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= b.nray) return;
  if (b.obs_skip && b.obs_skip[b.ray_obs[r]]) return;
  const AtmView a = atm_view(c, b, b.ray_obs[r]);
  const long long base = L.off[r];
  const int cap = L.count[r];
  double sft;
  const int n = walk<true>(c, ch, a, b.geo, b.nray, r, L, base, cap, &sft, err);
  L.sft[r] = sft;
  const long long nr = b.nray;
  double* tp = b.tp;
  // tangent point defaults to the view point (jurassic.c:4218-4220)
  tp[0 * nr + r] = b.geo[4 * nr + r];
  tp[1 * nr + r] = b.geo[5 * nr + r];
  tp[2 * nr + r] = b.geo[6 * nr + r];
  if (n <= 0) {
    L.count[r] = 0;
    return;
  }
  const double* z = L.z + base;
  const double* lo = L.lon + base;
  const double* la = L.lat + base;
  double* ds = L.ds + base;
  // tangent point (tangent_point, jurassic.c:5223-5263), before trapezoid
  int imin = 0;
  for (int i = 1; i < n; i++)
    if (z[i] < z[imin]) imin = i;
  if (imin <= 0 || imin >= n - 1) {
    tp[0 * nr + r] = z[n - 1];
    tp[1 * nr + r] = lo[n - 1];
    tp[2 * nr + r] = la[n - 1];
  } else {
    const double y0 = z[imin - 1], y1 = z[imin], y2 = z[imin + 1];
    const double x1 = sqrt(ds[imin] * ds[imin] - (y1 - y0) * (y1 - y0));
    const double x2 = x1 + sqrt(ds[imin + 1] * ds[imin + 1] - (y2 - y1) * (y2 - y1));
    const double aa = 1 / (x1 - x2) * (-(y0 - y1) / x1 + (y0 - y2) / x2);
    const double bb = -(y0 - y1) / x1 - aa * x1;
    const double cc = y0;
    const double xt = -bb / (2 * aa);
    tp[0 * nr + r] = aa * xt * xt + bb * xt + cc;
    double v0[3], v2[3], v[3], dummy, tlon, tlat;
    to_cart(z[imin - 1], lo[imin - 1], la[imin - 1], v0);
    to_cart(z[imin + 1], lo[imin + 1], la[imin + 1], v2);
    for (int i = 0; i < 3; i++) v[i] = lin(0.0, v0[i], x2, v2[i], xt);
    to_geo(v, &dummy, &tlon, &tlat);
    tp[1 * nr + r] = tlon;
    tp[2 * nr + r] = tlat;
  }
  double* e = L.ends + 6LL * r;
  e[0] = z[0];
  e[1] = lo[0];
  e[2] = la[0];
  e[3] = z[n - 1];
  e[4] = lo[n - 1];
  e[5] = la[n - 1];
  // trapezoid segment lengths
  for (int ip = n - 1; ip >= 1; ip--) ds[ip] = 0.5 * (ds[ip - 1] + ds[ip]);
  ds[0] *= 0.5;
  // column densities (q stored in the u plane) and Curtis-Godson means
  const double* p = L.p + base;
  const double* t = L.t + base;
  for (int ig = 0; ig < c.ng; ig++) {
    double* u = L.u + ig * L.cap + base;
    for (int ip = 0; ip < n; ip++) u[ip] = 10 * u[ip] * p[ip] / (kKB * t[ip]) * ds[ip];
    if (L.cga) {
      double* cgu = L.cgu + ig * L.cap + base;
      double* cgp = L.cgp + ig * L.cap + base;
      double* cgt = L.cgt + ig * L.cap + base;
      double su = u[0], sp = u[0] * p[0], st = u[0] * t[0];
      cgu[0] = su;
      cgp[0] = sp / su;
      cgt[0] = st / su;
      for (int ip = 1; ip < n; ip++) {
        su = su + u[ip];
        sp = sp + u[ip] * p[ip];
        st = st + u[ip] * t[ip];
        cgu[ip] = su;
        cgp[ip] = sp / su;
        cgt[ip] = st / su;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// tables

struct Row {
  const float* u;
  const float* e;
  int n;
};

__device__ inline Row row_at(const TblDev& T, long long dg, int ip, int it) {
  const long long r = (dg * T.tp + ip) * T.tt + it;
  Row w;
  w.u = T.u + r * T.tu;
  w.e = T.eps + r * T.tu;
  w.n = T.nu[r];
  return w;
}

// intpol_tbl_eps (jurassic.c:3895-3929)
__device__ inline double row_eps(const Row& r, double u) {
  if (u < (double)r.u[0]) return lin_f(0.0f, 0.0f, r.u[0], r.e[0], u);
  if (u > (double)r.u[r.n - 1]) {
    const double a = log((double)(1 - r.e[r.n - 1])) / (double)r.u[r.n - 1];
    return 1 - exp(a * u);
  }
  const int i = bracket_row(r.u, r.n, u);
  return lin_f(r.u[i], r.e[i], r.u[i + 1], r.e[i + 1], u);
}

// intpol_tbl_u (jurassic.c:3933-3967)
__device__ inline double row_u(const Row& r, double e) {
  if (e < (double)r.e[0]) return lin_f(0.0f, 0.0f, r.e[0], r.u[0], e);
  if (e > (double)r.e[r.n - 1]) {
    const double a = log((double)(1 - r.e[r.n - 1])) / (double)r.u[r.n - 1];
    return log(1 - e) / a;
  }
  const int i = bracket_row(r.e, r.n, e);
  return lin_f(r.e[i], r.u[i], r.e[i + 1], r.u[i + 1], e);
}

// Segment emissivity of one (channel, emitter) at one LOS point; updates
// the extended-path transmittance (intpol_tbl_ega / intpol_tbl_cga).
__device__ inline double gas_eps(const TblDev& T, long long dg, bool cga, double pq, double tq,
                                 double du, double ucg, double* tau_path) {
  const int np = T.np[dg];
  if (np < 30) return 0;
  if (*tau_path < 1e-9) return 1;
  const double* pg = T.p + dg * T.tp;
  const int* ntg = T.nt + dg * T.tp;
  const int ipr = bracket_irr(pg, np, pq);
  const double* t0g = T.t + (dg * T.tp + ipr) * T.tt;
  const double* t1g = t0g + T.tt;
  const int it0 = bracket_reg(t0g, ntg[ipr], tq);
  const int it1 = bracket_reg(t1g, ntg[ipr + 1], tq);
  if (ntg[ipr] < 2 || ntg[ipr + 1] < 2) return 0;
  const Row r00 = row_at(T, dg, ipr, it0), r01 = row_at(T, dg, ipr, it0 + 1);
  const Row r10 = row_at(T, dg, ipr + 1, it1), r11 = row_at(T, dg, ipr + 1, it1 + 1);
  if (r00.n < 2 || r01.n < 2 || r10.n < 2 || r11.n < 2) return 0;
  double e00, e01, e10, e11;
  if (cga) {
    e00 = row_eps(r00, ucg);
    e01 = row_eps(r01, ucg);
    e10 = row_eps(r10, ucg);
    e11 = row_eps(r11, ucg);
  } else {
    const double prev = 1 - *tau_path;
    e00 = row_eps(r00, row_u(r00, prev) + du);
    e01 = row_eps(r01, row_u(r01, prev) + du);
    e10 = row_eps(r10, row_u(r10, prev) + du);
    e11 = row_eps(r11, row_u(r11, prev) + du);
  }
  e00 = lin(t0g[it0], e00, t0g[it0 + 1], e01, tq);
  e11 = lin(t1g[it1], e10, t1g[it1 + 1], e11, tq);
  e00 = cga ? logx(pg[ipr], e00, pg[ipr + 1], e11, pq) : lin(pg[ipr], e00, pg[ipr + 1], e11, pq);
  e00 = e00 < 1 ? e00 : 1;
  e00 = e00 > 0 ? e00 : 0;
  return 1 - (1 - e00) / *tau_path;
}

// formod_srcfunc (jurassic.c:3483-3496) for one channel
__device__ inline double src_at(const TblDev& T, int nd, int id, double t) {
  const int it = bracket_reg(T.st, kNS, t);
  return lin(T.st[it], T.sr[(long long)it * nd + id], T.st[it + 1], T.sr[(long long)(it + 1) * nd + id], t);
}

// continua (ctmco2/ctmh2o/ctmn2/ctmo2 with the wavenumber-only factors
// precomputed per channel on the host, see ctm_coefficients in jgb_api.cu)
__device__ inline double continuum_beta(const CtlDev& c, const double* cc, double kext, double p,
                                        double t, double ds, double uco2, double uh2o,
                                        double qh2o, double nu) {
  double beta = kext;
  if (c.ctm_co2 && c.ig_co2 >= 0 && cc[0] != 0) {
    const double d230 = t - 230, d260 = t - 260, d296 = t - 296;
    const double ctw = d260 * 5.050505e-4 * d296 * cc[3] - d230 * 9.259259e-4 * d296 * cc[2] +
                       d230 * 4.208754e-4 * d260 * cc[1];
    beta += uco2 / kNA / 1000 * p / kP0 * ctw / ds;
  }
  if (c.ctm_h2o && c.ig_h2o >= 0 && cc[4] != 0) {
    const double self = cc[5] * pow(cc[6], (296 - t) / (296 - 260));
    const double a1 = nu * uh2o * tanh(.7193876 / t * nu);
    const double a2 = 296 / t;
    const double a3 = p / kP0 * (qh2o * self + (1 - qh2o) * cc[7]) * 1e-20;
    beta += a1 * a2 * a3 / ds;
  }
  if (c.ctm_n2 && cc[8] != 0) {
    const double qn = 0.79, t0 = 273.0, tr = 296.0;
    const double x = p / kP0 * t0 / t;
    beta += 0.1 * (x * x) * exp(cc[10] * (1 / tr - 1 / t)) * qn * cc[9] *
            (qn + (1 - qn) * (1.294 - 0.4545 * t / tr));
  }
  if (c.ctm_o2 && cc[11] != 0) {
    const double qo = 0.21, t0 = 273, tr = 296;
    const double x = p / kP0 * t0 / t;
    beta += 0.1 * (x * x) * exp(cc[13] * (1 / tr - 1 / t)) * qo * cc[12];
  }
  return beta;
}

// Solar zenith angle (sza, jurassic.c:5183-5219)
__device__ inline double solar_zenith(double sec, double lon, double lat) {
  const double d = sec / 86400 - 0.5;
  const double g = (357.529 + 0.98560028 * d) * (kPI / 180.0);
  const double q = 280.459 + 0.98564736 * d;
  const double l = (q + 1.915 * sin(g) + 0.020 * sin(2 * g)) * (kPI / 180.0);
  const double e = (23.439 - 0.00000036 * d) * (kPI / 180.0);
  const double dec = asin(sin(e) * sin(l));
  const double ra = atan2(cos(e) * sin(l), cos(l));
  const double gmst = 18.697374558 + 24.06570982441908 * d;
  const double lst = gmst + lon / 15;
  const double h = lst / 12 * kPI - ra;
  const double latr = lat * (kPI / 180.0);
  return acos(sin(latr) * sin(dec) + cos(latr) * cos(dec) * cos(h)) * (180.0 / kPI);
}

// Per-(observation, channel) constants derived from the atmosphere record.
__device__ inline void obs_channel_consts(const CtlDev& c, const ChanDev& ch, const double* s,
                                          int id, double* cloud, bool* has_cloud,
                                          double* sfeps) {
  const double nu = ch.nu[id];
  *has_cloud = c.ncl > 0 && s[1] > 0;
  *cloud = 0;
  if (*has_cloud) {
    const int icl = bracket_irr(ch.clnu, c.ncl, nu);
    *cloud = lin(ch.clnu[icl], s[2 + icl], ch.clnu[icl + 1], s[2 + icl + 1], nu);
  }
  *sfeps = 1.0;
  if (c.nsf > 0) {
    const double* se = s + 5 + c.ncl;
    const int isf = bracket_irr(ch.sfnu, c.nsf, nu);
    *sfeps = lin(ch.sfnu[isf], se[isf], ch.sfnu[isf + 1], se[isf + 1], nu);
  }
}

__global__ void k_path_fp64(CtlDev c, TblDev T, ChanDev ch, BatchDev b, LosDev L,
                            double* refl_scratch) {
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nray = b.nray;
  if (gid >= nray * c.nd) return;
  const int id = (int)(gid / nray);
  const int r = (int)(gid % nray);
  const int o = b.ray_obs[r];
  if (b.obs_skip && b.obs_skip[o]) return;
  const int n = b.skip_masked && b.mask[gid] ? 0 : L.count[r];  // gid = id * nray + r
  const long long base = L.off[r];
  const double nu = ch.nu[id];
  const double* cc = ch.ctm + (long long)id * kCtmStride;
  const double* s = b.scal + (long long)o * b.nscal;
  double cloud, sfeps;
  bool has_cloud;
  obs_channel_consts(c, ch, s, id, &cloud, &has_cloud, &sfeps);
  const int w = c.nw > 0 ? ch.window[id] : 0;
  double tau_path[kMaxG];
  for (int ig = 0; ig < c.ng; ig++) tau_path[ig] = 1;
  double rad = 0, tau = 1;
  const bool cga = c.formod == 0;
  const bool refl = c.sftype >= 2 && sfeps < 1 && L.sft[r] > 0 && c.sftype >= 1;
  double* sc = refl ? refl_scratch + 2 * base * c.nd : nullptr;

  for (int ip = 0; ip < n; ip++) {
    const long long q = base + ip;
    const double p = L.p[q], t = L.t[q], ds = L.ds[q];
    double tau_gas = 1;
    for (int ig = 0; ig < c.ng; ig++) {
      const long long dg = (long long)id * c.ng + ig;
      const double du = cga ? 0.0 : L.u[ig * L.cap + q];
      const double pq = cga ? L.cgp[ig * L.cap + q] : p;
      const double tq = cga ? L.cgt[ig * L.cap + q] : t;
      const double ucg = cga ? L.cgu[ig * L.cap + q] : 0.0;
      const double eps = gas_eps(T, dg, cga, pq, tq, du, ucg, &tau_path[ig]);
      tau_path[ig] *= (1 - eps);
      tau_gas *= (1 - eps);
    }
    double kext = c.nw > 0 ? L.kw[w * L.cap + q] : 0.0;
    if (has_cloud) kext += L.aux[q] * cloud;
    const double uco2 = c.ig_co2 >= 0 ? L.u[c.ig_co2 * L.cap + q] : 0.0;
    const double uh2o = c.ig_h2o >= 0 ? L.u[c.ig_h2o * L.cap + q] : 0.0;
    const double qh2o = c.ig_h2o >= 0 ? L.qh2o[q] : 0.0;
    const double beta = continuum_beta(c, cc, kext, p, t, ds, uco2, uh2o, qh2o, nu);
    const double src = src_at(T, c.nd, id, t);
    double eps = 0;
    if (tau_gas > 0) {
      eps = 1 - tau_gas * exp(-beta * ds);
      rad += src * eps * tau;
      tau *= (1 - eps);
    }
    if (sc) {
      sc[2 * ((long long)ip * c.nd + id)] = src;
      sc[2 * ((long long)ip * c.nd + id) + 1] = eps;
    }
  }

  // surface emission, reflection and solar term (jurassic.c:3264-3328)
  const double sft = L.sft[r];
  if (c.sftype >= 1 && sft > 0) {
    rad += sfeps * src_at(T, c.nd, id, sft) * tau;
    if (refl) {
      double tau_refl = 1;
      for (int ip = n - 1; ip >= 0; ip--) {
        const double src = sc[2 * ((long long)ip * c.nd + id)];
        const double e = sc[2 * ((long long)ip * c.nd + id) + 1];
        rad += src * e * tau_refl * tau * (1 - sfeps);
        tau_refl *= (1 - e);
      }
      if (c.sftype >= 3) {
        const double* e6 = L.ends + 6LL * r;
        const double sza2 = c.sfsza < 0 ? solar_zenith(b.geo[r], e6[4], e6[5]) : c.sfsza;
        if (sza2 < 89.999) {
          double x0[3], x1[3];
          to_cart(e6[3], e6[4], e6[5], x0);
          to_cart(e6[0], e6[1], e6[2], x1);
          for (int i = 0; i < 3; i++) x1[i] -= x0[i];
          const double cosa = (x0[0] * x1[0] + x0[1] * x1[1] + x0[2] * x1[2]) /
                              sqrt(x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2]) /
                              sqrt(x1[0] * x1[0] + x1[1] * x1[1] + x1[2] * x1[2]);
          const double rcos = cosa / cos(sza2 * (kPI / 180.0));
          rad += 6.764e-5 / (2. * kPI) * planck(kTSUN, nu) * tau_refl * (1 - sfeps) * tau * rcos;
        }
      }
    }
  }
  const long long oi = (long long)id * nray + r;
  if (c.fov) {  // pencil beam only: FOV convolution, BT and mask follow in k_fov
    b.rad[oi] = rad;
    b.tau[oi] = tau;
    return;
  }
  if (c.write_bbt) rad = kC2 * nu / log1p(kC1 * (nu * nu * nu) / rad);
  b.rad[oi] = b.mask[oi] ? __longlong_as_double(0x7ff8000000000000LL) : rad;
  b.tau[oi] = tau;
}

// init_srcfunc (jurassic.c:3631-3681): one thread per (temperature, channel)
__global__ void k_srcfunc(int nd, int id0, int nch, const int* fn_off, const double* fnu,
                          const double* f, const double* st, double* sr) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= kNS * nch) return;
  const int it = gid % kNS;
  const int j = gid / kNS;
  const int id = id0 + j;
  const double* x = fnu + fn_off[j];
  const double* y = f + fn_off[j];
  const int n = fn_off[j + 1] - fn_off[j];
  double dnu = 1.0;
  for (int i = 1; i < n; i++) dnu = (x[i] - x[i - 1]) < dnu ? (x[i] - x[i - 1]) : dnu;
  const double temp = st[it];
  double fsum = 0, acc = 0;
  for (double v = x[0]; v <= x[n - 1]; v += dnu) {
    const int i = bracket_irr(x, n, v);
    const double w = lin(x[i], y[i], x[i + 1], y[i + 1], v);
    fsum += w;
    acc += w * planck(temp, v);
  }
  sr[(long long)it * nd + id] = acc / fsum;
}

// hydrostatic (jurassic.c:3520-3582): one thread per profile
__global__ void k_hydrostatic(CtlDev c, BatchDev b, double* p_out) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= b.nobs || c.hydz < 0) return;
  if (b.obs_skip && b.obs_skip[o]) return;
  const int l0 = b.lev_off[o], np = b.lev_off[o + 1] - l0;
  const double* z = b.z + l0;
  const double* t = b.t + l0;
  const double* qw = c.ig_h2o >= 0 ? b.q + (long long)c.ig_h2o * b.nlev + l0 : nullptr;
  double* p = p_out + l0;
  const double mmair = 28.96456e-3, mmh2o = 18.0153e-3;
  const int npts = 20;
  double best = 1e99, e = 0;
  int iref = 0;
  for (int ip = 0; ip < np; ip++)
    if (fabs(z[ip] - c.hydz) < best) {
      best = fabs(z[ip] - c.hydz);
      iref = ip;
    }
  for (int ip = iref + 1; ip < np; ip++) {
    double mean = 0;
    for (int i = 0; i < npts; i++) {
      if (qw) e = lin(0.0, qw[ip - 1], npts - 1.0, qw[ip], (double)i);
      mean += (e * mmh2o + (1 - e) * mmair) * kG0 / kRI /
              lin(0.0, t[ip - 1], npts - 1.0, t[ip], (double)i) / npts;
    }
    p[ip] = exp(log(p[ip - 1]) - mean * 1000 * (z[ip] - z[ip - 1]));
  }
  for (int ip = iref - 1; ip >= 0; ip--) {
    double mean = 0;
    for (int i = 0; i < npts; i++) {
      if (qw) e = lin(0.0, qw[ip + 1], npts - 1.0, qw[ip], (double)i);
      mean += (e * mmh2o + (1 - e) * mmair) * kG0 / kRI /
              lin(0.0, t[ip + 1], npts - 1.0, t[ip], (double)i) / npts;
    }
    p[ip] = exp(log(p[ip + 1]) - mean * 1000 * (z[ip] - z[ip + 1]));
  }
}

// ---------------------------------------------------------------------------
// launch wrappers

void launch_trace_count(const CtlDev& c, const ChanDev& ch, const BatchDev& b, const LosDev& L,
                        unsigned* err, cudaStream_t s) {
  const int bs = 64;
  k_trace_count<<<(b.nray + bs - 1) / bs, bs, 0, s>>>(c, ch, b, L, err);
}

void launch_trace_fill(const CtlDev& c, const ChanDev& ch, const BatchDev& b, const LosDev& L,
                       unsigned* err, cudaStream_t s) {
  const int bs = 64;
  k_trace_fill<<<(b.nray + bs - 1) / bs, bs, 0, s>>>(c, ch, b, L, err);
}

void launch_path_fp64(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                      const LosDev& L, double* refl_scratch, cudaStream_t s) {
  const long long nth = (long long)b.nray * c.nd;
  const int bs = 128;
  k_path_fp64<<<(unsigned)((nth + bs - 1) / bs), bs, 0, s>>>(c, T, ch, b, L, refl_scratch);
}

void launch_srcfunc(int nd, int id0, int nch, const int* fn_off, const double* fnu,
                    const double* f, const double* st, double* sr, cudaStream_t s) {
  const int nth = kNS * nch, bs = 128;
  k_srcfunc<<<(nth + bs - 1) / bs, bs, 0, s>>>(nd, id0, nch, fn_off, fnu, f, st, sr);
}

// formod_fov (jurassic.c:3121-3192), then BRIGHT and the mask of formod
// (3057-3067): one thread per (ray, channel) reads the pencil beams of the
// rays within +-5 of its own in the same observation with the same time.
__global__ void k_fov(CtlDev c, BatchDev b, const double* prad, const double* ptau, int nfov,
                      const double* fdz, const double* fw, const double* nu, unsigned* err) {
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nray = b.nray;
  if (gid >= nray * c.nd) return;
  const int id = (int)(gid / nray);
  const int r = (int)(gid % nray);
  const int o = b.ray_obs[r];
  if (b.obs_skip && b.obs_skip[o]) return;
  const double* time = b.geo;
  const double* vpz = b.geo + 4 * nray;
  double zz[11];
  int ray[11], nz = 0;
  const int lo = r - 5 > 0 ? r - 5 : 0;
  const int hi = r + 6 < nray ? r + 6 : (int)nray;
  for (int r2 = lo; r2 < hi; r2++)
    if (b.ray_obs[r2] == o && time[r2] == time[r]) {
      zz[nz] = vpz[r2];
      ray[nz++] = r2;
    }
  if (nz < 2) {
    atomicOr(err, kErrFov);
    return;
  }
  const double* pr = prad + (long long)id * nray;
  const double* pt = ptau + (long long)id * nray;
  double rs = 0, ts = 0, wsum = 0;
  for (int i = 0; i < nfov; i++) {
    const double zf = vpz[r] + fdz[i];
    const int k = bracket_irr(zz, nz, zf);
    rs += fw[i] * lin(zz[k], pr[ray[k]], zz[k + 1], pr[ray[k + 1]], zf);
    ts += fw[i] * lin(zz[k], pt[ray[k]], zz[k + 1], pt[ray[k + 1]], zf);
    wsum += fw[i];
  }
  rs /= wsum;
  ts /= wsum;
  if (c.write_bbt) {
    const double v = nu[id];
    rs = kC2 * v / log1p(kC1 * (v * v * v) / rs);
  }
  const long long oi = (long long)id * nray + r;
  b.rad[oi] = b.mask[oi] ? __longlong_as_double(0x7ff8000000000000LL) : rs;
  b.tau[oi] = ts;
}

void launch_fov(const CtlDev& c, const BatchDev& b, const double* prad, const double* ptau,
                int nfov, const double* fdz, const double* fw, const double* nu, unsigned* err,
                cudaStream_t s) {
  const long long nth = (long long)b.nray * c.nd;
  const int bs = 128;
  k_fov<<<(unsigned)((nth + bs - 1) / bs), bs, 0, s>>>(c, b, prad, ptau, nfov, fdz, fw, nu, err);
}

void launch_hydrostatic(const CtlDev& c, const BatchDev& b, double* p_out, cudaStream_t s) {
  const int bs = 64;
  k_hydrostatic<<<(b.nobs + bs - 1) / bs, bs, 0, s>>>(c, b, p_out);
}

// Loads the FP64 forward-model kernels onto the current device (CUDA loads
// modules lazily, at a kernel's first launch or attribute query), so that a
// later first launch allocates no device memory for their code.
int preload_fp64_kernels() {
  cudaFuncAttributes a;
  const void* fns[] = {(const void*)k_trace_count, (const void*)k_trace_fill,
                       (const void*)k_path_fp64, (const void*)k_hydrostatic};
  for (const void* f : fns)
    if (cudaFuncGetAttributes(&a, f) != cudaSuccess) return JGB_ERR_CUDA;
  return JGB_OK;
}

}  // namespace jgb
