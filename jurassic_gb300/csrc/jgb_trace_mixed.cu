// Ray tracing for the mixed-precision forward model.
//
// Same algorithm, step rule, refraction scheme and clipping as raytrace
// (jurassic.c:4201-4438, restated in FP64 in jgb_fp64.cu), with numerics
// chosen for GB300, whose FP64 pipe is ~64x narrower than FP32:
//  * the position x stays FP64 (three adds per step), but the altitude is
//    carried as z (FP64) plus exact FP32 increments
//      dz = (2 r (xhat . d) + |d|^2) / (r + sqrt(r^2 + 2 r (xhat . d) + |d|^2))
//    (no cancellation, relative error ~1e-7 of the step), so no FP64 square
//    roots, divisions or cart2geo per step;
//  * atmosphere interpolation (log-linear p, linear T, q, k; intpol_atm,
//    jurassic.c:3685-3706) runs in FP32 with per-level constants;
//  * the refractivity finite difference of the reference,
//    (N(xh + h e_k) - N(xh)) / h with N = 7.753e-5 p / T and h = 20 m,
//    is evaluated without cancellation:
//      N(z + dl) - N(z) = c p / (T T') (T expm1(s_p dl) - s_T dl)
//    inside one level (split at a level boundary), where N itself would only
//    carry ~7 significant digits in FP32;
//  * longitude and latitude are computed only at the points that use them
//    (first, last and the neighbours of the lowest point, for the tangent
//    point and the solar geometry);
//  * trapezoid lengths, column densities and Curtis-Godson sums in FP32
//    (compensated sums), written by the walk itself when the next point is
//    placed; the point data go to FP32 planes (z stays FP64);
//  * finite-difference perturbations in large EGA batches take their base
//    ray's geometry or walk on from the base's walk (TraceResume).
// The count and fill passes share the walk, so they agree on the point count.
#include "jgb_common.cuh"
#include "jgb_internal.h"

namespace jgb {
namespace {

constexpr float kRefracC = 7.753e-05f;

struct AtmM {
  int np;
  long long stride;
  const double *z, *p, *t, *q, *k;
  double clz, cldz, sfz, sfp, sft;
};

__device__ inline AtmM atm_m(const BatchDev& b, const CtlDev& c, int o) {
  AtmM a;
  const int l0 = b.lev_off[o];
  a.np = b.lev_off[o + 1] - l0;
  a.stride = b.nlev;
  a.z = b.z + l0;
  a.p = b.p + l0;
  a.t = b.t + l0;
  a.q = b.q + l0;
  a.k = b.k + l0;
  const double* s = b.scal + (long long)o * b.nscal;
  a.clz = s[0];
  a.cldz = s[1];
  a.sfz = s[2 + c.ncl];
  a.sfp = s[3 + c.ncl];
  a.sft = s[4 + c.ncl];
  return a;
}

// One level interval [z_i, z_i+1] of the profile in FP32 form.  Points are
// placed in it by their FP32 offset dl = z - z_i, so checking whether a
// point (or a refraction sub-point) is still in the interval needs no load.
struct Lev {
  int i;
  double z0;        // z_i
  float dz;         // z_i+1 - z_i
  float p0, p1, t0, t1;
  float sp;         // log(p1/p0)/dz (log-linear p) or (p1-p0)/dz (linear fallback)
  float st;         // (t1-t0)/dz
  bool plog;
  bool first, last; // lowest / highest interval (extrapolation below / above)
};

__device__ inline void lev_load(const AtmM& a, int i, Lev& L) {
  L.i = i;
  L.first = i == 0;
  L.last = i == a.np - 2;
  L.z0 = a.z[i];
  L.dz = (float)(a.z[i + 1] - a.z[i]);
  L.p0 = (float)a.p[i];
  L.p1 = (float)a.p[i + 1];
  L.t0 = (float)a.t[i];
  L.t1 = (float)a.t[i + 1];
  L.plog = (a.p[i + 1] / a.p[i]) > 0;
  L.sp = L.plog ? logf(L.p1 / L.p0) / L.dz : (L.p1 - L.p0) / L.dz;
  L.st = (L.t1 - L.t0) / L.dz;
}

// Is offset dl inside the interval (locate_irr semantics: the lowest
// interval also takes points below the grid, the highest those above)?
// Only for an ascending grid; otherwise the caller brackets.
__device__ inline bool lev_holds(const Lev& L, float dl) {
  return L.i >= 0 && L.dz > 0.f && (dl >= 0.f || L.first) && (dl < L.dz || L.last);
}

// Interval of z with the cached interval as hint, then its neighbour towards
// z (a ray or a refraction sub-point mostly crosses one level at a time:
// one round of independent loads instead of a bisection's chain); returns
// dl = z - z_i.  An interval that holds z is the one the bisection finds,
// so the hints change no result.
__device__ inline float lev_find(const AtmM& a, double z, Lev& L) {
  if (L.i >= 0) {
    const float dl = (float)(z - L.z0);
    if (lev_holds(L, dl)) return dl;
    const int j = dl < 0.f ? L.i - 1 : L.i + 1;
    if (j >= 0 && j <= a.np - 2) {
      Lev M;
      lev_load(a, j, M);
      const float dm = (float)(z - M.z0);
      if (lev_holds(M, dm)) {
        L = M;
        return dm;
      }
    }
  }
  lev_load(a, bracket_irr(a.z, a.np, z), L);
  return (float)(z - L.z0);
}

__device__ inline void lev_pt(const Lev& L, float dl, float* p, float* t) {
  *p = L.plog ? L.p0 * __expf(L.sp * dl) : L.p0 + L.sp * dl;
  *t = L.t0 + L.st * dl;
}

// exp(x) - 1 for the small exponents of the refraction finite differences:
// the Taylor series to x^4 where |x| < 1/64 (truncation below x^4/120
// relative, far under FP32 rounding), else expm1f.
__device__ inline float expm1_small(float x) {
  if (fabsf(x) < 0.015625f)
    return x * (1.f + x * (0.5f + x * (0.16666667f + x * 0.041666668f)));
  return expm1f(x);
}

// N(z + dl) - N(z) inside one level, from p, T at z (no cancellation).
__device__ inline float dN_in(const Lev& L, float p, float t, float dl) {
  const float t2 = t + L.st * dl;
  if (L.plog) return kRefracC * p / (t * t2) * (t * expm1_small(L.sp * dl) - L.st * dl);
  return kRefracC * dl * (L.sp * t - p * L.st) / (t * t2);
}

// Altitude increment of a displacement d from a point at radius r with
// radial unit vector xh.
__device__ inline float dz_of(const float* xh, float r, const float* d) {
  const float u = xh[0] * d[0] + xh[1] * d[1] + xh[2] * d[2];
  const float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  const float num = 2.f * r * u + dd;
  return num / (r + sqrtf(r * r + num));
}

// Lon/lat bookkeeping of the fill pass (positions of the first and last
// point and of the neighbours of the lowest one).
struct GeoKeep {
  double x_first[3], x_m1[3], x_p1[3], x_last[3];
  double zmin_seen;
  double ds_clip;     // the clipped last segment (point n - 2) in FP64
  float ds_m, ds_p1;  // raw segment lengths of the lowest point and the next
  int imin;
  bool want_p1;
};

// The walk's state at LOS point n, for walking on from there: position,
// direction and altitude at the point, the previous point's position and
// altitude, and the previous point's level interval (the search hint).
struct WalkFrom {
  int n;
  double x[3], e[3], z;
  double x_last[3], z_last;
  int lev_last;
  float raw_last;  // raw segment length of the previous point
};

// Mixing ratio or extinction at offset dl in a level interval, from the
// level value v0 and the slope (v1 - v0) / dz, rounded after the product
// and after the sum (shared by the walk and the copies of a base's
// geometry, so both give the same bits).
__device__ __forceinline__ float qk_at(float v0, float slope, float dl) {
  return __fadd_rn(v0, __fmul_rn(slope, dl));
}

// Column density of a segment, 10 / k_B q p / T ds (p in hPa, ds in km).
__device__ __forceinline__ float col_density(float q, float p, float t, float ds) {
  return (float)(10.0 / kKB) * q * p / t * ds;
}

// Threads per block of the trace kernels (the fill pass keeps per-thread
// level caches in shared memory with this stride).
constexpr int kTraceThreads = 64;

// The emitter and window values of level i and their slopes (v1 - v0) / dz
// over interval i, into the per-thread cache qc (stride kTraceThreads):
// qc[k] = v0, qc[nqk + k] = slope, nqk = ng + nw.
__device__ __forceinline__ void level_values(const CtlDev& c, const AtmM& a, int i, float dz,
                                             float* qc) {
  const int nqk = c.ng + c.nw;
  for (int k = 0; k < nqk; k++) {
    const double* src = k < c.ng ? a.q + k * a.stride : a.k + (k - c.ng) * a.stride;
    const float v0 = (float)src[i], v1 = (float)src[i + 1];
    qc[k * kTraceThreads] = v0;
    qc[(nqk + k) * kTraceThreads] = (v1 - v0) / dz;
  }
}

// Per-thread shared memory of the fill pass, stride kTraceThreads: the
// current level's emitter and window values and slopes (qc[k], qc[nqk + k],
// nqk = ng + nw), the mixing ratios of the point waiting for its trapezoid
// length (pq[ig]) and, in CGA, the running compensated sums (cg[6 ig + j]).
__host__ __device__ inline int trace_smem_floats(const CtlDev& c) {
  return 2 * (c.ng + c.nw) + c.ng + (c.formod == 0 ? 6 * c.ng : 0);
}

// STORE places every point with its final values: its trapezoid length
// 0.5 (ds_(i-1) + ds_i), column densities 10 / k_B q p / T ds and CGA sums
// are written when the next point is placed (the clip of the last segment
// changes the previous point's raw length), so the walk keeps the raw
// lengths of the last two points.
// ROLE 1 keeps every point's position, direction, raw length and level
// interval in sv; ROLE 2 with wf walks on from the state wf (a base ray's
// walk).
template <bool STORE, int ROLE = 0>
__device__ int walk_m(const CtlDev& c, const AtmM& a, const double* g, long long nray, int r,
                      const LosDev& L, long long base, int cap, double* sft_out, GeoKeep* gk,
                      float* qc, unsigned* err, const WalkFrom* wf = nullptr,
                      const TraceResume* sv = nullptr) {
  const float h = 0.02f;
  const double zrefrac = 60;
  *sft_out = -999;
  const double obsz = g[1 * nray + r], obslon = g[2 * nray + r], obslat = g[3 * nray + r];
  const double vpz = g[4 * nray + r], vplon = g[5 * nray + r], vplat = g[6 * nray + r];
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

  // the direction stays FP64: renormalising an FP32 unit vector every step
  // would random-walk it by ~1e-7 rad per step (metres over a limb path)
  double x[3], ex0[3], z;
  double last_z = 0, x_last[3] = {0, 0, 0};
  Lev lv;
  lv.i = -1;
  int n = 0, stop = 0, qc_level = -1;
  if (ROLE == 2 && wf) {  // on from a base's walk
    for (int i = 0; i < 3; i++) {
      x[i] = wf->x[i];
      ex0[i] = wf->e[i];
      x_last[i] = wf->x_last[i];
    }
    z = wf->z;
    last_z = wf->z_last;
    n = wf->n;
    lev_load(a, wf->lev_last, lv);
  } else {
    double xobs[3], xvp[3];
    to_cart(obsz, obslon, obslat, xobs);
    to_cart(vpz, vplon, vplat, xvp);
    for (int i = 0; i < 3; i++) ex0[i] = xvp[i] - xobs[i];
    const double norm = sqrt(ex0[0] * ex0[0] + ex0[1] * ex0[1] + ex0[2] * ex0[2]);
    for (int i = 0; i < 3; i++) {
      ex0[i] /= norm;
      x[i] = xobs[i];
    }
    z = obsz;
    if (obsz > zmax) {  // entry into the atmosphere: bisection on the line of sight (FP64, once)
      double dmax = norm, dmin = 0;
      for (int guard = 0; fabs(dmin - dmax) > 0.001 && guard < 200; guard++) {
        const double d = (dmax + dmin) / 2;
        for (int i = 0; i < 3; i++) x[i] = xobs[i] + d * ex0[i];
        z = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]) - kRE;
        if (z <= zmax && z > zmax - 0.001) break;
        if (z < zmax - 0.0005) dmax = d; else dmin = d;
      }
    }
    z = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]) - kRE;
  }
  const int nqk = c.ng + c.nw;
  const float rayds = (float)c.rayds, raydz = (float)c.raydz;
  // the direction in FP32 (carried from the previous step's conversion)
  float ef[3] = {(float)ex0[0], (float)ex0[1], (float)ex0[2]};
  // the point waiting for its final values (STORE): raw lengths of it and
  // of the point before, its p and T; its mixing ratios in pq
  float* pq = STORE ? qc + 2 * nqk * kTraceThreads : nullptr;
  float* cg = STORE ? pq + c.ng * kTraceThreads : nullptr;
  float raw_before = 0.f, raw_pend = 0.f, pend_p = 0.f, pend_t = 0.f;
  const int n0 = n;
  if (ROLE == 2 && wf) raw_pend = wf->raw_last;
  if (STORE && L.cga)
    for (int k = 0; k < 6 * c.ng; k++) cg[k * kTraceThreads] = 0.f;
  auto finalize = [&](int k) {
    const long long sk = base + k;
    const float dsT = k == 0 ? 0.5f * raw_pend : 0.5f * (raw_before + raw_pend);
    L.f.ds[sk] = dsT;
    for (int ig = 0; ig < c.ng; ig++) {
      const float uu = col_density(pq[ig * kTraceThreads], pend_p, pend_t, dsT);
      L.f.u[ig * L.cap + sk] = uu;
      if (L.cga) {  // compensated running sums
        float* q = cg + 6 * ig * kTraceThreads;
        float su = q[0], sp = q[kTraceThreads], st = q[2 * kTraceThreads];
        float cu = q[3 * kTraceThreads], cp = q[4 * kTraceThreads], ct = q[5 * kTraceThreads];
        float y = uu - cu, s2 = su + y;
        cu = (s2 - su) - y;
        su = s2;
        y = uu * pend_p - cp;
        s2 = sp + y;
        cp = (s2 - sp) - y;
        sp = s2;
        y = uu * pend_t - ct;
        s2 = st + y;
        ct = (s2 - st) - y;
        st = s2;
        q[0] = su;
        q[kTraceThreads] = sp;
        q[2 * kTraceThreads] = st;
        q[3 * kTraceThreads] = cu;
        q[4 * kTraceThreads] = cp;
        q[5 * kTraceThreads] = ct;
        L.f.cgu[ig * L.cap + sk] = su;
        L.f.cgp[ig * L.cap + sk] = sp / su;
        L.f.cgt[ig * L.cap + sk] = st / su;
      }
    }
  };
  for (;;) {
    // radial unit vector and radius at x
    const double rr = z + kRE;
    const float rf = (float)rr, rinv = 1.f / rf;
    float xh[3] = {(float)x[0] * rinv, (float)x[1] * rinv, (float)x[2] * rinv};
    // step length from this point (jurassic.c:4278-4287)
    float step = rayds;
    if (raydz > 0) {
      const float cosa = fabsf(ef[0] * xh[0] + ef[1] * xh[1] + ef[2] * xh[2]);
      if (cosa != 0) step = rayds < raydz / cosa ? rayds : raydz / cosa;
    }
    // ground or top of the atmosphere: clip the last segment (4292-4306;
    // the previous point's step becomes this point's step times frac)
    if ((z < zmin || z > zmax) && n > 0) {
      if (!STORE) {
        if (n >= cap) {
          atomicOr(err, cap < c.nlos_max ? kErrSlabOverflow : kErrLosOverflow);
          return -1;
        }
        return n + 1;
      }
      stop = (z < zmin ? 2 : 1);
      const double frac = ((z < zmin ? zmin : zmax) - last_z) / (z - last_z);
      for (int i = 0; i < 3; i++) x[i] = x_last[i] + frac * (x[i] - x_last[i]);
      z = last_z + frac * (z - last_z);
      const double dsc = (double)step * frac;
      raw_pend = (float)dsc;
      if (ROLE == 1) sv->dsr[base + n - 1] = raw_pend;
      gk->ds_clip = dsc;
      step = 0.f;
    }
    if (n >= cap) {
      atomicOr(err, cap < c.nlos_max ? kErrSlabOverflow : kErrLosOverflow);
      return -1;
    }
    const float dl = lev_find(a, z, lv);
    float p, t;
    lev_pt(lv, dl, &p, &t);
    if (STORE) {
      if (n > n0) finalize(n - 1);
      const long long s = base + n;
      L.z[s] = z;
      L.f.p[s] = p;
      L.f.t[s] = t;
      raw_before = raw_pend;
      raw_pend = step;
      pend_p = p;
      pend_t = t;
      const int i = lv.i;
      if (i != qc_level) {  // a new level: its values and slopes q0 + (q1 - q0) / dz * dl
        qc_level = i;
        level_values(c, a, i, lv.dz, qc);
      }
      for (int ig = 0; ig < c.ng; ig++) {
        const float v = qk_at(qc[ig * kTraceThreads], qc[(nqk + ig) * kTraceThreads], dl);
        pq[ig * kTraceThreads] = v;
        if (ig == c.ig_h2o) L.f.qh2o[s] = v;
      }
      for (int iw = 0; iw < c.nw; iw++)
        L.f.kw[iw * L.cap + s] = qk_at(qc[(c.ng + iw) * kTraceThreads],
                                       qc[(nqk + c.ng + iw) * kTraceThreads], dl);
      if (ROLE == 1) {
        const long long bp = sv->bpts;
        for (int i2 = 0; i2 < 3; i2++) {
          sv->xs[i2 * bp + s] = x[i2];
          sv->es[i2 * bp + s] = ex0[i2];
        }
        sv->lev[s] = i;
        sv->dsr[s] = step;
      }
      if (c.ncl > 0 && a.cldz > 0) {
        const float v = (float)((z - a.clz) / a.cldz);
        L.f.aux[s] = expf(-0.5f * v * v);
      } else {
        L.f.aux[s] = 0.f;
      }
      // geometry kept for lon/lat of the points that need them
      if (n == 0)
        for (int i2 = 0; i2 < 3; i2++) gk->x_first[i2] = x[i2];
      if (gk->want_p1) {
        for (int i2 = 0; i2 < 3; i2++) gk->x_p1[i2] = x[i2];
        gk->ds_p1 = step;
        gk->want_p1 = false;
      }
      if (n == 0 || z < gk->zmin_seen) {
        gk->zmin_seen = z;
        gk->imin = n;
        gk->ds_m = step;
        for (int i2 = 0; i2 < 3; i2++) gk->x_m1[i2] = x_last[i2];   // the previous point
        gk->want_p1 = true;
      }
    }
    last_z = z;
    for (int i2 = 0; i2 < 3; i2++) x_last[i2] = x[i2];
    n++;
    if (stop) {
      if (c.nsf > 0 && a.sft > 0) t = (float)a.sft;
      *sft_out = (stop == 2 ? (c.nsf > 0 && a.sft > 0 ? a.sft : (double)t) : -999);
      if (STORE) {
        for (int i2 = 0; i2 < 3; i2++) gk->x_last[i2] = x[i2];
        finalize(n - 1);
      }
      break;
    }
    // refraction (jurassic.c:4388-4415): ex1 = (n ex0 + ds grad N) / |...|
    // = (ex0 + inc) / |ex0 + inc| with inc = ds grad N / n, the increment in
    // FP32 and the renormalisation as a series in delta = |ex0 + inc|^2 - 1
    const bool bend = c.refrac && z <= zrefrac;
    double ex1[3] = {ex0[0], ex0[1], ex0[2]};
    if (bend) {
      const float nref = 1.f + kRefracC * p / t;
      // midpoint xh = x + ds/2 ex0 and its radial unit vector
      const float d[3] = {0.5f * step * ef[0], 0.5f * step * ef[1], 0.5f * step * ef[2]};
      const float dzh = dz_of(xh, rf, d);
      const float rh = rf + dzh, rhinv = 1.f / rh;
      const float xhh[3] = {(xh[0] * rf + d[0]) * rhinv, (xh[1] * rf + d[1]) * rhinv,
                            (xh[2] * rf + d[2]) * rhinv};
      // midpoint offset in the point's interval (FP64 only when it leaves it)
      Lev lh = lv;
      float dlh = dl + dzh;
      if (!lev_holds(lh, dlh)) dlh = lev_find(a, z + dzh, lh);
      float ph, th;
      lev_pt(lh, dlh, &ph, &th);
      float inc[3];
      for (int k = 0; k < 3; k++) {
        float dk[3] = {0.f, 0.f, 0.f};
        dk[k] = h;
        const float dlk = dz_of(xhh, rh, dk);
        float dN;
        if (lev_holds(lh, dlh + dlk)) {
          dN = dN_in(lh, ph, th, dlk);
        } else {
          // split at the level boundary between the midpoint and zk
          const double zh = lh.z0 + (double)dlh, zk = zh + dlk;
          Lev lk = lh;
          const float dlk0 = lev_find(a, zk, lk);
          if (lk.i == lh.i) {
            dN = dN_in(lh, ph, th, dlk);
          } else {
            const bool up = lk.i > lh.i;
            const double zb = up ? a.z[lh.i + 1] : a.z[lh.i];
            const float d1 = (float)(zb - zh);
            const float dn1 = dN_in(lh, ph, th, d1);
            float pb, tb;
            const float dlb = (float)(zb - lk.z0);
            lev_pt(lk, dlb, &pb, &tb);
            dN = dn1 + dN_in(lk, pb, tb, dlk0 - dlb);
          }
        }
        inc[k] = step * (dN / h) / nref;
      }
      const float delta = 2.f * (ef[0] * inc[0] + ef[1] * inc[1] + ef[2] * inc[2]) +
                          (inc[0] * inc[0] + inc[1] * inc[1] + inc[2] * inc[2]);
      for (int k = 0; k < 3; k++) ex1[k] = ex0[k] + (double)inc[k];
      if (fabsf(delta) < 1e-3f) {
        const float corr = delta * (-0.5f + delta * (0.375f - 0.3125f * delta));
        for (int k = 0; k < 3; k++) ex1[k] += ex1[k] * (double)corr;
      } else {
        const double nn = sqrt(ex1[0] * ex1[0] + ex1[1] * ex1[1] + ex1[2] * ex1[2]);
        for (int k = 0; k < 3; k++) ex1[k] /= nn;
      }
    }
    float D[3], efn[3];
    for (int k = 0; k < 3; k++) {
      efn[k] = (float)ex1[k];
      D[k] = 0.5f * step * (ef[k] + efn[k]);
    }
    const float dzs = dz_of(xh, rf, D);
    for (int k = 0; k < 3; k++) {
      x[k] += (double)D[k];
      ex0[k] = ex1[k];
      ef[k] = efn[k];
    }
    z += dzs;
  }
  return n;
}

__global__ void k_trace_count_m(CtlDev c, BatchDev b, LosDev L, unsigned* err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= b.nray) return;
  if (b.obs_skip && b.obs_skip[b.ray_obs[r]]) {
    L.count[r] = 0;
    return;
  }
  const AtmM a = atm_m(b, c, b.ray_obs[r]);
  double sft;
  const int n = walk_m<false>(c, a, b.geo, b.nray, r, L, 0, c.nlos_max, &sft, nullptr, nullptr,
                              err);
  L.count[r] = n < 0 ? 0 : n;
}

// Upper bound of the LOS points of every ray, for tracing a large batch in
// one pass.  The step rule ds = min(RAYDS, RAYDZ/|cos a|) (jurassic.c:
// 4278-4287) makes every step either RAYDS long or move the point by RAYDZ
// along the local vertical, less the curvature term ds^2/(2 r) <=
// RAYDS^2/(2 RE).  A path of length S through a total altitude change V so
// takes at most S/RAYDS + V/(RAYDZ - RAYDS^2/(2 RE)) steps, plus the first
// and the clipped last point.  S and V come from the straight line of sight
// (entry at the top of the atmosphere, exit at the top or at the lowest
// level), with 10 % and, with refraction, 4 km of altitude as margins for
// the bending; the bound is scaled by jgb_set_los_bound_scale.  A ray that
// still outgrows its bound raises
// kErrSlabOverflow in the fill pass and the batch is traced again with
// exact counts, so the bound only decides the memory and the speed.
__global__ void k_los_bound_m(CtlDev c, BatchDev b, double scale, int* cap) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= b.nray) return;
  if (b.obs_skip && b.obs_skip[b.ray_obs[r]]) {
    cap[r] = 0;
    return;
  }
  const AtmM a = atm_m(b, c, b.ray_obs[r]);
  double zmin = a.z[0], zmax = a.z[0];
  for (int i = 1; i < a.np; i++) {
    zmin = fmin(zmin, a.z[i]);
    zmax = fmax(zmax, a.z[i]);
  }
  const long long nr = b.nray;
  const double* g = b.geo;
  const double obsz = g[1 * nr + r], vpz = g[4 * nr + r];
  if (vpz > zmax || obsz < zmin) {  // no LOS, or an error raised by the fill pass
    cap[r] = 2;
    return;
  }
  double xo[3], xv[3], d[3];
  to_cart(obsz, g[2 * nr + r], g[3 * nr + r], xo);
  to_cart(vpz, g[5 * nr + r], g[6 * nr + r], xv);
  const double dn = sqrt((xv[0] - xo[0]) * (xv[0] - xo[0]) + (xv[1] - xo[1]) * (xv[1] - xo[1]) +
                         (xv[2] - xo[2]) * (xv[2] - xo[2]));
  for (int i = 0; i < 3; i++) d[i] = dn > 0 ? (xv[i] - xo[i]) / dn : 0.0;
  // |xo + s d|^2 = r02 + 2 bb s + s^2
  const double bb = xo[0] * d[0] + xo[1] * d[1] + xo[2] * d[2];
  const double r02 = xo[0] * xo[0] + xo[1] * xo[1] + xo[2] * xo[2];
  const double rt = kRE + zmax, rb = kRE + zmin;
  const double disc_t = fmax(bb * bb - (r02 - rt * rt), 0.0);
  const double s_in = r02 > rt * rt ? fmax(-bb - sqrt(disc_t), 0.0) : 0.0;
  const double r_in = sqrt(fmax(r02 + 2 * bb * s_in + s_in * s_in, 0.0));
  const double s_t = -bb, rmin = sqrt(fmax(r02 - bb * bb, 0.0));
  double s_out, V;
  if (rmin < rb && s_t > s_in) {  // down to the lowest level
    s_out = -bb - sqrt(fmax(bb * bb - (r02 - rb * rb), 0.0));
    V = r_in - rb;
  } else {
    s_out = -bb + sqrt(disc_t);
    V = (s_t > s_in && s_t < s_out) ? (r_in - rmin) + (rt - rmin) : fabs(rt - r_in);
  }
  const double S = fmax(s_out - s_in, 0.0);
  double est = c.rayds > 0 ? S / c.rayds : 0.0;
  if (c.raydz > 0) {
    const double per = fmax(c.raydz - c.rayds * c.rayds / (2 * kRE), 0.5 * c.raydz);
    est += (V + (c.refrac ? 4.0 : 0.0)) / per;
  }
  const double bound = ceil(scale * 1.1 * est) + 16;
  cap[r] = bound >= (double)c.nlos_max ? c.nlos_max : (int)bound;
}

// Resumed perturbation of mode 2 (TraceResume): ray r takes base ray rb's
// LOS geometry, p, T, cloud weights, segment lengths, tangent point and
// ends, and evaluates its own mixing ratios and extinctions on the base's
// level intervals, as its own walk would.
__device__ void copy_base_geometry(const CtlDev& c, const BatchDev& b, const LosDev& L,
                                   const AtmM& a, int r, int rb, int cap, const TraceResume& R,
                                   float* qc, unsigned* err) {
  const long long base = L.off[r], ob = L.off[rb];
  const int n = L.count[rb];
  if (n > cap) {
    atomicOr(err, cap < c.nlos_max ? kErrSlabOverflow : kErrLosOverflow);
    return;
  }
  const long long nr = b.nray;
  for (int k = 0; k < 3; k++) b.tp[k * nr + r] = b.tp[k * nr + rb];
  for (int k = 0; k < 6; k++) L.ends[6LL * r + k] = L.ends[6LL * rb + k];
  L.sft[r] = L.sft[rb];
  L.count[r] = n;
  const int nqk = c.ng + c.nw;
  int qc_level = -1;
  double z0 = 0;
  for (int ip = 0; ip < n; ip++) {
    const long long q = ob + ip, s = base + ip;
    const double z = L.z[q];
    const float pf = L.f.p[q], tf = L.f.t[q], dsf = L.f.ds[q];
    L.z[s] = z;
    L.f.p[s] = pf;
    L.f.t[s] = tf;
    L.f.ds[s] = dsf;
    L.f.aux[s] = L.f.aux[q];
    const int i = R.lev[q];
    if (i != qc_level) {  // the walk's level values and slopes
      qc_level = i;
      z0 = a.z[i];
      level_values(c, a, i, (float)(a.z[i + 1] - a.z[i]), qc);
    }
    const float dl = (float)(z - z0);
    for (int ig = 0; ig < c.ng; ig++) {
      const float v = qk_at(qc[ig * kTraceThreads], qc[(nqk + ig) * kTraceThreads], dl);
      if (ig == c.ig_h2o) L.f.qh2o[s] = v;
      L.f.u[ig * L.cap + s] = col_density(v, pf, tf, dsf);
    }
    for (int iw = 0; iw < c.nw; iw++)
      L.f.kw[iw * L.cap + s] = qk_at(qc[(c.ng + iw) * kTraceThreads],
                                     qc[(nqk + c.ng + iw) * kTraceThreads], dl);
  }
}

// order (optional): thread t traces ray order[t], else ray r0 + t, so that a
// warp's rays have similar LOS capacities and finish together; each ray's
// outputs go to its own slots, so the order does not change any result.
// ROLE 0: plain rays; 1: base rays of resumed perturbations (their walks are
// kept in R); 2: the perturbations (R.plan; EGA only: the Curtis-Godson sums
// run from the first point).
template <int ROLE>
__global__ void k_trace_fill_m(CtlDev c, BatchDev b, LosDev L, const int* order, int r0, int nr_l,
                               TraceResume R, unsigned* err) {
  const int th = blockIdx.x * blockDim.x + threadIdx.x;
  if (th >= nr_l) return;
  const int r = order ? order[th] : r0 + th;
  if (b.obs_skip && b.obs_skip[b.ray_obs[r]]) {
    L.count[r] = 0;
    return;
  }
  const AtmM a = atm_m(b, c, b.ray_obs[r]);
  const long long base = L.off[r];
  const int cap = L.count[r];
  extern __shared__ float qcache[];  // trace_smem_floats(c) per thread
  int4 pl = make_int4(-1, 0, 0, 0);
  if (ROLE == 2) pl = R.plan[r];
  if (ROLE == 2 && pl.z == 2) {
    copy_base_geometry(c, b, L, a, r, pl.x, cap, R, qcache + threadIdx.x, err);
    return;
  }
  double sft;
  GeoKeep gk;
  gk.want_p1 = false;
  gk.imin = 0;
  gk.zmin_seen = 0;
  gk.ds_clip = 0;
  gk.ds_m = gk.ds_p1 = 0.f;
  for (int i = 0; i < 3; i++) gk.x_m1[i] = gk.x_p1[i] = gk.x_first[i] = gk.x_last[i] = 0;
  // mode 1: points [0, m) are the base's (final values); the walk goes on
  // from the base's state at m, its lon/lat bookkeeping restated from the
  // base's points before m
  int m = 0;
  long long ob = 0;
  WalkFrom wf;
  if (ROLE == 2 && pl.z == 1) {
    m = pl.y;
    ob = L.off[pl.x];
    if (m > cap) {
      atomicOr(err, cap < c.nlos_max ? kErrSlabOverflow : kErrLosOverflow);
      return;
    }
    const long long bp = R.bpts;
    for (int ip = 0; ip < m; ip++) {
      const long long q = ob + ip, s = base + ip;
      L.z[s] = L.z[q];
      L.f.p[s] = L.f.p[q];
      L.f.t[s] = L.f.t[q];
      L.f.ds[s] = L.f.ds[q];
      L.f.aux[s] = L.f.aux[q];
      if (c.ig_h2o >= 0) L.f.qh2o[s] = L.f.qh2o[q];
      for (int ig = 0; ig < c.ng; ig++) L.f.u[ig * L.cap + s] = L.f.u[ig * L.cap + q];
      for (int iw = 0; iw < c.nw; iw++) L.f.kw[iw * L.cap + s] = L.f.kw[iw * L.cap + q];
    }
    wf.n = m;
    for (int i = 0; i < 3; i++) {
      wf.x[i] = R.xs[i * bp + ob + m];
      wf.e[i] = R.es[i * bp + ob + m];
      wf.x_last[i] = R.xs[i * bp + ob + m - 1];
      gk.x_first[i] = R.xs[i * bp + ob];
    }
    wf.z = L.z[ob + m];
    wf.z_last = L.z[ob + m - 1];
    wf.lev_last = R.lev[ob + m - 1];
    wf.raw_last = R.dsr[ob + m - 1];
    // the first lowest point so far and its neighbours
    int imin = 0;
    double zmin = L.z[ob];
    for (int ip = 1; ip < m; ip++)
      if (L.z[ob + ip] < zmin) {
        zmin = L.z[ob + ip];
        imin = ip;
      }
    gk.imin = imin;
    gk.zmin_seen = zmin;
    gk.want_p1 = imin == m - 1;
    gk.ds_m = R.dsr[ob + imin];
    if (imin + 1 < m) gk.ds_p1 = R.dsr[ob + imin + 1];
    for (int i = 0; i < 3; i++) {
      gk.x_m1[i] = imin > 0 ? R.xs[i * bp + ob + imin - 1] : 0.0;
      gk.x_p1[i] = imin + 1 < m ? R.xs[i * bp + ob + imin + 1] : 0.0;
    }
  }
  const int n = walk_m<true, ROLE>(c, a, b.geo, b.nray, r, L, base, cap, &sft, &gk,
                                   qcache + threadIdx.x, err, m > 0 ? &wf : nullptr, &R);
  L.sft[r] = sft;
  if (n > 0) L.count[r] = n;
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
  double dummy, lon0, lat0, lonl, latl;
  to_geo(gk.x_first, &dummy, &lon0, &lat0);
  to_geo(gk.x_last, &dummy, &lonl, &latl);
  // tangent point (tangent_point, jurassic.c:5223-5263) from the raw lengths
  const int imin = gk.imin;
  if (imin <= 0 || imin >= n - 1) {
    tp[0 * nr + r] = z[n - 1];
    tp[1 * nr + r] = lonl;
    tp[2 * nr + r] = latl;
  } else {
    const double y0 = z[imin - 1], y1 = z[imin], y2 = z[imin + 1];
    // raw segment lengths (the clipped last one, of point n - 2, in FP64)
    const double d1 = imin == n - 2 ? gk.ds_clip : (double)gk.ds_m;
    const double d2 = imin + 1 == n - 2 ? gk.ds_clip : (double)gk.ds_p1;
    const double x1 = sqrt(d1 * d1 - (y1 - y0) * (y1 - y0));
    const double x2 = x1 + sqrt(d2 * d2 - (y2 - y1) * (y2 - y1));
    const double aa = 1 / (x1 - x2) * (-(y0 - y1) / x1 + (y0 - y2) / x2);
    const double bb = -(y0 - y1) / x1 - aa * x1;
    const double cc = y0;
    const double xt = -bb / (2 * aa);
    tp[0 * nr + r] = aa * xt * xt + bb * xt + cc;
    double v[3], tlon, tlat;
    for (int i = 0; i < 3; i++) v[i] = lin(0.0, gk.x_m1[i], x2, gk.x_p1[i], xt);
    to_geo(v, &dummy, &tlon, &tlat);
    tp[1 * nr + r] = tlon;
    tp[2 * nr + r] = tlat;
  }
  double* e = L.ends + 6LL * r;
  e[0] = z[0];
  e[1] = lon0;
  e[2] = lat0;
  e[3] = z[n - 1];
  e[4] = lonl;
  e[5] = latl;
}

}  // namespace

void launch_trace_count_mixed(const CtlDev& c, const BatchDev& b, const LosDev& L, unsigned* err,
                              cudaStream_t s) {
  const int bs = kTraceThreads;
  k_trace_count_m<<<(b.nray + bs - 1) / bs, bs, 0, s>>>(c, b, L, err);
}

void launch_los_bound_mixed(const CtlDev& c, const BatchDev& b, double scale, int* cap,
                            cudaStream_t s) {
  const int bs = 128;
  k_los_bound_m<<<(b.nray + bs - 1) / bs, bs, 0, s>>>(c, b, scale, cap);
}

void launch_trace_fill_mixed(const CtlDev& c, const BatchDev& b, const LosDev& L, const int* order,
                             unsigned* err, cudaStream_t s) {
  const int bs = kTraceThreads;
  const size_t smem = sizeof(float) * trace_smem_floats(c) * kTraceThreads;
  k_trace_fill_m<0><<<(b.nray + bs - 1) / bs, bs, smem, s>>>(c, b, L, order, 0, b.nray,
                                                              TraceResume{}, err);
}

int trace_fill_resident(int sms) {
  // blocks per SM are set by the registers (the shared memory of a few
  // emitters does not bind); computed once, thread-safely
  static const int per_sm = [] {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_trace_fill_m<2>, kTraceThreads, 0) !=
            cudaSuccess ||
        nb < 1)
      nb = 1;
    return nb * kTraceThreads;
  }();
  return per_sm * sms;
}

void launch_trace_fill_resumed(const CtlDev& c, const BatchDev& b, const LosDev& L,
                               const int* order, int r0, int nr, const TraceResume& R, int role,
                               unsigned* err, cudaStream_t s) {
  const int bs = kTraceThreads;
  if (nr <= 0) return;
  const size_t smem = sizeof(float) * trace_smem_floats(c) * kTraceThreads;
  if (role == 1)
    k_trace_fill_m<1><<<(nr + bs - 1) / bs, bs, smem, s>>>(c, b, L, order, r0, nr, R, err);
  else
    k_trace_fill_m<2><<<(nr + bs - 1) / bs, bs, smem, s>>>(c, b, L, order, r0, nr, R, err);
}

}  // namespace jgb
