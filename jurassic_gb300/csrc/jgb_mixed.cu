// Mixed-precision forward model: FP32 path loop with compensated sums.
//
// Work decomposition: rays are sorted by LOS length and grouped into tiles
// of 32 (one ray per lane); a warp walks one tile for one channel, so all
// lanes of a warp read the same emissivity table (same channel, emitter)
// at neighbouring rows and the same LOS plane entries (one 128-byte line
// per field and point).  A block holds 4 warps = 4 channels of one tile,
// which share the tile's LOS data through L1.
//
// Numerics (same algorithm as intpol_tbl_ega/cga, jurassic.c:3710-3891, and
// formod_pencil, 3196-3338):
//  * each (channel, emitter) carries its path transmittance t and path
//    emissivity e = 1 - t as two floats, each accurate where it is small,
//    so that neither 1 - t nor 1 - e is ever formed from a rounded value;
//  * segment emissivities are combined as E <- E + (1 - E) eps_g (no
//    cancellation for small eps), the continuum as -expm1(-beta ds);
//  * the radiance sum is Kahan-compensated.
#include "jgb_common.cuh"
#include "jgb_internal.h"

namespace jgb {

// Field indices of a tile plane: the point's p, t, ds, q_H2O and cloud
// factor, the extinction per window, then one block of kEmitterFields(CGA)
// fields per emitter, emitter g's at g0 + g * es + k (k constant, so that a
// warp addresses them from one base):
//   EGA: u, br, pw, wa, wb;  CGA: u, cgp, cgt, cgu, br, pw, wa, wb.
// For emitters whose p-T grids are shared by all channels, the
// channel-independent part of the table interpolation is done once per LOS
// point: br holds the rows of the point's p-T cell within a (channel,
// emitter) table, ipr * tt + it0 | ((ipr + 1) * tt + it1) << 16
// (kNoBracket: no table, kNoBracket | 2: no temperature rows at that
// pressure; tp * tt < 2^15), pw the pressure interpolation weight in that
// bracket (linear in EGA, log-linear in CGA), wa and wb the temperature
// weights at the lower and upper pressure of the bracket.
struct Fields {
  int p, t, ds, qh2o, aux, kw0, g0, es, n;
};
constexpr int kFU = 0;  // column of the segment (EGA) / of the path (continua)
constexpr int kFCgp = 1, kFCgt = 2, kFCgu = 3;  // CGA means
__host__ __device__ constexpr int kEmitterFields(bool cga) { return cga ? 8 : 5; }
__host__ __device__ constexpr int kFBr(bool cga) { return cga ? 4 : 1; }  // then pw, wa, wb

__host__ __device__ inline Fields fields_of(const CtlDev& c, unsigned brmask) {
  (void)brmask;
  Fields f;
  f.p = 0;
  f.t = 1;
  f.ds = 2;
  f.qh2o = 3;
  f.aux = 4;
  f.kw0 = 5;
  f.g0 = 5 + c.nw;
  f.es = kEmitterFields(c.formod == 0);
  f.n = f.g0 + c.ng * f.es;
  return f;
}

int mixed_nfield(const CtlDev& c, unsigned brmask) { return fields_of(c, brmask).n; }

constexpr unsigned kNoBracket = 0x80000000u;

// ---------------------------------------------------------------------------
// float table access with hinted searches
//
// Along a path the column density of every (channel, emitter) only grows
// and pressure/temperature change slowly, so the bracket found at one LOS
// point is almost always the bracket (or its neighbour) at the next point.
// Each search therefore first tests the remembered bracket and the next one
// with independent loads (one round trip) and falls back to bisection
// only on a miss.  Any valid bracket gives the same interpolated value, so
// the result does not depend on the hint.

struct RowF {
  unsigned off;          // row start in the u and eps arrays
  int n;
  float u0, un, e0, en;  // first/last entries of the row
  float t;               // temperature of the row
};

// Row r = (dg * tp + ip) * tt + it from its record; 32-bit row arithmetic
// (the table upload checks that rows x TU < 2^32).  EGA records are 32
// bytes, {u[0], u[n-1], eps[0], eps[n-1]} and {n (int bits), t, 0, 0}: both
// ends of a row are tested before any search (the path emissivity starts
// below the rows and saturates above them).  CGA records are 16 bytes,
// {n, t, u[0], eps[0]}: a column above a row brackets at n-2, and the
// search brings the row's last entries.
// With the temperature weights precomputed (PRE) a row's temperature is not
// needed: EGA then reads only the count n of the second half of the record.
template <bool CGA, bool PRE = false>
__device__ __forceinline__ RowF rowf_at(const TblDev& T, unsigned r) {
  RowF w;
  w.off = r * (unsigned)T.tu;
  if (CGA) {
    const float4 m = __ldg(T.rowmeta + r);
    w.n = __float_as_int(m.x);
    w.t = m.y;
    w.u0 = m.z;
    w.e0 = m.w;
    w.un = w.en = 0.f;
  } else {
    const float4 m = __ldg(T.rowmeta + 2 * r);
    if (PRE) {
      w.n = __ldg(reinterpret_cast<const int*>(T.rowmeta + 2 * r + 1));
      w.t = 0.f;
    } else {
      const float4 m2 = __ldg(T.rowmeta + 2 * r + 1);
      w.n = __float_as_int(m2.x);
      w.t = m2.y;
    }
    w.u0 = m.x;
    w.un = m.y;
    w.e0 = m.z;
    w.en = m.w;
  }
  return w;
}

// A bracket index i with the grid values at i and i + 1.
struct Bracket {
  int i;
  float a, b;
};

// Bracket i of x in component C (0: u, 1: eps) of an interleaved ascending
// row of n entries with C[0] <= x <= C[n-1], from hint h (locate_tbl
// semantics, jurassic.c:4152-4170), with both components at i and i + 1
// (reused from the probe loads on a hit).
struct Bracket2 {
  int i;
  float2 a, b;
};

template <int C>
__device__ __forceinline__ float comp(const float2 v) {
  return C == 0 ? v.x : v.y;
}

template <int C>
__device__ __forceinline__ int bisect2(const float2* g, int lo, int hi, float x) {
  const float* gc = reinterpret_cast<const float*>(g) + C;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(gc + 2 * mid) > x) hi = mid; else lo = mid;
  }
  return lo;
}

// The third probe g[h+2] is read even where h + 2 = n (the next row's first
// entry, or the one-entry pad after the last row) and then ignored.
template <int C>
__device__ __forceinline__ Bracket2 hunt2(const float2* g, int n, float x, int h) {
  h = min(max(h, 0), n - 2);
  const float2 A = __ldg(g + h), B = __ldg(g + h + 1), D = __ldg(g + h + 2);
  const float a = comp<C>(A), b = comp<C>(B), c = comp<C>(D);
  // bracket h or h + 1: every x >= a when the probes reach the row's end
  // (h >= n - 3; x at or above g[n-1] keeps n - 2, and h + 1 <= n - 2 is the
  // last bracket there), else x < g[h+2]
  const bool tail = h + 2 >= n - 1;
  if (a <= x && (x < c || tail)) {
    const bool up = x >= b && h + 2 < n;
    return up ? Bracket2{h + 1, B, D} : Bracket2{h, A, B};
  }
  const int i = a <= x ? bisect2<C>(g, h + 2, n - 1, x) : bisect2<C>(g, 0, h, x);
  return Bracket2{i, __ldg(g + i), __ldg(g + i + 1)};
}

// Emissivity of one table row (corner of the p-T cell) for the extended
// path: EGA u = intpol_tbl_u(e_path) + du, CGA u = ucg; then
// intpol_tbl_eps(u) (jurassic.c:3799-3891, 3895-3967).  In EGA the bracket
// that inverts e_path also brackets u_eq in the column row (the rows are
// monotone), and u_eq + du usually stays inside it: then the emissivity is
// interpolated from the entries already loaded, with no second search.
// The bracket is the same either way, so the value is too.  h is the
// search hint carried along the path: of the emissivity-row search in EGA,
// of the column-row search in CGA (EGA's column search starts from the
// emissivity bracket, or from the row start below the table).
template <bool CGA>
__device__ __forceinline__ float corner_eps(const TblDev& T, const RowF& r, float e_path, float du,
                                            float ucg, unsigned short& h) {
  const float2* row = T.ue + r.off;
  if (CGA) {  // intpol_tbl_eps(ucg), the row's last entries from the search
    const float uc = ucg;
    if (uc < r.u0) return r.e0 / r.u0 * uc;
    const Bracket2 k = hunt2<0>(row, r.n, uc, h);
    h = (unsigned short)k.i;
    if (uc > k.b.x) {
      const float a = log1pf(-k.b.y) / k.b.x;
      return -expm1f(a * uc);
    }
    return k.a.y + (k.b.y - k.a.y) / (k.b.x - k.a.x) * (uc - k.a.x);
  }
  float uq;
  int ib = -1;
  float u_lo = 0.f, u_hi = 0.f, e_lo = 0.f, e_hi = 0.f;
  if (CGA) {
    uq = ucg;
  } else {
    if (e_path < r.e0) {
      uq = r.u0 / r.e0 * e_path;
    } else if (e_path > r.en) {
      const float a = log1pf(-r.en) / r.un;
      uq = log1pf(-e_path) / a;
    } else {
      const Bracket2 k = hunt2<1>(row, r.n, e_path, h);
      h = (unsigned short)k.i;
      ib = k.i;
      e_lo = k.a.y;
      e_hi = k.b.y;
      u_lo = k.a.x;
      u_hi = k.b.x;
      uq = u_lo + (u_hi - u_lo) / (e_hi - e_lo) * (e_path - e_lo);
    }
    uq = uq + du;
  }
  if (uq < r.u0) return r.e0 / r.u0 * uq;
  if (uq > r.un) {
    const float a = log1pf(-r.en) / r.un;
    return -expm1f(a * uq);
  }
  if (!CGA && ib >= 0 && uq >= u_lo && uq < u_hi)
    return e_lo + (e_hi - e_lo) / (u_hi - u_lo) * (uq - u_lo);
  const Bracket2 k = hunt2<0>(row, r.n, uq, CGA ? (int)h : (ib >= 0 ? ib : 0));
  if (CGA) h = (unsigned short)k.i;
  return k.a.y + (k.b.y - k.a.y) / (k.b.x - k.a.x) * (uq - k.a.x);
}

__device__ __forceinline__ int bracket_regf(const float* g, int n, float x) {
  const float g0 = __ldg(g), g1 = __ldg(g + 1);
  const int i = (int)((x - g0) / (g1 - g0));
  return i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
}

__device__ __forceinline__ int bracket_irrf(const float* g, int n, float x) {
  int lo = 0, hi = n - 1, mid = (lo + hi) >> 1;
  const bool up = __ldg(g + mid) < __ldg(g + mid + 1);
  while (hi > lo + 1) {
    mid = (lo + hi) >> 1;
    const float v = __ldg(g + mid);
    const bool go_low = up ? (v > x) : (v <= x);
    if (go_low) hi = mid; else lo = mid;
  }
  return lo;
}

// One thread per (tile, point, lane) converts the FP64 LOS to float tiles.
__global__ void k_pack_tiles(CtlDev c, TblDev T, LosDev L, MixedPlan P, long long total) {
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total * 32) return;
  const int lane = (int)(gid & 31);
  const long long tp = gid >> 5;  // tile-point
  // locate the tile by binary search over tile offsets
  int lo = 0, hi = P.ntile;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (P.toff[mid] <= tp) lo = mid; else hi = mid;
  }
  const int tile = lo;
  const int ip = (int)(tp - P.toff[tile]);
  const int r = P.perm[tile * 32 + lane];
  const Fields F = fields_of(c, P.brmask);
  float* out = P.data + tp * (long long)F.n * 32 + lane;
  if (r < 0 || ip >= L.count[r]) {
    for (int f = 0; f < F.n; f++) out[f * 32] = 0.f;
    return;
  }
  const long long q = L.off[r] + ip;
  const LosDev::F32& Lf = L.f;
  out[F.p * 32] = Lf.p[q];
  out[F.t * 32] = Lf.t[q];
  out[F.ds * 32] = Lf.ds[q];
  out[F.qh2o * 32] = c.ig_h2o >= 0 ? Lf.qh2o[q] : 0.f;
  out[F.aux * 32] = Lf.aux[q];
  for (int w = 0; w < c.nw; w++) out[(F.kw0 + w) * 32] = Lf.kw[w * L.cap + q];
  const bool cgaf = c.formod == 0;
  for (int g = 0; g < c.ng; g++) {
    float* og = out + (F.g0 + g * F.es) * 32;
    og[kFU * 32] = Lf.u[g * L.cap + q];
    if (cgaf) {
      og[kFCgp * 32] = Lf.cgp[g * L.cap + q];
      og[kFCgt * 32] = Lf.cgt[g * L.cap + q];
      og[kFCgu * 32] = Lf.cgu[g * L.cap + q];
    }
    for (int k = 0; k < 4; k++) og[(kFBr(cgaf) + k) * 32] = 0.f;
  }
  // p-T brackets and interpolation weights on the grids of channel 0
  // (identical for every channel)
  for (int g = 0; P.brmask && g < c.ng; g++) {
    unsigned wd = kNoBracket;  // no table (np < 30)
    float pw = 0.f, wa = 0.f, wb = 0.f;
    const int np = __ldg(T.np + g);
    if (((P.brmask >> g) & 1u) && np >= 30) {
      const float pq = c.formod == 0 ? Lf.cgp[g * L.cap + q] : Lf.p[q];
      const float tq = c.formod == 0 ? Lf.cgt[g * L.cap + q] : Lf.t[q];
      const int ipr = bracket_irrf(T.pf + (long long)g * T.tp, np, pq);
      const int nt0 = __ldg(T.nt + (long long)g * T.tp + ipr);
      const int nt1 = __ldg(T.nt + (long long)g * T.tp + ipr + 1);
      wd = kNoBracket | 2u;      // temperature rows missing at this pressure
      if (nt0 >= 2 && nt1 >= 2) {
        const float* t0g = T.tf + ((long long)g * T.tp + ipr) * T.tt;
        const int it0 = bracket_regf(t0g, nt0, tq);
        const int it1 = bracket_regf(t0g + T.tt, nt1, tq);
        wd = (unsigned)(ipr * T.tt + it0) | ((unsigned)((ipr + 1) * T.tt + it1) << 16);
        // temperature weights at both pressures (LIN in T of
        // intpol_tbl_ega / intpol_tbl_cga)
        wa = (tq - t0g[it0]) / (t0g[it0 + 1] - t0g[it0]);
        wb = (tq - t0g[T.tt + it1]) / (t0g[T.tt + it1 + 1] - t0g[T.tt + it1]);
        // pressure weight: linear in EGA, log-linear in CGA
        const float* pg = T.pf + (long long)g * T.tp;
        const float pa = pg[ipr], pb = pg[ipr + 1];
        if (c.formod == 0 && pq / pa > 0.f && pb / pa > 0.f)
          pw = __logf(pq / pa) / __logf(pb / pa);
        else
          pw = (pq - pa) / (pb - pa);
      }
    }
    float* og = out + (F.g0 + g * F.es + kFBr(cgaf)) * 32;
    og[0] = __uint_as_float(wd);
    og[32] = pw;
    og[64] = wa;
    og[96] = wb;
  }
}

// Pressure bracket with a hint: keeps ipr while p lies inside its interval
// (or beyond the grid end it is clamped to), else bisects; with the grid
// values at ipr and ipr + 1.
__device__ __forceinline__ Bracket pbracket_f(const float* g, int n, float x, int ipr) {
  if (ipr >= 0) {
    const float a = __ldg(g + ipr), b = __ldg(g + ipr + 1);
    const float lo = fminf(a, b), hi = fmaxf(a, b);
    const bool low_end = (ipr == 0) && ((a < b) ? (x < a) : (x > a));
    const bool high_end = (ipr == n - 2) && ((a < b) ? (x >= b) : (x <= b));
    if ((x >= lo && x < hi) || low_end || high_end) return Bracket{ipr, a, b};
  }
  const int i = bracket_irrf(g, n, x);
  return Bracket{i, __ldg(g + i), __ldg(g + i + 1)};
}

constexpr int kStateWords = 5;  // t, e, ipr, 2 words of 16-bit corner hints
constexpr float kTauStop = 1e-12f;  // path transmittance below which the walk stops
constexpr int kChanConsts = 16;  // constants of a warp's channel
constexpr int kThreadFloats = 2;  // per-thread values kept in shared memory
constexpr int kPathThreads = 128;  // threads of a path block: 4 warps = 4 channels

// Per (channel, emitter) state carried along the path: transmittance t and
// emissivity e of the extended path (each accurate where it is small), the
// pressure bracket and the search hints of the four table corners (16 bit).
struct GasState {
  float t, e;
  int ipr;
  unsigned short h[4];
};

// One (channel, emitter) at one LOS point (intpol_tbl_ega / intpol_tbl_cga,
// jurassic.c:3710-3891).  Returns the segment emissivity; *sat is set where
// the reference's segment transmittance becomes zero.
// brw: packed bracket precomputed for the LOS point (grids shared by all
// channels), or kNoBracket | 1 to search here; wpre, wta, wtb: the pressure
// and temperature interpolation weights precomputed with it.
template <bool CGA>
__device__ __forceinline__ float gas_eps_f(const TblDev& T, long long dg, float pq,
                                           float tq, float du, float ucg, unsigned brw,
                                           float wpre, float wta, float wtb, GasState& s,
                                           bool& sat) {
  constexpr bool cga = CGA;
  const bool pre = brw != (kNoBracket | 1u);
  if (pre && brw == kNoBracket) return 0.f;   // np < 30
  const float* pg = T.pf + dg * T.tp;
  int np = 0;
  if (!pre) {
    np = __ldg(T.np + dg);
    if (np < 30) return 0.f;
  }
  if (s.t < 1e-9f) {
    s.t = 0.f;
    s.e = 1.f;
    sat = true;
    return 1.f;
  }
  unsigned ra, rc;
  float pa = 0.f, pb = 0.f;
  if (pre) {
    if (brw & kNoBracket) return 0.f;         // nt < 2 at this pressure
    const unsigned rb = (unsigned)dg * (unsigned)(T.tp * T.tt);
    ra = rb + (brw & 0xffffu);
    rc = rb + (brw >> 16);
  } else {
    const int* ntg = T.nt + dg * T.tp;
    const Bracket pb_ = pbracket_f(pg, np, pq, s.ipr);
    const int ipr = pb_.i;
    s.ipr = ipr;
    pa = pb_.a;
    pb = pb_.b;
    const int nt0 = __ldg(ntg + ipr), nt1 = __ldg(ntg + ipr + 1);
    if (nt0 < 2 || nt1 < 2) return 0.f;
    const int it0 = bracket_regf(T.tf + (dg * T.tp + ipr) * T.tt, nt0, tq);
    const int it1 = bracket_regf(T.tf + (dg * T.tp + ipr + 1) * T.tt, nt1, tq);
    const unsigned rp = (unsigned)dg * (unsigned)T.tp + (unsigned)ipr;
    ra = rp * (unsigned)T.tt + (unsigned)it0;
    rc = (rp + 1u) * (unsigned)T.tt + (unsigned)it1;
  }
  float ea, eb, w;
  if (pre) {
    const RowF r00 = rowf_at<CGA, true>(T, ra), r01 = rowf_at<CGA, true>(T, ra + 1u);
    const RowF r10 = rowf_at<CGA, true>(T, rc), r11 = rowf_at<CGA, true>(T, rc + 1u);
    if (r00.n < 2 || r01.n < 2 || r10.n < 2 || r11.n < 2) return 0.f;
    const float e00 = corner_eps<CGA>(T, r00, s.e, du, ucg, s.h[0]);
    const float e01 = corner_eps<CGA>(T, r01, s.e, du, ucg, s.h[1]);
    const float e10 = corner_eps<CGA>(T, r10, s.e, du, ucg, s.h[2]);
    const float e11 = corner_eps<CGA>(T, r11, s.e, du, ucg, s.h[3]);
    ea = e00 + (e01 - e00) * wta;
    eb = e10 + (e11 - e10) * wtb;
    w = wpre;
  } else {
    const RowF r00 = rowf_at<CGA>(T, ra), r01 = rowf_at<CGA>(T, ra + 1u);
    const RowF r10 = rowf_at<CGA>(T, rc), r11 = rowf_at<CGA>(T, rc + 1u);
    if (r00.n < 2 || r01.n < 2 || r10.n < 2 || r11.n < 2) return 0.f;
    const float e00 = corner_eps<CGA>(T, r00, s.e, du, ucg, s.h[0]);
    const float e01 = corner_eps<CGA>(T, r01, s.e, du, ucg, s.h[1]);
    const float e10 = corner_eps<CGA>(T, r10, s.e, du, ucg, s.h[2]);
    const float e11 = corner_eps<CGA>(T, r11, s.e, du, ucg, s.h[3]);
    const float ta = r00.t, tb = r01.t, tc = r10.t, td = r11.t;
    ea = e00 + (e01 - e00) / (tb - ta) * (tq - ta);
    eb = e10 + (e11 - e10) / (td - tc) * (tq - tc);
    if (cga && pq / pa > 0.f && pb / pa > 0.f)
      w = __logf(pq / pa) / __logf(pb / pa);
    else
      w = (pq - pa) / (pb - pa);
  }
  float e = ea + (eb - ea) * w;
  e = fminf(fmaxf(e, 0.f), 1.f);
  const float te = 1.f - e;  // exact for e >= 0.5
  const float eps = (s.e < 0.5f) ? (e - s.e) / s.t : 1.f - te / s.t;
  if (e >= 1.f) sat = true;
  s.t = te;
  s.e = e;
  return eps;
}

// The emitter loop runs over a runtime count with the per-emitter state in
// shared memory: unrolling it over the emitters multiplies the code size
// beyond the instruction cache and the register count beyond what keeps
// enough warps resident to hide load latency, and thread-local arrays spill
// through L1 into L2.
// MINB is the minimum number of resident blocks per SM requested from the
// register allocator (1 = no cap); the variants are chosen by the autotuner.
// SPLIT: the emitters' segment emissivities come from k_path_gas (P.seg_eps,
// P.seg_sat) instead of being computed here; everything else is this same
// code, so both forms give the same results.
// RESUME: rays start at P.start[r] from a saved state and save states for
// other rays (finite-difference perturbations that leave a path prefix
// unchanged); the arithmetic of every point is the same.
template <int MINB, bool CGA, bool SPLIT = false, bool RESUME = false, bool SHARE = false,
          int NT = kPathThreads>
__global__ void __launch_bounds__(NT, MINB) k_path_mixed(CtlDev c, TblDev T, ChanDev ch,
                                                          BatchDev b, LosDev L, MixedPlan P,
                                                          float* refl) {
  const int ng = c.ng;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  constexpr int W = NT / 32;  // warps of a block
  int tile, id;
  if (P.tile_major) {  // one channel of W consecutive tiles
    tile = P.tile0 + (int)(blockIdx.x / c.nd) * W + warp;
    id = (int)(blockIdx.x % c.nd);
  } else {             // W channels of one tile
    const int nchb = (c.nd + W - 1) / W;
    tile = P.tile0 + blockIdx.x / nchb;
    id = (blockIdx.x % nchb) * W + warp;
  }
  if (tile >= P.tile1 || id >= c.nd) return;
  int r = P.perm[tile * 32 + lane];
  if (r >= 0 && b.obs_skip && b.obs_skip[b.ray_obs[r]]) r = -1;  // lane idle, outputs untouched
  const bool skip = r >= 0 && b.skip_masked && b.mask[(long long)id * b.nray + r];
  const int n = r >= 0 && !skip ? L.count[r] : 0;
  const Fields F = fields_of(c, P.brmask);
  const float* base = P.data + P.toff[tile] * (long long)F.n * 32 + lane;
  constexpr bool cga = CGA;
  const double nud = ch.nu[id];
  const float nu = (float)nud;

  // per-(observation, channel) constants
  float cloud = 0.f, sfeps = 1.f;
  bool has_cloud = false;
  if (r >= 0) {
    const double* s = b.scal + (long long)b.ray_obs[r] * b.nscal;
    has_cloud = c.ncl > 0 && s[1] > 0;
    if (has_cloud) {
      const int icl = bracket_irr(ch.clnu, c.ncl, nud);
      cloud = (float)lin(ch.clnu[icl], s[2 + icl], ch.clnu[icl + 1], s[2 + icl + 1], nud);
    }
    if (c.nsf > 0) {
      const double* se = s + 5 + c.ncl;
      const int isf = bracket_irr(ch.sfnu, c.nsf, nud);
      sfeps = (float)lin(ch.sfnu[isf], se[isf], ch.sfnu[isf + 1], se[isf + 1], nud);
    }
  }
  const int w = c.nw > 0 ? ch.window[id] : 0;
  const double* cc = ch.ctm + (long long)id * kCtmStride;
  const bool co2_on = c.ctm_co2 && c.ig_co2 >= 0 && cc[0] != 0;
  const bool h2o_on = c.ctm_h2o && c.ig_h2o >= 0 && cc[4] != 0;
  const bool n2_on = c.ctm_n2 && cc[8] != 0;
  const bool o2_on = c.ctm_o2 && cc[11] != 0;
  const float st0 = (float)kTMIN, sdt = (float)((kTMAX - kTMIN) / (kNS - 1.0));

  // per-emitter path state in shared memory, word-major per thread:
  // sh[(g * kStateWords + w) * NT + threadIdx.x]
  extern __shared__ unsigned sh_state[];
  constexpr int nth = NT;
  const int tid = threadIdx.x;
  // behind the state: the channel's constants (kChanConsts words per warp:
  // continuum coefficients, [11] channel index, [12] window index) and
  // kThreadFloats per thread (cloud extinction, surface emissivity), read
  // where used so that they hold no registers across the emitter loop
  float* const sh_tail = reinterpret_cast<float*>(sh_state + kStateWords * nth * (ng > 0 ? ng : 1));
  volatile float* kc = sh_tail + warp * kChanConsts;
  volatile int* kci = reinterpret_cast<volatile int*>(sh_tail + warp * kChanConsts);
  volatile float* kthr = sh_tail + (nth / 32) * kChanConsts + tid;  // [0], [nth]
  if (lane == 0) {
    kc[0] = nu;
    kc[1] = (float)cc[1];
    kc[2] = (float)cc[2];
    kc[3] = (float)cc[3];
    kc[4] = (float)cc[5];
    kc[5] = (float)log(cc[6] > 0 ? cc[6] : 1.0);
    kc[6] = (float)cc[7];
    kc[7] = (float)cc[9];
    kc[8] = (float)cc[10];
    kc[9] = (float)cc[12];
    kc[10] = (float)cc[13];
    kci[11] = id;
    kci[12] = w;
  }
  kthr[0] = cloud;
  kthr[nth] = sfeps;
  __syncwarp();
  // the pressure-bracket word is only used where the bracket is searched
  // here (pre = false); with a precomputed bracket it keeps its initial -1
  auto sload = [&](int g, bool pre = false) {
    const unsigned* q = sh_state + (g * kStateWords) * nth + tid;
    GasState st;
    st.t = __uint_as_float(q[0]);
    st.e = __uint_as_float(q[nth]);
    st.ipr = pre ? -1 : (int)q[2 * nth];
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const unsigned hw = q[(3 + k) * nth];
      st.h[2 * k] = (unsigned short)(hw & 0xffffu);
      st.h[2 * k + 1] = (unsigned short)(hw >> 16);
    }
    return st;
  };
  auto sstore = [&](int g, const GasState& st, bool pre = false) {
    unsigned* q = sh_state + (g * kStateWords) * nth + tid;
    q[0] = __float_as_uint(st.t);
    q[nth] = __float_as_uint(st.e);
    if (!pre) q[2 * nth] = (unsigned)st.ipr;
#pragma unroll
    for (int k = 0; k < 2; k++)
      q[(3 + k) * nth] = (unsigned)st.h[2 * k] | ((unsigned)st.h[2 * k + 1] << 16);
  };
  for (int g = 0; g < ng && !SPLIT; g++) {
    GasState st;
    st.t = 1.f;
    st.e = 0.f;
    st.ipr = -1;
#pragma unroll
    for (int k = 0; k < 4; k++) st.h[k] = 0;
    sstore(g, st);
  }
  // split form: segment emissivities of (point, this channel, emitter g) at
  // seg0 + ip * segstride + g * 32
  const long long segstride = (long long)c.nd * ng * 32;
  const long long seg0 = SPLIT ? ((P.toff[tile] * c.nd + id) * ng) * 32 + lane : 0;
  const long long dg0 = (long long)id * ng;
  float rad = 0.f, comp = 0.f, tau = 1.f;
  const bool do_refl = refl != nullptr && r >= 0 && c.sftype >= 2 && sfeps < 1.f && L.sft[r] > 0;

  // resume: the state words of every emitter and rad, comp, tau
  const int sw = kStateWords * ng;
  auto snap_write = [&](int target) {
    float* q = P.snap + ((long long)target * c.nd + id) * (sw + 3);
    for (int k = 0; k < sw; k++) q[k] = __uint_as_float(sh_state[k * nth + tid]);
    q[sw] = rad;
    q[sw + 1] = comp;
    q[sw + 2] = tau;
  };
  int start = 0, sn = 0, se = 0;
  if (RESUME && n > 0) {
    start = P.start[r];
    if (start > 0) {
      const float* q = P.snap + ((long long)r * c.nd + id) * (sw + 3);
      for (int k = 0; k < sw; k++) sh_state[k * nth + tid] = __float_as_uint(q[k]);
      rad = q[sw];
      comp = q[sw + 1];
      tau = q[sw + 2];
    }
    sn = P.snap_off[r];
    se = P.snap_off[r + 1];
  }

  // emitters shared with the base ray (see MixedPlan): rb >= 0 takes every
  // emitter but pg from the base while ip < nvalid; a base lane writes them
  const bool seg_write = SHARE && P.reuse == nullptr && r >= 0 && n > 0;
  int rb = -1, pg = -1, nvalid = 0;
  if (SHARE && P.reuse != nullptr && r >= 0 && n > 0) {
    const int2 ru = P.reuse[r];
    rb = ru.x;
    pg = ru.y;
    if (rb >= 0) nvalid = P.seg_nvalid[(long long)rb * c.nd + id];
  }
  int walked = n;  // points this lane walked (a base lane records it)
  // LOS offset of the base ray whose entries this lane writes or reads
  const long long soff = !SHARE ? 0 : rb >= 0 ? L.off[rb] : seg_write ? L.off[r] : 0;

  // resumed lanes join the warp's walk at their own start point: every
  // iteration reads one point of the tile for all lanes (coalesced)
  int ip0 = start;
  if (RESUME) {
    const unsigned wmin = __reduce_min_sync(0xffffffffu, n > 0 ? (unsigned)start : 0xffffffffu);
    ip0 = wmin == 0xffffffffu ? 0 : (int)wmin;
  }
  for (int ip = ip0; ip < n; ip++) {
    if (RESUME && ip < start) continue;
    // opaque from here on: the rest of the path adds at most max(src) tau,
    // below 1e-10 of the radiance (not with surface reflection, whose sum
    // needs every point)
    if (tau < kTauStop && !do_refl) {
      walked = ip;
      break;
    }
    if (RESUME)
      for (; sn < se && P.snap_ip[sn] == ip; sn++) snap_write(P.snap_ray[sn]);
    // the base stopped here: the shared emitters continue from its final states
    if (SHARE && rb >= 0 && ip == nvalid) {
      const unsigned* q = P.seg_final + ((long long)rb * c.nd + id) * sw;
      for (int g2 = 0; g2 < ng; g2++)
        if (g2 != pg)
          for (int k = 0; k < kStateWords; k++)
            sh_state[(g2 * kStateWords + k) * nth + tid] = q[g2 * kStateWords + k];
    }
    const bool shared = SHARE && rb >= 0 && ip < nvalid;
    const long long sbase = SHARE ? (soff + ip) * c.nd + id : 0;
    const unsigned satm_in = shared ? P.seg_satm[sbase] : 0u;
    unsigned satm_out = 0u;
    const float* f = base + (long long)ip * F.n * 32;
    const float p = f[F.p * 32], t = f[F.t * 32], ds = f[F.ds * 32];
    float E = 0.f;
    bool sat = false;
#pragma unroll 1
    for (int g = 0; g < ng; g++) {
      float eg;
      if (SPLIT) {
        const long long o = seg0 + ip * segstride + g * 32;
        eg = P.seg_eps[o];
        if (P.seg_sat[o]) sat = true;
      } else if (SHARE && shared && g != pg) {
        eg = P.seg_base[sbase * ng + g];
        if ((satm_in >> g) & 1u) sat = true;
      } else {
        constexpr int es = kEmitterFields(CGA), kb = kFBr(CGA);
        const float* fg = f + (F.g0 + g * es) * 32;
        const float du = cga ? 0.f : fg[kFU * 32];
        const float pq = cga ? fg[kFCgp * 32] : p;
        const float tq = cga ? fg[kFCgt * 32] : t;
        const float ucg = cga ? fg[kFCgu * 32] : 0.f;
        const bool brg = (P.brmask >> g) & 1u;
        const unsigned brw = brg ? __float_as_uint(fg[kb * 32]) : (kNoBracket | 1u);
        const float wpre = brg ? fg[(kb + 1) * 32] : 0.f;
        const float wta = brg ? fg[(kb + 2) * 32] : 0.f;
        const float wtb = brg ? fg[(kb + 3) * 32] : 0.f;
        GasState st = sload(g, brg);
        const long long dg = dg0 + g;  // (channel, emitter)
        bool sg = false;
        eg = gas_eps_f<CGA>(T, dg, pq, tq, du, ucg, brw, wpre, wta, wtb, st, sg);
        sstore(g, st, brg);
        if (sg) sat = true;
        if (SHARE && seg_write) {
          P.seg_base[sbase * ng + g] = eg;
          if (sg) satm_out |= 1u << g;
        }
      }
      E = E + (1.f - E) * eg;
    }
    if (SHARE && seg_write) P.seg_satm[sbase] = satm_out;
    // extinction and continua
    float beta = c.nw > 0 ? f[(F.kw0 + w) * 32] : 0.f;
    if (has_cloud) beta += f[F.aux * 32] * kthr[0];
    const float pr = p / (float)kP0;
    if (co2_on) {
      const float co2_296 = kc[1], co2_260 = kc[2], co2_230 = kc[3];
      const float d230 = t - 230.f, d260 = t - 260.f, d296 = t - 296.f;
      const float ctw = d260 * 5.050505e-4f * d296 * co2_230 - d230 * 9.259259e-4f * d296 * co2_260 +
                        d230 * 4.208754e-4f * d260 * co2_296;
      const float uco2 = f[(F.g0 + c.ig_co2 * F.es + kFU) * 32];
      beta += (uco2 / ds) * (float)(1.0 / (kNA * 1000.0)) * pr * ctw;
    }
    if (h2o_on) {
      const float q = f[F.qh2o * 32];
      const float uh = f[(F.g0 + c.ig_h2o * F.es + kFU) * 32];
      const float nu = kc[0], h2o_s296 = kc[4], h2o_lr = kc[5], h2o_frn = kc[6];
      const float self = h2o_s296 * __expf(h2o_lr * (296.f - t) * (1.f / 36.f));
      const float a1 = nu * ((uh / ds) * 1e-20f) * tanhf(.7193876f / t * nu);
      beta += a1 * (296.f / t) * pr * (q * self + (1.f - q) * h2o_frn);
    }
    if (n2_on || o2_on) {
      const float n2_b = kc[7], n2_beta = kc[8], o2_b = kc[9], o2_beta = kc[10];
      const float x = pr * 273.f / t;
      const float x2 = 0.1f * x * x;
      if (n2_on)
        beta += x2 * __expf(n2_beta * (1.f / 296.f - 1.f / t)) * 0.79f * n2_b *
                (0.79f + 0.21f * (1.294f - 0.4545f * t / 296.f));
      if (o2_on) beta += x2 * __expf(o2_beta * (1.f / 296.f - 1.f / t)) * 0.21f * o2_b;
    }
    // source function (formod_srcfunc); the channel index is re-read from
    // shared memory so that the table pointer holds no registers in the loop
    const float* srf = T.srf + (long long)kci[11] * kNS;
    const float xs = (t - st0) / sdt;
    int is = (int)xs;
    is = is < 0 ? 0 : (is > kNS - 2 ? kNS - 2 : is);
    const float s0 = __ldg(srf + is), s1 = __ldg(srf + is + 1);
    const float src = s0 + (s1 - s0) * (xs - (float)is);
    float eps = 0.f;
    if (!sat) {
      eps = E + (1.f - E) * (-expm1f(-beta * ds));
      // Kahan-compensated radiance sum
      const float y = src * eps * tau - comp;
      const float tsum = rad + y;
      comp = (tsum - rad) - y;
      rad = tsum;
      tau *= (1.f - eps);
    }
    if (do_refl) {
      float* sc = refl + 2 * (L.off[r] * c.nd);
      sc[2 * ((long long)ip * c.nd + id)] = src;
      sc[2 * ((long long)ip * c.nd + id) + 1] = eps;
    }
  }
  // states for resume points beyond the end of this walk (a path that became
  // opaque earlier hands its final state on, so the resumed rays stop too)
  if (RESUME)
    for (; sn < se; sn++) snap_write(P.snap_ray[sn]);
  if (SHARE && seg_write) {  // what a perturbed ray needs past this walk
    P.seg_nvalid[(long long)r * c.nd + id] = walked;
    unsigned* q = P.seg_final + ((long long)r * c.nd + id) * sw;
    for (int k = 0; k < sw; k++) q[k] = sh_state[k * nth + tid];
  }
  if (r < 0) return;

  const double nud2 = ch.nu[id];
  const float sfeps2 = kthr[nth];
  const float* srf = T.srf + (long long)id * kNS;
  double radd = (double)rad;
  const double sft = L.sft[r];
  if (c.sftype >= 1 && sft > 0) {
    const float xs = ((float)sft - st0) / sdt;
    int is = (int)xs;
    is = is < 0 ? 0 : (is > kNS - 2 ? kNS - 2 : is);
    const float s0 = srf[is], s1 = srf[is + 1];
    const float ssf = s0 + (s1 - s0) * (xs - (float)is);
    radd += (double)(sfeps2 * ssf * tau);
    if (do_refl) {
      const float* sc = refl + 2 * (L.off[r] * c.nd);
      float tr = 1.f;
      double acc = 0;
      for (int ip = n - 1; ip >= 0; ip--) {
        const float src = sc[2 * ((long long)ip * c.nd + id)];
        const float e = sc[2 * ((long long)ip * c.nd + id) + 1];
        acc += (double)(src * e * tr);
        tr *= (1.f - e);
      }
      radd += acc * (double)tau * (double)(1.f - sfeps2);
      if (c.sftype >= 3) {
        const double* e6 = L.ends + 6LL * r;
        // solar zenith angle (sza, jurassic.c:5183-5219) and incidence
        const double d = b.geo[r] / 86400 - 0.5;
        const double g = (357.529 + 0.98560028 * d) * (kPI / 180.0);
        const double qq = 280.459 + 0.98564736 * d;
        const double l = (qq + 1.915 * sin(g) + 0.020 * sin(2 * g)) * (kPI / 180.0);
        const double ee = (23.439 - 0.00000036 * d) * (kPI / 180.0);
        const double dec = asin(sin(ee) * sin(l));
        const double ra = atan2(cos(ee) * sin(l), cos(l));
        const double lst = 18.697374558 + 24.06570982441908 * d + e6[4] / 15;
        const double h = lst / 12 * kPI - ra;
        const double latr = e6[5] * (kPI / 180.0);
        const double sza2 = c.sfsza < 0 ? acos(sin(latr) * sin(dec) + cos(latr) * cos(dec) * cos(h)) *
                                              (180.0 / kPI)
                                        : c.sfsza;
        if (sza2 < 89.999) {
          double x0[3], x1[3];
          to_cart(e6[3], e6[4], e6[5], x0);
          to_cart(e6[0], e6[1], e6[2], x1);
          for (int i = 0; i < 3; i++) x1[i] -= x0[i];
          const double cosa = (x0[0] * x1[0] + x0[1] * x1[1] + x0[2] * x1[2]) /
                              sqrt(x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2]) /
                              sqrt(x1[0] * x1[0] + x1[1] * x1[1] + x1[2] * x1[2]);
          const double rcos = cosa / cos(sza2 * (kPI / 180.0));
          radd += 6.764e-5 / (2. * kPI) * planck(kTSUN, nud2) * tr * (1 - sfeps2) * tau * rcos;
        }
      }
    }
  }
  const long long oi = (long long)id * b.nray + r;
  if (c.fov) {  // pencil beam only: FOV convolution, BT and mask follow in k_fov
    b.rad[oi] = radd;
    b.tau[oi] = (double)tau;
    return;
  }
  if (c.write_bbt) radd = kC2 * nud2 / log1p(kC1 * (nud2 * nud2 * nud2) / radd);
  b.rad[oi] = b.mask[oi] ? __longlong_as_double(0x7ff8000000000000LL) : radd;
  b.tau[oi] = (double)tau;
}

// Emitter path states of the split form: one warp per (tile, channel,
// emitter) walks the tile's points with the state of that emitter only and
// writes every segment emissivity and saturation flag.  The emitters' states
// are independent along the path (intpol_tbl_ega / intpol_tbl_cga keep one
// tau_path per emitter); only their combination per point couples them, and
// that is left to k_path_mixed<..., SPLIT>.  A latency-bound batch (few
// tiles) so runs ng warps where the fused form runs one.
template <bool CGA>
__global__ void __launch_bounds__(128) k_path_gas(CtlDev c, TblDev T, BatchDev b, LosDev L,
                                                  MixedPlan P) {
  const int lane = threadIdx.x & 31;
  const int ng = c.ng;
  const long long per_tile = (long long)c.nd * ng;
  const long long wg = (long long)blockIdx.x * 4 + (threadIdx.x >> 5);
  const int tile = (int)(wg / per_tile);
  if (tile >= P.ntile) return;
  const int rem = (int)(wg - (long long)tile * per_tile);
  const int id = rem / ng, g = rem - id * ng;
  int r = P.perm[tile * 32 + lane];
  if (r >= 0 && b.obs_skip && b.obs_skip[b.ray_obs[r]]) r = -1;
  const bool skip = r >= 0 && b.skip_masked && b.mask[(long long)id * b.nray + r];
  const int n = r >= 0 && !skip ? L.count[r] : 0;
  const Fields F = fields_of(c, P.brmask);
  const float* base = P.data + P.toff[tile] * (long long)F.n * 32 + lane;
  constexpr bool cga = CGA;
  const long long dg = (long long)id * ng + g;
  const long long segstride = (long long)c.nd * ng * 32;
  const long long seg0 = ((P.toff[tile] * c.nd + id) * ng + g) * 32 + lane;
  GasState st;
  st.t = 1.f;
  st.e = 0.f;
  st.ipr = -1;
#pragma unroll
  for (int k = 0; k < 4; k++) st.h[k] = 0;
  const unsigned brbit = (P.brmask >> g) & 1u;
  for (int ip = 0; ip < n; ip++) {
    const float* f = base + (long long)ip * F.n * 32;
    constexpr int es = kEmitterFields(CGA), kb = kFBr(CGA);
    const float* fg = f + (F.g0 + g * es) * 32;
    const float du = cga ? 0.f : fg[kFU * 32];
    const float pq = cga ? fg[kFCgp * 32] : f[F.p * 32];
    const float tq = cga ? fg[kFCgt * 32] : f[F.t * 32];
    const float ucg = cga ? fg[kFCgu * 32] : 0.f;
    const unsigned brw = brbit ? __float_as_uint(fg[kb * 32]) : (kNoBracket | 1u);
    const float wpre = brbit ? fg[(kb + 1) * 32] : 0.f;
    const float wta = brbit ? fg[(kb + 2) * 32] : 0.f;
    const float wtb = brbit ? fg[(kb + 3) * 32] : 0.f;
    bool sat = false;
    const float eg = gas_eps_f<CGA>(T, dg, pq, tq, du, ucg, brw, wpre, wta, wtb, st, sat);
    const long long o = seg0 + ip * segstride;
    P.seg_eps[o] = eg;
    P.seg_sat[o] = sat ? 1 : 0;
  }
}

// Row records of the mixed path (layouts at rowf_at); rows with fewer than
// two entries are never interpolated and get zeros.
__global__ void k_rowmeta(long long nrow, int tu, const int* nu, const float* u, const float* e,
                          const float* tf, int cga, float4* meta) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrow) return;
  const int n = nu[r];
  const float* ur = u + r * tu;
  const float* er = e + r * tu;
  if (cga) {
    meta[r] = make_float4(__int_as_float(n), tf[r], n >= 2 ? ur[0] : 0.f, n >= 2 ? er[0] : 0.f);
    return;
  }
  float4 m = make_float4(0.f, 0.f, 0.f, 0.f);
  if (n >= 2) m = make_float4(ur[0], ur[n - 1], er[0], er[n - 1]);
  meta[2 * r] = m;
  meta[2 * r + 1] = make_float4(__int_as_float(n), tf[r], 0.f, 0.f);
}

// The rows interleaved {u[i], eps[i]}: a probe of one brings the other.
__global__ void k_interleave(long long n, const float* u, const float* e, float2* ue) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) ue[i] = make_float2(u[i], e[i]);
}

void launch_rowmeta(long long nrow, int tu, const int* nu, const float* u, const float* e,
                    const float* tf, int cga, float4* meta, float2* ue, cudaStream_t s) {
  const int bs = 256;
  if (nrow > 0) {
    k_rowmeta<<<(unsigned)((nrow + bs - 1) / bs), bs, 0, s>>>(nrow, tu, nu, u, e, tf, cga, meta);
    const long long n = nrow * tu;
    k_interleave<<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(n, u, e, ue);
  }
}

__global__ void k_src_to_float(int nd, const double* sr, float* srf) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= nd * kNS) return;
  const int id = gid / kNS, it = gid % kNS;
  srf[gid] = (float)sr[(long long)it * nd + id];
}

__global__ void k_to_float(long long n, const double* src, float* dst) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

void launch_pack_tiles_n(const CtlDev& c, const TblDev& T, const LosDev& L, const MixedPlan& P,
                         long long total_tile_points, cudaStream_t s) {
  const long long nth = total_tile_points * 32;
  const int bs = 256;
  k_pack_tiles<<<(unsigned)((nth + bs - 1) / bs), bs, 0, s>>>(c, T, L, P, total_tile_points);
}

// register caps of the autotuner's variants (minimum resident blocks per SM),
// each with both 128-thread block shapes, and the tile-major shape with
// 256-thread blocks (one channel of 8 consecutive tiles) at two caps
int path_mixed_caps() { return 7; }
int path_mixed_variants() { return 2 * path_mixed_caps() + 2; }

size_t path_smem(const CtlDev& c, int nt) {
  return sizeof(unsigned) * kStateWords * nt * (size_t)(c.ng > 0 ? c.ng : 1) +
         sizeof(float) * ((nt / 32) * kChanConsts + kThreadFloats * nt);
}

template <typename K>
void launch_k(K kern, unsigned nblk, int nt, size_t smem, cudaStream_t s, const CtlDev& c,
              const TblDev& T, const ChanDev& ch, const BatchDev& b, const LosDev& L,
              const MixedPlan& P, float* refl) {
  if (smem > 48 * 1024)  // many emitters: opt in to the larger shared memory
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kern<<<nblk, nt, smem, s>>>(c, T, ch, b, L, P, refl);
}

template <bool CGA>
void launch_variant(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                    const LosDev& L, const MixedPlan& P, float* refl, int variant,
                    cudaStream_t s) {
  MixedPlan Pv = P;
  if (variant >= 2 * path_mixed_caps()) {  // 256 threads, one channel of 8 tiles
    Pv.tile_major = 1;
    const unsigned nblk = (unsigned)((long long)((P.ntile + 7) / 8) * c.nd);
    const size_t smem = path_smem(c, 256);
    if (variant == 2 * path_mixed_caps())
      launch_k(k_path_mixed<4, CGA, false, false, false, 256>, nblk, 256, smem, s, c, T, ch, b, L, Pv, refl);
    else
      launch_k(k_path_mixed<5, CGA, false, false, false, 256>, nblk, 256, smem, s, c, T, ch, b, L, Pv, refl);
    return;
  }
  Pv.tile_major = variant >= path_mixed_caps() ? 1 : 0;
  const int nchb = (c.nd + 3) / 4;
  const unsigned nblk = Pv.tile_major ? (unsigned)((long long)((P.ntile + 3) / 4) * c.nd)
                                      : (unsigned)((long long)P.ntile * nchb);
  // state, then kChanConsts per warp and kThreadFloats per thread
  const size_t smem = path_smem(c, kPathThreads);
  switch (variant % path_mixed_caps()) {
    case 1: launch_k(k_path_mixed<5, CGA>, nblk, kPathThreads, smem, s, c, T, ch, b, L, Pv, refl); break;
    case 2: launch_k(k_path_mixed<6, CGA>, nblk, kPathThreads, smem, s, c, T, ch, b, L, Pv, refl); break;
    case 3: launch_k(k_path_mixed<4, CGA>, nblk, kPathThreads, smem, s, c, T, ch, b, L, Pv, refl); break;
    case 4: launch_k(k_path_mixed<8, CGA>, nblk, kPathThreads, smem, s, c, T, ch, b, L, Pv, refl); break;
    case 5: launch_k(k_path_mixed<10, CGA>, nblk, kPathThreads, smem, s, c, T, ch, b, L, Pv, refl); break;
    case 6: launch_k(k_path_mixed<12, CGA>, nblk, kPathThreads, smem, s, c, T, ch, b, L, Pv, refl); break;
    default: launch_k(k_path_mixed<1, CGA>, nblk, kPathThreads, smem, s, c, T, ch, b, L, Pv, refl); break;
  }
}

void launch_path_mixed(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                       const LosDev& L, const MixedPlan& P, float* refl_scratch, int variant,
                       cudaStream_t s) {
  if (c.formod == 0)
    launch_variant<true>(c, T, ch, b, L, P, refl_scratch, variant, s);
  else
    launch_variant<false>(c, T, ch, b, L, P, refl_scratch, variant, s);
}

template <bool CGA>
void launch_split(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                  const LosDev& L, const MixedPlan& P, float* refl, size_t smem, cudaStream_t s) {
  const long long warps = (long long)P.ntile * c.nd * c.ng;
  k_path_gas<CGA><<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(c, T, b, L, P);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_path_mixed<1, CGA, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
  const unsigned nblk = (unsigned)((long long)P.ntile * ((c.nd + 3) / 4));
  k_path_mixed<1, CGA, true><<<nblk, kPathThreads, smem, s>>>(c, T, ch, b, L, P, refl);
}

void launch_path_split(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                       const LosDev& L, const MixedPlan& P, float* refl_scratch, cudaStream_t s) {
  const size_t smem = sizeof(unsigned) * kStateWords * kPathThreads * (size_t)(c.ng > 0 ? c.ng : 1) +
                      sizeof(float) * (4 * kChanConsts + kThreadFloats * kPathThreads);
  if (c.formod == 0)
    launch_split<true>(c, T, ch, b, L, P, refl_scratch, smem, s);
  else
    launch_split<false>(c, T, ch, b, L, P, refl_scratch, smem, s);
}

int path_state_words(const CtlDev& c) { return kStateWords * c.ng + 3; }

void launch_path_resume(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                        const LosDev& L, const MixedPlan& P0, cudaStream_t s) {
  // block = one channel of 4 consecutive tiles (the perturbations of one
  // observation share table rows)
  MixedPlan P = P0;
  P.tile_major = 1;
  const unsigned nblk = (unsigned)((long long)((P.tile1 - P.tile0 + 3) / 4) * c.nd);
  if (nblk == 0) return;
  const size_t smem = sizeof(unsigned) * kStateWords * kPathThreads * (size_t)(c.ng > 0 ? c.ng : 1) +
                      sizeof(float) * (4 * kChanConsts + kThreadFloats * kPathThreads);
  auto go = [&](auto kern) {
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<nblk, kPathThreads, smem, s>>>(c, T, ch, b, L, P, nullptr);
  };
  const bool share = P.seg_base != nullptr;
  if (c.formod == 0) {
    if (share) go(k_path_mixed<8, true, false, true, true>);
    else go(k_path_mixed<8, true, false, true, false>);
  } else {
    if (share) go(k_path_mixed<8, false, false, true, true>);
    else go(k_path_mixed<8, false, false, true, false>);
  }
}

void launch_src_to_float(int nd, const double* sr, float* srf, cudaStream_t s) {
  const int n = nd * kNS, bs = 256;
  k_src_to_float<<<(n + bs - 1) / bs, bs, 0, s>>>(nd, sr, srf);
}

void launch_tables_to_float(long long n, const double* src, float* dst, cudaStream_t s) {
  const int bs = 256;
  if (n > 0) k_to_float<<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(n, src, dst);
}

}  // namespace jgb
