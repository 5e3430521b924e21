// Host side of libjurassic_gb300: context, table and source-function
// upload, the batched forward-model driver and the C ABI.
//
// A context replaces the reference's process-global state (the static
// tables of formod_pencil, jurassic.c:3202-3217, and the emitter indices
// cached in formod_continua, 3081) with explicit, device-resident data:
// one context serves one control set, any number of contexts coexist.
#include <cub/cub.cuh>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/jurassic_gb300.h"
#include "jgb_common.cuh"
#include "jgb_internal.h"
#include "jgb_ctx.h"

extern "C" const double jgb_continua_blob[];
extern "C" const long jgb_continua_count;

using namespace jgb;

namespace {

// Offsets of the continuum tables inside the blob (order of continua.bin).
enum { CT_CO2_296 = 0, CT_CO2_260 = 2001, CT_CO2_230 = 4002, CT_H2O_296 = 6003,
       CT_H2O_260 = 8004, CT_H2O_FRN = 10005, CT_XFCREV = 12006, CT_N2_B = 12021,
       CT_N2_BETA = 12119, CT_N2_NU = 12217, CT_O2_B = 12315, CT_O2_BETA = 12405,
       CT_O2_NU = 12495, CT_TOTAL = 12585 };

// Wavenumber-only factors of ctmco2/ctmh2o/ctmn2/ctmo2
// (jurassic.c:1718-1741, 2762-2790, 2846-2857, 2906-2916), evaluated once
// per channel with the reference's operation order.
void ctm_coefficients(double nu, double* out) {
  const double* B = jgb_continua_blob;
  for (int i = 0; i < kCtmStride; i++) out[i] = 0;
  {
    const double xw = nu / 2 + 1;
    if (xw >= 1 && xw < 2001) {
      const int iw = (int)xw;
      const double dw = xw - iw, ew = 1 - dw;
      out[0] = 1;
      out[1] = ew * B[CT_CO2_296 + iw - 1] + dw * B[CT_CO2_296 + iw];
      out[2] = ew * B[CT_CO2_260 + iw - 1] + dw * B[CT_CO2_260 + iw];
      out[3] = ew * B[CT_CO2_230 + iw - 1] + dw * B[CT_CO2_230 + iw];
    }
  }
  {
    const double xw = nu / 10 + 1;
    if (xw >= 1 && xw < 2001) {
      const int iw = (int)xw;
      const double dw = xw - iw, ew = 1 - dw;
      const double c296 = ew * B[CT_H2O_296 + iw - 1] + dw * B[CT_H2O_296 + iw];
      const double c260 = ew * B[CT_H2O_260 + iw - 1] + dw * B[CT_H2O_260 + iw];
      const double cfrn = ew * B[CT_H2O_FRN + iw - 1] + dw * B[CT_H2O_FRN + iw];
      double sfac = 1;
      if (!(nu <= 820 || nu >= 960)) {
        const double xx = (nu - 820) / 10;
        const int ix = (int)xx;
        const double dx = xx - ix;
        sfac = (1 - dx) * B[CT_XFCREV + ix] + dx * B[CT_XFCREV + ix + 1];
      }
      const double vf2 = (nu - 370) * (nu - 370), vf6 = vf2 * vf2 * vf2;
      const double fscal = 36100 / (vf2 + vf6 * 1e-8 + 36100) * -.25 + 1;
      out[4] = 1;
      out[5] = sfac * c296;
      out[6] = c260 / c296;
      out[7] = cfrn * fscal;
    }
  }
  auto cia = [&](int ob, int obeta, int onu, int n, double* o) {
    const double* nua = B + onu;
    if (nu < nua[0] || nu > nua[n - 1]) return;
    int i = (int)((nu - nua[0]) / (nua[1] - nua[0]));
    i = i < 0 ? 0 : (i > n - 2 ? n - 2 : i);
    o[0] = 1;
    o[1] = lin(nua[i], B[ob + i], nua[i + 1], B[ob + i + 1], nu);
    o[2] = lin(nua[i], B[obeta + i], nua[i + 1], B[obeta + i + 1], nu);
  };
  cia(CT_N2_B, CT_N2_BETA, CT_N2_NU, 98, out + 8);
  cia(CT_O2_B, CT_O2_BETA, CT_O2_NU, 90, out + 11);
}

}  // namespace


namespace {

int fail(jgb_ctx* x, int code, const std::string& msg) {
  if (x) x->err = msg;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(x, JGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

bool iequal(const std::string& a, const char* b) {
  if (a.size() != strlen(b)) return false;
  for (size_t i = 0; i < a.size(); i++)
    if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
  return true;
}

TblDev tbl_view(const jgb_ctx* x) {
  TblDev T;
  T.tp = x->tp;
  T.tt = x->tt;
  T.tu = x->tu;
  T.np = x->t_np.as<int>();
  T.p = x->t_p.as<double>();
  T.nt = x->t_nt.as<int>();
  T.t = x->t_t.as<double>();
  T.nu = x->t_nu.as<int>();
  T.u = x->t_u.as<float>();
  T.eps = x->t_eps.as<float>();
  T.pf = x->t_pf.as<float>();
  T.tf = x->t_tf.as<float>();
  T.rowmeta = x->t_meta.as<float4>();
  T.ue = x->t_ue.as<float2>();
  T.sr = x->s_sr.as<double>();
  T.srf = x->s_srf.as<float>();
  T.st = x->s_st.as<double>();
  return T;
}

ChanDev chan_view(const jgb_ctx* x) {
  ChanDev ch;
  ch.nu = x->d_nu.as<double>();
  ch.window = x->d_window.as<int>();
  ch.clnu = x->d_clnu.as<double>();
  ch.sfnu = x->d_sfnu.as<double>();
  ch.ctm = x->d_ctm.as<double>();
  return ch;
}

__global__ void k_mask(long long n, const double* rad, unsigned char* mask) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) mask[i] = !isfinite(rad[i]);
}

__global__ void k_ray_obs(int nobs, const int* ray_off, int* ray_obs) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nobs) return;
  for (int r = ray_off[o]; r < ray_off[o + 1]; r++) ray_obs[r] = o;
}

__global__ void k_widen(int n, const int* a, long long* b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

// Batches of mixed precision with at most this many rays x NLOS points are
// traced in one pass into fixed per-ray slabs (small batches, e.g. the
// retrieval's damped trials, are latency-bound and the counting pass would
// double the ray-tracing time); larger ones count first.
constexpr long long kSinglePassPoints = 1LL << 23;

// Fixed slabs of LOS points per ray (single-pass tracing): ray r owns
// points [r*slab, (r+1)*slab) and may fill up to slab of them.
__global__ void k_slab_offsets(int nray, long long slab, long long* off, int* count) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > nray) return;
  off[r] = (long long)r * slab;
  if (r < nray) count[r] = (int)slab;
}

__global__ void k_iota(int n, int* v, int from = 0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = from + i;
}

// tile plan from the rays in sort order (descending key): the first nfirst
// rays fill tiles [0, tfirst), the next nsecond - nfirst tiles [tfirst,
// tsecond), the others start a new tile again (three groups that never share
// a tile; nsecond = nfirst, tsecond = tfirst: two; nfirst = nray, tfirst =
// ntile: one)
__global__ void k_tiles(int nray, int ntile, int nfirst, int tfirst, int nsecond, int tsecond,
                        const int* count, const int* sorted_ray, int* perm, int* tlen,
                        long long* tpts) {
  const int tile = blockIdx.x * blockDim.x + threadIdx.x;
  if (tile >= ntile) return;
  int k0, k1;
  if (tile < tfirst) {
    k0 = tile * 32;
    k1 = min(k0 + 32, nfirst);
  } else if (tile < tsecond) {
    k0 = nfirst + (tile - tfirst) * 32;
    k1 = min(k0 + 32, nsecond);
  } else {
    k0 = nsecond + (tile - tsecond) * 32;
    k1 = min(k0 + 32, nray);
  }
  int mx = 0;
  for (int l = 0; l < 32; l++) {
    const int k = k0 + l;
    perm[tile * 32 + l] = k < k1 ? sorted_ray[k] : -1;
    if (k < k1) mx = max(mx, count[sorted_ray[k]]);
  }
  tlen[tile] = mx;
  tpts[tile] = mx;
}

// Resume point of every ray of a batch of perturbations (ResumeSpec).  A
// perturbed level value changes the atmosphere only on the two intervals
// next to it, [z_lo, z_hi].  The position of LOS point p + 1 depends on the
// refraction evaluated between points p and p + 1 (the step's midpoint and
// sub-points 20 m away), whose altitudes lie within the segment's end
// altitudes less its curvature sag (metres) and the 20 m offsets; the data
// of point p on its own altitude.  So while segments stay margin away from
// [z_lo, z_hi], the perturbed ray's points and their data equal the base
// ray's, and the path state before the first segment that comes closer is
// the base's (one point earlier is taken as a safety margin).  Bases, and
// perturbations of other than level values, start at 0.
// First segment [zb[p], zb[p + 1]] of n LOS points (the last point alone)
// that comes within [z_lo, z_hi] of perturbation pr of observation e, each
// side widened by margin; n if none does.
__device__ int first_near(const BatchDev& b, int e, int4 pr, double margin, const double* zb,
                          int n) {
  const int l0 = b.lev_off[e], nl = b.lev_off[e + 1] - l0;
  const double z1 = b.z[l0 + max(pr.z - 1, 0)], z2 = b.z[l0 + min(pr.z + 1, nl - 1)];
  const double lo = fmin(z1, z2) - margin, hi = fmax(z1, z2) + margin;
  for (int p = 0; p < n; p++) {
    const double za = zb[p], zc = p + 1 < n ? zb[p + 1] : za;
    if (fmin(za, zc) <= hi && fmax(za, zc) >= lo) return p;
  }
  return n;
}

__global__ void k_resume_points(int nray, BatchDev b, LosDev L, int nbase, const int4* pert,
                                const int* base_obs, const int* ray_off, double margin,
                                int* start) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nray) return;
  const int e = b.ray_obs[r];
  const int4 pr = pert[e];
  if (e < nbase || pr.x < 0 || pr.x > 3) {
    start[r] = 0;
    return;
  }
  const int eb = base_obs[e];
  const int rb = ray_off[eb] + (r - ray_off[e]);
  const int n = min(L.count[rb], L.count[r]);
  const int p0 = first_near(b, e, pr, margin, L.z + L.off[rb], n);
  start[r] = max(p0 - 1, 0);
}

// Trace plan of the perturbed rays [nbase_rays, nray) of a resumed batch
// (TraceResume; the base rays are traced).  A perturbed mixing ratio
// (array 2) or extinction (array 3) leaves the walk alone: the step rule,
// refraction and the clipping at the ground and the top see z, p and T
// only, so the ray takes its base's geometry (mode 2).  A perturbed
// temperature (array 1) changes the walk only from the first segment that
// comes within margin of the perturbed levels' intervals, p0: before p0 the
// points, their data and the walk's state equal the base's, so the ray walks
// on from the base's state one point before p0 (mode 1, which needs that
// point unclipped: m < n_b - 1), or takes the base's geometry when no
// segment comes near (mode 2).  Everything else walks from the start
// (mode 0).  key: the points left to walk, for ordering the threads.
__global__ void k_trace_plan(int nray, int nbase_rays, BatchDev b, LosDev L, const int4* pert,
                             const int* base_obs, const int* ray_off, double margin, int4* plan,
                             int* key) {
  const int r = nbase_rays + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nray) return;
  const int e = b.ray_obs[r];
  const int4 pr = pert[e];
  int4 pl = make_int4(-1, 0, 0, 0);
  if (pr.x >= 1 && pr.x <= 3) {
    const int eb = base_obs[e];
    const int rb = ray_off[eb] + (r - ray_off[e]);
    const int nb = L.count[rb];
    if (nb > 0) {
      if (pr.x >= 2) {
        pl = make_int4(rb, 0, 2, 0);
      } else {
        const int p0 = first_near(b, e, pr, margin, L.z + L.off[rb], nb);
        if (p0 >= nb) pl = make_int4(rb, 0, 2, 0);
        else if (p0 - 1 >= 1) pl = make_int4(rb, p0 - 1, 1, 0);
      }
    }
  }
  plan[r] = pl;
  key[r - nbase_rays] = pl.z == 2 ? 0 : max(L.count[r] - pl.y, 0);
}

// Sort key of a resumed batch: bases first (their tiles run first and save
// the states), then by perturbation class (below: the perturbations that
// cannot share emitters, class 15, before those that can, so that the two
// form separate tile ranges), by measured channels, by the LOS points left
// to do in 64-point buckets (longest first, so that no long warp is left for
// the end) and by start point in 16-point buckets (so that the lanes of a
// warp walk nearly the same range of points).
// The perturbation class follows the channels: the perturbations of one
// emitter's mixing ratio (class 1 + emitter) and of extinctions (class 0)
// compute only that emitter (none) and take the others from their base, so
// a warp whose lanes share the class skips the others' work altogether.
__global__ void k_resume_keys(int nray, int nbase_rays, int nd, const unsigned char* mask,
                              int skip_masked, const int* count, const int* start,
                              const int4* pert, const int* ray_obs, int* key) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nray) return;
  int m = nd;
  if (skip_masked) {
    m = 0;
    for (int id = 0; id < nd; id++) m += mask[(long long)id * nray + r] ? 0 : 1;
  }
  const int left = count[r] - start[r];
  int cls = 0;
  if (pert) {  // emitters shared with the base
    const int4 pr = pert[ray_obs[r]];
    cls = pr.x == 2 ? 1 + min(pr.y, 13) : pr.x == 3 ? 0 : 15;
  }
  key[r] = ((r < nbase_rays ? 1 : 0) << 30) | (cls << 26) | (min(m, 511) << 17) |
           (min(left >> 6, 127) << 10) | (min(start[r] >> 4, 255) << 2);
}

// Sort key of a batch whose masked pairs are skipped: rays with the same
// number of measured channels first, then by LOS length, so that a tile's
// rays tend to share their masks and whole warps of unmeasured channels
// have nothing to do.
__global__ void k_mask_keys(int nray, int nd, const unsigned char* mask, const int* count,
                            int* key) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nray) return;
  int m = 0;
  for (int id = 0; id < nd; id++) m += mask[(long long)id * nray + r] ? 0 : 1;
  key[r] = (m << 13) | min(count[r], 8191);
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

}  // namespace

// Forward model of a device-resident batch (BatchDev pointers on device).
int jgb::run_core(jgb_ctx* x, BatchDev& b, int precision, bool timed_h2d) {
  cudaStream_t s = x->stream;
  const CtlDev& c = x->c;
  const int nray = b.nray;
  CK(x->err_word.reserve(sizeof(unsigned)));
  unsigned* d_err = x->err_word.as<unsigned>();
  x->stats.resume_skip = 0.0;
  CK(cudaMemsetAsync(d_err, 0, sizeof(unsigned), s));
  if (!timed_h2d) CK(cudaEventRecord(x->ev[1], s));

  // hydrostatic equilibrium (rewrites p in place)
  if (c.hydz >= 0) launch_hydrostatic(c, b, const_cast<double*>(b.p), s);
  CK(cudaEventRecord(x->ev[2], s));

  // ray tracing.  Mixed precision traces in one pass: a small batch into
  // fixed slabs of NLOS points per ray, a large one into capacities from a
  // geometric bound of every ray's LOS points; if a ray outgrows its bound,
  // or in FP64, the rays are counted first (count, scan, fill).
  const long long slab = c.nlos_max;
  // resumed perturbations (EGA; the Curtis-Godson sums run from the first
  // point) can be traced from their base rays' walks (TraceResume).  The
  // base rays are then traced before the others, which adds a whole walk to
  // the critical path (a batch within one wave takes as long as its longest
  // walk): measured, it gains nothing on a 1.3-wave Jacobian chunk and loses
  // on serving batches, so the automatic mode keeps it for batches of at
  // least four waves of the fill kernel; modes 2 and 3 force it.
  bool tres = x->resume && precision == JGB_MIXED && c.formod != 0;
  if (tres && x->fd_resume == 1) {
    const int nbr = x->resume->h_ray_off[x->resume->nbase];
    tres = (long long)(nray - nbr) >= 4LL * trace_fill_resident(x->sms);
  }
  int trace_launches = 0;  // kernels of the resumed tracing beyond one fill
  enum { kSlab, kBound, kCount } mode =
      precision != JGB_MIXED ? kCount
      : (long long)nray * slab <= kSinglePassPoints ? kSlab
      : x->los_bound_scale > 0 ? kBound : kCount;
  CK(x->los_cnt.reserve(sizeof(int) * (size_t)std::max(nray, 1)));
  CK(x->los_cnt64.reserve(sizeof(long long) * (size_t)(nray + 1)));
  CK(x->los_off.reserve(sizeof(long long) * (size_t)(nray + 1)));
  CK(x->los_sft.reserve(sizeof(double) * (size_t)std::max(nray, 1)));
  CK(x->los_ends.reserve(6 * sizeof(double) * (size_t)std::max(nray, 1)));
  LosDev L{};
  L.count = x->los_cnt.as<int>();
  L.off = x->los_off.as<long long>();
  L.sft = x->los_sft.as<double>();
  L.ends = x->los_ends.as<double>();
  L.ng = c.ng;
  L.nw = c.nw;
  L.cga = c.formod == 0;
  ChanDev ch = chan_view(x);
  long long* cnt64 = x->los_cnt64.as<long long>();
  size_t tmp_bytes = 0;
  long long total = 0, cap = 1;
  unsigned h_err = 0;
  int passes = 0;
  for (;;) {
    if (mode == kSlab) {
      k_slab_offsets<<<(nray + 1 + 255) / 256, 256, 0, s>>>(nray, slab, L.off, L.count);
      total = (long long)nray * slab;
    } else {
      // per-ray capacities (bound) or exact counts, then their offsets
      if (mode == kBound)
        launch_los_bound_mixed(c, b, x->los_bound_scale, L.count, s);
      else if (precision == JGB_MIXED)
        launch_trace_count_mixed(c, b, L, d_err, s);
      else
        launch_trace_count(c, ch, b, L, d_err, s);
      CK(cudaGetLastError());
      passes += mode == kCount;
      k_widen<<<(nray + 255) / 256, 256, 0, s>>>(nray, L.count, cnt64);
      CK(cudaMemsetAsync(L.off, 0, sizeof(long long), s));
      cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, cnt64, L.off + 1, nray, s);
      CK(x->scan_tmp.reserve(tmp_bytes + 16));
      cub::DeviceScan::InclusiveSum(x->scan_tmp.p, tmp_bytes, cnt64, L.off + 1, nray, s);
      CK(cudaMemcpyAsync(&total, L.off + nray, sizeof(long long), cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(&h_err, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (h_err & kErrObserverBelowSurface) return fail(x, JGB_ERR_SURFACE, "Observer below surface!");
      if (h_err & kErrLosOverflow) return fail(x, JGB_ERR_LOS, "Too many LOS points!");
    }
    cap = std::max(total, 1LL);
    const int nplanes = 8 + c.ng + c.nw + (c.formod == 0 ? 3 * c.ng : 0);
    const int nfplanes = 5 + c.ng + c.nw + (c.formod == 0 ? 3 * c.ng : 0);
    CK(x->los_planes.reserve(precision == JGB_MIXED
                                 ? (sizeof(double) + sizeof(float) * nfplanes) * (size_t)cap
                                 : sizeof(double) * (size_t)cap * nplanes));
    double* P = x->los_planes.as<double>();
    if (precision == JGB_MIXED) {  // z in FP64, the point data in FP32 planes
      float* F = reinterpret_cast<float*>(P + cap);
      L.f.p = F + 0 * cap;
      L.f.t = F + 1 * cap;
      L.f.ds = F + 2 * cap;
      L.f.aux = F + 3 * cap;
      L.f.qh2o = F + 4 * cap;
      L.f.u = F + 5 * cap;
      L.f.kw = L.f.u + (long long)c.ng * cap;
      L.f.cgp = L.f.kw + (long long)c.nw * cap;
      L.f.cgt = L.f.cgp + (long long)c.ng * cap;
      L.f.cgu = L.f.cgt + (long long)c.ng * cap;
    }
    L.cap = cap;
    L.z = P + 0 * cap;
    if (precision != JGB_MIXED) {
      L.lon = P + 1 * cap;
      L.lat = P + 2 * cap;
      L.p = P + 3 * cap;
      L.t = P + 4 * cap;
      L.ds = P + 5 * cap;
      L.aux = P + 6 * cap;
      L.qh2o = P + 7 * cap;
      L.u = P + 8 * cap;
      L.kw = L.u + (long long)c.ng * cap;
      L.cgp = L.kw + (long long)c.nw * cap;
      L.cgt = L.cgp + (long long)c.ng * cap;
      L.cgu = L.cgt + (long long)c.ng * cap;
    }
    if (tres) {
      // resumed perturbations: the base rays first, keeping their walks;
      // then the perturbed rays, by the points they have left to walk
      const int nbr = x->resume->h_ray_off[x->resume->nbase], npr = nray - nbr;
      long long bpts = (long long)nbr * slab;
      if (mode != kSlab) {
        CK(cudaMemcpyAsync(&bpts, L.off + nbr, sizeof(long long), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
      }
      bpts = std::max(bpts, 1LL);
      auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
      const size_t o_es = a16(sizeof(double) * 3 * (size_t)bpts);
      const size_t o_ds = o_es + o_es, o_lev = o_ds + a16(sizeof(float) * (size_t)bpts);
      const size_t o_plan = o_lev + a16(sizeof(int) * (size_t)bpts);
      const size_t o_key = o_plan + a16(sizeof(int4) * (size_t)nray);
      const size_t nk = (size_t)std::max(npr, 1);
      CK(x->rs_trace.reserve(o_key + 4 * a16(sizeof(int) * nk)));
      char* tb = x->rs_trace.as<char>();
      TraceResume R{};
      R.bpts = bpts;
      R.xs = reinterpret_cast<double*>(tb);
      R.es = reinterpret_cast<double*>(tb + o_es);
      R.dsr = reinterpret_cast<float*>(tb + o_ds);
      R.lev = reinterpret_cast<int*>(tb + o_lev);
      int4* plan = reinterpret_cast<int4*>(tb + o_plan);
      R.plan = plan;
      int* key = reinterpret_cast<int*>(tb + o_key);
      int* key2 = key + a16(sizeof(int) * nk) / sizeof(int);
      int* vin = key2 + a16(sizeof(int) * nk) / sizeof(int);
      int* vout = vin + a16(sizeof(int) * nk) / sizeof(int);
      launch_trace_fill_resumed(c, b, L, nullptr, 0, nbr, R, 1, d_err, s);
      if (npr > 0) {
        const ResumeSpec* rs = x->resume;
        k_trace_plan<<<(npr + 127) / 128, 128, 0, s>>>(nray, nbr, b, L, rs->pert, rs->base_obs,
                                                        rs->ray_off, 0.05, plan, key);
        k_iota<<<(npr + 255) / 256, 256, 0, s>>>(npr, vin, nbr);
        int bits = 1;
        while (bits < 31 && (1LL << bits) <= (long long)c.nlos_max) bits++;
        size_t sb = 0;
        cub::DeviceRadixSort::SortPairsDescending(nullptr, sb, key, key2, vin, vout, npr, 0, bits, s);
        CK(x->scan_tmp.reserve(sb + 16));
        cub::DeviceRadixSort::SortPairsDescending(x->scan_tmp.p, sb, key, key2, vin, vout, npr, 0,
                                                  bits, s);
        launch_trace_fill_resumed(c, b, L, vout, 0, npr, R, 2, d_err, s);
        trace_launches += 6;  // plan, iota, the sort's three passes, the fill
      }
    } else if (precision == JGB_MIXED) {
      // rays ordered by capacity (longest first) when the capacities are
      // bounds of the real lengths: a warp's rays then walk similar lengths
      const int* order = nullptr;
      if (mode == kBound && nray > 32) {
        CK(x->tiles_keys2.reserve(sizeof(int) * (size_t)nray));
        CK(x->tiles_vals.reserve(sizeof(int) * 2 * (size_t)nray));
        int* vin = x->tiles_vals.as<int>();
        int* vout = vin + nray;
        k_iota<<<(nray + 255) / 256, 256, 0, s>>>(nray, vin);
        int bits = 1;
        while (bits < 31 && (1LL << bits) <= (long long)c.nlos_max) bits++;
        size_t sb = 0;
        cub::DeviceRadixSort::SortPairsDescending(nullptr, sb, L.count, x->tiles_keys2.as<int>(),
                                                  vin, vout, nray, 0, bits, s);
        CK(x->scan_tmp.reserve(sb + 16));
        cub::DeviceRadixSort::SortPairsDescending(x->scan_tmp.p, sb, L.count,
                                                  x->tiles_keys2.as<int>(), vin, vout, nray, 0,
                                                  bits, s);
        order = vout;
      }
      launch_trace_fill_mixed(c, b, L, order, d_err, s);
    } else
      launch_trace_fill(c, ch, b, L, d_err, s);
    CK(cudaGetLastError());
    passes++;
    if (mode == kCount) break;
    // single pass: the fill pass set the counts; errors and the number of
    // LOS points
    k_widen<<<(nray + 255) / 256, 256, 0, s>>>(nray, L.count, cnt64);
    cub::DeviceReduce::Sum(nullptr, tmp_bytes, cnt64, cnt64 + nray, nray, s);
    CK(x->scan_tmp.reserve(tmp_bytes + 16));
    cub::DeviceReduce::Sum(x->scan_tmp.p, tmp_bytes, cnt64, cnt64 + nray, nray, s);
    CK(cudaMemcpyAsync(&total, cnt64 + nray, sizeof(long long), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&h_err, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (h_err & kErrObserverBelowSurface) return fail(x, JGB_ERR_SURFACE, "Observer below surface!");
    if (h_err & kErrLosOverflow) return fail(x, JGB_ERR_LOS, "Too many LOS points!");
    if (h_err & kErrSlabOverflow) {  // a bound was too small: count exactly
      CK(cudaMemsetAsync(d_err, 0, sizeof(unsigned), s));
      mode = kCount;
      continue;
    }
    break;
  }
  CK(cudaEventRecord(x->ev[3], s));

  // with a field of view the path kernels write pencil beams to scratch
  BatchDev bo = b;
  if (c.fov) {
    CK(x->fov_raw.reserve(sizeof(double) * 2 * (size_t)c.nd * nray));
    bo.rad = x->fov_raw.as<double>();
    bo.tau = bo.rad + (size_t)c.nd * nray;
  }
  // reflection needs per-point source and emissivity per channel
  const bool need_refl = c.sftype >= 2 && c.nsf > 0;
  TblDev T = tbl_view(x);
  int launches = 4 + (c.hydz >= 0) + trace_launches;
  if (precision == JGB_FP64) {
    double* refl = nullptr;
    if (need_refl) {
      CK(x->refl.reserve(sizeof(double) * 2 * (size_t)cap * c.nd));
      refl = x->refl.as<double>();
    }
    CK(cudaEventRecord(x->ev[4], s));
    launch_path_fp64(c, T, ch, bo, L, refl, s);
    launches += 1;
  } else {
    if (x->srf_stale) {
      launch_src_to_float(c.nd, x->s_sr.as<double>(), x->s_srf.as<float>(), s);
      x->srf_stale = false;
    }
    if (x->meta_stale) {
      // emitters whose (float) p and T grids are identical for all channels:
      // their brackets are found once per LOS point in the tile packing
      x->grid_mask = 0;
      if ((long long)x->tp * x->tt < 32768)  // rows of a p-T cell packed in 16 bits
        for (int g = 0; g < c.ng; g++) {
          bool same = x->h_np[g] >= 30;
          for (int id = 1; id < c.nd && same; id++) {
            const size_t a = (size_t)g, b = (size_t)id * c.ng + g;
            same = x->h_np[b] == x->h_np[a] &&
                   std::equal(x->h_nt.begin() + a * x->tp, x->h_nt.begin() + (a + 1) * x->tp,
                              x->h_nt.begin() + b * x->tp) &&
                   std::equal(x->h_pf.begin() + a * x->tp, x->h_pf.begin() + (a + 1) * x->tp,
                              x->h_pf.begin() + b * x->tp) &&
                   std::equal(x->h_tf.begin() + a * x->tp * x->tt,
                              x->h_tf.begin() + (a + 1) * x->tp * x->tt,
                              x->h_tf.begin() + b * x->tp * x->tt);
          }
          if (same) x->grid_mask |= 1u << g;
        }
      launch_rowmeta((long long)c.nd * c.ng * x->tp * x->tt, x->tu, x->t_nu.as<int>(),
                     x->t_u.as<float>(), x->t_eps.as<float>(), x->t_tf.as<float>(),
                     c.formod == 0, x->t_meta.as<float4>(), x->t_ue.as<float2>(), s);
      x->meta_stale = false;
    }
    // resumed perturbations: start points and the base rays' snapshot lists
    const ResumeSpec* rs = x->resume;
    const int nchb = (c.nd + 3) / 4;
    int nbase_rays = nray, tfirst = 0;
    int nplain_end = nray, tsecond = 0;  // resumed: end of the rays that share no emitter
    double resume_skip = 0.0;
    int* rstart = nullptr;
    int *snap_off = nullptr, *snap_ip = nullptr, *snap_ray = nullptr;
    // emitters shared between a perturbed ray and its base (see MixedPlan)
    float* seg_base = nullptr;
    unsigned *seg_satm = nullptr, *seg_final = nullptr;
    int* seg_nvalid = nullptr;
    const int2* seg_reuse = nullptr;
    bool share_emitters = false;
    if (rs) {
      nbase_rays = rs->h_ray_off[rs->nbase];
      // sharing emitters with the base pays where most of the perturbed
      // lookups can be taken from it (several emitters, mostly mixing-ratio
      // perturbations); elsewhere its bookkeeping and the registers of the
      // sharing kernel cost more than it saves
      double shr = 0, tot = 0;
      for (int e = rs->nbase; e < b.nobs; e++) {
        const double wr = rs->h_ray_off[e + 1] - rs->h_ray_off[e];
        const int4 pr = rs->h_pert[e];
        tot += wr;
        if (pr.x == 2 && c.ng > 1) shr += wr * (c.ng - 1.0) / c.ng;
        else if (pr.x == 3) shr += wr;
      }
      share_emitters = x->fd_resume == 3 || (tot > 0 && shr / tot >= 0.3);
      CK(x->rs_start.reserve(sizeof(int) * (size_t)nray));
      rstart = x->rs_start.as<int>();
      k_resume_points<<<(nray + 127) / 128, 128, 0, s>>>(nray, b, L, rs->nbase, rs->pert,
                                                          rs->base_obs, rs->ray_off,
                                                          0.05, rstart);
      CK(cudaGetLastError());
      CK(x->tiles_keys.reserve(sizeof(int) * (size_t)nray));
      k_resume_keys<<<(nray + 255) / 256, 256, 0, s>>>(nray, nbase_rays, c.nd, b.mask, b.skip_masked,
                                                        L.count, rstart,
                                                        share_emitters ? rs->pert : nullptr,
                                                        b.ray_obs, x->tiles_keys.as<int>());
      std::vector<int> hs(nray), ray_obs(nray), hc(nray), hk(nray);
      CK(cudaMemcpyAsync(hs.data(), rstart, sizeof(int) * nray, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(hc.data(), L.count, sizeof(int) * nray, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(hk.data(), x->tiles_keys.p, sizeof(int) * nray, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      long long skipped = 0, points = 0;
      for (int r = nbase_rays; r < nray; r++) {
        skipped += hs[r];
        points += hc[r];
      }
      resume_skip = points > 0 ? (double)skipped / (double)points : 0.0;
      // Does resuming pay?  Lanes of a warp walk the union of their point
      // ranges, and the base tiles run before the others.  Estimate both
      // schedules from their tile plans: a group of tiles takes the longer
      // of its work over the tiles the device holds at once and its longest
      // tile.
      const double conc = std::max(1.0, (double)x->sms * 8.0 / nchb);
      double waves = 0;  // of the plain plan: work over the longest tile
      auto group_time = [&](const std::vector<int>& order, int k0, int k1, bool resumed) {
        double sum = 0, mx = 0;
        for (int t = k0; t < k1; t += 32) {
          int hi = 0, lo = 1 << 30;
          for (int l = t; l < std::min(t + 32, k1); l++) {
            hi = std::max(hi, hc[order[l]]);
            lo = std::min(lo, resumed ? hs[order[l]] : 0);
          }
          sum += hi - lo;
          mx = std::max(mx, (double)(hi - lo));
        }
        waves = mx > 0 ? sum / conc / mx : 0;
        return std::max(sum / conc, mx);
      };
      std::vector<int> ord(nray);
      for (int r = 0; r < nray; r++) ord[r] = r;
      std::stable_sort(ord.begin(), ord.end(), [&](int a, int b2) { return hk[a] > hk[b2]; });
      const double t_res = group_time(ord, 0, nbase_rays, false) + group_time(ord, nbase_rays, nray, true);
      // the plain plan: measured channels (key bits 17-25), then LOS length
      std::stable_sort(ord.begin(), ord.end(), [&](int a, int b2) {
        const int ma = (hk[a] >> 17) & 511, mb = (hk[b2] >> 17) & 511;
        return ma != mb ? ma > mb : hc[a] > hc[b2];
      });
      const double t_plain = group_time(ord, 0, nray, false);
      // measured: resumed chunks win from about ten waves on (48 serving
      // requests: -6 %; 2048 nadir observations x 405 perturbations: +55 %
      // throughput) and lose on a few waves, where the base tiles, which
      // run first, cost more than the skipped points save
      if (x->fd_resume == 1 && !(t_res < 0.9 * t_plain && waves >= 8.0)) {
        rs = nullptr;  // run the batch plainly (the base copies are computed too)
        nbase_rays = nray;
        resume_skip = 0.0;
      }
    }
    if (rs) {
      std::vector<int> hs(nray), ray_obs(nray);
      CK(cudaMemcpyAsync(hs.data(), rstart, sizeof(int) * nray, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      for (int o = 0; o < b.nobs; o++)
        for (int r = rs->h_ray_off[o]; r < rs->h_ray_off[o + 1]; r++) ray_obs[r] = o;
      std::vector<int> off(nray + 1, 0);
      std::vector<int> rb_of(nray, -1);
      for (int r = nbase_rays; r < nray; r++)
        if (hs[r] > 0) {
          const int e = ray_obs[r], eb = rs->h_base_obs[e];
          rb_of[r] = rs->h_ray_off[eb] + (r - rs->h_ray_off[e]);
          off[rb_of[r] + 1]++;
        }
      for (int r = 0; r < nray; r++) off[r + 1] += off[r];
      const int nsnap = off[nray];
      std::vector<int> sip(nsnap), sray(nsnap), fill(off.begin(), off.end() - 1);
      for (int r = nbase_rays; r < nray; r++)
        if (rb_of[r] >= 0) {
          const int k = fill[rb_of[r]]++;
          sip[k] = hs[r];
          sray[k] = r;
        }
      for (int rb = 0; rb < nbase_rays; rb++) {  // each list in point order
        std::vector<std::pair<int, int>> v;
        for (int k = off[rb]; k < off[rb + 1]; k++) v.emplace_back(sip[k], sray[k]);
        std::sort(v.begin(), v.end());
        for (size_t k = 0; k < v.size(); k++) {
          sip[off[rb] + k] = v[k].first;
          sray[off[rb] + k] = v[k].second;
        }
      }
      CK(x->rs_lists.reserve(sizeof(int) * ((size_t)nray + 1 + 2 * (size_t)std::max(nsnap, 1))));
      snap_off = x->rs_lists.as<int>();
      snap_ip = snap_off + nray + 1;
      snap_ray = snap_ip + std::max(nsnap, 1);
      CK(cudaMemcpyAsync(snap_off, off.data(), sizeof(int) * (nray + 1), cudaMemcpyHostToDevice, s));
      if (nsnap) {
        CK(cudaMemcpyAsync(snap_ip, sip.data(), sizeof(int) * nsnap, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(snap_ray, sray.data(), sizeof(int) * nsnap, cudaMemcpyHostToDevice, s));
      }
      CK(x->rs_snap.reserve(sizeof(float) * (size_t)nray * c.nd * path_state_words(c)));
      // a perturbation of one emitter's mixing ratio (array 2) or of an
      // extinction (array 3) leaves the LOS (refraction needs p and T only)
      // and the other emitters' inputs and states equal to the base's: those
      // emitters' segment emissivities are taken from the base's walk
      std::vector<int2> reuse(nray, make_int2(-1, -1));
      bool any_reuse = false;
      for (int r = nbase_rays; r < nray && share_emitters; r++) {
        const int e = ray_obs[r];
        const int4 pr = rs->h_pert[e];
        if (pr.x == 2 || pr.x == 3) {
          const int eb = rs->h_base_obs[e];
          reuse[r] = make_int2(rs->h_ray_off[eb] + (r - rs->h_ray_off[e]), pr.x == 2 ? pr.y : -1);
          any_reuse = true;
        }
      }
      if (any_reuse) {
        long long bpts = 0;
        CK(cudaMemcpyAsync(&bpts, L.off + nbase_rays, sizeof(long long), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        const size_t nseg = (size_t)std::max(bpts, 1LL) * c.nd;
        const size_t nst = (size_t)nbase_rays * c.nd;
        const size_t sw = (size_t)path_state_words(c) - 3;
        auto a16 = [](size_t b) { return (b + 15) & ~size_t(15); };
        const size_t b_eps = a16(sizeof(float) * nseg * c.ng), b_satm = a16(sizeof(unsigned) * nseg);
        const size_t b_nv = a16(sizeof(int) * nst), b_fin = a16(sizeof(unsigned) * nst * sw);
        const size_t b_ru = a16(sizeof(int2) * (size_t)nray);
        CK(x->rs_seg.reserve(b_eps + b_satm + b_nv + b_fin + b_ru));
        char* sp = x->rs_seg.as<char>();
        seg_base = reinterpret_cast<float*>(sp);
        seg_satm = reinterpret_cast<unsigned*>(sp + b_eps);
        seg_nvalid = reinterpret_cast<int*>(sp + b_eps + b_satm);
        seg_final = reinterpret_cast<unsigned*>(sp + b_eps + b_satm + b_nv);
        int2* d_reuse = reinterpret_cast<int2*>(sp + b_eps + b_satm + b_nv + b_fin);
        CK(cudaMemcpyAsync(d_reuse, reuse.data(), sizeof(int2) * (size_t)nray, cudaMemcpyHostToDevice, s));
        seg_reuse = d_reuse;
      }
      CK(cudaStreamSynchronize(s));  // the host lists go out of scope
      tfirst = (nbase_rays + 31) / 32;
      // the perturbations that share no emitter sort before those that do
      int nplain = 0;
      for (int r = nbase_rays; r < nray; r++) nplain += reuse[r].x < 0 ? 1 : 0;
      nplain_end = nbase_rays + nplain;
      tsecond = tfirst + (nplain + 31) / 32;
    }
    // tile plan: rays sorted by LOS length, 32 per tile (resumed batches:
    // base tiles first, then the perturbations that share no emitter with
    // their base, then those that do)
    const int ntile = rs ? tsecond + (nray - nplain_end + 31) / 32 : (nray + 31) / 32;
    if (!rs) {
      tfirst = tsecond = ntile;
      nplain_end = nray;
    }
    CK(x->tiles_keys.reserve(sizeof(int) * (size_t)nray));
    CK(x->tiles_keys2.reserve(sizeof(int) * (size_t)nray));
    CK(x->tiles_vals.reserve(sizeof(int) * 2 * (size_t)nray));
    CK(x->tiles_perm.reserve(sizeof(int) * 32 * (size_t)ntile));
    CK(x->tiles_len.reserve(sizeof(int) * (size_t)ntile));
    CK(x->tiles_off.reserve(sizeof(long long) * (size_t)(2 * ntile + 2)));
    int* vals_in = x->tiles_vals.as<int>();
    int* vals_out = vals_in + nray;
    k_iota<<<(nray + 255) / 256, 256, 0, s>>>(nray, vals_in);
    const int* keys = L.count;
    if (rs) {
      k_resume_keys<<<(nray + 255) / 256, 256, 0, s>>>(nray, nbase_rays, c.nd, b.mask, b.skip_masked,
                                                        L.count, rstart,
                                                        share_emitters ? rs->pert : nullptr,
                                                        b.ray_obs, x->tiles_keys.as<int>());
      keys = x->tiles_keys.as<int>();
    } else if (b.skip_masked) {
      k_mask_keys<<<(nray + 255) / 256, 256, 0, s>>>(nray, c.nd, b.mask, L.count,
                                                      x->tiles_keys.as<int>());
      keys = x->tiles_keys.as<int>();
    }
    size_t sbytes = 0;
    cub::DeviceRadixSort::SortPairsDescending(nullptr, sbytes, keys, x->tiles_keys2.as<int>(),
                                              vals_in, vals_out, nray, 0, 32, s);
    CK(x->scan_tmp.reserve(std::max(sbytes, tmp_bytes) + 16));
    cub::DeviceRadixSort::SortPairsDescending(x->scan_tmp.p, sbytes, keys,
                                              x->tiles_keys2.as<int>(), vals_in, vals_out, nray,
                                              0, 32, s);
    long long* tpts = x->tiles_off.as<long long>() + ntile + 1;
    long long* toff = x->tiles_off.as<long long>();
    MixedPlan Pm{};
    Pm.ntile = ntile;
    Pm.perm = x->tiles_perm.as<int>();
    Pm.tlen = x->tiles_len.as<int>();
    Pm.toff = toff;
    Pm.tile0 = 0;
    Pm.tile1 = ntile;
    k_tiles<<<(ntile + 127) / 128, 128, 0, s>>>(nray, ntile, rs ? nbase_rays : nray, tfirst,
                                                 nplain_end, tsecond, L.count, vals_out, Pm.perm,
                                                 Pm.tlen, tpts);
    CK(cudaMemsetAsync(toff, 0, sizeof(long long), s));
    size_t sb2 = 0;
    cub::DeviceScan::InclusiveSum(nullptr, sb2, tpts, toff + 1, ntile, s);
    CK(x->scan_tmp.reserve(std::max(std::max(sbytes, tmp_bytes), sb2) + 16));
    cub::DeviceScan::InclusiveSum(x->scan_tmp.p, sb2, tpts, toff + 1, ntile, s);
    long long tile_points = 0;
    CK(cudaMemcpyAsync(&tile_points, toff + ntile, sizeof(long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    Pm.brmask = x->grid_mask;
    Pm.nfield = mixed_nfield(c, Pm.brmask);
    CK(x->tiles_data.reserve(sizeof(float) * 32 * (size_t)std::max(tile_points, 1LL) * Pm.nfield));
    Pm.data = x->tiles_data.as<float>();
    launch_pack_tiles_n(c, tbl_view(x), L, Pm, tile_points, s);
    CK(cudaGetLastError());
    float* refl = nullptr;
    if (need_refl) {
      CK(x->refl.reserve(sizeof(float) * 2 * (size_t)cap * c.nd));
      refl = x->refl.as<float>();
    }
    // a batch with too few tiles to fill the device is latency-bound: split
    // the path over the emitters (ng warps per tile and channel)
    const long long split_warps = (long long)ntile * c.nd * c.ng;
    const bool split = !rs && c.ng > 1 &&
                       (x->path_split == 1 || (x->path_split < 0 && split_warps <= 32LL * x->sms));
    Pm.seg_eps = nullptr;
    Pm.seg_sat = nullptr;
    if (rs) {
      // bases (saving the states), then the perturbations (starting from them)
      Pm.start = rstart;
      Pm.snap_off = snap_off;
      Pm.snap_ip = snap_ip;
      Pm.snap_ray = snap_ray;
      Pm.snap = x->rs_snap.as<float>();
      Pm.seg_base = seg_base;
      Pm.seg_satm = seg_satm;
      Pm.seg_nvalid = seg_nvalid;
      Pm.seg_final = seg_final;
      CK(cudaEventRecord(x->ev[4], s));
      Pm.tile0 = 0;
      Pm.tile1 = tfirst;
      Pm.reuse = nullptr;       // the bases write their emitters' values
      launch_path_resume(c, T, ch, bo, L, Pm, s);
      MixedPlan Pp = Pm;        // perturbations that share no emitter
      Pp.tile0 = tfirst;
      Pp.tile1 = tsecond;
      Pp.seg_base = nullptr;
      launch_path_resume(c, T, ch, bo, L, Pp, s);
      Pm.tile0 = tsecond;
      Pm.tile1 = ntile;
      Pm.reuse = seg_reuse;     // the perturbations that do read them
      launch_path_resume(c, T, ch, bo, L, Pm, s);
      launches += 10;
      x->stats.resume_skip = resume_skip;
    } else if (split) {
      const size_t nseg = (size_t)std::max(tile_points, 1LL) * c.nd * c.ng * 32;
      CK(x->seg.reserve(nseg * (sizeof(float) + 1)));
      Pm.seg_eps = x->seg.as<float>();
      Pm.seg_sat = reinterpret_cast<unsigned char*>(Pm.seg_eps + nseg);
      CK(cudaEventRecord(x->ev[4], s));
      launch_path_split(c, T, ch, bo, L, Pm, refl, s);
      launches += 7;
    } else if (x->path_variant < 0 && !rs) {
      // autotune: time every register cap with both block shapes on this
      // batch (results are identical)
      const char* force = getenv("JGB_PATH_VARIANT");
      if (force) {
        x->path_variant = atoi(force) % path_mixed_variants();
      } else {
        float best = 1e30f;
        x->tune_ms.clear();
        auto trial = [&](int v) -> int {
          CK(cudaEventRecord(x->ev[4], s));
          launch_path_mixed(c, T, ch, bo, L, Pm, refl, v, s);
          CK(cudaEventRecord(x->ev[5], s));
          CK(cudaEventSynchronize(x->ev[5]));
          const float ms = elapsed(x->ev[4], x->ev[5]);
          x->tune_ms.push_back(ms);
          if (ms < best) {
            best = ms;
            x->path_variant = v;
          }
          return JGB_OK;
        };
        for (int v = 0; v < path_mixed_variants(); v++) {
          const int rc = trial(v);
          if (rc) return rc;
        }
      }
    }
    if (!split && !rs) {
      CK(cudaEventRecord(x->ev[4], s));
      launch_path_mixed(c, T, ch, bo, L, Pm, refl, x->path_variant, s);
      launches += 6;
    }
  }
  CK(cudaGetLastError());
  if (c.fov) {
    const double* fd = x->d_fov.as<double>();
    launch_fov(c, b, bo.rad, bo.tau, x->nfov, fd, fd + x->nfov, ch.nu, d_err, s);
    launches += 1;
    CK(cudaMemcpyAsync(&h_err, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (h_err & kErrFov) return fail(x, JGB_ERR_ARG, "Cannot apply FOV convolution!");
  }
  CK(cudaEventRecord(x->ev[5], s));
  x->stats.los_points = total;
  x->stats.trace_passes = passes;
  x->stats.path_launches = launches;
  x->stats.path_variant = x->path_variant;
  for (int v = 0; v < 16; v++) x->stats.tune_ms[v] = v < (int)x->tune_ms.size() ? x->tune_ms[v] : 0.f;
  return JGB_OK;
}

namespace {

int check_ready(jgb_ctx* x) {
  if (!x->tables_init) return fail(x, JGB_ERR_STATE, "emissivity tables not set");
  for (int id = 0; id < x->c.nd; id++)
    if (!x->src_set[id]) return fail(x, JGB_ERR_STATE, "source function of a channel not set");
  return JGB_OK;
}

// ---------------------------------------------------------------------------
// finite-difference Jacobian (kernel, jurassic.c:4004-4099)

__device__ inline int upper_index(const int* off, int n, long long v) {
  // largest e in [0, n-1] with off[e] <= v
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= v) lo = mid; else hi = mid;
  }
  return lo;
}

// Copy levels of the source observation into every expanded copy.
__global__ void k_expand_levels(int ne, const int* eoff, const int* esrc, const int* boff,
                                int nplanes, long long nlev_b, const double* lb,
                                long long nlev_e, double* le) {
  const long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nlev_e) return;
  const int e = upper_index(eoff, ne, l);
  const long long src = boff[esrc[e]] + (l - eoff[e]);
  for (int k = 0; k < nplanes; k++) le[k * nlev_e + l] = lb[k * nlev_b + src];
}

// Copy rays (geometry and input mask) and scal records into the copies.
__global__ void k_expand_rays(int ne, const int* eoff, const int* esrc, const int* boff,
                              long long nray_b, const double* geo_b, const double* rad_b,
                              int nd, long long nray_e, double* geo_e, double* rad_e) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nray_e) return;
  const int e = upper_index(eoff, ne, r);
  const long long src = boff[esrc[e]] + (r - eoff[e]);
  for (int k = 0; k < 7; k++) geo_e[k * nray_e + r] = geo_b[k * nray_b + src];
  for (int id = 0; id < nd; id++) rad_e[id * nray_e + r] = rad_b[id * nray_b + src];
}

__global__ void k_expand_scal(int ne, const int* esrc, int nscal, const double* sb, double* se) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  for (int k = 0; k < nscal; k++) se[(long long)e * nscal + k] = sb[(long long)esrc[e] * nscal + k];
}

// Raise the perturbed element of every copy by the step of kernel().
// pert[e] = {arr, plane, level-in-copy or scal slot, hkind}.
__global__ void k_perturb(int ne, const int4* pert, const int* eoff, long long nlev_e, int nscal,
                          double* le_p, double* le_t, double* le_q, double* le_k, double* se,
                          double* hout) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int4 pr = pert[e];
  if (pr.x < 0) {  // an unperturbed base copy
    hout[e] = 0.0;
    return;
  }
  double* v;
  const long long l = (long long)eoff[e] + pr.z;
  switch (pr.x) {
    case 0: v = le_p + l; break;
    case 1: v = le_t + l; break;
    case 2: v = le_q + pr.y * nlev_e + l; break;
    case 3: v = le_k + pr.y * nlev_e + l; break;
    default: v = se + (long long)e * nscal + pr.z; break;
  }
  const double x0 = *v;
  double h;
  switch (pr.w) {
    case 0: h = fabs(0.01 * x0) > 1e-7 ? fabs(0.01 * x0) : 1e-7; break;
    case 2: h = fabs(0.01 * x0) > 1e-15 ? fabs(0.01 * x0) : 1e-15; break;
    case 1: h = 1.0; break;
    case 3: h = 1e-4; break;
    case 4: h = 0.1; break;
    case 5: h = 10.0; break;
    default: h = 1e-2; break;
  }
  *v = x0 + h;
  hout[e] = h;
}

// K[row][col] = (y_col - y0) / h for every observation of the chunk.
// ymap[row] = (ray within observation, channel); kb: block offsets;
// e0[i]: first copy of observation i (copy of element col = e0[i] + col).
__global__ void k_fd(int nobs, const long long* kb, const int* mcount, const int* ncount,
                     const int* yoff, const int2* ymap, const int* e0, const int* eray,
                     const double* rad_e, long long nray_e, const int* bray,
                     const double* rad0, long long nray0, const double* h,
                     const long long* kdst, double* K) {
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= kb[nobs]) return;
  int lo = 0, hi = nobs;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (kb[mid] <= g) lo = mid; else hi = mid;
  }
  const int i = lo;
  const long long k = g - kb[i];
  const int n = ncount[i];
  const int row = (int)(k / n), col = (int)(k % n);
  const int2 ym = ymap[yoff[i] + row];
  const int e = e0[i] + col;
  const double y1 = rad_e[(long long)ym.y * nray_e + eray[e] + ym.x];
  const double y0 = rad0[(long long)ym.y * nray0 + bray[i] + ym.x];
  K[kdst[i] + k] = (y1 - y0) / h[e];
}

}  // namespace

namespace jgb {

int ctx_view(jgb_ctx* x, CtxView* out) {
  if (!x || !out) return JGB_ERR_ARG;
  out->device = x->device;
  out->stream = x->stream;
  out->c = x->c;
  out->T = tbl_view(x);
  out->ch = chan_view(x);
  return check_ready(x);
}

int ctx_fail(jgb_ctx* x, int code, const char* msg) { return fail(x, code, msg); }
void ctx_lock(jgb_ctx* x) { x->mu.lock(); }
void ctx_unlock(jgb_ctx* x) { x->mu.unlock(); }
int ctx_error(jgb_ctx* x, int code, const std::string& msg) { return fail(x, code, msg); }

}  // namespace jgb

namespace jgb {

void state_layout(const jgb_ctx* x, const double* z, int nl, std::vector<Elem>& out) {
  const CtlDev& c = x->c;
  out.clear();
  for (int ip = 0; ip < nl; ip++)
    if (z[ip] >= x->retp_zmin && z[ip] <= x->retp_zmax) out.push_back({0, 0, ip, 0});
  for (int ip = 0; ip < nl; ip++)
    if (z[ip] >= x->rett_zmin && z[ip] <= x->rett_zmax) out.push_back({1, 0, ip, 1});
  for (int ig = 0; ig < c.ng; ig++)
    for (int ip = 0; ip < nl; ip++)
      if (z[ip] >= x->retq_zmin[ig] && z[ip] <= x->retq_zmax[ig]) out.push_back({2, ig, ip, 2});
  for (int iw = 0; iw < c.nw; iw++)
    for (int ip = 0; ip < nl; ip++)
      if (z[ip] >= x->retk_zmin[iw] && z[ip] <= x->retk_zmax[iw]) out.push_back({3, iw, ip, 3});
  if (x->ret_flags[0]) out.push_back({4, 0, -1, 1});
  if (x->ret_flags[1]) out.push_back({4, 1, -1, 1});
  if (x->ret_flags[2])
    for (int icl = 0; icl < c.ncl; icl++) out.push_back({4, 2 + icl, -1, 3});
  const int o = 2 + c.ncl;
  if (x->ret_flags[3]) out.push_back({4, o, -1, 4});
  if (x->ret_flags[4]) out.push_back({4, o + 1, -1, 5});
  if (x->ret_flags[5]) out.push_back({4, o + 2, -1, 1});
  if (x->ret_flags[6])
    for (int isf = 0; isf < c.nsf; isf++) out.push_back({4, o + 3 + isf, -1, 6});
}

void launch_ray_obs_mask(int nobs, const int* ray_off, int* ray_obs, long long n, const double* rad,
                         unsigned char* mask, cudaStream_t s) {
  k_ray_obs<<<(nobs + 127) / 128, 128, 0, s>>>(nobs, ray_off, ray_obs);
  k_mask<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, rad, mask);
}

int fd_layout(jgb_ctx* x, int nobs, const int* lev_off, const int* ray_off, const double* z,
              const double* rad_mask, FdLayout& H) {
  const CtlDev& c = x->c;
  const int nray = ray_off[nobs];
  H.nobs = nobs;
  H.lev_off.assign(lev_off, lev_off + nobs + 1);
  H.ray_off.assign(ray_off, ray_off + nobs + 1);
  H.lay.assign(nobs, {});
  H.mcnt.assign(nobs, 0);
  H.ncnt.assign(nobs, 0);
  H.yoff.assign(nobs + 1, 0);
  H.ymap.clear();
  H.kb.assign(nobs + 1, 0);
  for (int i = 0; i < nobs; i++) {
    state_layout(x, z + lev_off[i], lev_off[i + 1] - lev_off[i], H.lay[i]);
    H.ncnt[i] = (int)H.lay[i].size();
    for (int r = ray_off[i]; r < ray_off[i + 1]; r++)
      for (int id = 0; id < c.nd; id++)
        if (std::isfinite(rad_mask[(size_t)id * nray + r])) H.ymap.push_back(make_int2(r - ray_off[i], id));
    H.yoff[i + 1] = (int)H.ymap.size();
    H.mcnt[i] = H.yoff[i + 1] - H.yoff[i];
    if (H.ncnt[i] == 0 || H.mcnt[i] == 0) return fail(x, JGB_ERR_ARG, "Check problem definition!");
    H.kb[i + 1] = H.kb[i] + (long long)H.mcnt[i] * H.ncnt[i];
  }
  return JGB_OK;
}

// Finite-difference Jacobians of the observations in `list` of a device
// batch: every state element of every listed observation becomes one
// perturbed copy; chunks of copies (bounded by LOS points) run through the
// forward model as one batch; K blocks are written at K + H.kb[obs].
int fd_core(jgb_ctx* x, const FdLayout& H, const FdInput& in, const std::vector<int>& list,
            double* K, int precision) {
  const CtlDev& c = x->c;
  cudaStream_t s = x->stream;
  const int nscal = 5 + c.ncl + c.nsf;
  const int nplanes = 6 + c.ng + c.nw;
  const long long nlev = H.lev_off[H.nobs], nray = H.ray_off[H.nobs];
  const long long budget = 60000000LL;
  // Mixed-precision perturbations resume from their base's path state
  // (run_core with a ResumeSpec): exact when nothing but the perturbed
  // levels' neighbourhood changes the LOS, i.e. without hydrostatic
  // pressures, a field of view or surface reflection (its sum runs over the
  // whole path).
  const bool resume = precision == JGB_MIXED && x->fd_resume && c.hydz < 0 && !c.fov &&
                      !(c.sftype >= 2 && c.nsf > 0);
  size_t i0 = 0;
  while (i0 < list.size()) {
    long long pts = 0;
    size_t i1 = i0;
    while (i1 < list.size()) {
      const int o = list[i1];
      long long p_i = 0;
      for (int r = H.ray_off[o]; r < H.ray_off[o + 1]; r++) p_i += in.cnt[r] + 2;
      p_i *= H.ncnt[o];
      if (i1 > i0 && pts + p_i > budget) break;
      pts += p_i;
      i1++;
    }
    const int nob = (int)(i1 - i0);
    std::vector<int> eoff_l(1, 0), eoff_r(1, 0), esrc, e0(nob), ebase;
    std::vector<int4> pert;
    // by default only chunks of many tile waves resume (see run_core)
    bool res_chunk = resume;
    if (resume && x->fd_resume == 1) {
      long long prays = 0;
      for (size_t q = i0; q < i1; q++) {
        const int o = list[q];
        prays += (long long)H.ncnt[o] * (H.ray_off[o + 1] - H.ray_off[o]);
      }
      const double waves = (double)((prays + 31) / 32) * ((c.nd + 3) / 4) / (8.0 * x->sms);
      res_chunk = waves >= 8.0;
    }
    if (res_chunk)  // unperturbed base copies first
      for (size_t q = i0; q < i1; q++) {
        const int o = list[q];
        esrc.push_back(o);
        eoff_l.push_back(eoff_l.back() + (H.lev_off[o + 1] - H.lev_off[o]));
        eoff_r.push_back(eoff_r.back() + (H.ray_off[o + 1] - H.ray_off[o]));
        pert.push_back(make_int4(-1, 0, 0, 0));
        ebase.push_back((int)(q - i0));
      }
    for (size_t q = i0; q < i1; q++) {
      const int o = list[q];
      e0[q - i0] = (int)esrc.size();
      const int nl = H.lev_off[o + 1] - H.lev_off[o];
      const int nr = H.ray_off[o + 1] - H.ray_off[o];
      for (const Elem& el : H.lay[o]) {
        esrc.push_back(o);
        eoff_l.push_back(eoff_l.back() + nl);
        eoff_r.push_back(eoff_r.back() + nr);
        pert.push_back(make_int4(el.arr, el.idx, el.arr == 4 ? el.idx : el.lev, el.hkind));
        ebase.push_back(res_chunk ? (int)(q - i0) : 0);
      }
    }
    const int ne = (int)esrc.size();
    const long long nlev_e = eoff_l.back(), nray_e = eoff_r.back();
    CK(x->kx_levoff.reserve(sizeof(int) * (ne + 1)));
    CK(x->kx_rayoff.reserve(sizeof(int) * (ne + 1)));
    CK(x->kx_src.reserve(sizeof(int) * ne));
    CK(x->kx_pert.reserve(sizeof(int4) * ne));
    CK(x->kx_h.reserve(sizeof(double) * ne));
    CK(x->kx_lev.reserve(sizeof(double) * (size_t)nlev_e * nplanes));
    CK(x->kx_scal.reserve(sizeof(double) * (size_t)ne * nscal));
    CK(x->kx_geo.reserve(sizeof(double) * 7 * (size_t)nray_e));
    CK(x->kx_tp.reserve(sizeof(double) * ((size_t)c.nd * 2 + 3) * (size_t)nray_e));
    CK(x->kx_mask.reserve((size_t)c.nd * nray_e));
    CK(x->kx_rayobs.reserve(sizeof(int) * nray_e));
    CK(cudaMemcpyAsync(x->kx_levoff.p, eoff_l.data(), sizeof(int) * (ne + 1), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(x->kx_rayoff.p, eoff_r.data(), sizeof(int) * (ne + 1), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(x->kx_src.p, esrc.data(), sizeof(int) * ne, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(x->kx_pert.p, pert.data(), sizeof(int4) * ne, cudaMemcpyHostToDevice, s));
    double* le = x->kx_lev.as<double>();
    double* rad_e = x->kx_tp.as<double>();
    double* tau_e = rad_e + (size_t)c.nd * nray_e;
    double* tp_e = tau_e + (size_t)c.nd * nray_e;
    k_expand_levels<<<(unsigned)((nlev_e + 255) / 256), 256, 0, s>>>(
        ne, x->kx_levoff.as<int>(), x->kx_src.as<int>(), in.lev_off, nplanes, nlev, in.lev, nlev_e, le);
    k_expand_rays<<<(unsigned)((nray_e + 255) / 256), 256, 0, s>>>(
        ne, x->kx_rayoff.as<int>(), x->kx_src.as<int>(), in.ray_off, nray, in.geo, in.radmask,
        c.nd, nray_e, x->kx_geo.as<double>(), rad_e);
    k_expand_scal<<<(ne + 127) / 128, 128, 0, s>>>(ne, x->kx_src.as<int>(), nscal, in.scal,
                                                    x->kx_scal.as<double>());
    k_perturb<<<(ne + 127) / 128, 128, 0, s>>>(ne, x->kx_pert.as<int4>(), x->kx_levoff.as<int>(),
                                               nlev_e, nscal, le + 4 * nlev_e, le + 5 * nlev_e,
                                               le + 6 * nlev_e, le + (6 + (size_t)c.ng) * nlev_e,
                                               x->kx_scal.as<double>(), x->kx_h.as<double>());
    BatchDev b{};
    b.nobs = ne;
    b.nlev = (int)nlev_e;
    b.nray = (int)nray_e;
    b.nscal = nscal;
    b.lev_off = x->kx_levoff.as<int>();
    b.ray_obs = x->kx_rayobs.as<int>();
    b.time = le;
    b.z = le + nlev_e;
    b.lon = le + 2 * nlev_e;
    b.lat = le + 3 * nlev_e;
    b.p = le + 4 * nlev_e;
    b.t = le + 5 * nlev_e;
    b.q = le + 6 * nlev_e;
    b.k = le + (6 + (size_t)c.ng) * nlev_e;
    b.scal = x->kx_scal.as<double>();
    b.geo = x->kx_geo.as<double>();
    b.rad = rad_e;
    b.tau = tau_e;
    b.tp = tp_e;
    b.mask = x->kx_mask.as<unsigned char>();
    // only measured (finite) entries enter K; with a field of view every
    // pencil beam may feed a measured neighbour
    b.skip_masked = c.fov ? 0 : 1;
    k_ray_obs<<<(ne + 127) / 128, 128, 0, s>>>(ne, x->kx_rayoff.as<int>(), x->kx_rayobs.as<int>());
    const long long nm = (long long)c.nd * nray_e;
    k_mask<<<(unsigned)((nm + 255) / 256), 256, 0, s>>>(nm, rad_e, x->kx_mask.as<unsigned char>());
    CK(cudaGetLastError());
    CK(cudaEventRecord(x->ev[0], s));
    ResumeSpec rsp{};
    if (res_chunk) {
      CK(x->rs_base.reserve(sizeof(int) * (size_t)ne));
      CK(cudaMemcpyAsync(x->rs_base.p, ebase.data(), sizeof(int) * ne, cudaMemcpyHostToDevice, s));
      rsp.nbase = nob;
      rsp.pert = x->kx_pert.as<int4>();
      rsp.base_obs = x->rs_base.as<int>();
      rsp.ray_off = x->kx_rayoff.as<int>();
      rsp.h_ray_off = eoff_r.data();
      rsp.h_base_obs = ebase.data();
      rsp.h_pert = pert.data();
      x->resume = &rsp;
    }
    int rc = run_core(x, b, precision, false);
    x->resume = nullptr;
    if (rc) return rc;
    // finite differences
    std::vector<long long> kbl(nob + 1, 0), kdst(nob);
    std::vector<int> mc(nob), nc(nob), yo(nob), bray(nob);
    for (int q = 0; q < nob; q++) {
      const int o = list[i0 + q];
      kbl[q + 1] = kbl[q] + (long long)H.mcnt[o] * H.ncnt[o];
      kdst[q] = H.kb[o];
      mc[q] = H.mcnt[o];
      nc[q] = H.ncnt[o];
      yo[q] = H.yoff[o];
      bray[q] = H.ray_off[o];
    }
    // bookkeeping arrays carved from one buffer, each 16-byte aligned
    size_t off = 0;
    auto carve = [&](size_t bytes) {
      const size_t o = off;
      off = (off + bytes + 15) & ~size_t(15);
      return o;
    };
    const size_t o_kb = carve(sizeof(long long) * (nob + 1)), o_kd = carve(sizeof(long long) * nob);
    const size_t o_mc = carve(sizeof(int) * nob), o_nc = carve(sizeof(int) * nob);
    const size_t o_yo = carve(sizeof(int) * nob), o_e0 = carve(sizeof(int) * nob);
    const size_t o_br = carve(sizeof(int) * nob), o_ym = carve(sizeof(int2) * H.ymap.size());
    CK(x->kx_ymap.reserve(off + 16));
    char* qp = x->kx_ymap.as<char>();
    long long* d_kb = reinterpret_cast<long long*>(qp + o_kb);
    long long* d_kd = reinterpret_cast<long long*>(qp + o_kd);
    int* d_mc = reinterpret_cast<int*>(qp + o_mc);
    int* d_nc = reinterpret_cast<int*>(qp + o_nc);
    int* d_yo = reinterpret_cast<int*>(qp + o_yo);
    int* d_e0 = reinterpret_cast<int*>(qp + o_e0);
    int* d_br = reinterpret_cast<int*>(qp + o_br);
    int2* d_ym = reinterpret_cast<int2*>(qp + o_ym);
    CK(cudaMemcpyAsync(d_kb, kbl.data(), sizeof(long long) * (nob + 1), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_kd, kdst.data(), sizeof(long long) * nob, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_mc, mc.data(), sizeof(int) * nob, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_nc, nc.data(), sizeof(int) * nob, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_yo, yo.data(), sizeof(int) * nob, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_e0, e0.data(), sizeof(int) * nob, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_br, bray.data(), sizeof(int) * nob, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_ym, H.ymap.data(), sizeof(int2) * H.ymap.size(), cudaMemcpyHostToDevice, s));
    const long long nk = kbl[nob];
    k_fd<<<(unsigned)((nk + 255) / 256), 256, 0, s>>>(nob, d_kb, d_mc, d_nc, d_yo, d_ym, d_e0,
                                                       x->kx_rayoff.as<int>(), rad_e, nray_e,
                                                       d_br, in.rad0, nray, x->kx_h.as<double>(),
                                                       d_kd, K);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    i0 = i1;
  }
  return JGB_OK;
}

}  // namespace jgb

// ===========================================================================
// C ABI

constexpr int kL2ReadThreads = 512;

// passes sweeps over a buffer small enough to stay in L2 (loads that skip
// L1), one sum per thread written out so that no load is dropped
__global__ void __launch_bounds__(kL2ReadThreads)
    k_l2_read(const float4* __restrict__ a, long long n4, int passes, float* __restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  float sx = 0.f, sy = 0.f, sz = 0.f, sw = 0.f;
  for (int p = 0; p < passes; p++)
    for (long long i = t; i < n4; i += stride) {
      const float4 v = __ldcg(a + i);
      sx += v.x;
      sy += v.y;
      sz += v.z;
      sw += v.w;
    }
  out[t] = sx + sy + sz + sw;
}

extern "C" {

int jgb_create(const jgb_ctl* ctl, int device, jgb_ctx** out) {
  if (!ctl || !out) return JGB_ERR_ARG;
  *out = nullptr;
  if (ctl->ng < 0 || ctl->ng > kMaxG || ctl->nd <= 0 || ctl->nw < 0 || ctl->nw > kMaxW ||
      ctl->ncl < 0 || ctl->ncl == 1 || ctl->nsf < 0 || ctl->nsf == 1)
    return JGB_ERR_ARG;
  if (ctl->formod != 0 && ctl->formod != 1) return JGB_ERR_UNSUPPORTED;
  jgb_ctx* x = new jgb_ctx();
  x->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete x;
    return JGB_ERR_CUDA;
  }
  for (auto& e : x->ev) cudaEventCreate(&e);
  for (auto& e : x->pev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  cudaDeviceGetAttribute(&x->sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&x->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
    jgb_destroy(x);
    return JGB_ERR_CUDA;
  }
  // the allocation-free entry point's scratch array and kernels go onto the
  // device here, so that its calls load nothing (a failure is retried and
  // reported by its first call)
  (void)jgb::noalloc_prepare(device);
  CtlDev& c = x->c;
  c.ng = ctl->ng;
  c.nd = ctl->nd;
  c.nw = ctl->nw;
  c.ncl = ctl->ncl;
  c.nsf = ctl->nsf;
  c.sftype = ctl->sftype;
  c.sfsza = ctl->sfsza;
  c.hydz = ctl->hydz;
  c.ctm_co2 = ctl->ctm_co2;
  c.ctm_h2o = ctl->ctm_h2o;
  c.ctm_n2 = ctl->ctm_n2;
  c.ctm_o2 = ctl->ctm_o2;
  c.refrac = ctl->refrac;
  c.formod = ctl->formod;
  c.write_bbt = ctl->write_bbt;
  c.rayds = ctl->rayds;
  c.raydz = ctl->raydz;
  c.nlos_max = ctl->nlos_max > 0 ? ctl->nlos_max : 4096;
  c.ig_co2 = c.ig_h2o = -1;
  for (int ig = 0; ig < c.ng; ig++) {
    x->emitter.push_back(ctl->emitter && ctl->emitter[ig] ? ctl->emitter[ig] : "");
    if (c.ig_co2 < 0 && iequal(x->emitter.back(), "CO2")) c.ig_co2 = ig;
    if (c.ig_h2o < 0 && iequal(x->emitter.back(), "H2O")) c.ig_h2o = ig;
  }
  x->nu.assign(ctl->nu, ctl->nu + c.nd);
  x->window.assign(c.nd, 0);
  if (ctl->window)
    for (int id = 0; id < c.nd; id++) x->window[id] = ctl->window[id];
  for (int id = 0; id < c.nd; id++)
    if (c.nw > 0 && (x->window[id] < 0 || x->window[id] >= c.nw)) {
      jgb_destroy(x);
      return JGB_ERR_ARG;
    }
  x->clnu.assign(ctl->clnu, ctl->clnu + c.ncl);
  x->sfnu.assign(ctl->sfnu, ctl->sfnu + c.nsf);
  x->retp_zmin = ctl->retp_zmin;
  x->retp_zmax = ctl->retp_zmax;
  x->rett_zmin = ctl->rett_zmin;
  x->rett_zmax = ctl->rett_zmax;
  for (int ig = 0; ig < c.ng; ig++) {
    x->retq_zmin.push_back(ctl->retq_zmin ? ctl->retq_zmin[ig] : -999);
    x->retq_zmax.push_back(ctl->retq_zmax ? ctl->retq_zmax[ig] : -999);
  }
  for (int iw = 0; iw < c.nw; iw++) {
    x->retk_zmin.push_back(ctl->retk_zmin ? ctl->retk_zmin[iw] : -999);
    x->retk_zmax.push_back(ctl->retk_zmax ? ctl->retk_zmax[iw] : -999);
  }
  const int rf[7] = {ctl->ret_clz, ctl->ret_cldz, ctl->ret_clk, ctl->ret_sfz,
                     ctl->ret_sfp, ctl->ret_sft, ctl->ret_sfeps};
  std::memcpy(x->ret_flags, rf, sizeof(rf));
  // per-channel constants
  std::vector<double> ctm((size_t)c.nd * kCtmStride);
  for (int id = 0; id < c.nd; id++) ctm_coefficients(x->nu[id], &ctm[(size_t)id * kCtmStride]);
  std::vector<double> st(kNS);
  for (int it = 0; it < kNS; it++) st[it] = lin(0.0, kTMIN, kNS - 1.0, kTMAX, (double)it);
  bool ok = x->d_nu.reserve(sizeof(double) * c.nd) == cudaSuccess &&
            x->d_window.reserve(sizeof(int) * c.nd) == cudaSuccess &&
            x->d_clnu.reserve(sizeof(double) * (c.ncl + 1)) == cudaSuccess &&
            x->d_sfnu.reserve(sizeof(double) * (c.nsf + 1)) == cudaSuccess &&
            x->d_ctm.reserve(sizeof(double) * ctm.size()) == cudaSuccess &&
            x->s_st.reserve(sizeof(double) * kNS) == cudaSuccess &&
            x->s_sr.reserve(sizeof(double) * kNS * c.nd) == cudaSuccess &&
            x->s_srf.reserve(sizeof(float) * kNS * c.nd) == cudaSuccess;
  ok = ok && cudaMemcpy(x->d_nu.p, x->nu.data(), sizeof(double) * c.nd, cudaMemcpyHostToDevice) == cudaSuccess;
  ok = ok && cudaMemcpy(x->d_window.p, x->window.data(), sizeof(int) * c.nd, cudaMemcpyHostToDevice) == cudaSuccess;
  if (c.ncl) ok = ok && cudaMemcpy(x->d_clnu.p, x->clnu.data(), sizeof(double) * c.ncl, cudaMemcpyHostToDevice) == cudaSuccess;
  if (c.nsf) ok = ok && cudaMemcpy(x->d_sfnu.p, x->sfnu.data(), sizeof(double) * c.nsf, cudaMemcpyHostToDevice) == cudaSuccess;
  ok = ok && cudaMemcpy(x->d_ctm.p, ctm.data(), sizeof(double) * ctm.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  ok = ok && cudaMemcpy(x->s_st.p, st.data(), sizeof(double) * kNS, cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    jgb_destroy(x);
    return JGB_ERR_CUDA;
  }
  x->src_set.assign(c.nd, 0);
  *out = x;
  return JGB_OK;
}

void jgb_destroy(jgb_ctx* x) {
  if (!x) return;
  {
    jgb::CtxLock lock(x);  // calls still running on other threads end first
    cudaSetDevice(x->device);
    if (x->stream) cudaStreamSynchronize(x->stream);
    // engines still open lose their memory now and their context
    for (jgb_engine* E : x->engines) engine_detach(E);
    x->engines.clear();
  }
  DevBuf* bufs[] = {&x->d_nu, &x->d_window, &x->d_clnu, &x->d_sfnu, &x->d_ctm, &x->t_np,
                    &x->t_p, &x->t_nt, &x->t_t, &x->t_nu, &x->t_u, &x->t_eps, &x->t_pf,
                    &x->t_tf, &x->t_meta, &x->t_ue, &x->s_st, &x->s_sr, &x->s_srf, &x->b_levoff, &x->b_rayoff,
                    &x->b_rayobs, &x->b_lev, &x->b_scal, &x->b_geo, &x->b_rad, &x->b_tau,
                    &x->b_tp, &x->b_mask, &x->b_p, &x->los_off, &x->los_cnt, &x->los_cnt64,
                    &x->los_sft, &x->los_ends, &x->los_planes, &x->scan_tmp, &x->err_word,
                    &x->tiles_perm, &x->tiles_keys, &x->tiles_keys2, &x->tiles_vals,
                    &x->tiles_off, &x->tiles_len, &x->tiles_data, &x->refl, &x->seg,
                    &x->rs_start, &x->rs_lists, &x->rs_snap, &x->rs_base, &x->rs_seg, &x->rs_trace,
                    &x->d_fov, &x->fov_raw,
                    &x->kx_levoff, &x->kx_rayoff, &x->kx_rayobs, &x->kx_src, &x->kx_lev,
                    &x->kx_scal, &x->kx_geo, &x->kx_rad, &x->kx_tau, &x->kx_tp, &x->kx_mask,
                    &x->kx_pert, &x->kx_h, &x->kx_ymap, &x->kx_K, &x->kx_base_rayoff,
                    &x->kx_base_levoff};
  for (DevBuf* b : bufs) b->release();
  if (x->copy_stream) cudaStreamSynchronize(x->copy_stream);
  for (auto& e : x->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : x->pev)
    if (e) cudaEventDestroy(e);
  if (x->copy_stream) cudaStreamDestroy(x->copy_stream);
  if (x->stream) cudaStreamDestroy(x->stream);
  delete x;
}

const char* jgb_last_error(const jgb_ctx* x) { return x ? x->err.c_str() : "null context"; }

int jgb_tables_init(jgb_ctx* x, int tp, int tt, int tu) {
  jgb::CtxLock lock(x);
  if (!x || tp < 2 || tt < 2 || tu < 2) return fail(x, JGB_ERR_ARG, "bad table capacities");
  cudaSetDevice(x->device);
  const CtlDev& c = x->c;
  const size_t ndg = (size_t)c.nd * c.ng;
  if ((double)ndg * tp * tt * tu >= 4294967296.0)
    return fail(x, JGB_ERR_ARG, "emissivity tables larger than 2^32 entries per array");
  x->tp = tp;
  x->tt = tt;
  x->tu = tu;
  x->h_np.assign(ndg, -1);
  x->h_nt.assign(ndg * tp, 0);
  x->h_pf.assign(ndg * tp, 0.f);
  x->h_tf.assign(ndg * tp * tt, 0.f);
  CK(x->t_np.reserve(sizeof(int) * std::max<size_t>(ndg, 1)));
  CK(x->t_p.reserve(sizeof(double) * std::max<size_t>(ndg * tp, 1)));
  CK(x->t_nt.reserve(sizeof(int) * std::max<size_t>(ndg * tp, 1)));
  CK(x->t_t.reserve(sizeof(double) * std::max<size_t>(ndg * tp * tt, 1)));
  CK(x->t_nu.reserve(sizeof(int) * std::max<size_t>(ndg * tp * tt, 1)));
  CK(x->t_u.reserve(sizeof(float) * std::max<size_t>(ndg * tp * tt * tu, 1)));
  CK(x->t_eps.reserve(sizeof(float) * std::max<size_t>(ndg * tp * tt * tu, 1)));
  CK(x->t_pf.reserve(sizeof(float) * std::max<size_t>(ndg * tp, 1)));
  CK(x->t_tf.reserve(sizeof(float) * std::max<size_t>(ndg * tp * tt, 1)));
  CK(x->t_meta.reserve(2 * sizeof(float4) * std::max<size_t>(ndg * tp * tt, 1)));
  // one entry of padding after the last row (the row search reads a third
  // probe that it ignores at a row's end)
  CK(x->t_ue.reserve(sizeof(float2) * (ndg * tp * tt * tu + 1)));
  x->meta_stale = true;
  CK(cudaMemcpy(x->t_np.p, x->h_np.data(), sizeof(int) * ndg, cudaMemcpyHostToDevice));
  CK(cudaMemset(x->t_nt.p, 0, sizeof(int) * ndg * tp));
  CK(cudaMemset(x->t_nu.p, 0, sizeof(int) * ndg * tp * tt));
  CK(cudaMemset(x->t_p.p, 0, sizeof(double) * ndg * tp));
  CK(cudaMemset(x->t_t.p, 0, sizeof(double) * ndg * tp * tt));
  x->tables_init = true;
  return JGB_OK;
}

int jgb_set_table(jgb_ctx* x, int id, int ig, int np, const double* p, const int* nt,
                  const double* t, const int* nu, const float* u, const float* eps, int tt_cap,
                  int tu_cap) {
  jgb::CtxLock lock(x);
  if (!x || !x->tables_init) return fail(x, JGB_ERR_STATE, "jgb_tables_init not called");
  const CtlDev& c = x->c;
  if (id < 0 || id >= c.nd || ig < 0 || ig >= c.ng) return fail(x, JGB_ERR_ARG, "table index");
  if (np > x->tp) return fail(x, JGB_ERR_ARG, "Too many pressure levels!");
  cudaSetDevice(x->device);
  const size_t dg = (size_t)id * c.ng + ig;
  x->h_np[dg] = np;
  x->meta_stale = true;
  CK(cudaMemcpy(x->t_np.as<int>() + dg, &np, sizeof(int), cudaMemcpyHostToDevice));
  if (np <= 0) return JGB_OK;
  std::vector<int> ntv(x->tp, 0), nuv((size_t)x->tp * x->tt, 0);
  std::vector<double> pv(x->tp, 0), tv((size_t)x->tp * x->tt, 0);
  std::vector<float> pf(x->tp, 0), tf((size_t)x->tp * x->tt, 0);
  for (int ip = 0; ip < np; ip++) {
    if (nt[ip] > x->tt) return fail(x, JGB_ERR_ARG, "Too many temperatures!");
    pv[ip] = p[ip];
    pf[ip] = (float)p[ip];
    ntv[ip] = nt[ip];
    for (int it = 0; it < nt[ip]; it++) {
      const int n = nu[(size_t)ip * tt_cap + it];
      if (n > x->tu) return fail(x, JGB_ERR_ARG, "Too many column densities!");
      tv[(size_t)ip * x->tt + it] = t[(size_t)ip * tt_cap + it];
      tf[(size_t)ip * x->tt + it] = (float)t[(size_t)ip * tt_cap + it];
      nuv[(size_t)ip * x->tt + it] = n;
    }
  }
  std::copy(ntv.begin(), ntv.end(), x->h_nt.begin() + dg * x->tp);
  std::copy(pf.begin(), pf.end(), x->h_pf.begin() + dg * x->tp);
  std::copy(tf.begin(), tf.end(), x->h_tf.begin() + dg * x->tp * x->tt);
  CK(cudaMemcpy(x->t_p.as<double>() + dg * x->tp, pv.data(), sizeof(double) * x->tp, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(x->t_pf.as<float>() + dg * x->tp, pf.data(), sizeof(float) * x->tp, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(x->t_nt.as<int>() + dg * x->tp, ntv.data(), sizeof(int) * x->tp, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(x->t_t.as<double>() + dg * x->tp * x->tt, tv.data(), sizeof(double) * x->tp * x->tt, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(x->t_tf.as<float>() + dg * x->tp * x->tt, tf.data(), sizeof(float) * x->tp * x->tt, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(x->t_nu.as<int>() + dg * x->tp * x->tt, nuv.data(), sizeof(int) * x->tp * x->tt, cudaMemcpyHostToDevice));
  // rows: (ip, it) -> device row of tu floats; source rows have pitch tu_cap
  const size_t rows = (size_t)x->tp * x->tt;
  float* du = x->t_u.as<float>() + dg * rows * x->tu;
  float* de = x->t_eps.as<float>() + dg * rows * x->tu;
  for (int ip = 0; ip < np; ip++) {
    const int ntt = nt[ip];
    const size_t w = std::min(tu_cap, x->tu);
    CK(cudaMemcpy2D(du + (size_t)ip * x->tt * x->tu, sizeof(float) * x->tu,
                    u + (size_t)ip * tt_cap * tu_cap, sizeof(float) * tu_cap, sizeof(float) * w,
                    ntt, cudaMemcpyHostToDevice));
    CK(cudaMemcpy2D(de + (size_t)ip * x->tt * x->tu, sizeof(float) * x->tu,
                    eps + (size_t)ip * tt_cap * tu_cap, sizeof(float) * tu_cap,
                    sizeof(float) * w, ntt, cudaMemcpyHostToDevice));
  }
  return JGB_OK;
}

int jgb_set_fd_resume(jgb_ctx* x, int mode) {
  jgb::CtxLock lock(x);
  if (!x || mode < 0 || mode > 3) return fail(x, JGB_ERR_ARG, "bad resume setting");
  x->fd_resume = mode;
  return JGB_OK;
}

int jgb_set_path_split(jgb_ctx* x, int mode) {
  jgb::CtxLock lock(x);
  if (!x || mode < -1 || mode > 1) return fail(x, JGB_ERR_ARG, "bad path split mode");
  x->path_split = mode;
  return JGB_OK;
}

int jgb_set_los_bound_scale(jgb_ctx* x, double scale) {
  jgb::CtxLock lock(x);
  if (!x || !(scale >= 0) || scale > 1e6) return fail(x, JGB_ERR_ARG, "bad LOS bound scale");
  x->los_bound_scale = scale;
  return JGB_OK;
}

int jgb_set_fov(jgb_ctx* x, int n, const double* dz, const double* w) {
  jgb::CtxLock lock(x);
  if (!x || n < 0 || (n > 0 && (!dz || !w))) return fail(x, JGB_ERR_ARG, "bad field of view");
  if (n == 1) return fail(x, JGB_ERR_ARG, "Could not read any data!");  // read_shape needs >= 2
  if (n > 20000) return fail(x, JGB_ERR_ARG, "Too many data points!");  // NSHAPE
  cudaSetDevice(x->device);
  x->nfov = n;
  x->c.fov = n > 0;
  if (n == 0) return JGB_OK;
  CK(x->d_fov.reserve(sizeof(double) * 2 * n));
  CK(cudaMemcpy(x->d_fov.as<double>(), dz, sizeof(double) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(x->d_fov.as<double>() + n, w, sizeof(double) * n, cudaMemcpyHostToDevice));
  return JGB_OK;
}

int jgb_set_filter(jgb_ctx* x, int id, int n, const double* fnu, const double* f) {
  jgb::CtxLock lock(x);
  if (!x || id < 0 || id >= x->c.nd || n < 2 || !fnu || !f)
    return fail(x, JGB_ERR_ARG, "bad filter function");
  cudaSetDevice(x->device);
  DevBuf tmp;
  const size_t bytes = sizeof(double) * 2 * n + 2 * sizeof(int) + 16;
  CK(tmp.reserve(bytes));
  double* dx = tmp.as<double>();
  double* dy = dx + n;
  int* off = reinterpret_cast<int*>(dy + n);
  const int hoff[2] = {0, n};
  CK(cudaMemcpy(dx, fnu, sizeof(double) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dy, f, sizeof(double) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(off, hoff, sizeof(hoff), cudaMemcpyHostToDevice));
  launch_srcfunc(x->c.nd, id, 1, off, dx, dy, x->s_st.as<double>(), x->s_sr.as<double>(), x->stream);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(x->stream));
  tmp.release();
  x->src_set[id] = 1;
  x->srf_stale = true;
  return JGB_OK;
}

int jgb_set_srcfunc(jgb_ctx* x, const double* sr) {
  jgb::CtxLock lock(x);
  if (!x || !sr) return fail(x, JGB_ERR_ARG, "null source function");
  cudaSetDevice(x->device);
  CK(cudaMemcpy(x->s_sr.p, sr, sizeof(double) * kNS * x->c.nd, cudaMemcpyHostToDevice));
  std::fill(x->src_set.begin(), x->src_set.end(), 1);
  x->srf_stale = true;
  return JGB_OK;
}

int jgb_get_srcfunc(jgb_ctx* x, double* st, double* sr) {
  jgb::CtxLock lock(x);
  if (!x) return JGB_ERR_ARG;
  cudaSetDevice(x->device);
  if (st) CK(cudaMemcpy(st, x->s_st.p, sizeof(double) * kNS, cudaMemcpyDeviceToHost));
  if (sr) CK(cudaMemcpy(sr, x->s_sr.p, sizeof(double) * kNS * x->c.nd, cudaMemcpyDeviceToHost));
  return JGB_OK;
}

// Forward model of a batch in host memory.  A large batch runs as two
// chunks of whole observations, each a compact sub-batch on the device: the
// first eighth is copied in and computed while the rest is copied in on the
// copy stream, and its results go back while the rest is computed, so only
// the first chunk's inputs and the last chunk's results move while the
// device waits.  Rays are independent, so the results are those of one batch.
int jgb_formod_batch(jgb_ctx* x, const jgb_batch* hb, int precision) {
  jgb::CtxLock lock(x);
  if (!x || !hb || hb->nobs <= 0) return fail(x, JGB_ERR_ARG, "empty batch");
  if (precision != JGB_FP64 && precision != JGB_MIXED) return fail(x, JGB_ERR_ARG, "precision");
  int rc = check_ready(x);
  if (rc) return rc;
  cudaSetDevice(x->device);
  const CtlDev& c = x->c;
  cudaStream_t s = x->stream, cs = x->copy_stream;
  const int nobs = hb->nobs;
  const int nlev = hb->lev_off[nobs], nray = hb->ray_off[nobs];
  if (nlev <= 0 || nray <= 0) return fail(x, JGB_ERR_ARG, "no levels or rays");
  for (int o = 0; o < nobs; o++)
    if (hb->lev_off[o + 1] - hb->lev_off[o] < 2)
      return fail(x, JGB_ERR_ARG, "an atmosphere needs at least two levels");
  const int nscal = 5 + c.ncl + c.nsf;
  const int nlevf = 6 + c.ng + c.nw;  // time z lon lat p t q[] k[]
  // chunks of observations [ob[k], ob[k+1])
  int nchunk = 1, ob[3] = {0, nobs, nobs};
  const double in_bytes = 8.0 * ((double)nlev * nlevf + (double)nobs * nscal + 7.0 * nray +
                                 (double)c.nd * nray);
  if (nobs >= 16 && in_bytes >= 64.0 * (1 << 20)) {
    const int o1 = nobs / 8;
    if (hb->ray_off[o1] > 0 && hb->ray_off[o1] < nray) {
      nchunk = 2;
      ob[1] = o1;
    }
  }
  CK(x->b_levoff.reserve(sizeof(int) * (nobs + 2)));
  CK(x->b_rayoff.reserve(sizeof(int) * (nobs + 2)));
  CK(x->b_rayobs.reserve(sizeof(int) * nray));
  CK(x->b_lev.reserve(sizeof(double) * (size_t)nlev * nlevf));
  CK(x->b_scal.reserve(sizeof(double) * (size_t)nobs * nscal));
  CK(x->b_geo.reserve(sizeof(double) * 7 * (size_t)nray));
  CK(x->b_rad.reserve(sizeof(double) * (size_t)c.nd * nray));
  CK(x->b_tau.reserve(sizeof(double) * (size_t)c.nd * nray));
  CK(x->b_tp.reserve(sizeof(double) * 3 * (size_t)nray));
  CK(x->b_mask.reserve((size_t)c.nd * nray));
  struct Chunk {
    int o0, o1, l0, l1, r0, r1;
    BatchDev b;
    int* rayoff;
    std::vector<int> hlev, hray;  // offsets relative to the chunk
  };
  Chunk ck[2];
  for (int k = 0; k < nchunk; k++) {
    Chunk& h = ck[k];
    h.o0 = ob[k];
    h.o1 = ob[k + 1];
    h.l0 = hb->lev_off[h.o0];
    h.l1 = hb->lev_off[h.o1];
    h.r0 = hb->ray_off[h.o0];
    h.r1 = hb->ray_off[h.o1];
    const int no = h.o1 - h.o0, nl = h.l1 - h.l0, nr = h.r1 - h.r0;
    h.hlev.resize(no + 1);
    h.hray.resize(no + 1);
    for (int o = 0; o <= no; o++) {
      h.hlev[o] = hb->lev_off[h.o0 + o] - h.l0;
      h.hray[o] = hb->ray_off[h.o0 + o] - h.r0;
    }
    double* lev = x->b_lev.as<double>() + (size_t)nlevf * h.l0;  // compact planes of stride nl
    BatchDev& b = h.b;
    b = BatchDev{};
    b.nobs = no;
    b.nlev = nl;
    b.nray = nr;
    b.nscal = nscal;
    b.lev_off = x->b_levoff.as<int>() + h.o0 + k;
    h.rayoff = x->b_rayoff.as<int>() + h.o0 + k;
    b.ray_obs = x->b_rayobs.as<int>() + h.r0;
    b.time = lev;
    b.z = lev + (size_t)nl;
    b.lon = lev + 2 * (size_t)nl;
    b.lat = lev + 3 * (size_t)nl;
    b.p = lev + 4 * (size_t)nl;
    b.t = lev + 5 * (size_t)nl;
    b.q = lev + 6 * (size_t)nl;
    b.k = lev + (6 + (size_t)c.ng) * nl;
    b.scal = x->b_scal.as<double>() + (size_t)nscal * h.o0;
    b.geo = x->b_geo.as<double>() + 7 * (size_t)h.r0;
    b.rad = x->b_rad.as<double>() + (size_t)c.nd * h.r0;
    b.tau = x->b_tau.as<double>() + (size_t)c.nd * h.r0;
    b.tp = x->b_tp.as<double>() + 3 * (size_t)h.r0;
    b.mask = x->b_mask.as<unsigned char>() + (size_t)c.nd * h.r0;
  }
  const size_t D = sizeof(double);
  auto upload = [&](const Chunk& h, cudaStream_t st) -> cudaError_t {
    const BatchDev& b = h.b;
    const size_t nl = (size_t)b.nlev, nr = (size_t)b.nray, no = (size_t)b.nobs;
    cudaError_t e = cudaMemcpyAsync((void*)b.lev_off, h.hlev.data(), sizeof(int) * (no + 1),
                                    cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h.rayoff, h.hray.data(), sizeof(int) * (no + 1), cudaMemcpyHostToDevice, st);
    const double* src[6] = {hb->time, hb->z, hb->lon, hb->lat, hb->p, hb->t};
    const double* dst[6] = {b.time, b.z, b.lon, b.lat, b.p, b.t};
    for (int i = 0; i < 6 && e == cudaSuccess; i++)
      e = cudaMemcpyAsync((void*)dst[i], src[i] + h.l0, D * nl, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && c.ng)
      e = cudaMemcpy2DAsync((void*)b.q, D * nl, hb->q + h.l0, D * nlev, D * nl, c.ng,
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && c.nw)
      e = cudaMemcpy2DAsync((void*)b.k, D * nl, hb->k + h.l0, D * nlev, D * nl, c.nw,
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync((void*)b.scal, hb->scal + (size_t)nscal * h.o0, D * no * nscal,
                          cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync((void*)b.geo, D * nr, hb->geo + h.r0, D * nray, D * nr, 7,
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(b.rad, D * nr, hb->rad + h.r0, D * nray, D * nr, c.nd,
                            cudaMemcpyHostToDevice, st);
    return e;
  };
  auto download = [&](const Chunk& h, cudaStream_t st) -> cudaError_t {
    const BatchDev& b = h.b;
    const size_t nr = (size_t)b.nray;
    cudaError_t e = cudaMemcpy2DAsync(hb->rad + h.r0, D * nray, b.rad, D * nr, D * nr, c.nd,
                                      cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(hb->tau + h.r0, D * nray, b.tau, D * nr, D * nr, c.nd,
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(hb->tp + h.r0, D * nray, b.tp, D * nr, D * nr, 3,
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && c.hydz >= 0)
      e = cudaMemcpyAsync(hb->p + h.l0, b.p, D * (size_t)b.nlev, cudaMemcpyDeviceToHost, st);
    return e;
  };
  // on an error, let the copy stream finish with the caller's buffers
  auto bail = [&](int code) {
    cudaStreamSynchronize(cs);
    return code;
  };
  CK(cudaEventRecord(x->ev[0], s));
  CK(upload(ck[0], s));
  if (nchunk > 1) {
    CK(cudaStreamWaitEvent(cs, x->ev[0], 0));
    CK(upload(ck[1], cs));
    CK(cudaEventRecord(x->pev[0], cs));
  }
  double acc[4] = {0, 0, 0, 0}, h2d_ms = 0;
  long long los = 0;
  int launches = 0, passes = 0;
  for (int k = 0; k < nchunk; k++) {
    Chunk& h = ck[k];
    if (k > 0) CK(cudaStreamWaitEvent(s, x->pev[0], 0));
    const int no = h.b.nobs;
    k_ray_obs<<<(no + 127) / 128, 128, 0, s>>>(no, h.rayoff, const_cast<int*>(h.b.ray_obs));
    const long long nm = (long long)c.nd * h.b.nray;
    k_mask<<<(unsigned)((nm + 255) / 256), 256, 0, s>>>(nm, h.b.rad,
                                                        const_cast<unsigned char*>(h.b.mask));
    CK(cudaEventRecord(x->ev[1], s));
    rc = run_core(x, h.b, precision, true);
    if (rc) return bail(rc);
    if (k + 1 < nchunk) {
      CK(cudaEventRecord(x->pev[1], s));
      CK(cudaStreamWaitEvent(cs, x->pev[1], 0));
      CK(download(h, cs));
      CK(cudaEventRecord(x->pev[2], cs));
      // the next chunk's first host synchronisation waits for this one anyway
      CK(cudaEventSynchronize(x->ev[5]));
      if (k == 0) h2d_ms = elapsed(x->ev[0], x->ev[1]);
      acc[0] += elapsed(x->ev[1], x->ev[2]);
      acc[1] += elapsed(x->ev[2], x->ev[3]);
      acc[2] += elapsed(x->ev[3], x->ev[4]);
      acc[3] += elapsed(x->ev[4], x->ev[5]);
      los += x->stats.los_points;
      launches += x->stats.path_launches;
      passes = std::max(passes, x->stats.trace_passes);
    } else {
      CK(download(h, s));
    }
  }
  if (nchunk > 1) CK(cudaStreamWaitEvent(s, x->pev[2], 0));
  CK(cudaEventRecord(x->ev[6], s));
  CK(cudaStreamSynchronize(s));
  if (nchunk == 1) h2d_ms = elapsed(x->ev[0], x->ev[1]);
  x->stats.h2d_ms = h2d_ms;
  x->stats.hydro_ms = acc[0] + elapsed(x->ev[1], x->ev[2]);
  x->stats.trace_ms = acc[1] + elapsed(x->ev[2], x->ev[3]);
  x->stats.pack_ms = acc[2] + elapsed(x->ev[3], x->ev[4]);
  x->stats.path_ms = acc[3] + elapsed(x->ev[4], x->ev[5]);
  x->stats.d2h_ms = elapsed(x->ev[5], x->ev[6]);
  x->stats.total_ms = elapsed(x->ev[0], x->ev[6]);
  x->stats.los_points += los;
  x->stats.path_launches += launches;
  x->stats.trace_passes = std::max(passes, x->stats.trace_passes);
  return JGB_OK;
}

int jgb_formod_batch_dev(jgb_ctx* x, const jgb_batch* db, int precision) {
  jgb::CtxLock lock(x);
  if (!x || !db || db->nobs <= 0) return fail(x, JGB_ERR_ARG, "empty batch");
  if (precision != JGB_FP64 && precision != JGB_MIXED) return fail(x, JGB_ERR_ARG, "precision");
  int rc = check_ready(x);
  if (rc) return rc;
  cudaSetDevice(x->device);
  const CtlDev& c = x->c;
  cudaStream_t s = x->stream;
  const int nobs = db->nobs;
  int nlev = 0, nray = 0;
  CK(cudaMemcpy(&nlev, db->lev_off + nobs, sizeof(int), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(&nray, db->ray_off + nobs, sizeof(int), cudaMemcpyDeviceToHost));
  if (nlev <= 0 || nray <= 0) return fail(x, JGB_ERR_ARG, "no levels or rays");
  CK(x->b_rayobs.reserve(sizeof(int) * nray));
  CK(x->b_mask.reserve((size_t)c.nd * nray));
  BatchDev b{};
  b.nobs = nobs;
  b.nlev = nlev;
  b.nray = nray;
  b.nscal = 5 + c.ncl + c.nsf;
  b.lev_off = db->lev_off;
  b.ray_obs = x->b_rayobs.as<int>();
  b.time = db->time;
  b.z = db->z;
  b.lon = db->lon;
  b.lat = db->lat;
  b.p = db->p;
  b.t = db->t;
  b.q = db->q;
  b.k = db->k;
  b.scal = db->scal;
  b.geo = db->geo;
  b.rad = db->rad;
  b.tau = db->tau;
  b.tp = db->tp;
  b.mask = x->b_mask.as<unsigned char>();
  CK(cudaEventRecord(x->ev[0], s));
  k_ray_obs<<<(nobs + 127) / 128, 128, 0, s>>>(nobs, db->ray_off, x->b_rayobs.as<int>());
  const long long nm = (long long)c.nd * nray;
  k_mask<<<(unsigned)((nm + 255) / 256), 256, 0, s>>>(nm, b.rad, x->b_mask.as<unsigned char>());
  rc = run_core(x, b, precision, false);
  if (rc) return rc;
  CK(cudaEventRecord(x->ev[6], s));
  CK(cudaStreamSynchronize(s));
  x->stats.h2d_ms = 0;
  x->stats.hydro_ms = elapsed(x->ev[1], x->ev[2]);
  x->stats.trace_ms = elapsed(x->ev[2], x->ev[3]);
  x->stats.pack_ms = elapsed(x->ev[3], x->ev[4]);
  x->stats.path_ms = elapsed(x->ev[4], x->ev[5]);
  x->stats.d2h_ms = 0;
  x->stats.total_ms = elapsed(x->ev[0], x->ev[6]);
  return JGB_OK;
}

int jgb_formod(jgb_ctx* x, int np, const double* time, const double* z, const double* lon,
               const double* lat, double* p, const double* t, const double* q, const double* k,
               const double* scal, int nr, const double* geo, double* rad, double* tau,
               double* tp, int precision) {
  jgb::CtxLock lock(x);
  const int lev_off[2] = {0, np};
  const int ray_off[2] = {0, nr};
  jgb_batch b{};
  b.nobs = 1;
  b.lev_off = lev_off;
  b.time = time;
  b.z = z;
  b.lon = lon;
  b.lat = lat;
  b.p = p;
  b.t = t;
  b.q = q;
  b.k = k;
  b.scal = scal;
  b.ray_off = ray_off;
  b.geo = geo;
  b.rad = rad;
  b.tau = tau;
  b.tp = tp;
  return jgb_formod_batch(x, &b, precision);
}

int jgb_kernel_sizes(jgb_ctx* x, const jgb_batch* hb, int* m, int* n) {
  jgb::CtxLock lock(x);
  if (!x || !hb || !m || !n || hb->nobs <= 0) return fail(x, JGB_ERR_ARG, "bad arguments");
  const CtlDev& c = x->c;
  const int nray = hb->ray_off[hb->nobs];
  std::vector<Elem> el;
  for (int i = 0; i < hb->nobs; i++) {
    const int l0 = hb->lev_off[i];
    state_layout(x, hb->z + l0, hb->lev_off[i + 1] - l0, el);
    n[i] = (int)el.size();
    int mm = 0;
    for (int r = hb->ray_off[i]; r < hb->ray_off[i + 1]; r++)
      for (int id = 0; id < c.nd; id++) mm += std::isfinite(hb->rad[(size_t)id * nray + r]) ? 1 : 0;
    m[i] = mm;
  }
  return JGB_OK;
}

int jgb_kernel_batch(jgb_ctx* x, const jgb_batch* hb, double* kmat, int precision) {
  jgb::CtxLock lock(x);
  if (!x || !hb || !kmat || hb->nobs <= 0) return fail(x, JGB_ERR_ARG, "bad arguments");
  cudaSetDevice(x->device);
  const CtlDev& c = x->c;
  const int nobs = hb->nobs;
  const int nray = hb->ray_off[nobs], nlev = hb->lev_off[nobs];
  FdLayout H;
  int rc = fd_layout(x, nobs, hb->lev_off, hb->ray_off, hb->z, hb->rad, H);
  if (rc) return rc;
  // keep the caller's mask: the base forward model overwrites rad
  std::vector<double> rad_in(hb->rad, hb->rad + (size_t)c.nd * nray);
  // base forward model (also applies hydrostatic equilibrium to p)
  rc = jgb_formod_batch(x, hb, precision);
  if (rc) return rc;
  std::vector<int> cnt(nray);
  CK(cudaMemcpy(cnt.data(), x->los_cnt.p, sizeof(int) * nray, cudaMemcpyDeviceToHost));
  // snapshot of the post-hydrostatic base batch (the perturbed runs reuse b_*)
  const int nscal = 5 + c.ncl + c.nsf, nplanes = 6 + c.ng + c.nw;
  DevBuf snap;
  const size_t nb_lev = (size_t)nlev * nplanes, nb_scal = (size_t)nobs * nscal,
               nb_geo = 7 * (size_t)nray, nb_rad = (size_t)c.nd * nray;
  CK(snap.reserve(sizeof(double) * (nb_lev + nb_scal + nb_geo + 2 * nb_rad) + sizeof(int) * 2 * (nobs + 1)));
  double* lev = snap.as<double>();
  double* scal = lev + nb_lev;
  double* geo = scal + nb_scal;
  double* radm = geo + nb_geo;
  double* rad0 = radm + nb_rad;
  int* loff = reinterpret_cast<int*>(rad0 + nb_rad);
  int* roff = loff + nobs + 1;
  CK(cudaMemcpy(lev, x->b_lev.p, sizeof(double) * nb_lev, cudaMemcpyDeviceToDevice));
  CK(cudaMemcpy(scal, x->b_scal.p, sizeof(double) * nb_scal, cudaMemcpyDeviceToDevice));
  CK(cudaMemcpy(geo, x->b_geo.p, sizeof(double) * nb_geo, cudaMemcpyDeviceToDevice));
  CK(cudaMemcpy(rad0, x->b_rad.p, sizeof(double) * nb_rad, cudaMemcpyDeviceToDevice));
  CK(cudaMemcpy(radm, rad_in.data(), sizeof(double) * nb_rad, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(loff, hb->lev_off, sizeof(int) * (nobs + 1), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(roff, hb->ray_off, sizeof(int) * (nobs + 1), cudaMemcpyHostToDevice));
  FdInput in{lev, scal, geo, radm, loff, roff, rad0, cnt.data()};
  DevBuf kd;
  CK(kd.reserve(sizeof(double) * (size_t)std::max(H.kb[nobs], 1LL)));
  std::vector<int> all(nobs);
  for (int i = 0; i < nobs; i++) all[i] = i;
  rc = fd_core(x, H, in, all, kd.as<double>(), precision);
  if (rc) return rc;
  CK(cudaMemcpy(kmat, kd.p, sizeof(double) * (size_t)H.kb[nobs], cudaMemcpyDeviceToHost));
  return JGB_OK;
}

int jgb_get_stats(const jgb_ctx* x, jgb_stats* out) {
  jgb::CtxLock lock(x);
  if (!x || !out) return JGB_ERR_ARG;
  *out = x->stats;
  return JGB_OK;
}

// The slot of one state element in the caller's arrays (atm2x / x2atm
// order, jurassic.c:29-83 and 5896-5946): p, t, q[ig][ip], k[iw][ip], or
// the scalar block clz cldz clk[] sfz sfp sft sfeps[].
static double* state_slot(const jgb::Elem& e, int np, double* p, double* t, double* q, double* k,
                          double* scal) {
  switch (e.arr) {
    case 0: return p ? p + e.lev : nullptr;
    case 1: return t ? t + e.lev : nullptr;
    case 2: return q ? q + (long long)e.idx * np + e.lev : nullptr;
    case 3: return k ? k + (long long)e.idx * np + e.lev : nullptr;
    default: return scal ? scal + e.idx : nullptr;
  }
}

int jgb_atm2x(jgb_ctx* x, int np, const double* z, const double* p, const double* t,
              const double* q, const double* k, const double* scal, double* xv, int* n) {
  jgb::CtxLock lock(x);
  if (!x || np <= 0 || !z || !n) return JGB_ERR_ARG;
  std::vector<Elem> lay;
  state_layout(x, z, np, lay);
  *n = (int)lay.size();
  if (!xv) return JGB_OK;
  for (size_t j = 0; j < lay.size(); j++) {
    double* s = state_slot(lay[j], np, const_cast<double*>(p), const_cast<double*>(t),
                           const_cast<double*>(q), const_cast<double*>(k), const_cast<double*>(scal));
    if (!s) return ctx_fail(x, JGB_ERR_ARG, "state element in an array that was not given");
    xv[j] = *s;
  }
  return JGB_OK;
}

int jgb_x2atm(jgb_ctx* x, int np, const double* z, const double* xv, double* p, double* t,
              double* q, double* k, double* scal) {
  jgb::CtxLock lock(x);
  if (!x || np <= 0 || !z || !xv) return JGB_ERR_ARG;
  std::vector<Elem> lay;
  state_layout(x, z, np, lay);
  for (size_t j = 0; j < lay.size(); j++) {
    double* s = state_slot(lay[j], np, p, t, q, k, scal);
    if (!s) return ctx_fail(x, JGB_ERR_ARG, "state element in an array that was not given");
    *s = xv[j];
  }
  return JGB_OK;
}

int jgb_read_shape(const char* path, int nmax, double* xs, double* ys, int* n) {
  if (!path || nmax < 2 || !xs || !ys || !n) return JGB_ERR_ARG;
  *n = 0;
  FILE* in = fopen(path, "r");
  if (!in) return JGB_ERR_IO;
  // lines of two numbers; other lines (comments, headers) are skipped
  std::vector<char> line(1 << 16);
  while (fgets(line.data(), (int)line.size(), in)) {
    double a, b;
    if (sscanf(line.data(), "%lg %lg", &a, &b) == 2) {
      if (*n >= nmax) {
        fclose(in);
        return JGB_ERR_ARG;
      }
      xs[*n] = a;
      ys[*n] = b;
      (*n)++;
    }
  }
  fclose(in);
  return *n < 2 ? JGB_ERR_IO : JGB_OK;
}

void* jgb_host_alloc(unsigned long long bytes) {
  void* p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) return nullptr;
  return p;
}

void jgb_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

void* jgb_dev_alloc(unsigned long long bytes) {
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

void jgb_dev_free(void* p) {
  if (p) cudaFree(p);
}

int jgb_memcpy_h2d(void* dst, const void* src, unsigned long long bytes) {
  return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess ? JGB_OK : JGB_ERR_CUDA;
}

int jgb_memcpy_d2h(void* dst, const void* src, unsigned long long bytes) {
  return cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? JGB_OK : JGB_ERR_CUDA;
}

int jgb_measure_l2_read(unsigned long long bytes, int passes, double* gbs) {
  if (!gbs || bytes < 16 || passes < 1) return JGB_ERR_ARG;
  *gbs = 0.0;
  const long long n4 = (long long)(bytes / 16);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return JGB_ERR_CUDA;
  const int grid = sms * 4;
  float4* a = nullptr;
  float* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = JGB_ERR_CUDA;
  if (cudaMalloc(&a, n4 * 16) == cudaSuccess &&
      cudaMalloc(&out, (size_t)grid * kL2ReadThreads * 4) == cudaSuccess &&
      cudaMemset(a, 0, n4 * 16) == cudaSuccess && cudaEventCreate(&e0) == cudaSuccess &&
      cudaEventCreate(&e1) == cudaSuccess) {
    k_l2_read<<<grid, kL2ReadThreads>>>(a, n4, 1, out);  // brings the buffer into L2
    float best = 0.f;
    bool ok = cudaGetLastError() == cudaSuccess;
    for (int run = 0; ok && run < 5; run++) {
      cudaEventRecord(e0);
      k_l2_read<<<grid, kL2ReadThreads>>>(a, n4, passes, out);
      cudaEventRecord(e1);
      float ms = 0.f;
      ok = cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      if (ok && (best == 0.f || ms < best)) best = ms;
    }
    if (ok && best > 0.f) {
      *gbs = (double)n4 * 16.0 * passes / (best * 1e-3) / 1e9;
      st = JGB_OK;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(a);
  cudaFree(out);
  return st;
}

}  // extern "C"

// Emitter contributions (TASK c, formod.c:200-249): with the continua
// switched off, one forward model per emitter with every other emitter's
// volume mixing ratio and all extinction set to zero, then one with all
// mixing ratios zero and the extinction kept ("EXTINCT").  All ng + 1
// variants of every observation run as one batch.
extern "C" int jgb_formod_contrib(jgb_ctx* x, const jgb_batch* hb, double* rad_out,
                                  double* tau_out, int precision) {
  jgb::CtxLock lock(x);
  if (!x || !hb || hb->nobs <= 0 || !rad_out) return fail(x, JGB_ERR_ARG, "bad arguments");
  const CtlDev c = x->c;
  const int nobs = hb->nobs, ng = c.ng, nw = c.nw, nv = ng + 1;
  const long long nlev = hb->lev_off[nobs], nray = hb->ray_off[nobs];
  const int nscal = 5 + c.ncl + c.nsf;
  if ((long long)nobs * nv > 0x7fffffffLL || nlev * nv > 0x7fffffffLL || nray * nv > 0x7fffffffLL)
    return fail(x, JGB_ERR_ARG, "batch too large");
  const long long NL = nlev * nv, NR = nray * nv;
  std::vector<int> lo(nobs * nv + 1, 0), ro(nobs * nv + 1, 0);
  std::vector<double> time(NL), z(NL), lon(NL), lat(NL), p(NL), t(NL), q((size_t)ng * NL),
      k((size_t)nw * NL), scal((size_t)nobs * nv * nscal), geo(7 * (size_t)NR),
      rad((size_t)c.nd * NR), tau((size_t)c.nd * NR), tp(3 * (size_t)NR);
  // variant v of observation o is batch entry v * nobs + o
  for (int v = 0; v < nv; v++)
    for (int o = 0; o < nobs; o++) {
      const int e = v * nobs + o;
      lo[e + 1] = lo[e] + (hb->lev_off[o + 1] - hb->lev_off[o]);
      ro[e + 1] = ro[e] + (hb->ray_off[o + 1] - hb->ray_off[o]);
    }
  for (int v = 0; v < nv; v++) {
    const long long l0 = v * nlev, r0 = v * nray;
    std::memcpy(&time[l0], hb->time, sizeof(double) * nlev);
    std::memcpy(&z[l0], hb->z, sizeof(double) * nlev);
    std::memcpy(&lon[l0], hb->lon, sizeof(double) * nlev);
    std::memcpy(&lat[l0], hb->lat, sizeof(double) * nlev);
    std::memcpy(&p[l0], hb->p, sizeof(double) * nlev);
    std::memcpy(&t[l0], hb->t, sizeof(double) * nlev);
    for (int g = 0; g < ng; g++)
      if (v == g) std::memcpy(&q[(size_t)g * NL + l0], hb->q + (size_t)g * nlev, sizeof(double) * nlev);
    for (int w = 0; w < nw; w++)
      if (v == ng) std::memcpy(&k[(size_t)w * NL + l0], hb->k + (size_t)w * nlev, sizeof(double) * nlev);
    std::memcpy(&scal[(size_t)v * nobs * nscal], hb->scal, sizeof(double) * nobs * nscal);
    for (int f = 0; f < 7; f++) std::memcpy(&geo[f * NR + r0], hb->geo + f * nray, sizeof(double) * nray);
    for (int id = 0; id < c.nd; id++)
      std::memcpy(&rad[id * NR + r0], hb->rad + id * nray, sizeof(double) * nray);
  }
  jgb_batch eb{};
  eb.nobs = nobs * nv;
  eb.lev_off = lo.data();
  eb.time = time.data();
  eb.z = z.data();
  eb.lon = lon.data();
  eb.lat = lat.data();
  eb.p = p.data();
  eb.t = t.data();
  eb.q = q.data();
  eb.k = k.data();
  eb.scal = scal.data();
  eb.ray_off = ro.data();
  eb.geo = geo.data();
  eb.rad = rad.data();
  eb.tau = tau.data();
  eb.tp = tp.data();
  // continua off for these runs (formod.c:203-207)
  x->c.ctm_co2 = x->c.ctm_h2o = x->c.ctm_n2 = x->c.ctm_o2 = 0;
  const int rc = jgb_formod_batch(x, &eb, precision);
  x->c = c;
  if (rc) return rc;
  // rad/tau are [nd][nv*nray]; reorder to [nv][nd][nray]
  for (int v = 0; v < nv; v++)
    for (int id = 0; id < c.nd; id++) {
      std::memcpy(rad_out + ((size_t)v * c.nd + id) * nray, &rad[id * NR + v * nray], sizeof(double) * nray);
      if (tau_out)
        std::memcpy(tau_out + ((size_t)v * c.nd + id) * nray, &tau[id * NR + v * nray], sizeof(double) * nray);
    }
  return JGB_OK;
}
