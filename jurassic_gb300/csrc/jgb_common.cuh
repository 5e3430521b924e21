// Shared device helpers and internal structures of libjurassic_gb300.
//
// FP64 helpers reproduce the reference's expression order so that the FP64
// path agrees with the reference to rounding (translation units that use
// them are compiled without FMA contraction).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace jgb {

// Physical constants (jurassic.h:254-345).
constexpr double kC1 = 1.19104259e-8;
constexpr double kC2 = 1.43877506;
constexpr double kG0 = 9.80665;
constexpr double kKB = 1.3806504e-23;
constexpr double kNA = 6.02214199e23;
constexpr double kRE = 6367.421;
constexpr double kRI = 8.3144598;
constexpr double kP0 = 1013.25;
constexpr double kTMIN = 100.0;
constexpr double kTMAX = 400.0;
constexpr double kTSUN = 5780.0;
constexpr int kNS = 1200;  // source-function temperatures (TBLNS)
constexpr double kPI = 3.14159265358979323846;
constexpr int kMaxG = 16;  // emitters handled by the device path
constexpr int kMaxW = 8;   // spectral windows handled by the device path

// Error flags raised by kernels (bit mask in a device word).
enum : unsigned {
  kErrLosOverflow = 1u,
  kErrObserverBelowSurface = 2u,
  kErrBadInput = 4u,
  kErrFov = 8u,
  kErrSlabOverflow = 16u,  // a ray outgrew its estimated capacity (traced again)
};

// ---------------------------------------------------------------------------
// FP64 helpers (LIN/LOGX/LOGY jurassic.h:164-175; locate_* jurassic.c:4103-4170)

__host__ __device__ inline double lin(double x0, double y0, double x1, double y1, double x) {
  return y0 + (y1 - y0) / (x1 - x0) * (x - x0);
}

__host__ __device__ inline double logx(double x0, double y0, double x1, double y1, double x) {
  if (x / x0 > 0 && x1 / x0 > 0) return y0 + (y1 - y0) * log(x / x0) / log(x1 / x0);
  return lin(x0, y0, x1, y1, x);
}

__host__ __device__ inline double logy(double x0, double y0, double x1, double y1, double x) {
  if (y1 / y0 > 0) return y0 * exp(log(y1 / y0) / (x1 - x0) * (x - x0));
  return lin(x0, y0, x1, y1, x);
}

// Interpolation between two float table entries: the slope is formed in
// single precision, as the reference's LIN macro does on float operands.
__host__ __device__ inline double lin_f(float x0, float y0, float x1, float y1, double x) {
  const float slope = (y1 - y0) / (x1 - x0);
  return (double)y0 + (double)slope * (x - (double)x0);
}

// Lower bracket on an ascending or descending grid (bisection).
template <typename T>
__host__ __device__ inline int bracket_irr(const T* g, int n, double x) {
  int lo = 0, hi = n - 1, mid = (lo + hi) >> 1;
  const bool up = g[mid] < g[mid + 1];
  while (hi > lo + 1) {
    mid = (lo + hi) >> 1;
    const bool go_low = up ? ((double)g[mid] > x) : ((double)g[mid] <= x);
    if (go_low) hi = mid; else lo = mid;
  }
  return lo;
}

// Direct index on a regular grid, clamped to [0, n-2].
__host__ __device__ inline int bracket_reg(const double* g, int n, double x) {
  const int i = (int)((x - g[0]) / (g[1] - g[0]));
  if (i < 0) return 0;
  if (i > n - 2) return n - 2;
  return i;
}

// Bisection on an ascending float row.
__host__ __device__ inline int bracket_row(const float* g, int n, double x) {
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    const int mid = (lo + hi) >> 1;
    if ((double)g[mid] > x) hi = mid; else lo = mid;
  }
  return lo;
}

__host__ __device__ inline void to_geo(const double* x, double* z, double* lon, double* lat) {
  const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  *lat = asin(x[2] / r) * (180.0 / kPI);
  *lon = atan2(x[1], x[0]) * (180.0 / kPI);
  *z = r - kRE;
}

__host__ __device__ inline void to_cart(double z, double lon, double lat, double* x) {
  const double r = z + kRE;
  const double la = lat / 180. * kPI, lo = lon / 180. * kPI;
  const double cl = cos(la);
  x[0] = r * cl * cos(lo);
  x[1] = r * cl * sin(lo);
  x[2] = r * sin(la);
}

__host__ __device__ inline double planck(double t, double nu) {
  return kC1 * (nu * nu * nu) / expm1(kC2 * nu / t);
}

// ---------------------------------------------------------------------------
// Device-resident views (plain pointers into context-owned buffers)

struct CtlDev {
  int ng, nd, nw, ncl, nsf;
  int sftype;
  double sfsza, hydz;
  int ctm_co2, ctm_h2o, ctm_n2, ctm_o2;
  int refrac, formod, write_bbt;
  double rayds, raydz;
  int ig_co2, ig_h2o;
  int nlos_max;
  int fov;   // field-of-view convolution on: path kernels write pencil values only
};

// Emissivity tables, dense with capacities tp x tt x tu per (channel, emitter).
struct TblDev {
  int tp, tt, tu;
  const int* np;       // [nd*ng]
  const double* p;     // [nd*ng*tp]
  const int* nt;       // [nd*ng*tp]
  const double* t;     // [nd*ng*tp*tt]
  const int* nu;       // [nd*ng*tp*tt]
  const float* u;      // [nd*ng*tp*tt*tu]
  const float* eps;    // [nd*ng*tp*tt*tu]
  const float* pf;     // float copies of p and t for the mixed path
  const float* tf;
  const float4* rowmeta;  // row records of the mixed path (EGA: 2 float4 per row, CGA: 1)
  const float2* ue;    // rows interleaved {u[i], eps[i]} (mixed path)
  const double* sr;    // source function [kNS][nd]
  const float* srf;    // source function, channel-major float [nd][kNS]
  const double* st;    // source-function temperatures [kNS]
};

// Per-channel constants: wavenumber, window, continuum coefficients.
struct ChanDev {
  const double* nu;     // [nd]
  const int* window;    // [nd]
  const double* clnu;   // [ncl]
  const double* sfnu;   // [nsf]
  const double* ctm;    // [nd][kCtmStride] continuum coefficients (see jgb_api.cu)
};
constexpr int kCtmStride = 16;

// A packed batch of observations on the device.
struct BatchDev {
  int nobs, nlev, nray, nscal;
  const int* lev_off;   // [nobs+1]
  const int* ray_obs;   // [nray] observation of each ray
  const double *time, *z, *lon, *lat, *p, *t, *q, *k, *scal;
  const double* geo;    // [7][nray]
  double* rad;          // [nd][nray]
  double* tau;          // [nd][nray]
  double* tp;           // [3][nray]
  const unsigned char* mask;  // [nd][nray] 1 = masked
  // [nobs] 1 = observation not computed: its rays get no LOS and its
  // outputs (rad, tau, tp) and pressures are left untouched (nullptr: none)
  const unsigned char* obs_skip;
  // 1: masked (ray, channel) pairs need no radiance (their outputs are only
  // NaN-masked), so the path loop skips them; 0: every pair is computed
  unsigned char skip_masked;
};

// Lines of sight, ray-major with per-ray offsets, SoA planes of FP64.
struct LosDev {
  long long* off;       // [nray+1]
  int* count;           // [nray]
  double* sft;          // [nray]  surface temperature or -999
  double* ends;         // [nray][6]: z,lon,lat of first and last point
  long long cap;        // capacity in points
  int ng, nw;
  bool cga;
  // planes [point]
  double *z, *lon, *lat, *p, *t, *ds, *aux, *qh2o;
  double* u;            // [ng][cap]
  double* kw;           // [nw][cap]
  double *cgp, *cgt, *cgu;  // [ng][cap] (CGA only)
  // mixed precision: the point data as FP32 planes (the values are FP32
  // numbers; z above stays FP64)
  struct F32 {
    float *p, *t, *ds, *aux, *qh2o;
    float* u;             // [ng][cap]
    float* kw;            // [nw][cap]
    float *cgp, *cgt, *cgu;  // [ng][cap] (CGA only)
  } f;
};

// Float LOS tiles for the mixed path: 32 rays per tile (rays sorted by
// length), point-major inside a tile, one float plane per field.
struct TileDev {
  int ntile;
  const int* perm;          // [ntile*32] ray of (tile, lane), -1 = empty lane
  const long long* off;     // [ntile+1] point offsets (points of a tile x 32)
  const int* len;           // [ntile] longest ray of the tile
  int nfield;
  float* data;              // [total_points*32][nfield] as [tile-point][field][lane]
};

}  // namespace jgb
