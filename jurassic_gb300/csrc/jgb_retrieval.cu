// Optimal-estimation retrieval on the device (optimal_estimation,
// retrieval.c:448-749), batched over independent retrievals.
//
// All retrievals of a batch advance in lockstep through the Levenberg-
// Marquardt iterations, each with its own damping parameter, inner-loop
// state and convergence flag.  Per outer iteration: finite-difference
// Jacobian (fd_core, one batched forward-model launch sequence for every
// perturbation of every active retrieval), normal-equation products (3xTF32
// tensor cores or FP64), then up to 20 damped steps, each an FP64 Cholesky
// solve plus one batched forward model of the retrievals still trying.
// FP64 is used for the a-priori covariance and its inverse, the Cholesky
// solves, the cost function and the convergence test.
//
// This translation unit is compiled without FMA contraction: the FP64 linear
// algebra follows the textbook loop orders of the reference's helpers
// (cost_function retrieval.c:340-369, matrix_invert 373-399, Cholesky
// decomposition/solution as used at 588-589).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "jgb_ctx.h"
#include "jgb_internal.h"

namespace jgb {
namespace {

#define RCK(call)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return ctx_error(x, JGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Per-retrieval offsets into the concatenated vectors and matrices.
struct RetDesc {
  int n, m;
  long long xo, yo, so, ko;   // offsets: state vectors, measurement vectors, n*n, m*n
};

// ---------------------------------------------------------------------------
// state <-> atmosphere (atm2x / x2atm, jurassic.c:29-104, 5896-5958)

// Level arrays of the current iterate: [6+ng+nw][nlev] like the forward batch.
struct AtmArrays {
  double* lev;
  double* scal;
  long long nlev;
  int nscal, ng;
};

__device__ inline double* elem_ptr(const AtmArrays& a, int lev0, long long o, int4 el) {
  switch (el.x) {
    case 0: return a.lev + 4 * a.nlev + lev0 + el.z;
    case 1: return a.lev + 5 * a.nlev + lev0 + el.z;
    case 2: return a.lev + (6 + el.y) * a.nlev + lev0 + el.z;
    case 3: return a.lev + (6 + a.ng + el.y) * a.nlev + lev0 + el.z;
    default: return a.scal + o * a.nscal + el.z;
  }
}

__global__ void k_gather_state(int nret, const RetDesc* d, const int* lev_off, const int4* elems,
                               AtmArrays a, double* xv) {
  const int i = blockIdx.x;
  if (i >= nret) return;
  for (int j = threadIdx.x; j < d[i].n; j += blockDim.x)
    xv[d[i].xo + j] = *elem_ptr(a, lev_off[i], i, elems[d[i].xo + j]);
}

// Current iterate = a-priori copy with the state vector scattered in and
// the clamps of retrieval.c:596-614 applied.  Only retrievals with
// active[i] != 0 are updated.
__global__ void k_set_iterate(int nret, const RetDesc* d, const int* lev_off, const int4* elems,
                              const int* active, AtmArrays apr, AtmArrays cur, const double* xv,
                              int nw, int ncl, int nsf) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  const int l0 = lev_off[i], nl = lev_off[i + 1] - l0;
  const int nplanes = 6 + cur.ng + nw;
  for (int k = 0; k < nplanes; k++)
    for (int l = threadIdx.x; l < nl; l += blockDim.x)
      cur.lev[k * cur.nlev + l0 + l] = apr.lev[k * apr.nlev + l0 + l];
  for (int k = threadIdx.x; k < cur.nscal; k += blockDim.x)
    cur.scal[(long long)i * cur.nscal + k] = apr.scal[(long long)i * apr.nscal + k];
  __syncthreads();
  for (int j = threadIdx.x; j < d[i].n; j += blockDim.x)
    *elem_ptr(cur, l0, i, elems[d[i].xo + j]) = xv[d[i].xo + j];
  __syncthreads();
  for (int l = threadIdx.x; l < nl; l += blockDim.x) {
    double* p = cur.lev + 4 * cur.nlev + l0 + l;
    double* t = cur.lev + 5 * cur.nlev + l0 + l;
    *p = fmin(fmax(*p, 5e-7), 5e4);
    *t = fmin(fmax(*t, 100.0), 400.0);
    for (int g = 0; g < cur.ng; g++) {
      double* q = cur.lev + (6 + g) * cur.nlev + l0 + l;
      *q = fmin(fmax(*q, 0.0), 1.0);
    }
    for (int w = 0; w < nw; w++) {
      double* kk = cur.lev + (6 + cur.ng + w) * cur.nlev + l0 + l;
      *kk = fmax(*kk, 0.0);
    }
  }
  if (threadIdx.x == 0) {
    double* s = cur.scal + (long long)i * cur.nscal;
    s[0] = fmax(s[0], 0.0);
    s[1] = fmax(s[1], 0.1);
    for (int c = 0; c < ncl; c++) s[2 + c] = fmax(s[2 + c], 0.0);
    const int o = 2 + ncl;
    s[o] = fmax(s[o], 0.0);
    s[o + 1] = fmax(s[o + 1], 0.0);
    s[o + 2] = fmin(fmax(s[o + 2], 100.0), 400.0);
    for (int f = 0; f < nsf; f++) s[o + 3 + f] = fmin(fmax(s[o + 3 + f], 0.0), 1.0);
  }
}

// y_i (obs2y order) from the forward-model results of retrieval i.
__global__ void k_gather_y(int nret, const RetDesc* d, const int* ray_off, const int2* ymap,
                           const double* rad, long long nray, double* yv) {
  const int i = blockIdx.x;
  if (i >= nret) return;
  for (int r = threadIdx.x; r < d[i].m; r += blockDim.x) {
    const int2 ym = ymap[d[i].yo + r];
    yv[d[i].yo + r] = rad[(long long)ym.y * nray + ray_off[i] + ym.x];
  }
}

// dx = x - x_a, dy = y_m - y (retrieval.c:537-541, 622-625)
__global__ void k_residuals(int nret, const RetDesc* d, const int* active, const double* xv,
                            const double* xa, const double* ym, const double* yv, double* dx,
                            double* dy) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  for (int j = threadIdx.x; j < d[i].n; j += blockDim.x) dx[d[i].xo + j] = xv[d[i].xo + j] - xa[d[i].xo + j];
  for (int r = threadIdx.x; r < d[i].m; r += blockDim.x) dy[d[i].yo + r] = ym[d[i].yo + r] - yv[d[i].yo + r];
}

// chi^2/m (cost_function, retrieval.c:340-369): serial sums in the
// reference's order, one thread per retrieval.
__global__ void k_cost(int nret, const RetDesc* d, const int* active, const double* dx,
                       const double* dy, const double* sainv, const double* w, double* chisq) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nret || !active[i]) return;
  const RetDesc r = d[i];
  double chim = 0, chia = 0;
  for (int k = 0; k < r.m; k++) {
    const double v = dy[r.yo + k] * w[r.yo + k];
    chim += v * v;
  }
  const double* S = sainv + r.so;
  for (int a = 0; a < r.n; a++) {
    double s = 0;
    for (int b = 0; b < r.n; b++) s += S[(long long)a * r.n + b] * dx[r.xo + b];
    chia += dx[r.xo + a] * s;
  }
  chisq[i] = (chim + chia) / (double)r.m;
}

// b = -S_a^-1 dx + K^T W dy (retrieval.c:573-577)
__global__ void k_gradient(int nret, const RetDesc* d, const int* active, const double* sainv,
                           const double* dx, double* b) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  const RetDesc r = d[i];
  const double* S = sainv + r.so;
  for (int a = threadIdx.x; a < r.n; a += blockDim.x) {
    double s = 0;
    for (int c = 0; c < r.n; c++) s += S[(long long)a * r.n + c] * dx[r.xo + c];
    b[r.xo + a] = -1.0 * s + 1.0 * b[r.xo + a];
  }
}

// A = (1 + lmpar) S_a^-1 + K^T W K (retrieval.c:583-585)
__global__ void k_lm_matrix(int nret, const RetDesc* d, const int* active, const double* lmpar,
                            const double* sainv, const double* cov, double* A) {
  const int i = blockIdx.y;
  if (i >= nret || !active[i]) return;
  const RetDesc r = d[i];
  const long long nn = (long long)r.n * r.n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x)
    A[r.so + e] = sainv[r.so + e] * (1 + lmpar[i]) + cov[r.so + e];
}

// In-place Cholesky factor (lower triangle, mirrored into the upper one),
// one block per retrieval; dot products are serial per entry so the result
// is the textbook column algorithm's.  status[i] = 1 if not positive definite.
__global__ void k_chol_factor(int nret, const RetDesc* d, const int* active, double* Aall,
                              int* status) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  const int n = d[i].n;
  double* A = Aall + d[i].so;
  __shared__ double ljj;
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  for (int j = 0; j < n; j++) {
    if (threadIdx.x == 0) {
      double s = A[(long long)j * n + j];
      for (int k = 0; k < j; k++) s -= A[(long long)j * n + k] * A[(long long)j * n + k];
      if (!(s > 0)) bad = 1;
      ljj = sqrt(s);
      A[(long long)j * n + j] = ljj;
    }
    __syncthreads();
    if (bad) break;
    for (int r = j + 1 + threadIdx.x; r < n; r += blockDim.x) {
      double s = A[(long long)r * n + j];
      for (int k = 0; k < j; k++) s -= A[(long long)r * n + k] * A[(long long)j * n + k];
      A[(long long)r * n + j] = s / ljj;
    }
    __syncthreads();
  }
  if (bad) {
    if (threadIdx.x == 0) status[i] = 1;
    return;
  }
  for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
    const int r = (int)(e / n), c = (int)(e % n);
    if (c > r) A[e] = A[(long long)c * n + r];
  }
}

__device__ void chol_solve_serial(const double* L, int n, const double* b, double* xs,
                                  long long stride) {
  for (int r = 0; r < n; r++) xs[r * stride] = b[r * stride];
  for (int r = 0; r < n; r++) {
    double s = xs[r * stride];
    for (int k = 0; k < r; k++) s -= L[(long long)r * n + k] * xs[k * stride];
    xs[r * stride] = s / L[(long long)r * n + r];
  }
  for (int r = n - 1; r >= 0; r--) {
    double s = xs[r * stride];
    for (int k = r + 1; k < n; k++) s -= L[(long long)k * n + r] * xs[k * stride];
    xs[r * stride] = s / L[(long long)r * n + r];
  }
}

// step = A^-1 b from the factor (retrieval.c:589), one thread per retrieval
__global__ void k_chol_solve(int nret, const RetDesc* d, const int* active, const double* L,
                             const double* b, double* step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nret || !active[i]) return;
  chol_solve_serial(L + d[i].so, d[i].n, b + d[i].xo, step + d[i].xo, 1);
}

// Inverse from the factor: column solves of L L^T X = I, symmetrised
// (matrix_invert, retrieval.c:373-399, non-diagonal branch).
__global__ void k_chol_inverse(int nret, const RetDesc* d, const int* active, const double* L,
                               double* work, double* out) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  const int n = d[i].n;
  double* W = work + d[i].so;
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    // solve for unit vector e_c, stored in column c of W (stride n)
    for (int r = 0; r < n; r++) W[(long long)r * n + c] = (r == c) ? 1.0 : 0.0;
    chol_solve_serial(L + d[i].so, n, W + c, W + c, n);
  }
  __syncthreads();
  for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
    const int r = (int)(e / n), c = (int)(e % n);
    out[d[i].so + e] = 0.5 * (W[(long long)r * n + c] + W[(long long)c * n + r]);
  }
}

__global__ void k_diag_inverse(int nret, const RetDesc* d, const int* active, double* S) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  for (int j = threadIdx.x; j < d[i].n; j += blockDim.x) {
    double* v = S + d[i].so + (long long)j * d[i].n + j;
    *v = 1 / *v;
  }
}

// a-priori covariance (set_cov_apr, retrieval.c:808-920): per element
// sigma, quantity, correlation lengths and location (lon, lat, z).
struct SaElem {
  double sigma, cz, ch, lon, lat, z;
  int iq;
};

__global__ void k_build_sa(int nret, const RetDesc* d, const SaElem* el, double* S) {
  const int i = blockIdx.y;
  if (i >= nret) return;
  const RetDesc r = d[i];
  const long long nn = (long long)r.n * r.n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(e / r.n), b = (int)(e % r.n);
    const SaElem ea = el[r.xo + a], eb = el[r.xo + b];
    double v = 0;
    if (a == b) {
      v = ea.sigma * ea.sigma;
    } else if (ea.iq == eb.iq && ea.cz > 0 && ea.ch > 0) {
      double x0[3], x1[3];
      to_cart(0, ea.lon, ea.lat, x0);
      to_cart(0, eb.lon, eb.lat, x1);
      const double dist = sqrt((x0[0] - x1[0]) * (x0[0] - x1[0]) + (x0[1] - x1[1]) * (x0[1] - x1[1]) +
                               (x0[2] - x1[2]) * (x0[2] - x1[2]));
      const double rho = exp(-dist / ea.ch - fabs(ea.z - eb.z) / ea.cz);
      v = ea.sigma * eb.sigma * rho;
    }
    S[r.so + e] = v;
  }
}

__global__ void k_axpy_state(int nret, const RetDesc* d, const int* active, double sign,
                             const double* step, double* xv) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  for (int j = threadIdx.x; j < d[i].n; j += blockDim.x)
    xv[d[i].xo + j] = sign > 0 ? xv[d[i].xo + j] + step[d[i].xo + j] : xv[d[i].xo + j] - step[d[i].xo + j];
}

__global__ void k_dot_state(int nret, const RetDesc* d, const int* active, const double* a,
                            const double* b, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nret || !active[i]) return;
  double s = 0;
  for (int j = 0; j < d[i].n; j++) s += a[d[i].xo + j] * b[d[i].xo + j];
  out[i] = s;
}

__global__ void k_add(long long n, const double* a, double* b) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) b[e] += a[e];
}

}  // namespace
}  // namespace jgb

using namespace jgb;

extern "C" int jgb_retrieve_batch(jgb_ctx* x, const jgb_ret* ret, const jgb_batch* hb,
                                  double* x_out, double* cov_out, double* costs, int* iters,
                                  int precision) {
  if (!x || !ret || !hb || !x_out || hb->nobs <= 0) return ctx_error(x, JGB_ERR_ARG, "bad arguments");
  if (ret->conv_itmax < 0 || ret->kernel_recomp <= 0) return ctx_error(x, JGB_ERR_ARG, "bad retrieval settings");
  if (hb->nobs > 65535) return ctx_error(x, JGB_ERR_ARG, "at most 65535 retrievals per batch");
  cudaSetDevice(x->device);
  const CtlDev& c = x->c;
  cudaStream_t s = x->stream;
  const int nret = hb->nobs;
  const int nray = hb->ray_off[nret], nlev = hb->lev_off[nret];
  const int nscal = 5 + c.ncl + c.nsf, nplanes = 6 + c.ng + c.nw;
  // ---- layouts (host) ----
  FdLayout H;
  int rc = fd_layout(x, nret, hb->lev_off, hb->ray_off, hb->z, hb->rad, H);
  if (rc) return rc;
  std::vector<RetDesc> desc(nret);
  long long nx = 0, ny = 0, nss = 0, nk = 0;
  for (int i = 0; i < nret; i++) {
    desc[i] = RetDesc{H.ncnt[i], H.mcnt[i], nx, (long long)H.yoff[i], nss, H.kb[i]};
    nx += H.ncnt[i];
    nss += (long long)H.ncnt[i] * H.ncnt[i];
    nk += (long long)H.ncnt[i] * H.mcnt[i];
  }
  ny = (long long)H.ymap.size();
  // measured y and its errors (set_cov_meas, retrieval.c:924-964)
  std::vector<double> ymeas(ny), winv(ny);
  for (int i = 0; i < nret; i++)
    for (int k = 0; k < H.mcnt[i]; k++) {
      const int2 ym = H.ymap[H.yoff[i] + k];
      const double v = hb->rad[(size_t)ym.y * nray + hb->ray_off[i] + ym.x];
      const double sn = ret->err_noise ? ret->err_noise[ym.y] : 0.0;
      const double sf = fabs((ret->err_formod ? ret->err_formod[ym.y] : 0.0) / 100 * v);
      ymeas[H.yoff[i] + k] = v;
      winv[H.yoff[i] + k] = 1 / sqrt(sn * sn + sf * sf);
      if (!(winv[H.yoff[i] + k] > 0))
        return ctx_error(x, JGB_ERR_ARG, "Check measurement errors (zero standard deviation)!");
    }
  // state element tables and a-priori sigmas
  std::vector<int4> elems(nx);
  std::vector<SaElem> sael(nx);
  std::vector<char> sa_diag(nret, 1);
  for (int i = 0; i < nret; i++) {
    const int l0 = hb->lev_off[i];
    for (int j = 0; j < H.ncnt[i]; j++) {
      const Elem& e = H.lay[i][j];
      elems[desc[i].xo + j] = make_int4(e.arr, e.idx, e.arr == 4 ? e.idx : e.lev, e.hkind);
      SaElem se{};
      const double* scal = hb->scal + (size_t)i * nscal;
      double xv = 0;
      switch (e.arr) {
        case 0: xv = hb->p[l0 + e.lev]; break;
        case 1: xv = hb->t[l0 + e.lev]; break;
        case 2: xv = hb->q[(size_t)e.idx * nlev + l0 + e.lev]; break;
        case 3: xv = hb->k[(size_t)e.idx * nlev + l0 + e.lev]; break;
        default: xv = scal[e.idx]; break;
      }
      int iq;
      if (e.arr == 0) { iq = 0; se.sigma = ret->err_press / 100 * xv; se.cz = ret->err_press_cz; se.ch = ret->err_press_ch; }
      else if (e.arr == 1) { iq = 1; se.sigma = ret->err_temp; se.cz = ret->err_temp_cz; se.ch = ret->err_temp_ch; }
      else if (e.arr == 2) { iq = 2 + e.idx; se.sigma = ret->err_q[e.idx] / 100 * xv; se.cz = ret->err_q_cz[e.idx]; se.ch = ret->err_q_ch[e.idx]; }
      else if (e.arr == 3) { iq = 2 + c.ng + e.idx; se.sigma = ret->err_k[e.idx]; se.cz = ret->err_k_cz[e.idx]; se.ch = ret->err_k_ch[e.idx]; }
      else {
        const int o = 2 + c.ncl;
        se.cz = se.ch = 0;
        if (e.idx == 0) { iq = 2 + c.ng + c.nw; se.sigma = ret->err_clz; }
        else if (e.idx == 1) { iq = 3 + c.ng + c.nw; se.sigma = ret->err_cldz; }
        else if (e.idx < o) { iq = 4 + c.ng + c.nw + (e.idx - 2); se.sigma = ret->err_clk[e.idx - 2]; }
        else if (e.idx == o) { iq = 4 + c.ng + c.nw + c.ncl; se.sigma = ret->err_sfz; }
        else if (e.idx == o + 1) { iq = 5 + c.ng + c.nw + c.ncl; se.sigma = ret->err_sfp; }
        else if (e.idx == o + 2) { iq = 6 + c.ng + c.nw + c.ncl; se.sigma = ret->err_sft; }
        else { iq = 7 + c.ng + c.nw + c.ncl + (e.idx - o - 3); se.sigma = ret->err_sfeps[e.idx - o - 3]; }
      }
      if (!(se.sigma * se.sigma > 0))
        return ctx_error(x, JGB_ERR_ARG, "Check a priori data (zero standard deviation)!");
      se.iq = iq;
      const int lv = e.arr == 4 ? 0 : e.lev;
      se.lon = hb->lon[l0 + lv];
      se.lat = hb->lat[l0 + lv];
      se.z = hb->z[l0 + lv];
      sael[desc[i].xo + j] = se;
    }
    // diagonal iff no pair of the same quantity has both correlation lengths > 0
    for (int j = 0; j < H.ncnt[i] && sa_diag[i]; j++) {
      const SaElem& a = sael[desc[i].xo + j];
      if (a.cz > 0 && a.ch > 0)
        for (int k = 0; k < H.ncnt[i]; k++)
          if (k != j && sael[desc[i].xo + k].iq == a.iq) { sa_diag[i] = 0; break; }
    }
  }
  // ---- device buffers ----
  DevBuf mem;
  const size_t dbl = sizeof(double);
  const size_t bytes = dbl * ((size_t)nlev * nplanes * 2 + (size_t)nret * nscal * 2 + 7 * (size_t)nray +
                              (size_t)c.nd * nray * 4 + (size_t)nx * 8 + (size_t)ny * 4 + (size_t)nss * 5 +
                              (size_t)nk + (size_t)nret * 4) +
                       sizeof(int4) * nx + sizeof(SaElem) * nx + sizeof(RetDesc) * nret +
                       sizeof(int) * (4 * (size_t)nret + 4) + sizeof(int2) * ny + normal_desc_bytes(nret) +
                       64 * 256;  // alignment padding of the sub-arrays carved below (< 64 of them)
  RCK(mem.reserve(bytes));
  char* mp = mem.as<char>();
  auto take = [&](size_t nbytes) {
    char* p = mp;
    mp += (nbytes + 255) & ~size_t(255);
    return p;
  };
  double* apr_lev = (double*)take(dbl * (size_t)nlev * nplanes);
  double* cur_lev = (double*)take(dbl * (size_t)nlev * nplanes);
  double* apr_scal = (double*)take(dbl * (size_t)nret * nscal);
  double* cur_scal = (double*)take(dbl * (size_t)nret * nscal);
  double* geo = (double*)take(dbl * 7 * (size_t)nray);
  double* radm = (double*)take(dbl * (size_t)c.nd * nray);
  double* rad = (double*)take(dbl * (size_t)c.nd * nray);
  double* tau = (double*)take(dbl * (size_t)c.nd * nray);
  double* tp = (double*)take(dbl * 3 * (size_t)nray);
  double* xa = (double*)take(dbl * nx);
  double* xi = (double*)take(dbl * nx);
  double* dx = (double*)take(dbl * nx);
  double* bvec = (double*)take(dbl * nx);
  double* step = (double*)take(dbl * nx);
  double* xfin = (double*)take(dbl * nx);
  double* ym_d = (double*)take(dbl * ny);
  double* yi = (double*)take(dbl * ny);
  double* dy = (double*)take(dbl * ny);
  double* w_d = (double*)take(dbl * ny);
  double* sainv = (double*)take(dbl * nss);
  double* cov = (double*)take(dbl * nss);
  double* Amat = (double*)take(dbl * nss);
  double* work = (double*)take(dbl * nss);
  double* Kd = (double*)take(dbl * std::max(nk, 1LL));
  double* chisq_d = (double*)take(dbl * nret);
  double* lmpar_d = (double*)take(dbl * nret);
  double* disq_d = (double*)take(dbl * nret);
  int4* elems_d = (int4*)take(sizeof(int4) * nx);
  SaElem* sael_d = (SaElem*)take(sizeof(SaElem) * nx);
  RetDesc* desc_d = (RetDesc*)take(sizeof(RetDesc) * nret);
  int* active_d = (int*)take(sizeof(int) * nret);
  int* status_d = (int*)take(sizeof(int) * nret);
  int* levoff_d = (int*)take(sizeof(int) * (nret + 1));
  int* rayoff_d = (int*)take(sizeof(int) * (nret + 1));
  int2* ymap_d = (int2*)take(sizeof(int2) * ny);
  void* nedesc_d = take(normal_desc_bytes(nret));
  // upload
  const size_t L = (size_t)nlev * dbl;
  const double* src_lev[6] = {hb->time, hb->z, hb->lon, hb->lat, hb->p, hb->t};
  for (int k = 0; k < 6; k++) RCK(cudaMemcpyAsync(apr_lev + (size_t)k * nlev, src_lev[k], L, cudaMemcpyHostToDevice, s));
  if (c.ng) RCK(cudaMemcpyAsync(apr_lev + 6 * (size_t)nlev, hb->q, L * c.ng, cudaMemcpyHostToDevice, s));
  if (c.nw) RCK(cudaMemcpyAsync(apr_lev + (6 + (size_t)c.ng) * nlev, hb->k, L * c.nw, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(apr_scal, hb->scal, dbl * (size_t)nret * nscal, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(geo, hb->geo, dbl * 7 * (size_t)nray, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(radm, hb->rad, dbl * (size_t)c.nd * nray, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(ym_d, ymeas.data(), dbl * ny, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(w_d, winv.data(), dbl * ny, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(elems_d, elems.data(), sizeof(int4) * nx, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(sael_d, sael.data(), sizeof(SaElem) * nx, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(desc_d, desc.data(), sizeof(RetDesc) * nret, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(levoff_d, hb->lev_off, sizeof(int) * (nret + 1), cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(rayoff_d, hb->ray_off, sizeof(int) * (nret + 1), cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(ymap_d, H.ymap.data(), sizeof(int2) * ny, cudaMemcpyHostToDevice, s));
  RCK(cudaMemcpyAsync(cur_lev, apr_lev, dbl * (size_t)nlev * nplanes, cudaMemcpyDeviceToDevice, s));
  RCK(cudaMemcpyAsync(cur_scal, apr_scal, dbl * (size_t)nret * nscal, cudaMemcpyDeviceToDevice, s));
  RCK(cudaMemsetAsync(status_d, 0, sizeof(int) * nret, s));
  std::vector<int> active(nret, 1), trying(nret, 0), converged(nret, 0);
  std::vector<double> lmpar(nret, 0.001), chisq(nret), chisq_old(nret), disq(nret);
  std::vector<int> niter(nret, 0);
  const int ncost = ret->conv_itmax + 1;
  if (costs)
    for (long long k = 0; k < (long long)nret * ncost; k++) costs[k] = NAN;
  auto put_active = [&](const std::vector<int>& a) {
    return cudaMemcpyAsync(active_d, a.data(), sizeof(int) * nret, cudaMemcpyHostToDevice, s);
  };
  AtmArrays apr{apr_lev, apr_scal, nlev, nscal, c.ng};
  AtmArrays cur{cur_lev, cur_scal, nlev, nscal, c.ng};
  BatchDev bd{};
  bd.nobs = nret;
  bd.nlev = nlev;
  bd.nray = nray;
  bd.nscal = nscal;
  bd.lev_off = levoff_d;
  bd.time = cur_lev;
  bd.z = cur_lev + nlev;
  bd.lon = cur_lev + 2 * (size_t)nlev;
  bd.lat = cur_lev + 3 * (size_t)nlev;
  bd.p = cur_lev + 4 * (size_t)nlev;
  bd.t = cur_lev + 5 * (size_t)nlev;
  bd.q = cur_lev + 6 * (size_t)nlev;
  bd.k = cur_lev + (6 + (size_t)c.ng) * nlev;
  bd.scal = cur_scal;
  bd.geo = geo;
  bd.rad = rad;
  bd.tau = tau;
  bd.tp = tp;
  RCK(x->b_rayobs.reserve(sizeof(int) * nray));
  RCK(x->b_mask.reserve((size_t)c.nd * nray));
  bd.ray_obs = x->b_rayobs.as<int>();
  bd.mask = x->b_mask.as<unsigned char>();
  std::vector<int> cnt(nray);
  // forward model of the current iterates: results in rad, y_i gathered
  auto forward = [&]() -> int {
    RCK(cudaMemcpyAsync(rad, radm, dbl * (size_t)c.nd * nray, cudaMemcpyDeviceToDevice, s));
    launch_ray_obs_mask(nret, rayoff_d, const_cast<int*>(bd.ray_obs), (long long)c.nd * nray, rad,
                        const_cast<unsigned char*>(bd.mask), s);
    const int r2 = run_core(x, bd, precision, false);
    if (r2) return r2;
    k_gather_y<<<nret, 128, 0, s>>>(nret, desc_d, rayoff_d, ymap_d, rad, nray, yi);
    RCK(cudaGetLastError());
    return JGB_OK;
  };
  auto jacobian = [&](const std::vector<int>& list) -> int {
    RCK(cudaMemcpy(cnt.data(), x->los_cnt.p, sizeof(int) * nray, cudaMemcpyDeviceToHost));
    FdInput in{cur_lev, cur_scal, geo, radm, levoff_d, rayoff_d, rad, cnt.data()};
    return fd_core(x, H, in, list, Kd, precision);
  };
  auto normal = [&](const std::vector<int>& a) -> int {
    // cov = K^T W K and bvec = K^T W dy for the listed retrievals (all
    // retrievals are computed; inactive ones are recomputed harmlessly)
    std::vector<int> m(nret), n(nret);
    for (int i = 0; i < nret; i++) {
      m[i] = H.mcnt[i];
      n[i] = H.ncnt[i];
    }
    (void)a;
    return normal_equations_dev(nret, m.data(), n.data(), Kd, w_d, dy, cov, bvec, precision, nedesc_d, s);
  };

  // ---- initialisation (retrieval.c:503-556) ----
  rc = forward();
  if (rc) return rc;
  RCK(put_active(active));
  k_gather_state<<<nret, 128, 0, s>>>(nret, desc_d, levoff_d, elems_d, apr, xa);
  k_gather_state<<<nret, 128, 0, s>>>(nret, desc_d, levoff_d, elems_d, cur, xi);
  {
    dim3 g(64, nret);
    k_build_sa<<<g, 256, 0, s>>>(nret, desc_d, sael_d, sainv);
  }
  std::vector<int> nondiag(nret), diag(nret);
  bool any_nondiag = false;
  for (int i = 0; i < nret; i++) {
    nondiag[i] = !sa_diag[i];
    diag[i] = sa_diag[i];
    any_nondiag |= !sa_diag[i];
  }
  RCK(put_active(diag));
  k_diag_inverse<<<nret, 128, 0, s>>>(nret, desc_d, active_d, sainv);
  if (any_nondiag) {
    RCK(put_active(nondiag));
    RCK(cudaMemcpyAsync(work, sainv, dbl * nss, cudaMemcpyDeviceToDevice, s));
    k_chol_factor<<<nret, 256, 0, s>>>(nret, desc_d, active_d, work, status_d);
    k_chol_inverse<<<nret, 128, 0, s>>>(nret, desc_d, active_d, work, Amat, sainv);
  }
  RCK(put_active(active));
  k_residuals<<<nret, 128, 0, s>>>(nret, desc_d, active_d, xi, xa, ym_d, yi, dx, dy);
  k_cost<<<(nret + 63) / 64, 64, 0, s>>>(nret, desc_d, active_d, dx, dy, sainv, w_d, chisq_d);
  RCK(cudaMemcpyAsync(chisq.data(), chisq_d, dbl * nret, cudaMemcpyDeviceToHost, s));
  RCK(cudaStreamSynchronize(s));
  for (int i = 0; i < nret; i++)
    if (costs) costs[(size_t)i * ncost] = chisq[i];
  {
    std::vector<int> all(nret);
    for (int i = 0; i < nret; i++) all[i] = i;
    rc = jacobian(all);
    if (rc) return rc;
  }
  // ---- Levenberg-Marquardt (retrieval.c:559-652) ----
  for (int it = 1; it <= ret->conv_itmax; it++) {
    std::vector<int> act;
    for (int i = 0; i < nret; i++)
      if (active[i]) act.push_back(i);
    if (act.empty()) break;
    chisq_old = chisq;
    if (it > 1 && it % ret->kernel_recomp == 0) {
      rc = jacobian(act);
      if (rc) return rc;
    }
    RCK(put_active(active));
    if (it == 1 || it % ret->kernel_recomp == 0) {
      rc = normal(active);
      if (rc) return rc;
    } else {
      // b needs K^T W dy with the current dy even when cov is kept
      RCK(cudaMemcpyAsync(work, cov, dbl * nss, cudaMemcpyDeviceToDevice, s));
      rc = normal(active);
      if (rc) return rc;
      RCK(cudaMemcpyAsync(cov, work, dbl * nss, cudaMemcpyDeviceToDevice, s));
    }
    k_gradient<<<nret, 128, 0, s>>>(nret, desc_d, active_d, sainv, dx, bvec);
    trying = active;
    for (int it2 = 0; it2 < 20; it2++) {
      bool any = false;
      for (int i = 0; i < nret; i++) any |= trying[i] != 0;
      if (!any) break;
      RCK(put_active(trying));
      RCK(cudaMemcpyAsync(lmpar_d, lmpar.data(), dbl * nret, cudaMemcpyHostToDevice, s));
      {
        dim3 g(64, nret);
        k_lm_matrix<<<g, 256, 0, s>>>(nret, desc_d, active_d, lmpar_d, sainv, cov, Amat);
      }
      k_chol_factor<<<nret, 256, 0, s>>>(nret, desc_d, active_d, Amat, status_d);
      k_chol_solve<<<(nret + 63) / 64, 64, 0, s>>>(nret, desc_d, active_d, Amat, bvec, step);
      k_axpy_state<<<nret, 128, 0, s>>>(nret, desc_d, active_d, +1.0, step, xi);
      k_set_iterate<<<nret, 256, 0, s>>>(nret, desc_d, levoff_d, elems_d, active_d, apr, cur, xi,
                                          c.nw, c.ncl, c.nsf);
      rc = forward();
      if (rc) return rc;
      k_residuals<<<nret, 128, 0, s>>>(nret, desc_d, active_d, xi, xa, ym_d, yi, dx, dy);
      k_cost<<<(nret + 63) / 64, 64, 0, s>>>(nret, desc_d, active_d, dx, dy, sainv, w_d, chisq_d);
      std::vector<double> cnew(nret);
      std::vector<int> st(nret);
      RCK(cudaMemcpyAsync(cnew.data(), chisq_d, dbl * nret, cudaMemcpyDeviceToHost, s));
      RCK(cudaMemcpyAsync(st.data(), status_d, sizeof(int) * nret, cudaMemcpyDeviceToHost, s));
      RCK(cudaStreamSynchronize(s));
      std::vector<int> reject(nret, 0);
      for (int i = 0; i < nret; i++) {
        if (!trying[i]) continue;
        if (st[i]) return ctx_error(x, JGB_ERR_NUMERIC, "normal matrix is not positive definite");
        chisq[i] = cnew[i];
        if (chisq[i] > chisq_old[i]) {
          lmpar[i] *= 10;
          reject[i] = 1;
        } else {
          lmpar[i] /= 10;
          trying[i] = 0;
        }
      }
      RCK(put_active(reject));
      k_axpy_state<<<nret, 128, 0, s>>>(nret, desc_d, active_d, -1.0, step, xi);
      for (int i = 0; i < nret; i++)
        if (!reject[i]) trying[i] = 0;
    }
    RCK(put_active(active));
    k_dot_state<<<(nret + 63) / 64, 64, 0, s>>>(nret, desc_d, active_d, step, bvec, disq_d);
    RCK(cudaMemcpyAsync(disq.data(), disq_d, dbl * nret, cudaMemcpyDeviceToHost, s));
    RCK(cudaStreamSynchronize(s));
    for (int i : act) {
      if (costs) costs[(size_t)i * ncost + it] = chisq[i];
      niter[i] = it;
      const double dq = disq[i] / (double)H.ncnt[i];
      if ((it == 1 || it % ret->kernel_recomp == 0) && dq < ret->conv_dmin) active[i] = 0;
    }
  }
  // ---- results (retrieval.c:658-661, 668-684) ----
  std::vector<int> all(nret, 1);
  RCK(put_active(all));
  k_gather_state<<<nret, 128, 0, s>>>(nret, desc_d, levoff_d, elems_d, cur, xfin);
  RCK(cudaMemcpyAsync(x_out, xfin, dbl * nx, cudaMemcpyDeviceToHost, s));
  RCK(cudaMemcpyAsync(hb->rad, rad, dbl * (size_t)c.nd * nray, cudaMemcpyDeviceToHost, s));
  RCK(cudaMemcpyAsync(hb->tau, tau, dbl * (size_t)c.nd * nray, cudaMemcpyDeviceToHost, s));
  RCK(cudaMemcpyAsync(hb->tp, tp, dbl * 3 * (size_t)nray, cudaMemcpyDeviceToHost, s));
  RCK(cudaMemcpyAsync(hb->p, cur_lev + 4 * (size_t)nlev, L, cudaMemcpyDeviceToHost, s));
  if (ret->err_ana && cov_out) {
    rc = normal(all);
    if (rc) return rc;
    k_add<<<(unsigned)((nss + 255) / 256), 256, 0, s>>>(nss, sainv, cov);
    k_chol_factor<<<nret, 256, 0, s>>>(nret, desc_d, active_d, cov, status_d);
    k_chol_inverse<<<nret, 128, 0, s>>>(nret, desc_d, active_d, cov, work, Amat);
    RCK(cudaMemcpyAsync(cov_out, Amat, dbl * nss, cudaMemcpyDeviceToHost, s));
  }
  RCK(cudaStreamSynchronize(s));
  if (iters)
    for (int i = 0; i < nret; i++) iters[i] = niter[i];
  return JGB_OK;
}
