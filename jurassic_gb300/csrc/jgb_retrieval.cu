// Optimal-estimation retrieval on the device (optimal_estimation,
// retrieval.c:448-749), batched over independent retrievals and served by a
// continuous-batching engine (see the engine section below).
//
// Every retrieval keeps its own Levenberg-Marquardt state (iteration count,
// damping parameter, inner-loop trials, convergence).  Per iteration:
// finite-difference Jacobian (fd_core, one batched forward-model launch
// sequence for every perturbation of every retrieval that needs it),
// normal-equation products (3xTF32 tensor cores or FP64), then up to 20
// damped steps, each an FP64 Cholesky solve plus one forward model of the
// retrievals still trying.  FP64 is used for the a-priori covariance and its
// inverse, the Cholesky solves, the cost function, the convergence test and
// the error analysis (retrieval.c:668-726).
//
// This translation unit is compiled without FMA contraction: the FP64 linear
// algebra follows the textbook loop orders of the reference's helpers
// (cost_function retrieval.c:340-369, matrix_invert 373-399, Cholesky
// decomposition/solution as used at 588-589, matrix_product 403-444).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
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

// sum over the 32 lanes of a warp (butterfly: every lane gets the same sum)
__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

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
                               const int* active, AtmArrays a, double* xv) {
  const int i = blockIdx.x;
  if (i >= nret || (active && !active[i])) return;
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
                           const int* active, const double* rad, long long nray, double* yv) {
  const int i = blockIdx.x;
  if (i >= nret || (active && !active[i])) return;
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

// chi^2/m (cost_function, retrieval.c:340-369), one block per retrieval:
// chi_m = sum_k (w_k dy_k)^2 and chi_a = sum_a dx_a (S_a^-1 dx)_a, a warp per
// row of S_a^-1 (lanes along the row) and per stretch of dy, the partial
// sums combined in a fixed order (deterministic).
__global__ void k_cost(int nret, const RetDesc* d, const int* active, const double* dx,
                       const double* dy, const double* sainv, const double* w, double* chisq) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  const RetDesc r = d[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  __shared__ double part_m[32], part_a[32];
  double pm = 0, pa = 0;
  for (int k = threadIdx.x; k < r.m; k += blockDim.x) {
    const double v = dy[r.yo + k] * w[r.yo + k];
    pm += v * v;
  }
  pm = warp_sum_d(pm);
  const double* S = sainv + r.so;
  for (int a = warp; a < r.n; a += nwarp) {
    double s = 0;
    for (int b = lane; b < r.n; b += 32) s += S[(long long)a * r.n + b] * dx[r.xo + b];
    s = warp_sum_d(s);
    pa += dx[r.xo + a] * s;
  }
  if (lane == 0) {
    part_m[warp] = pm;
    part_a[warp] = pa;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double chim = 0, chia = 0;
    for (int k = 0; k < nwarp; k++) {
      chim += part_m[k];
      chia += part_a[k];
    }
    chisq[i] = (chim + chia) / (double)r.m;
  }
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

// In-place Cholesky factor (lower triangle, mirrored into the upper one;
// gsl_linalg_cholesky_decomp of matrix_invert / the LM step, retrieval.c:
// 373-399, 588-589), one block per retrieval.  Column j: warp 0 forms the
// diagonal L_jj = sqrt(A_jj - sum_k L_jk^2), then every warp takes rows
// r > j in turn, L_rj = (A_rj - sum_k L_rk L_jk) / L_jj, the 32 lanes of a
// warp summing over k < j along the two rows (coalesced) and reducing by
// shuffles.  status[i] = 1 if not positive definite.
__global__ void k_chol_factor(int nret, const RetDesc* d, const int* active, double* Aall,
                              int* status) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  const int n = d[i].n;
  double* A = Aall + d[i].so;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  __shared__ double ljj;
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < n; j++) {
    const double* Aj = A + (long long)j * n;
    if (warp == 0) {
      double s = 0;
      for (int k = lane; k < j; k += 32) s += Aj[k] * Aj[k];
      s = warp_sum_d(s);
      if (lane == 0) {
        const double dj = Aj[j] - s;
        if (!(dj > 0)) bad = 1;
        ljj = sqrt(dj);
        A[(long long)j * n + j] = ljj;
      }
    }
    __syncthreads();
    if (bad) break;
    const double lj = ljj;
    for (int r = j + 1 + warp; r < n; r += nwarp) {
      const double* Ar = A + (long long)r * n;
      double s = 0;
      for (int k = lane; k < j; k += 32) s += Ar[k] * Aj[k];
      s = warp_sum_d(s);
      if (lane == 0) A[(long long)r * n + j] = (Ar[j] - s) / lj;
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

// L L^T x = e_c (column c of the identity) in place in xs (stride apart).
// The forward sweep's entries above c are exactly +0 (1 or 0 minus products
// with zeros), so the sweep starts at row c and its sums at column c: the
// same values as the full sweep, a third of its work.
__device__ void chol_solve_unit(const double* L, int n, int c, double* xs, long long stride) {
  for (int r = 0; r < n; r++) xs[r * stride] = r == c ? 1.0 : 0.0;
  for (int r = c; r < n; r++) {
    double s = xs[r * stride];
    for (int k = c; k < r; k++) s -= L[(long long)r * n + k] * xs[k * stride];
    xs[r * stride] = s / L[(long long)r * n + r];
  }
  for (int r = n - 1; r >= 0; r--) {
    double s = xs[r * stride];
    for (int k = r + 1; k < n; k++) s -= L[(long long)k * n + r] * xs[k * stride];
    xs[r * stride] = s / L[(long long)r * n + r];
  }
}

// step = A^-1 b from the factor (gsl_linalg_cholesky_solve, retrieval.c:
// 589), one block per retrieval, the vector in shared memory (n doubles).
// Forward L y = b by column sweeps: once y_r is final, every thread
// subtracts L_kr y_r from its rows k > r, so each row sees its subtractions
// in the serial order.  Backward L^T x = y the same way from the last row.
// L's upper triangle holds L^T (k_chol_factor mirrors it), so both sweeps
// read rows of the matrix, coalesced.
__global__ void k_chol_solve(int nret, const RetDesc* d, const int* active, const double* L,
                             const double* b, double* step) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  const int n = d[i].n;
  const double* Li = L + d[i].so;
  extern __shared__ double xs[];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int r = tid; r < n; r += nt) xs[r] = b[d[i].xo + r];
  __syncthreads();
  for (int r = 0; r < n; r++) {
    const double* row = Li + (long long)r * n;   // row r: L_rk for k < r, L_kr for k > r
    const double yr = xs[r] / row[r];
    for (int k = r + 1 + tid; k < n; k += nt) xs[k] -= row[k] * yr;
    __syncthreads();
    if (tid == 0) xs[r] = yr;
    __syncthreads();
  }
  for (int r = n - 1; r >= 0; r--) {
    const double* row = Li + (long long)r * n;
    const double xr = xs[r] / row[r];
    for (int k = tid; k < r; k += nt) xs[k] -= row[k] * xr;
    __syncthreads();
    if (tid == 0) xs[r] = xr;
    __syncthreads();
  }
  for (int r = tid; r < n; r += nt) step[d[i].xo + r] = xs[r];
}

// Inverse from the factor: column solves of L L^T X = I, symmetrised
// (matrix_invert, retrieval.c:373-399, non-diagonal branch).  The column
// solves are independent: thread c of the block (blockIdx.x, i) solves for
// column blockIdx.x * blockDim.x + c (its loads of X run along rows across
// the threads, L is read by all threads alike), so a retrieval's columns
// spread over several blocks; k_sym_half then forms (X + X^T) / 2.
__global__ void k_chol_inverse_cols(int nret, const RetDesc* d, const int* active,
                                    const double* L, double* work) {
  const int i = blockIdx.y;
  if (i >= nret || !active[i]) return;
  const int n = d[i].n;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  chol_solve_unit(L + d[i].so, n, c, work + d[i].so + c, n);
}

__global__ void k_sym_half(int nret, const RetDesc* d, const int* active, const double* work,
                           double* out) {
  const int i = blockIdx.y;
  if (i >= nret || !active[i]) return;
  const int n = d[i].n;
  const double* W = work + d[i].so;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < (long long)n * n;
       e += (long long)gridDim.x * blockDim.x) {
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

// The diagonal test of matrix_invert (retrieval.c:379-385: any element right
// of the diagonal other than 0, NaN included, makes the matrix full):
// diag[i] / full[i] select the two branches, status[i] starts at 0.
__global__ void k_invert_flags(int nret, const RetDesc* d, const double* A, int* diag, int* full,
                               int* status) {
  const int i = blockIdx.x;
  if (i >= nret) return;
  const int n = d[i].n;
  const double* M = A + d[i].so;
  int nz = 0;
  for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
    const int r = (int)(e / n), c = (int)(e % n);
    if (c > r && M[e] != 0) nz = 1;
  }
  nz = __syncthreads_or(nz);
  if (threadIdx.x == 0) {
    diag[i] = !nz;
    full[i] = nz;
    status[i] = 0;
  }
}

// Matrices whose factor failed (status 1) take no inverse: they keep their
// input.
__global__ void k_drop_failed(int nret, const int* status, int* full) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nret && status[i]) full[i] = 0;
}

// a-priori covariance (set_cov_apr, retrieval.c:808-920): per element
// sigma, quantity, correlation lengths and location (lon, lat, z).
struct SaElem {
  double sigma, cz, ch, lon, lat, z;
  int iq;
};

__global__ void k_build_sa(int nret, const RetDesc* d, const int* active, const SaElem* el,
                           double* S) {
  const int i = blockIdx.y;
  if (i >= nret || (active && !active[i])) return;
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

__global__ void k_dot_state(int nret, const RetDesc* d, const int* active, const double* a,
                            const double* b, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nret || !active[i]) return;
  double s = 0;
  for (int j = 0; j < d[i].n; j++) s += a[d[i].xo + j] * b[d[i].xo + j];
  out[i] = s;
}

}  // namespace
}  // namespace jgb


// ===========================================================================
// Retrieval engine: continuous batching of independent retrievals.
//
// Requests (one observation each) wait in a queue and are admitted while the
// number of active requests and the device memory of their working set stay
// within the engine's limits.  The working set is one contiguous allocation
// holding, for every active request, its a-priori and current atmosphere,
// geometry, measurement, forward model, state vectors, S_a^-1, K, K^T W K
// and the LM scratch.  When requests leave or join, a new working set is
// built in a second allocation and the iterate state of the requests that
// stay is moved there on the device (segment copies), so no request's state
// goes back to the host between its iterations.
//
// One engine step = admission, the initialisation (a-priori forward model,
// S_a^-1, cost, first Jacobian) of newly admitted requests, then one
// Levenberg-Marquardt iteration of every initialised request, each at its
// own iteration count, damping parameter and kernel-recomputation phase.
// Forward models run on the whole working set with the requests that are
// not part of the current sub-step flagged off (no LOS, outputs untouched),
// so every request sees exactly the arithmetic it would see alone.

namespace jgb {
namespace {

// Segment copies: seg[3k] source, seg[3k+1] destination (device addresses),
// seg[3k+2] length in doubles.  blockIdx.y strides over segments.
__global__ void k_copy_segments(int nseg, const unsigned long long* seg) {
  for (int k = blockIdx.y; k < nseg; k += gridDim.y) {
    const double* src = reinterpret_cast<const double*>(seg[3 * k]);
    double* dst = reinterpret_cast<double*>(seg[3 * k + 1]);
    const long long nw = (long long)seg[3 * k + 2];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nw;
         i += (long long)gridDim.x * blockDim.x)
      dst[i] = src[i];
  }
}

// Damped-trial candidates of one request, k = 0..count-1 at cand first+k:
// the iterate of candidate k is what the sequential loop (retrieval.c:
// 580-633) would form at trial k after k rejections: x_k = b_k + s_k with
// b_0 = x and b_{k+1} = x_k - s_k (the rejected step taken back), in the
// same floating-point operations.  xrest receives b_{k+1}.
__global__ void k_spec_chain(int nreq, const int* first, const int* count, const RetDesc* d,
                             double* xi, const double* step, double* xrest) {
  const int r = blockIdx.x;
  if (r >= nreq) return;
  const int c0 = first[r], K = count[r], n = d[c0].n;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double base = xi[d[c0].xo + j];
    for (int k = 0; k < K; k++) {
      const long long o = d[c0 + k].xo + j;
      const double v = base + step[o];
      xi[o] = v;
      base = v - step[o];
      xrest[o] = base;
    }
  }
}

// LOS point counts of the rays that were traced (skip flag clear).
__global__ void k_keep_counts(int nray, const int* ray_obs, const unsigned char* skip,
                              const int* src, int* dst) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < nray && !skip[ray_obs[r]]) dst[r] = src[r];
}

// dst = src on the n x n blocks of the selected retrievals.
__global__ void k_select_nn(int nret, const RetDesc* d, const int* sel, const double* src,
                            double* dst) {
  const int i = blockIdx.y;
  if (i >= nret || !sel[i]) return;
  const long long nn = (long long)d[i].n * d[i].n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x)
    dst[d[i].so + e] = src[d[i].so + e];
}

// b += a on the n x n blocks (gsl_matrix_add(cov, s_a_inv), retrieval.c:673)
__global__ void k_add_nn(int nret, const RetDesc* d, const int* active, const double* a,
                         double* b) {
  const int i = blockIdx.y;
  if (i >= nret || !active[i]) return;
  const long long nn = (long long)d[i].n * d[i].n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x)
    b[d[i].so + e] = b[d[i].so + e] + a[d[i].so + e];
}

// Gain G = cov K^T diag(w^2), n x m at offset ko (retrieval.c:694-701).
__global__ void k_gain(int nret, const RetDesc* d, const int* active, const double* cov,
                       const double* K, const double* w, double* G) {
  const int i = blockIdx.y;
  if (i >= nret || !active[i]) return;
  const RetDesc r = d[i];
  const double* C = cov + r.so;
  const double* Ki = K + r.ko;
  const long long nm = (long long)r.n * r.m;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nm;
       e += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(e / r.m), j = (int)(e % r.m);
    const double wj = w[r.yo + j];
    double s = 0;
    for (int b = 0; b < r.n; b++) s += C[(long long)a * r.n + b] * (Ki[(long long)j * r.n + b] * (wj * wj));
    G[r.ko + e] = s;
  }
}

// sqrt(diag(G diag(sig^2) G^T)): error propagation of noise or forward-model
// errors (matrix_product(gain, sig, 2, a) + write_stddev, retrieval.c:705-711).
__global__ void k_err_diag(int nret, const RetDesc* d, const int* active, const double* G,
                           const double* sig, double* out) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  const RetDesc r = d[i];
  for (int a = threadIdx.x; a < r.n; a += blockDim.x) {
    double s = 0;
    for (int j = 0; j < r.m; j++) {
      const double v = G[r.ko + (long long)a * r.m + j] * sig[r.yo + j];
      s += v * v;
    }
    out[r.xo + a] = sqrt(s);
  }
}

__global__ void k_sqrt_diag(int nret, const RetDesc* d, const int* active, const double* S,
                            double* out) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  for (int a = threadIdx.x; a < d[i].n; a += blockDim.x)
    out[d[i].xo + a] = sqrt(S[d[i].so + (long long)a * d[i].n + a]);
}

// Averaging kernel A = G K, n x n (retrieval.c:714-715).
__global__ void k_avk(int nret, const RetDesc* d, const int* active, const double* G,
                      const double* K, double* A) {
  const int i = blockIdx.y;
  if (i >= nret || !active[i]) return;
  const RetDesc r = d[i];
  const long long nn = (long long)r.n * r.n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nn;
       e += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(e / r.n), b = (int)(e % r.n);
    double s = 0;
    for (int j = 0; j < r.m; j++) s += G[r.ko + (long long)a * r.m + j] * K[r.ko + (long long)j * r.n + b];
    A[r.so + e] = s;
  }
}

// analyze_avk (retrieval.c:257-336): per state element, the row sum of the
// averaging kernel over the elements of the same quantity (added to the
// value copy_atm(..., init=1) leaves there: 1 for surface emissivities,
// else 0) and the inverse diagonal.
__global__ void k_avk_analyze(int nret, const RetDesc* d, const int* active, const double* A,
                              const SaElem* el, int iq_sfeps, double* cont, double* res) {
  const int i = blockIdx.x;
  if (i >= nret || !active[i]) return;
  const RetDesc r = d[i];
  for (int a = threadIdx.x; a < r.n; a += blockDim.x) {
    const int iq = el[r.xo + a].iq;
    int n0 = -1, n1 = 0;
    for (int j = 0; j < r.n; j++)
      if (el[r.xo + j].iq == iq) {
        if (n0 < 0) n0 = j;
        n1 = j - n0 + 1;
      }
    double s = iq >= iq_sfeps ? 1.0 : 0.0;
    for (int j = 0; j < n1; j++) s += A[r.so + (long long)a * r.n + n0 + j];
    cont[r.xo + a] = s;
    res[r.xo + a] = 1 / A[r.so + (long long)a * r.n + a];
  }
}

// One retrieval request: its inputs, host-side LM scalars and results.
struct Request {
  unsigned long long id = 0;
  int np = 0, nr = 0, n = 0, m = 0;
  std::vector<double> lev;    // [6+ng+nw][np]: time z lon lat p t q[] k[]
  std::vector<double> scal;   // [nscal]
  std::vector<double> geo;    // [7][nr]
  std::vector<double> rad;    // [nd][nr] measurement, NaN = channel not used
  std::vector<Elem> lay;      // state layout (atm2x order)
  std::vector<int2> ymap;     // (ray, channel) of each measurement element
  std::vector<int4> elems;    // device form of lay
  std::vector<SaElem> sael;   // a-priori sigma, correlation lengths, location
  std::vector<double> ymeas, winv, sn, sf;  // y_m, 1/sigma_eps, noise, formod errors
  bool sa_diag = true;
  size_t bytes = 0;           // working-set bytes of this request
  int slot = -1;              // index in the current working set
  int state = 0;              // 0 waiting for initialisation, 1 iterating, 2 finished
  int it = 0;                 // LM iterations done
  double lmpar = 0.001, chisq = 0, chisq_old = 0;
  int status = JGB_OK;
  std::vector<double> costs;
  // results
  std::vector<double> x, cov, avk, gain, err_total, err_noise, err_formod, cont, res;
  std::vector<double> rad_out, tau_out, tp_out, p_out;
};

// Contiguous device working set of the active requests.
struct WorkSet {
  int nret = 0;
  long long nlev = 0, nray = 0, nx = 0, ny = 0, nss = 0, nk = 0;
  FdLayout H;
  std::vector<RetDesc> desc;
  std::vector<int> mvec, nvec;
  DevBuf mem;
  double *apr_lev = nullptr, *cur_lev = nullptr, *apr_scal = nullptr, *cur_scal = nullptr;
  double *geo = nullptr, *radm = nullptr, *rad = nullptr, *tau = nullptr, *tp = nullptr;
  double *xa = nullptr, *xi = nullptr, *dx = nullptr, *bvec = nullptr, *step = nullptr, *xfin = nullptr;
  double *e_tot = nullptr, *e_noise = nullptr, *e_formod = nullptr, *cont = nullptr, *res = nullptr;
  double *ym = nullptr, *yi = nullptr, *dy = nullptr, *w = nullptr, *sn = nullptr, *sf = nullptr;
  double *sainv = nullptr, *cov = nullptr, *covn = nullptr, *Amat = nullptr, *work = nullptr;
  double *Kd = nullptr, *G = nullptr;
  double *chisq = nullptr, *lmpar = nullptr, *disq = nullptr;
  int4* elems = nullptr;
  SaElem* sael = nullptr;
  RetDesc* desc_d = nullptr;
  int *active = nullptr, *status = nullptr, *levoff = nullptr, *rayoff = nullptr;
  int *rayobs = nullptr, *cnt = nullptr;
  unsigned char *skip = nullptr, *mask = nullptr;
  int2* ymap = nullptr;
  void* nedesc = nullptr;
};

// Device bytes of a working set with these totals (the carving below).
size_t workset_bytes(const CtlDev& c, long long nret, long long nlev, long long nray, long long nx,
                     long long ny, long long nss, long long nk, bool err_ana) {
  const long long nscal = 5 + c.ncl + c.nsf, nplanes = 6 + c.ng + c.nw;
  const size_t dbl = sizeof(double);
  return dbl * (size_t)(nlev * nplanes * 2 + nret * nscal * 2 + 7 * nray + c.nd * nray * 3 +
                        3 * nray + nx * 11 + ny * 6 + nss * 5 + nk * (err_ana ? 2 : 1) + nret * 3) +
         sizeof(int4) * nx + sizeof(SaElem) * nx + sizeof(RetDesc) * nret +
         sizeof(int) * (4 * nret + 2 + 2 * nray) + (size_t)nret + (size_t)c.nd * nray +
         sizeof(int2) * ny + normal_desc_bytes((int)nret) + 64 * 256;
}

}  // namespace
}  // namespace jgb

struct jgb_engine {
  jgb_ctx* x = nullptr;
  int precision = JGB_FP64;
  unsigned long long budget = 0;
  int max_active = 0;
  int keep_gain = 0;
  jgb_ret ret{};
  std::vector<double> v_formod, v_noise, v_q, v_qcz, v_qch, v_k, v_kcz, v_kch, v_clk, v_sfeps;
  unsigned long long next_id = 1;
  std::deque<jgb::Request*> queue;
  std::vector<jgb::Request*> active;
  std::map<unsigned long long, jgb::Request*> done;
  jgb::WorkSet ws[2];
  jgb::WorkSet cw;              // damped-trial candidates of one round
  jgb::DevBuf chainbuf;
  int cur = 0;
  bool have_ws = false, dirty = true;
  unsigned long long used = 0;
  jgb::DevBuf segbuf, stage;
  double* pinned = nullptr;
  size_t pinned_n = 0;
  jgb_engine_stats st{};
  ~jgb_engine() {
    for (jgb::Request* r : queue) delete r;
    for (jgb::Request* r : active) delete r;
    for (auto& kv : done) delete kv.second;
    if (pinned) cudaFreeHost(pinned);
  }
};

using namespace jgb;

namespace {

#define ECK(call)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return ctx_error(E->x, JGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Host-side checks and tables of one request (set_cov_apr, set_cov_meas,
// retrieval.c:808-964; errors as the reference reports them).
int prepare_request(jgb_engine* E, Request* q) {
  jgb_ctx* x = E->x;
  const CtlDev& c = x->c;
  const jgb_ret* ret = &E->ret;
  FdLayout H;
  const int lev_off[2] = {0, q->np}, ray_off[2] = {0, q->nr};
  int rc = fd_layout(x, 1, lev_off, ray_off, q->lev.data() + q->np, q->rad.data(), H);
  if (rc) return rc;
  q->lay = H.lay[0];
  q->ymap = H.ymap;
  q->n = H.ncnt[0];
  q->m = H.mcnt[0];
  q->ymeas.resize(q->m);
  q->winv.resize(q->m);
  q->sn.resize(q->m);
  q->sf.resize(q->m);
  for (int k = 0; k < q->m; k++) {
    const int2 ym = q->ymap[k];
    const double v = q->rad[(size_t)ym.y * q->nr + ym.x];
    const double sn = ret->err_noise ? ret->err_noise[ym.y] : 0.0;
    const double sf = fabs((ret->err_formod ? ret->err_formod[ym.y] : 0.0) / 100 * v);
    q->ymeas[k] = v;
    q->sn[k] = sn;
    q->sf[k] = sf;
    q->winv[k] = 1 / sqrt(sn * sn + sf * sf);
    if (!(q->winv[k] > 0))
      return ctx_error(x, JGB_ERR_ARG, "Check measurement errors (zero standard deviation)!");
  }
  q->elems.resize(q->n);
  q->sael.resize(q->n);
  const double* L = q->lev.data();
  const size_t np = q->np;
  for (int j = 0; j < q->n; j++) {
    const Elem& e = q->lay[j];
    q->elems[j] = make_int4(e.arr, e.idx, e.arr == 4 ? e.idx : e.lev, e.hkind);
    SaElem se{};
    double xv;
    switch (e.arr) {
      case 0: xv = L[4 * np + e.lev]; break;
      case 1: xv = L[5 * np + e.lev]; break;
      case 2: xv = L[(6 + (size_t)e.idx) * np + e.lev]; break;
      case 3: xv = L[(6 + (size_t)c.ng + e.idx) * np + e.lev]; break;
      default: xv = q->scal[e.idx]; break;
    }
    if (e.arr == 0) { se.iq = 0; se.sigma = ret->err_press / 100 * xv; se.cz = ret->err_press_cz; se.ch = ret->err_press_ch; }
    else if (e.arr == 1) { se.iq = 1; se.sigma = ret->err_temp; se.cz = ret->err_temp_cz; se.ch = ret->err_temp_ch; }
    else if (e.arr == 2) { se.iq = 2 + e.idx; se.sigma = ret->err_q[e.idx] / 100 * xv; se.cz = ret->err_q_cz[e.idx]; se.ch = ret->err_q_ch[e.idx]; }
    else if (e.arr == 3) { se.iq = 2 + c.ng + e.idx; se.sigma = ret->err_k[e.idx]; se.cz = ret->err_k_cz[e.idx]; se.ch = ret->err_k_ch[e.idx]; }
    else {
      const int o = 2 + c.ncl;
      se.cz = se.ch = 0;
      if (e.idx == 0) { se.iq = 2 + c.ng + c.nw; se.sigma = ret->err_clz; }
      else if (e.idx == 1) { se.iq = 3 + c.ng + c.nw; se.sigma = ret->err_cldz; }
      else if (e.idx < o) { se.iq = 4 + c.ng + c.nw + (e.idx - 2); se.sigma = ret->err_clk[e.idx - 2]; }
      else if (e.idx == o) { se.iq = 4 + c.ng + c.nw + c.ncl; se.sigma = ret->err_sfz; }
      else if (e.idx == o + 1) { se.iq = 5 + c.ng + c.nw + c.ncl; se.sigma = ret->err_sfp; }
      else if (e.idx == o + 2) { se.iq = 6 + c.ng + c.nw + c.ncl; se.sigma = ret->err_sft; }
      else { se.iq = 7 + c.ng + c.nw + c.ncl + (e.idx - o - 3); se.sigma = ret->err_sfeps[e.idx - o - 3]; }
    }
    if (!(se.sigma * se.sigma > 0))
      return ctx_error(x, JGB_ERR_ARG, "Check a priori data (zero standard deviation)!");
    const int lv = e.arr == 4 ? 0 : e.lev;
    se.lon = L[2 * np + lv];
    se.lat = L[3 * np + lv];
    se.z = L[1 * np + lv];
    q->sael[j] = se;
  }
  // S_a is diagonal unless two elements of one quantity correlate (retrieval.c:901)
  q->sa_diag = true;
  for (int j = 0; j < q->n && q->sa_diag; j++) {
    const SaElem& a = q->sael[j];
    if (a.cz > 0 && a.ch > 0)
      for (int k = 0; k < q->n; k++)
        if (k != j && q->sael[k].iq == a.iq) {
          q->sa_diag = false;
          break;
        }
  }
  const long long n = q->n, m = q->m;
  q->bytes = workset_bytes(c, 1, q->np, q->nr, n, m, n * n, n * m, E->ret.err_ana != 0);
  q->costs.assign(E->ret.conv_itmax + 1, NAN);
  return JGB_OK;
}

// Grow-only pinned staging buffer for results.
int ensure_pinned(jgb_engine* E, size_t words) {
  if (words <= E->pinned_n) return JGB_OK;
  if (E->pinned) cudaFreeHost(E->pinned);
  E->pinned = nullptr;
  E->pinned_n = 0;
  const size_t want = words + words / 4 + 1024;
  ECK(cudaMallocHost(reinterpret_cast<void**>(&E->pinned), want * sizeof(double)));
  E->pinned_n = want;
  return JGB_OK;
}

// Run segment copies (device addresses, lengths in doubles).
int run_segments(jgb_engine* E, const std::vector<unsigned long long>& seg) {
  if (seg.empty()) return JGB_OK;
  cudaStream_t s = E->x->stream;
  ECK(E->segbuf.reserve(sizeof(unsigned long long) * seg.size()));
  ECK(cudaMemcpyAsync(E->segbuf.p, seg.data(), sizeof(unsigned long long) * seg.size(),
                      cudaMemcpyHostToDevice, s));
  const int nseg = (int)(seg.size() / 3);
  dim3 grid(8, (unsigned)std::min(nseg, 65535));
  k_copy_segments<<<grid, 256, 0, s>>>(nseg, E->segbuf.as<unsigned long long>());
  ECK(cudaGetLastError());
  // the host vector is reused by the caller: wait for the upload
  ECK(cudaStreamSynchronize(s));
  return JGB_OK;
}

// Build working set `w` for the requests `reqs` (inputs uploaded from their
// host records); with `old`, requests with slot >= 0 bring their iterate
// state from it; with `carry`, their slots become their index in `w`.
int build_workset(jgb_engine* E, WorkSet& w, WorkSet* old, const std::vector<Request*>& reqs,
                  bool carry) {
  jgb_ctx* x = E->x;
  const CtlDev& c = x->c;
  cudaStream_t s = x->stream;
  const int nret = (int)reqs.size();
  const int nscal = 5 + c.ncl + c.nsf, nplanes = 6 + c.ng + c.nw;
  w.nret = nret;
  FdLayout& H = w.H;
  H.nobs = nret;
  H.lev_off.assign(nret + 1, 0);
  H.ray_off.assign(nret + 1, 0);
  H.lay.assign(nret, {});
  H.mcnt.assign(nret, 0);
  H.ncnt.assign(nret, 0);
  H.yoff.assign(nret + 1, 0);
  H.kb.assign(nret + 1, 0);
  H.ymap.clear();
  w.desc.assign(nret, RetDesc{});
  w.mvec.assign(nret, 0);
  w.nvec.assign(nret, 0);
  long long nx = 0, nss = 0;
  for (int i = 0; i < nret; i++) {
    const Request* q = reqs[i];
    H.lev_off[i + 1] = H.lev_off[i] + q->np;
    H.ray_off[i + 1] = H.ray_off[i] + q->nr;
    H.lay[i] = q->lay;
    H.ncnt[i] = q->n;
    H.mcnt[i] = q->m;
    H.ymap.insert(H.ymap.end(), q->ymap.begin(), q->ymap.end());
    H.yoff[i + 1] = H.yoff[i] + q->m;
    H.kb[i + 1] = H.kb[i] + (long long)q->m * q->n;
    w.desc[i] = RetDesc{q->n, q->m, nx, (long long)H.yoff[i], nss, H.kb[i]};
    w.mvec[i] = q->m;
    w.nvec[i] = q->n;
    nx += q->n;
    nss += (long long)q->n * q->n;
  }
  w.nlev = H.lev_off[nret];
  w.nray = H.ray_off[nret];
  w.nx = nx;
  w.nss = nss;
  w.ny = H.yoff[nret];
  w.nk = H.kb[nret];
  const bool err_ana = E->ret.err_ana != 0;
  // host staging of the inputs
  std::vector<double> lev((size_t)w.nlev * nplanes), scal((size_t)nret * nscal), geo(7 * (size_t)w.nray),
      radm((size_t)c.nd * w.nray), yv(4 * (size_t)w.ny);
  std::vector<int4> elems(nx);
  std::vector<SaElem> sael(nx);
  for (int i = 0; i < nret; i++) {
    const Request* q = reqs[i];
    const int l0 = H.lev_off[i], r0 = H.ray_off[i];
    for (int k = 0; k < nplanes; k++)
      std::memcpy(&lev[(size_t)k * w.nlev + l0], &q->lev[(size_t)k * q->np], sizeof(double) * q->np);
    std::memcpy(&scal[(size_t)i * nscal], q->scal.data(), sizeof(double) * nscal);
    for (int k = 0; k < 7; k++)
      std::memcpy(&geo[(size_t)k * w.nray + r0], &q->geo[(size_t)k * q->nr], sizeof(double) * q->nr);
    for (int k = 0; k < c.nd; k++)
      std::memcpy(&radm[(size_t)k * w.nray + r0], &q->rad[(size_t)k * q->nr], sizeof(double) * q->nr);
    const size_t yo = H.yoff[i];
    std::memcpy(&yv[yo], q->ymeas.data(), sizeof(double) * q->m);
    std::memcpy(&yv[w.ny + yo], q->winv.data(), sizeof(double) * q->m);
    std::memcpy(&yv[2 * w.ny + yo], q->sn.data(), sizeof(double) * q->m);
    std::memcpy(&yv[3 * w.ny + yo], q->sf.data(), sizeof(double) * q->m);
    std::copy(q->elems.begin(), q->elems.end(), elems.begin() + w.desc[i].xo);
    std::copy(q->sael.begin(), q->sael.end(), sael.begin() + w.desc[i].xo);
  }
  const size_t bytes = workset_bytes(c, nret, w.nlev, w.nray, nx, w.ny, nss, w.nk, err_ana);
  ECK(w.mem.reserve(bytes));
  char* mp = w.mem.as<char>();
  auto take = [&](size_t nbytes) {
    char* p = mp;
    mp += (nbytes + 255) & ~size_t(255);
    return p;
  };
  const size_t dbl = sizeof(double);
  w.apr_lev = (double*)take(dbl * (size_t)w.nlev * nplanes);
  w.cur_lev = (double*)take(dbl * (size_t)w.nlev * nplanes);
  w.apr_scal = (double*)take(dbl * (size_t)nret * nscal);
  w.cur_scal = (double*)take(dbl * (size_t)nret * nscal);
  w.geo = (double*)take(dbl * 7 * (size_t)w.nray);
  w.radm = (double*)take(dbl * (size_t)c.nd * w.nray);
  w.rad = (double*)take(dbl * (size_t)c.nd * w.nray);
  w.tau = (double*)take(dbl * (size_t)c.nd * w.nray);
  w.tp = (double*)take(dbl * 3 * (size_t)w.nray);
  double** xs[11] = {&w.xa, &w.xi, &w.dx, &w.bvec, &w.step, &w.xfin, &w.e_tot, &w.e_noise, &w.e_formod, &w.cont, &w.res};
  for (double** p : xs) *p = (double*)take(dbl * nx);
  w.ym = (double*)take(dbl * 4 * w.ny);
  w.w = w.ym + w.ny;
  w.sn = w.ym + 2 * w.ny;
  w.sf = w.ym + 3 * w.ny;
  w.yi = (double*)take(dbl * w.ny);
  w.dy = (double*)take(dbl * w.ny);
  double** ss[5] = {&w.sainv, &w.cov, &w.covn, &w.Amat, &w.work};
  for (double** p : ss) *p = (double*)take(dbl * nss);
  w.Kd = (double*)take(dbl * std::max(w.nk, 1LL));
  w.G = err_ana ? (double*)take(dbl * std::max(w.nk, 1LL)) : nullptr;
  w.chisq = (double*)take(dbl * nret);
  w.lmpar = (double*)take(dbl * nret);
  w.disq = (double*)take(dbl * nret);
  w.elems = (int4*)take(sizeof(int4) * nx);
  w.sael = (SaElem*)take(sizeof(SaElem) * nx);
  w.desc_d = (RetDesc*)take(sizeof(RetDesc) * nret);
  w.active = (int*)take(sizeof(int) * nret);
  w.status = (int*)take(sizeof(int) * nret);
  w.levoff = (int*)take(sizeof(int) * (nret + 1));
  w.rayoff = (int*)take(sizeof(int) * (nret + 1));
  w.rayobs = (int*)take(sizeof(int) * w.nray);
  w.cnt = (int*)take(sizeof(int) * w.nray);
  w.skip = (unsigned char*)take(nret);
  w.mask = (unsigned char*)take((size_t)c.nd * w.nray);
  w.ymap = (int2*)take(sizeof(int2) * w.ny);
  w.nedesc = take(normal_desc_bytes(nret));
  if ((size_t)(mp - w.mem.as<char>()) > w.mem.n)
    return ctx_error(x, JGB_ERR_CUDA, "retrieval working set overflow");
  ECK(cudaMemcpyAsync(w.apr_lev, lev.data(), dbl * lev.size(), cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.apr_scal, scal.data(), dbl * scal.size(), cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.geo, geo.data(), dbl * geo.size(), cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.radm, radm.data(), dbl * radm.size(), cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.ym, yv.data(), dbl * yv.size(), cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.elems, elems.data(), sizeof(int4) * nx, cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.sael, sael.data(), sizeof(SaElem) * nx, cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.desc_d, w.desc.data(), sizeof(RetDesc) * nret, cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.levoff, H.lev_off.data(), sizeof(int) * (nret + 1), cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.rayoff, H.ray_off.data(), sizeof(int) * (nret + 1), cudaMemcpyHostToDevice, s));
  ECK(cudaMemcpyAsync(w.ymap, H.ymap.data(), sizeof(int2) * w.ny, cudaMemcpyHostToDevice, s));
  ECK(cudaMemsetAsync(w.status, 0, sizeof(int) * nret, s));
  ECK(cudaMemsetAsync(w.cnt, 0, sizeof(int) * w.nray, s));
  launch_ray_obs_mask(nret, w.rayoff, w.rayobs, (long long)c.nd * w.nray, w.radm, w.mask, s);
  ECK(cudaGetLastError());
  // fresh requests start from the a priori
  ECK(cudaMemcpyAsync(w.cur_lev, w.apr_lev, dbl * lev.size(), cudaMemcpyDeviceToDevice, s));
  ECK(cudaMemcpyAsync(w.cur_scal, w.apr_scal, dbl * scal.size(), cudaMemcpyDeviceToDevice, s));
  // requests that stay bring their iterate state
  std::vector<unsigned long long> seg;
  auto add = [&](const double* src, double* dst, long long nwords) {
    if (nwords <= 0) return;
    seg.push_back((unsigned long long)src);
    seg.push_back((unsigned long long)dst);
    seg.push_back((unsigned long long)nwords);
  };
  std::vector<int> cnt_keep;
  if (old)
    for (int i = 0; i < nret; i++) {
      const Request* q = reqs[i];
      const int j = q->slot;
      if (j < 0 || q->state == 0) continue;
      const long long ol = old->H.lev_off[j], orr = old->H.ray_off[j];
      const long long nl = H.lev_off[i], nr = H.ray_off[i];
      for (int k = 0; k < nplanes; k++) add(old->cur_lev + k * old->nlev + ol, w.cur_lev + k * w.nlev + nl, q->np);
      add(old->cur_scal + (long long)j * nscal, w.cur_scal + (long long)i * nscal, nscal);
      for (int k = 0; k < c.nd; k++) {
        add(old->rad + k * old->nray + orr, w.rad + k * w.nray + nr, q->nr);
        add(old->tau + k * old->nray + orr, w.tau + k * w.nray + nr, q->nr);
      }
      for (int k = 0; k < 3; k++) add(old->tp + k * old->nray + orr, w.tp + k * w.nray + nr, q->nr);
      const RetDesc& od = old->desc[j];
      const RetDesc& nd = w.desc[i];
      add(old->xa + od.xo, w.xa + nd.xo, od.n);
      add(old->xi + od.xo, w.xi + nd.xo, od.n);
      add(old->dx + od.xo, w.dx + nd.xo, od.n);
      add(old->yi + od.yo, w.yi + nd.yo, od.m);
      add(old->dy + od.yo, w.dy + nd.yo, od.m);
      add(old->sainv + od.so, w.sainv + nd.so, (long long)od.n * od.n);
      // K and K^T W K are reused unless the next iteration recomputes them
      const int nit = q->it + 1;
      if (!(nit == 1 || nit % E->ret.kernel_recomp == 0)) {
        add(old->cov + od.so, w.cov + nd.so, (long long)od.n * od.n);
        add(old->Kd + od.ko, w.Kd + nd.ko, (long long)od.n * od.m);
      }
      // LOS point counts (ints) travel as pairs packed in doubles where
      // aligned; simpler to copy them through the host below
      cnt_keep.push_back(i);
    }
  int rc = run_segments(E, seg);
  if (rc) return rc;
  if (!cnt_keep.empty()) {
    std::vector<int> oc(old->nray), nc(w.nray, 0);
    ECK(cudaMemcpy(oc.data(), old->cnt, sizeof(int) * old->nray, cudaMemcpyDeviceToHost));
    for (int i : cnt_keep) {
      const int j = reqs[i]->slot;
      std::memcpy(&nc[H.ray_off[i]], &oc[old->H.ray_off[j]], sizeof(int) * reqs[i]->nr);
    }
    ECK(cudaMemcpyAsync(w.cnt, nc.data(), sizeof(int) * w.nray, cudaMemcpyHostToDevice, s));
    ECK(cudaStreamSynchronize(s));
  }
  if (carry)
    for (int i = 0; i < nret; i++) reqs[i]->slot = i;
  return JGB_OK;
}

// Inverse of every flagged retrieval's matrix from its Cholesky factor L
// (matrix_invert): the column solves spread over blocks of 64 columns, then
// the symmetrised result in out.
void chol_inverse(int nret, const WorkSet& w, const double* L, double* work, double* out,
                  cudaStream_t s) {
  int nmax = 1;
  for (int i = 0; i < nret; i++) nmax = std::max(nmax, w.desc[i].n);
  k_chol_inverse_cols<<<dim3((nmax + 63) / 64, nret), 64, 0, s>>>(nret, w.desc_d, w.active, L, work);
  k_sym_half<<<dim3(16, nret), 256, 0, s>>>(nret, w.desc_d, w.active, work, out);
}

int put_flags(jgb_engine* E, WorkSet& w, const std::vector<int>& f) {
  ECK(cudaMemcpyAsync(w.active, f.data(), sizeof(int) * w.nret, cudaMemcpyHostToDevice, E->x->stream));
  return JGB_OK;
}

AtmArrays apr_arrays(const jgb_engine* E, const WorkSet& w) {
  const CtlDev& c = E->x->c;
  return AtmArrays{w.apr_lev, w.apr_scal, w.nlev, 5 + c.ncl + c.nsf, c.ng};
}
AtmArrays cur_arrays(const jgb_engine* E, const WorkSet& w) {
  const CtlDev& c = E->x->c;
  return AtmArrays{w.cur_lev, w.cur_scal, w.nlev, 5 + c.ncl + c.nsf, c.ng};
}

// Forward model of the flagged requests of the working set; y_i gathered.
// Leaves w.active = flags.
int forward(jgb_engine* E, WorkSet& w, const std::vector<int>& flags) {
  jgb_ctx* x = E->x;
  const CtlDev& c = x->c;
  cudaStream_t s = x->stream;
  const int nret = w.nret;
  std::vector<unsigned char> skip(nret);
  for (int i = 0; i < nret; i++) skip[i] = flags[i] ? 0 : 1;
  ECK(cudaMemcpyAsync(w.skip, skip.data(), nret, cudaMemcpyHostToDevice, s));
  int rc = put_flags(E, w, flags);
  if (rc) return rc;
  BatchDev bd{};
  bd.nobs = nret;
  bd.nlev = (int)w.nlev;
  bd.nray = (int)w.nray;
  bd.nscal = 5 + c.ncl + c.nsf;
  bd.lev_off = w.levoff;
  bd.ray_obs = w.rayobs;
  bd.time = w.cur_lev;
  bd.z = w.cur_lev + w.nlev;
  bd.lon = w.cur_lev + 2 * w.nlev;
  bd.lat = w.cur_lev + 3 * w.nlev;
  bd.p = w.cur_lev + 4 * w.nlev;
  bd.t = w.cur_lev + 5 * w.nlev;
  bd.q = w.cur_lev + 6 * w.nlev;
  bd.k = w.cur_lev + (6 + (long long)c.ng) * w.nlev;
  bd.scal = w.cur_scal;
  bd.geo = w.geo;
  bd.rad = w.rad;
  bd.tau = w.tau;
  bd.tp = w.tp;
  bd.mask = w.mask;
  bd.obs_skip = w.skip;
  rc = run_core(x, bd, E->precision, false);
  if (rc) return rc;
  E->st.forward_calls++;
  k_keep_counts<<<(unsigned)((w.nray + 255) / 256), 256, 0, s>>>((int)w.nray, w.rayobs, w.skip,
                                                                  x->los_cnt.as<int>(), w.cnt);
  k_gather_y<<<nret, 128, 0, s>>>(nret, w.desc_d, w.rayoff, w.ymap, w.active, w.rad, w.nray, w.yi);
  ECK(cudaGetLastError());
  return JGB_OK;
}

int jacobian(jgb_engine* E, WorkSet& w, const std::vector<int>& flags) {
  std::vector<int> list;
  for (int i = 0; i < w.nret; i++)
    if (flags[i]) list.push_back(i);
  if (list.empty()) return JGB_OK;
  std::vector<int> cnt(w.nray);
  ECK(cudaMemcpyAsync(cnt.data(), w.cnt, sizeof(int) * w.nray, cudaMemcpyDeviceToHost, E->x->stream));
  ECK(cudaStreamSynchronize(E->x->stream));
  FdInput in{w.cur_lev, w.cur_scal, w.geo, w.radm, w.levoff, w.rayoff, w.rad, cnt.data()};
  E->st.jacobians += list.size();
  const double t0 = now_ms();
  const int rc = fd_core(E->x, w.H, in, list, w.Kd, E->precision);
  E->st.jacobian_ms += now_ms() - t0;
  return rc;
}

// Initialisation of the flagged requests (retrieval.c:503-556).
int init_requests(jgb_engine* E, WorkSet& w, const std::vector<int>& F) {
  jgb_ctx* x = E->x;
  cudaStream_t s = x->stream;
  const int nret = w.nret;
  int rc = forward(E, w, F);
  if (rc) return rc;
  k_gather_state<<<nret, 128, 0, s>>>(nret, w.desc_d, w.levoff, w.elems, w.active, apr_arrays(E, w), w.xa);
  k_gather_state<<<nret, 128, 0, s>>>(nret, w.desc_d, w.levoff, w.elems, w.active, cur_arrays(E, w), w.xi);
  k_build_sa<<<dim3(64, nret), 256, 0, s>>>(nret, w.desc_d, w.active, w.sael, w.sainv);
  std::vector<int> diag(nret, 0), nondiag(nret, 0);
  bool any_nd = false;
  for (int i = 0; i < nret; i++) {
    if (!F[i]) continue;
    if (E->active[i]->sa_diag) diag[i] = 1;
    else nondiag[i] = 1, any_nd = true;
  }
  rc = put_flags(E, w, diag);
  if (rc) return rc;
  k_diag_inverse<<<nret, 128, 0, s>>>(nret, w.desc_d, w.active, w.sainv);
  if (any_nd) {
    rc = put_flags(E, w, nondiag);
    if (rc) return rc;
    k_select_nn<<<dim3(16, nret), 256, 0, s>>>(nret, w.desc_d, w.active, w.sainv, w.work);
    k_chol_factor<<<nret, 1024, 0, s>>>(nret, w.desc_d, w.active, w.work, w.status);
    chol_inverse(nret, w, w.work, w.Amat, w.sainv, s);
  }
  rc = put_flags(E, w, F);
  if (rc) return rc;
  k_residuals<<<nret, 128, 0, s>>>(nret, w.desc_d, w.active, w.xi, w.xa, w.ym, w.yi, w.dx, w.dy);
  k_cost<<<nret, 256, 0, s>>>(nret, w.desc_d, w.active, w.dx, w.dy, w.sainv, w.w, w.chisq);
  std::vector<double> chisq(nret);
  std::vector<int> st(nret);
  ECK(cudaMemcpyAsync(chisq.data(), w.chisq, sizeof(double) * nret, cudaMemcpyDeviceToHost, s));
  ECK(cudaMemcpyAsync(st.data(), w.status, sizeof(int) * nret, cudaMemcpyDeviceToHost, s));
  ECK(cudaStreamSynchronize(s));
  std::vector<int> J(nret, 0);
  for (int i = 0; i < nret; i++) {
    if (!F[i]) continue;
    Request* q = E->active[i];
    q->chisq = chisq[i];
    q->costs[0] = chisq[i];
    q->state = 1;
    if (st[i]) {
      q->status = JGB_ERR_NUMERIC;
      q->state = 2;
    } else if (E->ret.conv_itmax == 0) {
      q->state = 2;
    }
    J[i] = q->state == 1;
  }
  return jacobian(E, w, J);
}

// Candidates per request in the first and later rounds of damped trials,
// and the rays of a first round up to which it takes several.
constexpr int kTrialFirst = 3, kTrialLater = 4;
constexpr long long kTrialRays = 2048;

// One round of damped trials (retrieval.c:580-633) for the requests flagged
// in `trying`.  Request i evaluates up to `kk` damping values at once,
// lambda_i, 10 lambda_i, 100 lambda_i, ... (at most 20 trials per iteration
// in all): every candidate is a copy of the request in a candidate working
// set, with the iterate the sequential loop would form after the preceding
// rejections (k_spec_chain), and all candidates share one forward-model call.
// The decisions are then taken in lambda order exactly as the sequential
// loop takes them (first candidate with chi^2 <= the previous iteration's is
// accepted), and the state of the accepted candidate, or of the last one if
// all were rejected, moves back into `w`.  The results are the sequential
// loop's; only fewer latency-bound forward-model calls are made.
int trial_round(jgb_engine* E, WorkSet& w, std::vector<int>& trying, std::vector<int>& A,
                std::vector<int>& trials, int kk) {
  jgb_ctx* x = E->x;
  const CtlDev& c = x->c;
  cudaStream_t s = x->stream;
  const int nret = w.nret;
  const int nscal = 5 + c.ncl + c.nsf, nplanes = 6 + c.ng + c.nw;
  std::vector<Request*> creq;
  std::vector<int> csrc, first, count, who;
  std::vector<double> lam;
  for (int i = 0; i < nret; i++) {
    if (!trying[i]) continue;
    Request* q = E->active[i];
    const int K = std::max(1, std::min(kk, 20 - trials[i]));
    first.push_back((int)creq.size());
    count.push_back(K);
    who.push_back(i);
    double l = q->lmpar;
    for (int k = 0; k < K; k++) {
      creq.push_back(q);
      csrc.push_back(i);
      lam.push_back(l);
      l *= 10;
    }
  }
  const int nc = (int)creq.size(), nq = (int)who.size();
  if (nc == 0) return JGB_OK;
  WorkSet& cw = E->cw;
  int rc = build_workset(E, cw, nullptr, creq, false);
  if (rc) return rc;
  std::vector<unsigned long long> seg;
  auto add = [&](const double* src, double* dst, long long nwords) {
    if (nwords <= 0) return;
    seg.push_back((unsigned long long)src);
    seg.push_back((unsigned long long)dst);
    seg.push_back((unsigned long long)nwords);
  };
  for (int k = 0; k < nc; k++) {
    const RetDesc& d = w.desc[csrc[k]];
    const RetDesc& e = cw.desc[k];
    add(w.xa + d.xo, cw.xa + e.xo, d.n);
    add(w.xi + d.xo, cw.xi + e.xo, d.n);
    add(w.bvec + d.xo, cw.bvec + e.xo, d.n);
    add(w.sainv + d.so, cw.sainv + e.so, (long long)d.n * d.n);
    add(w.cov + d.so, cw.cov + e.so, (long long)d.n * d.n);
  }
  rc = run_segments(E, seg);
  if (rc) return rc;
  std::vector<int> all(nc, 1);
  rc = put_flags(E, cw, all);
  if (rc) return rc;
  ECK(cudaMemcpyAsync(cw.lmpar, lam.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, s));
  k_lm_matrix<<<dim3(64, nc), 256, 0, s>>>(nc, cw.desc_d, cw.active, cw.lmpar, cw.sainv, cw.cov, cw.Amat);
  k_chol_factor<<<nc, 1024, 0, s>>>(nc, cw.desc_d, cw.active, cw.Amat, cw.status);
  int nmax = 1;
  for (int k = 0; k < nc; k++) nmax = std::max(nmax, cw.desc[k].n);
  const size_t solve_smem = sizeof(double) * (size_t)nmax;
  if (solve_smem > 48 * 1024)
    ECK(cudaFuncSetAttribute(k_chol_solve, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)solve_smem));
  k_chol_solve<<<nc, 128, solve_smem, s>>>(nc, cw.desc_d, cw.active, cw.Amat, cw.bvec, cw.step);
  std::vector<int> fc(2 * (size_t)nq);
  for (int r = 0; r < nq; r++) {
    fc[r] = first[r];
    fc[nq + r] = count[r];
  }
  ECK(E->chainbuf.reserve(sizeof(int) * fc.size()));
  ECK(cudaMemcpyAsync(E->chainbuf.p, fc.data(), sizeof(int) * fc.size(), cudaMemcpyHostToDevice, s));
  k_spec_chain<<<nq, 128, 0, s>>>(nq, E->chainbuf.as<int>(), E->chainbuf.as<int>() + nq, cw.desc_d,
                                  cw.xi, cw.step, cw.xfin);
  k_set_iterate<<<nc, 256, 0, s>>>(nc, cw.desc_d, cw.levoff, cw.elems, cw.active, apr_arrays(E, cw),
                                    cur_arrays(E, cw), cw.xi, c.nw, c.ncl, c.nsf);
  ECK(cudaGetLastError());
  const double tfw = now_ms();
  rc = forward(E, cw, all);
  if (rc) return rc;
  ECK(cudaStreamSynchronize(s));
  E->st.trial_fwd_ms += now_ms() - tfw;
  {
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, x->ev[2], x->ev[3]);
    cudaEventElapsedTime(&b, x->ev[4], x->ev[5]);
    E->st.trial_trace_ms += a;
    E->st.trial_path_ms += b;
  }
  k_residuals<<<nc, 128, 0, s>>>(nc, cw.desc_d, cw.active, cw.xi, cw.xa, cw.ym, cw.yi, cw.dx, cw.dy);
  k_cost<<<nc, 256, 0, s>>>(nc, cw.desc_d, cw.active, cw.dx, cw.dy, cw.sainv, cw.w, cw.chisq);
  std::vector<double> cnew(nc);
  std::vector<int> st(nc);
  ECK(cudaMemcpyAsync(cnew.data(), cw.chisq, sizeof(double) * nc, cudaMemcpyDeviceToHost, s));
  ECK(cudaMemcpyAsync(st.data(), cw.status, sizeof(int) * nc, cudaMemcpyDeviceToHost, s));
  ECK(cudaStreamSynchronize(s));
  E->st.lm_trials++;
  // the sequential loop's decisions, candidate by candidate in lambda order
  // stepped: the iterate keeps the step (accepted, or the trial failed);
  // otherwise the last rejected step was taken back
  std::vector<int> chosen(nret, -1), accepted(nret, 0), stepped(nret, 0);
  for (int r = 0; r < nq; r++) {
    const int i = who[r];
    Request* q = E->active[i];
    for (int k = 0; k < count[r]; k++) {
      const int cidx = first[r] + k;
      trials[i]++;
      if (st[cidx]) {  // normal matrix not positive definite: the request fails
        q->status = JGB_ERR_NUMERIC;
        q->state = 2;
        A[i] = 0;
        chosen[i] = cidx;
        stepped[i] = 1;
        break;
      }
      q->chisq = cnew[cidx];
      chosen[i] = cidx;
      if (q->chisq > q->chisq_old) {
        q->lmpar *= 10;
      } else {
        q->lmpar /= 10;
        accepted[i] = stepped[i] = 1;
        break;
      }
    }
    trying[i] = A[i] && !accepted[i] && trials[i] < 20;
  }
  // state of the chosen candidates back into the working set
  seg.clear();
  std::vector<int> cnt_c(cw.nray), cnt_w(w.nray);
  bool any_chosen = false;
  for (int i = 0; i < nret; i++) {
    const int k = chosen[i];
    if (k < 0) continue;
    any_chosen = true;
    const Request* q = E->active[i];
    const RetDesc& d = w.desc[i];
    const RetDesc& e = cw.desc[k];
    const long long lw = w.H.lev_off[i], lc = cw.H.lev_off[k];
    const long long rw = w.H.ray_off[i], rcw = cw.H.ray_off[k];
    for (int pl = 0; pl < nplanes; pl++)
      add(cw.cur_lev + pl * cw.nlev + lc, w.cur_lev + pl * w.nlev + lw, q->np);
    add(cw.cur_scal + (long long)k * nscal, w.cur_scal + (long long)i * nscal, nscal);
    for (int id = 0; id < c.nd; id++) {
      add(cw.rad + id * cw.nray + rcw, w.rad + id * w.nray + rw, q->nr);
      add(cw.tau + id * cw.nray + rcw, w.tau + id * w.nray + rw, q->nr);
    }
    for (int pl = 0; pl < 3; pl++) add(cw.tp + pl * cw.nray + rcw, w.tp + pl * w.nray + rw, q->nr);
    add(cw.yi + e.yo, w.yi + d.yo, d.m);
    add(cw.dy + e.yo, w.dy + d.yo, d.m);
    add(cw.dx + e.xo, w.dx + d.xo, d.n);
    add(cw.step + e.xo, w.step + d.xo, d.n);
    add((stepped[i] ? cw.xi : cw.xfin) + e.xo, w.xi + d.xo, d.n);
  }
  if (!any_chosen) return JGB_OK;
  rc = run_segments(E, seg);
  if (rc) return rc;
  // LOS point counts (they size the chunks of later Jacobians)
  ECK(cudaMemcpyAsync(cnt_c.data(), cw.cnt, sizeof(int) * cw.nray, cudaMemcpyDeviceToHost, s));
  ECK(cudaMemcpyAsync(cnt_w.data(), w.cnt, sizeof(int) * w.nray, cudaMemcpyDeviceToHost, s));
  ECK(cudaStreamSynchronize(s));
  for (int i = 0; i < nret; i++)
    if (chosen[i] >= 0)
      std::memcpy(&cnt_w[w.H.ray_off[i]], &cnt_c[cw.H.ray_off[chosen[i]]],
                  sizeof(int) * E->active[i]->nr);
  ECK(cudaMemcpyAsync(w.cnt, cnt_w.data(), sizeof(int) * w.nray, cudaMemcpyHostToDevice, s));
  ECK(cudaStreamSynchronize(s));
  return JGB_OK;
}

// One LM iteration (retrieval.c:559-652) of every iterating request.
int lm_iteration(jgb_engine* E, WorkSet& w) {
  jgb_ctx* x = E->x;
  cudaStream_t s = x->stream;
  const int nret = w.nret;
  const int kr = E->ret.kernel_recomp;
  std::vector<int> A(nret, 0), J(nret, 0), N(nret, 0);
  bool any = false;
  for (int i = 0; i < nret; i++) {
    Request* q = E->active[i];
    if (q->state != 1) continue;
    const int it = q->it + 1;
    A[i] = 1;
    any = true;
    J[i] = it > 1 && it % kr == 0;
    N[i] = it == 1 || it % kr == 0;
    q->chisq_old = q->chisq;
  }
  if (!any) return JGB_OK;
  int rc = jacobian(E, w, J);
  if (rc) return rc;
  double t0 = now_ms();
  // K^T W K into covn and K^T W dy into bvec; covn replaces cov where the
  // kernel was (re)computed for this iteration
  rc = normal_equations_dev(nret, w.mvec.data(), w.nvec.data(), w.Kd, w.w, w.dy, w.covn, w.bvec,
                            E->precision, A.data(), w.nedesc, s);
  if (rc) return ctx_error(x, rc, "normal-equation kernel failed");
  rc = put_flags(E, w, N);
  if (rc) return rc;
  k_select_nn<<<dim3(16, nret), 256, 0, s>>>(nret, w.desc_d, w.active, w.covn, w.cov);
  rc = put_flags(E, w, A);
  if (rc) return rc;
  k_gradient<<<nret, 128, 0, s>>>(nret, w.desc_d, w.active, w.sainv, w.dx, w.bvec);
  ECK(cudaStreamSynchronize(s));
  E->st.normal_ms += now_ms() - t0;
  t0 = now_ms();
  // damped trials in rounds of candidates: several damping values per
  // request while the candidates of a round stay few enough rays for the
  // forward model to remain latency-bound, else one
  std::vector<int> trying = A, trials(nret, 0);
  for (int round = 0;; round++) {
    long long rays = 0;
    int ntry = 0;
    for (int i = 0; i < nret; i++)
      if (trying[i]) {
        rays += E->active[i]->nr;
        ntry++;
      }
    if (ntry == 0) break;
    int kk = round ? kTrialLater : kTrialFirst;
    while (kk > 1 && rays * kk > kTrialRays) kk--;
    rc = trial_round(E, w, trying, A, trials, kk);
    if (rc) return rc;
  }
  E->st.trial_ms += now_ms() - t0;
  rc = put_flags(E, w, A);
  if (rc) return rc;
  k_dot_state<<<(nret + 63) / 64, 64, 0, s>>>(nret, w.desc_d, w.active, w.step, w.bvec, w.disq);
  std::vector<double> disq(nret);
  ECK(cudaMemcpyAsync(disq.data(), w.disq, sizeof(double) * nret, cudaMemcpyDeviceToHost, s));
  ECK(cudaStreamSynchronize(s));
  for (int i = 0; i < nret; i++) {
    if (!A[i]) continue;
    Request* q = E->active[i];
    q->it++;
    q->costs[q->it] = q->chisq;
    const double dq = disq[i] / (double)q->n;
    if ((q->it == 1 || q->it % kr == 0) && dq < E->ret.conv_dmin) q->state = 2;
    if (q->it >= E->ret.conv_itmax) q->state = 2;
  }
  return JGB_OK;
}

// Results of the finished requests: final state, forward model, error
// analysis (retrieval.c:658-726), moved to the host in one staged copy.
int finish_requests(jgb_engine* E, WorkSet& w) {
  jgb_ctx* x = E->x;
  const CtlDev& c = x->c;
  cudaStream_t s = x->stream;
  const int nret = w.nret;
  std::vector<int> Fin(nret, 0), ok(nret, 0);
  bool any = false, any_ok = false;
  for (int i = 0; i < nret; i++) {
    const Request* q = E->active[i];
    if (q->state != 2) continue;
    Fin[i] = 1;
    any = true;
    ok[i] = q->status == JGB_OK;
    any_ok |= ok[i] != 0;
  }
  if (!any) return JGB_OK;
  const bool err_ana = E->ret.err_ana != 0;
  int rc = put_flags(E, w, Fin);
  if (rc) return rc;
  k_gather_state<<<nret, 128, 0, s>>>(nret, w.desc_d, w.levoff, w.elems, w.active, cur_arrays(E, w), w.xfin);
  std::vector<int> st(nret, 0);
  if (err_ana && any_ok) {
    // the final covariance is FP64 in both precision modes
    rc = normal_equations_dev(nret, w.mvec.data(), w.nvec.data(), w.Kd, w.w, w.dy, w.covn, w.bvec,
                              JGB_FP64, ok.data(), w.nedesc, s);
    if (rc) return ctx_error(x, rc, "normal-equation kernel failed");
    rc = put_flags(E, w, ok);
    if (rc) return rc;
    ECK(cudaMemsetAsync(w.status, 0, sizeof(int) * nret, s));
    k_add_nn<<<dim3(16, nret), 256, 0, s>>>(nret, w.desc_d, w.active, w.sainv, w.covn);
    k_chol_factor<<<nret, 1024, 0, s>>>(nret, w.desc_d, w.active, w.covn, w.status);
    chol_inverse(nret, w, w.covn, w.work, w.Amat, s);
    k_gain<<<dim3(64, nret), 256, 0, s>>>(nret, w.desc_d, w.active, w.Amat, w.Kd, w.w, w.G);
    k_sqrt_diag<<<nret, 128, 0, s>>>(nret, w.desc_d, w.active, w.Amat, w.e_tot);
    k_err_diag<<<nret, 128, 0, s>>>(nret, w.desc_d, w.active, w.G, w.sn, w.e_noise);
    k_err_diag<<<nret, 128, 0, s>>>(nret, w.desc_d, w.active, w.G, w.sf, w.e_formod);
    k_avk<<<dim3(64, nret), 256, 0, s>>>(nret, w.desc_d, w.active, w.G, w.Kd, w.work);
    k_avk_analyze<<<nret, 128, 0, s>>>(nret, w.desc_d, w.active, w.work, w.sael,
                                        7 + c.ng + c.nw + c.ncl, w.cont, w.res);
    ECK(cudaGetLastError());
    ECK(cudaMemcpyAsync(st.data(), w.status, sizeof(int) * nret, cudaMemcpyDeviceToHost, s));
  }
  // stage every result of every finished request into one device buffer
  std::vector<unsigned long long> seg;
  size_t words = 0;
  struct Dst {
    std::vector<double>* v;
    size_t off, len;
  };
  std::vector<Dst> dst;
  auto add = [&](const double* src, long long len, std::vector<double>* v, size_t voff) {
    if (len <= 0) return;
    seg.push_back((unsigned long long)src);
    seg.push_back(words);  // relocated to the staging address below
    seg.push_back((unsigned long long)len);
    dst.push_back(Dst{v, voff, (size_t)len});
    words += (size_t)len;
  };
  for (int i = 0; i < nret; i++) {
    if (!Fin[i]) continue;
    Request* q = E->active[i];
    const RetDesc& d = w.desc[i];
    const long long n = q->n, nr = q->nr, r0 = w.H.ray_off[i];
    q->x.assign(n, 0);
    q->rad_out.assign((size_t)c.nd * nr, 0);
    q->tau_out.assign((size_t)c.nd * nr, 0);
    q->tp_out.assign(3 * (size_t)nr, 0);
    q->p_out.assign(q->np, 0);
    add(w.xfin + d.xo, n, &q->x, 0);
    for (int k = 0; k < c.nd; k++) {
      add(w.rad + k * w.nray + r0, nr, &q->rad_out, (size_t)k * nr);
      add(w.tau + k * w.nray + r0, nr, &q->tau_out, (size_t)k * nr);
    }
    for (int k = 0; k < 3; k++) add(w.tp + k * w.nray + r0, nr, &q->tp_out, (size_t)k * nr);
    add(w.cur_lev + 4 * w.nlev + w.H.lev_off[i], q->np, &q->p_out, 0);
    if (err_ana && ok[i] && !st[i]) {
      q->cov.assign(n * n, 0);
      q->avk.assign(n * n, 0);
      q->err_total.assign(n, 0);
      q->err_noise.assign(n, 0);
      q->err_formod.assign(n, 0);
      q->cont.assign(n, 0);
      q->res.assign(n, 0);
      add(w.Amat + d.so, n * n, &q->cov, 0);
      add(w.work + d.so, n * n, &q->avk, 0);
      add(w.e_tot + d.xo, n, &q->err_total, 0);
      add(w.e_noise + d.xo, n, &q->err_noise, 0);
      add(w.e_formod + d.xo, n, &q->err_formod, 0);
      add(w.cont + d.xo, n, &q->cont, 0);
      add(w.res + d.xo, n, &q->res, 0);
      if (E->keep_gain) {
        q->gain.assign(n * q->m, 0);
        add(w.G + d.ko, n * q->m, &q->gain, 0);
      }
    } else if (err_ana && ok[i] && st[i]) {
      q->status = JGB_ERR_NUMERIC;
    }
  }
  ECK(E->stage.reserve(sizeof(double) * std::max(words, (size_t)1)));
  double* sd = E->stage.as<double>();
  for (size_t k = 0; k < seg.size(); k += 3) seg[k + 1] = (unsigned long long)(sd + seg[k + 1]);
  rc = run_segments(E, seg);
  if (rc) return rc;
  rc = ensure_pinned(E, words);
  if (rc) return rc;
  ECK(cudaMemcpyAsync(E->pinned, sd, sizeof(double) * words, cudaMemcpyDeviceToHost, s));
  ECK(cudaStreamSynchronize(s));
  size_t o = 0;
  for (const Dst& d : dst) {
    std::memcpy(d.v->data() + d.off, E->pinned + o, sizeof(double) * d.len);
    o += d.len;
  }
  // retire
  std::vector<Request*> keep;
  for (int i = 0; i < nret; i++) {
    Request* q = E->active[i];
    if (Fin[i]) {
      E->used -= q->bytes;
      E->done[q->id] = q;
      E->st.finished++;
      if (q->status) E->st.failed++;
    } else {
      keep.push_back(q);
    }
  }
  E->active.swap(keep);
  E->dirty = true;
  return JGB_OK;
}

int engine_step(jgb_engine* E) {
  jgb_ctx* x = E->x;
  cudaSetDevice(x->device);
  const double t0 = now_ms();
  // admission by slots and working-set bytes
  while (!E->queue.empty() && (int)E->active.size() < E->max_active) {
    Request* q = E->queue.front();
    if (!E->active.empty() && E->used + q->bytes > E->budget) break;
    E->queue.pop_front();
    q->slot = -1;
    E->active.push_back(q);
    E->used += q->bytes;
    E->dirty = true;
  }
  if (E->active.empty()) return JGB_OK;
  if (E->dirty) {
    const double tb = now_ms();
    WorkSet& nw = E->ws[1 - E->cur];
    int rc = build_workset(E, nw, E->have_ws ? &E->ws[E->cur] : nullptr, E->active, true);
    if (rc) return rc;
    ECK(cudaStreamSynchronize(x->stream));
    E->st.rebuild_ms += now_ms() - tb;
    E->cur = 1 - E->cur;
    E->have_ws = true;
    E->dirty = false;
    E->st.rebuilds++;
  }
  WorkSet& w = E->ws[E->cur];
  std::vector<int> F(w.nret, 0);
  bool anyf = false;
  for (int i = 0; i < w.nret; i++) {
    F[i] = E->active[i]->state == 0;
    anyf |= F[i] != 0;
  }
  int rc = JGB_OK;
  if (anyf) {
    const double ti = now_ms(), j0 = E->st.jacobian_ms;
    rc = init_requests(E, w, F);
    E->st.init_ms += now_ms() - ti - (E->st.jacobian_ms - j0);
  }
  if (!rc) rc = lm_iteration(E, w);
  if (!rc) {
    const double tf = now_ms();
    rc = finish_requests(E, w);
    E->st.finish_ms += now_ms() - tf;
  }
  E->st.steps++;
  E->st.step_ms += now_ms() - t0;
  return rc;
}

}  // namespace

// ===========================================================================
// C ABI of the engine

extern "C" int jgb_engine_create(jgb_ctx* x, const jgb_ret* ret, int precision,
                                 unsigned long long mem_budget, int max_active, int keep_gain,
                                 jgb_engine** out) {
  jgb::CtxLock lock(x);
  if (!x || !ret || !out) return ctx_error(x, JGB_ERR_ARG, "bad arguments");
  *out = nullptr;
  if (ret->conv_itmax < 0 || ret->kernel_recomp <= 0) return ctx_error(x, JGB_ERR_ARG, "bad retrieval settings");
  if (precision != JGB_FP64 && precision != JGB_MIXED) return ctx_error(x, JGB_ERR_ARG, "bad precision");
  CtxView v;
  int rc = ctx_view(x, &v);
  if (rc) return rc;
  const CtlDev& c = x->c;
  jgb_engine* E = new jgb_engine();
  E->x = x;
  x->engines.push_back(E);
  E->precision = precision;
  E->budget = mem_budget ? mem_budget : ~0ULL;
  E->max_active = max_active > 0 ? std::min(max_active, 65535) : 65535;
  E->keep_gain = keep_gain;
  E->ret = *ret;
  auto cp = [](std::vector<double>& v, const double* p, int n) -> const double* {
    if (!p || n <= 0) return nullptr;
    v.assign(p, p + n);
    return v.data();
  };
  E->ret.err_formod = cp(E->v_formod, ret->err_formod, c.nd);
  E->ret.err_noise = cp(E->v_noise, ret->err_noise, c.nd);
  E->ret.err_q = cp(E->v_q, ret->err_q, c.ng);
  E->ret.err_q_cz = cp(E->v_qcz, ret->err_q_cz, c.ng);
  E->ret.err_q_ch = cp(E->v_qch, ret->err_q_ch, c.ng);
  E->ret.err_k = cp(E->v_k, ret->err_k, c.nw);
  E->ret.err_k_cz = cp(E->v_kcz, ret->err_k_cz, c.nw);
  E->ret.err_k_ch = cp(E->v_kch, ret->err_k_ch, c.nw);
  E->ret.err_clk = cp(E->v_clk, ret->err_clk, c.ncl);
  E->ret.err_sfeps = cp(E->v_sfeps, ret->err_sfeps, c.nsf);
  *out = E;
  return JGB_OK;
}

void jgb::engine_detach(jgb_engine* E) {
  for (jgb::WorkSet& w : E->ws) w.mem.release();
  E->cw.mem.release();
  E->chainbuf.release();
  E->segbuf.release();
  E->stage.release();
  if (E->pinned) cudaFreeHost(E->pinned);
  E->pinned = nullptr;
  E->pinned_n = 0;
  E->have_ws = false;
  E->x = nullptr;
}

extern "C" void jgb_engine_destroy(jgb_engine* E) {
  if (!E) return;
  jgb_ctx* x = E->x;
  if (!x) {  // detached by jgb_destroy: its memory is gone already
    delete E;
    return;
  }
  jgb::CtxLock lock(x);
  cudaSetDevice(x->device);
  cudaStreamSynchronize(x->stream);
  x->engines.erase(std::remove(x->engines.begin(), x->engines.end(), E), x->engines.end());
  delete E;
}

extern "C" int jgb_engine_submit(jgb_engine* E, const jgb_batch* hb, unsigned long long* ids) {
  jgb::CtxLock lock(E ? E->x : nullptr);
  if (!E || !hb || hb->nobs <= 0) return ctx_error(E ? E->x : nullptr, JGB_ERR_ARG, "bad arguments");
  if (!E->x) return JGB_ERR_STATE;  // context destroyed
  jgb_ctx* x = E->x;
  const CtlDev& c = x->c;
  const int nobs = hb->nobs;
  const int nlev = hb->lev_off[nobs], nray = hb->ray_off[nobs];
  const int nscal = 5 + c.ncl + c.nsf;
  std::vector<Request*> made;
  for (int i = 0; i < nobs; i++) {
    Request* q = new Request();
    const int l0 = hb->lev_off[i], r0 = hb->ray_off[i];
    q->np = hb->lev_off[i + 1] - l0;
    q->nr = hb->ray_off[i + 1] - r0;
    int rc = JGB_OK;
    if (q->np < 1 || q->nr < 1) rc = ctx_error(x, JGB_ERR_ARG, "empty observation");
    if (!rc) {
      const int nplanes = 6 + c.ng + c.nw;
      q->lev.resize((size_t)nplanes * q->np);
      const double* src[6] = {hb->time, hb->z, hb->lon, hb->lat, hb->p, hb->t};
      for (int k = 0; k < 6; k++) std::memcpy(&q->lev[(size_t)k * q->np], src[k] + l0, sizeof(double) * q->np);
      for (int g = 0; g < c.ng; g++)
        std::memcpy(&q->lev[(size_t)(6 + g) * q->np], hb->q + (size_t)g * nlev + l0, sizeof(double) * q->np);
      for (int k = 0; k < c.nw; k++)
        std::memcpy(&q->lev[(size_t)(6 + c.ng + k) * q->np], hb->k + (size_t)k * nlev + l0, sizeof(double) * q->np);
      q->scal.assign(hb->scal + (size_t)i * nscal, hb->scal + (size_t)(i + 1) * nscal);
      q->geo.resize(7 * (size_t)q->nr);
      for (int k = 0; k < 7; k++)
        std::memcpy(&q->geo[(size_t)k * q->nr], hb->geo + (size_t)k * nray + r0, sizeof(double) * q->nr);
      q->rad.resize((size_t)c.nd * q->nr);
      for (int k = 0; k < c.nd; k++)
        std::memcpy(&q->rad[(size_t)k * q->nr], hb->rad + (size_t)k * nray + r0, sizeof(double) * q->nr);
      rc = prepare_request(E, q);
    }
    if (rc) {
      delete q;
      for (Request* r : made) delete r;
      return rc;
    }
    made.push_back(q);
  }
  for (size_t i = 0; i < made.size(); i++) {
    made[i]->id = E->next_id++;
    if (ids) ids[i] = made[i]->id;
    E->queue.push_back(made[i]);
  }
  E->st.submitted += made.size();
  return JGB_OK;
}

extern "C" int jgb_engine_step(jgb_engine* E, int* n_active, int* n_queued, int* n_done) {
  jgb::CtxLock lock(E ? E->x : nullptr);
  if (!E) return JGB_ERR_ARG;
  if (!E->x) return JGB_ERR_STATE;  // context destroyed
  const int rc = engine_step(E);
  if (n_active) *n_active = (int)E->active.size();
  if (n_queued) *n_queued = (int)E->queue.size();
  if (n_done) *n_done = (int)E->done.size();
  return rc;
}

extern "C" int jgb_engine_finished(jgb_engine* E, unsigned long long* ids, int max, int* count) {
  jgb::CtxLock lock(E ? E->x : nullptr);
  if (!E || !count) return JGB_ERR_ARG;
  if (!E->x) return JGB_ERR_STATE;  // context destroyed
  int k = 0;
  for (auto it = E->done.begin(); it != E->done.end() && k < max; ++it) ids[k++] = it->first;
  *count = k;
  return JGB_OK;
}

extern "C" int jgb_engine_sizes(jgb_engine* E, unsigned long long id, int* n, int* m, int* np, int* nr) {
  jgb::CtxLock lock(E ? E->x : nullptr);
  if (!E) return JGB_ERR_ARG;
  if (!E->x) return JGB_ERR_STATE;  // context destroyed
  auto it = E->done.find(id);
  if (it == E->done.end()) return ctx_error(E->x, JGB_ERR_ARG, "unknown or unfinished request");
  const Request* q = it->second;
  if (n) *n = q->n;
  if (m) *m = q->m;
  if (np) *np = q->np;
  if (nr) *nr = q->nr;
  return JGB_OK;
}

extern "C" int jgb_engine_result(jgb_engine* E, unsigned long long id, jgb_ret_out* o) {
  jgb::CtxLock lock(E ? E->x : nullptr);
  if (!E || !o) return JGB_ERR_ARG;
  if (!E->x) return JGB_ERR_STATE;  // context destroyed
  auto it = E->done.find(id);
  if (it == E->done.end()) return ctx_error(E->x, JGB_ERR_ARG, "unknown or unfinished request");
  Request* q = it->second;
  auto put = [](double* dst, const std::vector<double>& v) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), sizeof(double) * v.size());
  };
  put(o->x, q->x);
  put(o->cov, q->cov);
  put(o->costs, q->costs);
  put(o->rad, q->rad_out);
  put(o->tau, q->tau_out);
  put(o->tp, q->tp_out);
  put(o->p, q->p_out);
  put(o->gain, q->gain);
  put(o->avk, q->avk);
  put(o->err_total, q->err_total);
  put(o->err_noise, q->err_noise);
  put(o->err_formod, q->err_formod);
  put(o->cont, q->cont);
  put(o->res, q->res);
  o->iters = q->it;
  o->status = q->status;
  o->has_err_ana = q->cov.empty() ? 0 : 1;
  E->done.erase(it);
  delete q;
  return JGB_OK;
}

extern "C" int jgb_engine_get_stats(const jgb_engine* E, jgb_engine_stats* out) {
  jgb::CtxLock lock(E ? E->x : nullptr);
  if (!E || !out) return JGB_ERR_ARG;
  if (!E->x) return JGB_ERR_STATE;  // context destroyed
  *out = E->st;
  out->active = (int)E->active.size();
  out->queued = (int)E->queue.size();
  out->done = (int)E->done.size();
  out->used_bytes = E->used;
  return JGB_OK;
}

// Lockstep-free batch retrieval on top of the engine: every observation is a
// request, all are admitted at once and stepped until done.
extern "C" int jgb_retrieve_batch(jgb_ctx* x, const jgb_ret* ret, const jgb_batch* hb,
                                  double* x_out, double* cov_out, double* costs, int* iters,
                                  int precision) {
  jgb::CtxLock lock(x);
  if (!x || !ret || !hb || !x_out || hb->nobs <= 0) return ctx_error(x, JGB_ERR_ARG, "bad arguments");
  if (hb->nobs > 65535) return ctx_error(x, JGB_ERR_ARG, "at most 65535 retrievals per batch");
  const CtlDev& c = x->c;
  jgb_engine* E = nullptr;
  int rc = jgb_engine_create(x, ret, precision, 0, hb->nobs, 0, &E);
  if (rc) return rc;
  const int nret = hb->nobs;
  std::vector<unsigned long long> ids(nret);
  rc = jgb_engine_submit(E, hb, ids.data());
  while (!rc && (int)E->done.size() < nret) rc = engine_step(E);
  if (rc) {
    jgb_engine_destroy(E);
    return rc;
  }
  const int nray = hb->ray_off[nret];
  const int ncost = ret->conv_itmax + 1;
  int first_err = JGB_OK;
  long long xo = 0, so = 0;
  for (int i = 0; i < nret; i++) {
    Request* q = E->done[ids[i]];
    std::memcpy(x_out + xo, q->x.data(), sizeof(double) * q->n);
    if (cov_out && !q->cov.empty()) std::memcpy(cov_out + so, q->cov.data(), sizeof(double) * q->cov.size());
    if (costs) std::memcpy(costs + (size_t)i * ncost, q->costs.data(), sizeof(double) * ncost);
    if (iters) iters[i] = q->it;
    const int r0 = hb->ray_off[i];
    for (int k = 0; k < c.nd; k++) {
      std::memcpy(hb->rad + (size_t)k * nray + r0, &q->rad_out[(size_t)k * q->nr], sizeof(double) * q->nr);
      std::memcpy(hb->tau + (size_t)k * nray + r0, &q->tau_out[(size_t)k * q->nr], sizeof(double) * q->nr);
    }
    for (int k = 0; k < 3; k++)
      std::memcpy(hb->tp + (size_t)k * nray + r0, &q->tp_out[(size_t)k * q->nr], sizeof(double) * q->nr);
    std::memcpy(hb->p + hb->lev_off[i], q->p_out.data(), sizeof(double) * q->np);
    if (q->status && !first_err) first_err = q->status;
    xo += q->n;
    so += (long long)q->n * q->n;
  }
  jgb_engine_destroy(E);
  if (first_err == JGB_ERR_NUMERIC) return ctx_error(x, first_err, "normal matrix is not positive definite");
  return first_err;
}

// Batched matrix_invert (retrieval.c:373-399) on the device: the diagonal
// test, reciprocal diagonals, and for the other matrices the engine's
// Cholesky factor and column-solve inverse, symmetrised.
extern "C" int jgb_matrix_invert_dev(jgb_ctx* x, int nret, const int* n, double* A, int* status,
                                     float* kernel_ms) {
  jgb::CtxLock lock(x);
  if (!x || nret <= 0 || !n || !A) return ctx_error(x, JGB_ERR_ARG, "bad arguments");
  if (nret > 65535) return ctx_error(x, JGB_ERR_ARG, "at most 65535 matrices per call");
  CtxView v;
  int rc = ctx_view(x, &v);  // only the device and the stream are needed
  if (rc != JGB_OK && rc != JGB_ERR_STATE) return rc;
  rc = JGB_OK;  // tables are not needed: a context without them is fine
  cudaSetDevice(v.device);
  (void)cudaGetLastError();  // launch errors below are this call's
  std::vector<RetDesc> desc(nret);
  long long so = 0;
  int nmax = 1;
  for (int i = 0; i < nret; i++) {
    if (n[i] <= 0) return ctx_error(x, JGB_ERR_ARG, "empty matrix");
    desc[i] = RetDesc{n[i], 0, 0, 0, so, 0};
    so += (long long)n[i] * n[i];
    nmax = std::max(nmax, n[i]);
  }
  // scratch: descriptors, flags and status, the factors, the column solves
  const size_t b_desc = (sizeof(RetDesc) * (size_t)nret + 255) & ~size_t(255);
  const size_t b_flags = (sizeof(int) * 3 * (size_t)nret + 255) & ~size_t(255);
  void* buf = nullptr;
  if (cudaMalloc(&buf, b_desc + b_flags + sizeof(double) * 2 * (size_t)so) != cudaSuccess)
    return ctx_error(x, JGB_ERR_CUDA, "cudaMalloc failed");
  char* p = static_cast<char*>(buf);
  RetDesc* d = reinterpret_cast<RetDesc*>(p);
  int* diag = reinterpret_cast<int*>(p + b_desc);
  int* full = diag + nret;
  int* st = full + nret;
  double* L = reinterpret_cast<double*>(p + b_desc + b_flags);
  double* W = L + so;
  cudaStream_t s = v.stream;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaMemcpyAsync(d, desc.data(), sizeof(RetDesc) * nret, cudaMemcpyHostToDevice, s);
  cudaEventRecord(e0, s);
  k_invert_flags<<<nret, 256, 0, s>>>(nret, d, A, diag, full, st);
  k_diag_inverse<<<nret, 128, 0, s>>>(nret, d, diag, A);
  k_select_nn<<<dim3(16, nret), 256, 0, s>>>(nret, d, full, A, L);
  k_chol_factor<<<nret, 1024, 0, s>>>(nret, d, full, L, st);
  k_drop_failed<<<(nret + 255) / 256, 256, 0, s>>>(nret, st, full);
  k_chol_inverse_cols<<<dim3((nmax + 63) / 64, nret), 64, 0, s>>>(nret, d, full, L, W);
  k_sym_half<<<dim3(16, nret), 256, 0, s>>>(nret, d, full, W, A);
  cudaEventRecord(e1, s);
  cudaError_t err = cudaGetLastError();
  std::vector<int> hst(nret);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(hst.data(), st, sizeof(int) * nret, cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess) err = cudaStreamSynchronize(s);
  if (err == cudaSuccess && kernel_ms) cudaEventElapsedTime(kernel_ms, e0, e1);
  if (err == cudaSuccess && status) std::memcpy(status, hst.data(), sizeof(int) * nret);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (err != cudaSuccess)
    return ctx_error(x, JGB_ERR_CUDA,
                     std::string("matrix inversion kernels: ") + cudaGetErrorString(err));
  return JGB_OK;
}

extern "C" int jgb_matrix_invert(jgb_ctx* x, int nret, const int* n, double* A, int* status) {
  jgb::CtxLock lock(x);
  if (!x || nret <= 0 || !n || !A) return ctx_error(x, JGB_ERR_ARG, "bad arguments");
  long long so = 0;
  for (int i = 0; i < nret; i++) {
    if (n[i] <= 0) return ctx_error(x, JGB_ERR_ARG, "empty matrix");
    so += (long long)n[i] * n[i];
  }
  CtxView v;
  int rc = ctx_view(x, &v);
  if (rc != JGB_OK && rc != JGB_ERR_STATE) return rc;
  cudaSetDevice(v.device);
  jgb::DevBuf dA;
  if (dA.reserve(sizeof(double) * (size_t)so) != cudaSuccess)
    return ctx_error(x, JGB_ERR_CUDA, "cudaMalloc failed");
  if (cudaMemcpyAsync(dA.p, A, sizeof(double) * so, cudaMemcpyHostToDevice, v.stream) != cudaSuccess)
    return ctx_error(x, JGB_ERR_CUDA, "copy to the device failed");
  rc = jgb_matrix_invert_dev(x, nret, n, dA.as<double>(), status, nullptr);
  if (rc) return rc;
  if (cudaMemcpyAsync(A, dA.p, sizeof(double) * so, cudaMemcpyDeviceToHost, v.stream) != cudaSuccess ||
      cudaStreamSynchronize(v.stream) != cudaSuccess)
    return ctx_error(x, JGB_ERR_CUDA, "copy to the host failed");
  return JGB_OK;
}
