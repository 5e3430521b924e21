// Normal-equation products of the optimal-estimation retrieval:
//   A = K^T W K  and  b = K^T W dy,   W = diag(w^2)
// (matrix_product, retrieval.c:403-444, and the gsl_blas_dgemv of
// retrieval.c:573-577), batched over retrievals of different sizes.
//
// Mixed precision: 3xTF32 on the tensor cores.  Every operand x = sqrt(W)K is
// split into a TF32 head and a TF32 residual (x = hi + lo); the product uses
// hi*hi + hi*lo + lo*hi with FP32 accumulation, which recovers ~FP32
// accuracy from TF32 inputs.  dy is appended to K as column n so that b is
// the last column of the same product.  Only the lower triangle of output
// tiles is computed; the upper one is mirrored.
//
// FP64: the same products on the FP64 pipes (the plain reference arithmetic).
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <utility>

#include "../../include/jurassic_gb300.h"
#include "jgb_common.cuh"
#include "jgb_internal.h"

namespace jgb {

namespace {

constexpr int kTile = 64;   // output tile (kTile x kTile) per block
constexpr int kChunk = 32;  // rows of K per smem stage

struct NeDesc {
  int m, n;                 // rows of K, columns of K (state size)
  long long koff, moff, aoff, boff;
  long long xoff;           // offset of the problem's X planes (m x (n+1))
};

__device__ __forceinline__ unsigned tf32_of(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float* c, const unsigned* a, const unsigned* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Exact float -> double widening with integer operations (the FP64 pipe of
// GB300 is narrow); zero, subnormal, infinite and NaN inputs take the
// conversion instruction.
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const unsigned long long s = (unsigned long long)(u >> 31) << 63;
  const unsigned long long ex = (unsigned long long)(e + 896u) << 52;   // rebias 127 -> 1023
  const unsigned long long mt = (unsigned long long)(u & 0x7fffffu) << 29;
  return __longlong_as_double((long long)(s | ex | mt));
}

// X = sqrt(W)[K | dy] of every problem, formed once in FP64 and split into
// a TF32 high part and an FP32 remainder (row-major m x (n+1) per problem):
// one block per row, threads over the columns.
__global__ void k_split_x(const NeDesc* desc, const double* Kall, const double* wall,
                          const double* dyall, float* xhi, float* xlo) {
  const NeDesc d = desc[blockIdx.y];
  const int na = d.n + 1;
  for (int row = blockIdx.x; row < d.m; row += gridDim.x) {
    const double wr = wall[d.moff + row];
    const double* Kr = Kall + d.koff + (long long)row * d.n;
    const long long o = d.xoff + (long long)row * na;
    for (int col = threadIdx.x; col < na; col += blockDim.x) {
      const double v = col < d.n ? Kr[col] : dyall[d.moff + row];
      const float x = (float)(v * wr);
      const float hi = __uint_as_float(tf32_of(x));
      xhi[o + col] = hi;
      xlo[o + col] = x - hi;
    }
  }
}

// One block: output tile (ti, tj) with ti >= tj of retrieval blockIdx.z.
// 4 warps in a 2x2 arrangement, each a 32x32 sub-tile = 2 (M16) x 4 (N8)
// mma tiles.
__global__ void __launch_bounds__(128) k_normal_3xtf32(const NeDesc* desc, const float* xhi,
                                                       const float* xlo, double* Aall,
                                                       double* ball) {
  const NeDesc d = desc[blockIdx.z];
  const int na = d.n + 1;  // augmented columns
  const int nt = (na + kTile - 1) / kTile;
  // blockIdx.x enumerates lower-triangular tile pairs
  int t = blockIdx.x, ti = 0;
  while (t > ti) {
    t -= ti + 1;
    ti++;
  }
  const int tj = t;
  if (ti >= nt) return;
  const float* XH = xhi + d.xoff;
  const float* XL = xlo + d.xoff;
  __shared__ float hi_i[kChunk][kTile + 8], lo_i[kChunk][kTile + 8];  // +8: conflict-free fragment reads
  __shared__ float hi_j[kChunk][kTile + 8], lo_j[kChunk][kTile + 8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wr = (warp >> 1) * 32, wc = (warp & 1) * 32;  // warp sub-tile origin
  const int g = lane >> 2, tg = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;

  for (int k0 = 0; k0 < d.m; k0 += kChunk) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < kChunk * kTile; idx += blockDim.x) {
      const int r = idx / kTile, cidx = idx % kTile;
      const int row = k0 + r, ci = ti * kTile + cidx, cj = tj * kTile + cidx;
      const bool rin = row < d.m;
      const long long o = (long long)row * na;
      hi_i[r][cidx] = (rin && ci < na) ? __ldg(XH + o + ci) : 0.f;
      lo_i[r][cidx] = (rin && ci < na) ? __ldg(XL + o + ci) : 0.f;
      hi_j[r][cidx] = (rin && cj < na) ? __ldg(XH + o + cj) : 0.f;
      lo_j[r][cidx] = (rin && cj < na) ? __ldg(XL + o + cj) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kChunk; kk += 8) {
      // A fragments: rows = output rows (columns of X in tile i), cols = k
      unsigned ah[2][4], al[2][4];
#pragma unroll
      for (int a = 0; a < 2; a++) {
        const int r0 = wr + a * 16 + g;
        ah[a][0] = tf32_of(hi_i[kk + tg][r0]);
        ah[a][1] = tf32_of(hi_i[kk + tg][r0 + 8]);
        ah[a][2] = tf32_of(hi_i[kk + tg + 4][r0]);
        ah[a][3] = tf32_of(hi_i[kk + tg + 4][r0 + 8]);
        al[a][0] = tf32_of(lo_i[kk + tg][r0]);
        al[a][1] = tf32_of(lo_i[kk + tg][r0 + 8]);
        al[a][2] = tf32_of(lo_i[kk + tg + 4][r0]);
        al[a][3] = tf32_of(lo_i[kk + tg + 4][r0 + 8]);
      }
#pragma unroll
      for (int bq = 0; bq < 4; bq++) {
        const int c0 = wc + bq * 8 + g;
        unsigned bh[2], bl[2];
        bh[0] = tf32_of(hi_j[kk + tg][c0]);
        bh[1] = tf32_of(hi_j[kk + tg + 4][c0]);
        bl[0] = tf32_of(lo_j[kk + tg][c0]);
        bl[1] = tf32_of(lo_j[kk + tg + 4][c0]);
#pragma unroll
        for (int a = 0; a < 2; a++) {
          mma_tf32(acc[a][bq], al[a], bh);
          mma_tf32(acc[a][bq], ah[a], bl);
          mma_tf32(acc[a][bq], ah[a], bh);
        }
      }
    }
  }
  // store: rows/cols < n go to A (and the mirror), column n goes to b
  double* A = Aall + d.aoff;
  double* bv = ball + d.boff;
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int bq = 0; bq < 4; bq++)
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const int row = ti * kTile + wr + a * 16 + g + (c >= 2 ? 8 : 0);
        const int col = tj * kTile + wc + bq * 8 + 2 * tg + (c & 1);
        const double v = f2d_bits(acc[a][bq][c]);
        if (row < d.n && col < d.n) {
          if (row >= col) {
            A[(long long)row * d.n + col] = v;
            A[(long long)col * d.n + row] = v;
          }
        } else if (row == d.n && col < d.n) {
          bv[col] = v;
        }
      }
}

// FP64 reference products: one thread per lower-triangle element (+ b).
__global__ void k_normal_fp64(const NeDesc* desc, const double* Kall, const double* wall,
                              const double* dyall, double* Aall, double* ball) {
  const NeDesc d = desc[blockIdx.y];
  const long long nel = (long long)d.n * (d.n + 1) / 2 + d.n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nel;
       e += (long long)gridDim.x * blockDim.x) {
    const double* K = Kall + d.koff;
    const double* w = wall + d.moff;
    const double* dy = dyall + d.moff;
    if (e < (long long)d.n * (d.n + 1) / 2) {
      int i = (int)((sqrt(8.0 * (double)e + 1.0) - 1.0) / 2.0);
      while ((long long)(i + 1) * (i + 2) / 2 <= e) i++;
      while ((long long)i * (i + 1) / 2 > e) i--;
      const int j = (int)(e - (long long)i * (i + 1) / 2);
      double s = 0;  // sum of (w K)_ki (w K)_kj, the order of matrix_product
      for (int k = 0; k < d.m; k++)
        s += (w[k] * K[(long long)k * d.n + i]) * (w[k] * K[(long long)k * d.n + j]);
      Aall[d.aoff + (long long)i * d.n + j] = s;
      Aall[d.aoff + (long long)j * d.n + i] = s;
    } else {
      const int j = (int)(e - (long long)d.n * (d.n + 1) / 2);
      double s = 0;
      for (int k = 0; k < d.m; k++) s += K[(long long)k * d.n + j] * (dy[k] * (w[k] * w[k]));
      ball[d.boff + j] = s;
    }
  }
}

}  // namespace

// Grow-only scratch for the split X planes, one per device; calls that use
// it are ordered on their stream (the engine and the entry points run on
// their context's stream; concurrent streams on one device would share it).
static float* split_buffer(size_t bytes, cudaStream_t s) {
  static std::mutex mu;
  static std::map<int, std::pair<void*, size_t>> bufs;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  auto& b = bufs[dev];
  if (b.second < bytes) {
    if (b.first) {
      cudaStreamSynchronize(s);
      cudaFree(b.first);
    }
    b.first = nullptr;
    b.second = 0;
    const size_t want = bytes + bytes / 4;
    if (cudaMalloc(&b.first, want) != cudaSuccess) return nullptr;
    b.second = want;
  }
  return static_cast<float*>(b.first);
}

int normal_equations_dev(int nret, const int* m, const int* n, const double* K, const double* w,
                         const double* dy, double* A, double* b, int precision, const int* sel,
                         void* desc_dev, cudaStream_t s) {
  // descriptors of the selected problems (host -> device scratch provided by
  // the caller); offsets follow the concatenation of all nret problems
  NeDesc* hd = new NeDesc[nret];
  long long ko = 0, mo = 0, ao = 0, bo = 0, xo = 0;
  int maxtiles = 0, maxn = 0, maxm = 0, nsel = 0;
  for (int i = 0; i < nret; i++) {
    if (!sel || sel[i]) {
      hd[nsel++] = NeDesc{m[i], n[i], ko, mo, ao, bo, xo};
      xo += (long long)m[i] * (n[i] + 1);
      maxm = m[i] > maxm ? m[i] : maxm;
      const int nt = (n[i] + 1 + kTile - 1) / kTile;
      maxtiles = nt * (nt + 1) / 2 > maxtiles ? nt * (nt + 1) / 2 : maxtiles;
      maxn = n[i] > maxn ? n[i] : maxn;
    }
    ko += (long long)m[i] * n[i];
    mo += m[i];
    ao += (long long)n[i] * n[i];
    bo += n[i];
  }
  if (nsel == 0) {
    delete[] hd;
    return JGB_OK;
  }
  if (nsel > 65535) {
    delete[] hd;
    return JGB_ERR_ARG;
  }
  cudaError_t e = cudaMemcpyAsync(desc_dev, hd, sizeof(NeDesc) * nsel, cudaMemcpyHostToDevice, s);
  cudaStreamSynchronize(s);
  delete[] hd;
  if (e != cudaSuccess) return JGB_ERR_CUDA;
  if (precision == JGB_MIXED) {
    // X planes in a grow-only buffer of the current device (held to exit)
    float* xbuf = split_buffer(sizeof(float) * 2 * (size_t)xo, s);
    if (!xbuf) return JGB_ERR_CUDA;
    const NeDesc* dd = static_cast<const NeDesc*>(desc_dev);
    k_split_x<<<dim3((unsigned)(maxm < 1024 ? maxm : 1024), nsel), 128, 0, s>>>(dd, K, w, dy, xbuf,
                                                                                  xbuf + xo);
    dim3 grid(maxtiles, 1, nsel);
    k_normal_3xtf32<<<grid, 128, 0, s>>>(dd, xbuf, xbuf + xo, A, b);
  } else {
    const long long nel = (long long)maxn * (maxn + 1) / 2 + maxn;
    dim3 grid((unsigned)((nel + 127) / 128 < 4096 ? (nel + 127) / 128 : 4096), nsel);
    k_normal_fp64<<<grid, 128, 0, s>>>(static_cast<const NeDesc*>(desc_dev), K, w, dy, A, b);
  }
  return cudaGetLastError() == cudaSuccess ? JGB_OK : JGB_ERR_CUDA;
}

size_t normal_desc_bytes(int nret) { return sizeof(NeDesc) * (size_t)nret; }

}  // namespace jgb

using namespace jgb;

// Host-buffer entry point: copies in, computes, copies out.
extern "C" int jgb_normal_equations(jgb_ctx* x, int nret, const int* m, const int* n,
                                    const double* K, const double* w, const double* dy,
                                    double* A, double* b, int precision) {
  if (!x || nret <= 0 || !m || !n || !K || !w || !dy || !A || !b)
    return ctx_fail(x, JGB_ERR_ARG, "bad arguments");
  CtxView v;
  int rc = ctx_view(x, &v);  // tables are not needed here: only device and stream
  if (rc != JGB_OK && rc != JGB_ERR_STATE) return rc;
  cudaSetDevice(v.device);
  long long sk = 0, sm = 0, sa = 0, sb = 0;
  for (int i = 0; i < nret; i++) {
    if (m[i] <= 0 || n[i] <= 0) return ctx_fail(x, JGB_ERR_ARG, "empty retrieval");
    sk += (long long)m[i] * n[i];
    sm += m[i];
    sa += (long long)n[i] * n[i];
    sb += n[i];
  }
  void* buf = nullptr;
  const size_t bytes = sizeof(double) * (size_t)(sk + 2 * sm + sa + sb) + normal_desc_bytes(nret) + 64;
  if (cudaMalloc(&buf, bytes) != cudaSuccess) return ctx_fail(x, JGB_ERR_CUDA, "cudaMalloc failed");
  double* dK = static_cast<double*>(buf);
  double* dw = dK + sk;
  double* ddy = dw + sm;
  double* dA = ddy + sm;
  double* db = dA + sa;
  void* ddesc = db + sb;
  cudaStream_t s = v.stream;
  cudaMemcpyAsync(dK, K, sizeof(double) * sk, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dw, w, sizeof(double) * sm, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(ddy, dy, sizeof(double) * sm, cudaMemcpyHostToDevice, s);
  rc = normal_equations_dev(nret, m, n, dK, dw, ddy, dA, db, precision, nullptr, ddesc, s);
  if (rc == JGB_OK) {
    cudaMemcpyAsync(A, dA, sizeof(double) * sa, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(b, db, sizeof(double) * sb, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) rc = JGB_ERR_CUDA;
  }
  cudaFree(buf);
  return rc ? ctx_fail(x, rc, "normal-equation kernel failed") : JGB_OK;
}

// Device-buffer entry point: K, w, dy, A, b on the device, m and n on the
// host; runs on the context's stream and returns when the products are
// done.  *kernel_ms (optional) receives the CUDA-event time of the kernel.
extern "C" int jgb_normal_equations_dev(jgb_ctx* x, int nret, const int* m, const int* n,
                                        const double* K, const double* w, const double* dy,
                                        double* A, double* b, int precision, float* kernel_ms) {
  if (!x || nret <= 0 || !m || !n || !K || !w || !dy || !A || !b)
    return ctx_fail(x, JGB_ERR_ARG, "bad arguments");
  if (nret > 65535) return ctx_fail(x, JGB_ERR_ARG, "at most 65535 problems per call");
  CtxView v;
  int rc = ctx_view(x, &v);
  if (rc != JGB_OK && rc != JGB_ERR_STATE) return rc;
  cudaSetDevice(v.device);
  for (int i = 0; i < nret; i++)
    if (m[i] <= 0 || n[i] <= 0) return ctx_fail(x, JGB_ERR_ARG, "empty retrieval");
  void* ddesc = nullptr;
  if (cudaMalloc(&ddesc, normal_desc_bytes(nret)) != cudaSuccess)
    return ctx_fail(x, JGB_ERR_CUDA, "cudaMalloc failed");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaStream_t s = v.stream;
  // descriptors are uploaded (and the stream synchronised) inside; the
  // events bracket the kernel launch that follows
  rc = normal_equations_dev(nret, m, n, K, w, dy, A, b, precision, nullptr, ddesc, s);
  // time a second identical launch only when asked: the first one above
  // included the descriptor upload
  if (rc == JGB_OK && kernel_ms) {
    cudaEventRecord(e0, s);
    rc = normal_equations_dev(nret, m, n, K, w, dy, A, b, precision, nullptr, ddesc, s);
    cudaEventRecord(e1, s);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) rc = JGB_ERR_CUDA;
  if (rc == JGB_OK && kernel_ms) cudaEventElapsedTime(kernel_ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(ddesc);
  return rc ? ctx_fail(x, rc, "normal-equation kernel failed") : JGB_OK;
}
