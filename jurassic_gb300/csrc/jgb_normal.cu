// Normal-equation products of the optimal-estimation retrieval:
//   A = K^T W K  and  b = K^T W dy,   W = diag(w^2)
// (matrix_product, retrieval.c:403-444, and the gsl_blas_dgemv of
// retrieval.c:573-577), batched over retrievals of different sizes.
//
// Mixed precision: 3xTF32 on the 5th-generation tensor cores (tcgen05, FP32
// accumulators in tensor memory).  Every operand x = sqrt(W)K is split into
// a TF32 head and a TF32 residual (x = hi + lo); the product uses
// hi*hi + hi*lo + lo*hi with FP32 accumulation, which recovers ~FP32
// accuracy from TF32 inputs.  dy is appended to K as column n so that b is
// the last row of the same product.  Only the lower triangle of output
// tiles is computed; the upper one is mirrored.
//
// FP64: the same products on the FP64 pipes (the plain reference arithmetic).
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <utility>

#include "../../include/jurassic_gb300.h"
#include "jgb_common.cuh"
#include "jgb_internal.h"

namespace jgb {

namespace {

constexpr int kTile = 128;  // output tile (kTile x kTile) per block
constexpr int kChunk = 16;  // rows of X per shared-memory stage
constexpr int kPlaneBytes = kTile * kChunk * 4;  // one operand plane of a stage (8 KB)
constexpr int kStageBytes = 4 * kPlaneBytes;     // A hi, A lo, B hi, B lo
constexpr int kTcSmem = 2 * kStageBytes + 64;    // two stages, barriers, TMEM address
constexpr int kHalf = kTile / 2;                 // epilogue columns per pass

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

__device__ unsigned g_tc_err;  // a tensor-core wait gave up (results invalid)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of element (row, k) in a 128 x kChunk K-major operand plane of
// 8-row x 16-byte core matrices: [k / 8][row / 8][k % 8 / 4][row % 8][k % 4];
// one MMA (K = 8 TF32) reads a [row / 8][2 core matrices] slice of 4 KB.
__device__ __forceinline__ int tc_off(int row, int k) {
  return (k >> 3) * 4096 + (row >> 3) * 256 + ((k & 7) >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

// Shared-memory matrix descriptor of such a slice (no swizzle): start
// address >> 4, leading byte offset 128 (the two core matrices along K),
// stride byte offset 256 (8-row groups), descriptor version 0b001 at bit 46.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) |
         ((uint64_t)(256u >> 4) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, N = M = kTile.
constexpr uint32_t kTcIdesc = (1u << 4) | (2u << 7) | (2u << 10) |
                              ((uint32_t)(kTile >> 3) << 17) | ((uint32_t)(kTile >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kTcIdesc), "r"(acc));
}

// Bounded wait for phase `parity` of an mbarrier.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (int it = 0; it < (1 << 20); it++) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
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
// a TF32 high part and a TF32-rounded remainder (row-major m x (n+1) per
// problem): one block per row, threads over the columns.
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
      xlo[o + col] = __uint_as_float(tf32_of(x - hi));
    }
  }
}

// One CTA: output tile (ti, tj), ti >= tj, of problem blockIdx.z, C = X^T X
// over the augmented columns.  Rows of X stream through two shared-memory
// stages of kChunk rows (A = columns of tile ti, B = columns of tile tj; on
// a diagonal tile B is A), copied element by element with cp.async straight
// into the core-matrix layout while the previous stage is multiplied.  One
// thread issues the 3 x 2 tcgen05.mma of a stage into a 128 x 128 FP32
// accumulator in tensor memory and commits them to the stage's mbarrier,
// which the threads wait on before refilling the stage.  The accumulator is
// read back with tcgen05.ld in two column halves, staged in shared memory,
// and written as FP64 with coalesced rows (direct and mirrored).  64 KB of
// shared memory: three CTAs per SM.
__global__ void __launch_bounds__(128, 3) k_normal_tc(const NeDesc* desc, const float* xhi,
                                                      const float* xlo, double* Aall,
                                                      double* ball) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
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
  if (ti >= nt) return;  // the whole CTA, before any barrier or tensor memory
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool diag = ti == tj;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(tc_smem + 2 * kStageBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tc_smem + 2 * kStageBytes + 16);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kTile));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;
  const float* XH = xhi + d.xoff;
  const float* XL = xlo + d.xoff;
  const int ci = ti * kTile + tid, cj = tj * kTile + tid;  // this thread's columns
  const bool iin = ci < na, jin = cj < na;
  const int nch = (d.m + kChunk - 1) / kChunk;
  const uint32_t sbase = smem_u32(tc_smem);
  // cp.async of chunk c into stage st (4-byte copies; out-of-range elements
  // are zero-filled from the problem's first element)
  auto load = [&](int c, int st) {
    const uint32_t base = sbase + st * kStageBytes;
#pragma unroll 4
    for (int k = 0; k < kChunk; k++) {
      const int row = c * kChunk + k;
      const bool rin = row < d.m;
      const long long o = (long long)row * na;
      const uint32_t off = (uint32_t)tc_off(tid, k);
      const uint32_t ni = rin && iin ? 4u : 0u, nj = rin && jin ? 4u : 0u;
      const float* hi = ni ? XH + o + ci : XH;
      const float* lo = ni ? XL + o + ci : XL;
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(base + off), "l"(hi), "r"(ni));
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(base + kPlaneBytes + off),
                   "l"(lo), "r"(ni));
      if (!diag) {
        const float* hj = nj ? XH + o + cj : XH;
        const float* lj = nj ? XL + o + cj : XL;
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(base + 2 * kPlaneBytes + off),
                     "l"(hj), "r"(nj));
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(base + 3 * kPlaneBytes + off),
                     "l"(lj), "r"(nj));
      }
    }
  };
  bool ok = true;
  load(0, 0);
  asm volatile("cp.async.commit_group;");
  for (int c = 0; c < nch; c++) {
    const int st = c & 1;
    if (c + 1 < nch) {
      // the other stage's MMAs (chunk c - 1) must be done before refilling it
      if (c >= 1) ok = mbar_wait(smem_u32(&mbar[st ^ 1]), ((c - 1) >> 1) & 1);
      ok = __syncthreads_and(ok);
      if (!ok) break;
      load(c + 1, st ^ 1);
    }
    asm volatile("cp.async.commit_group;");
    asm volatile("cp.async.wait_group 1;");  // chunk c has landed
    asm volatile("fence.proxy.async.shared::cta;");  // generic writes -> tensor-core reads
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = sbase + st * kStageBytes;
      const uint32_t b0 = diag ? a0 : a0 + 2 * kPlaneBytes;
#pragma unroll
      for (int s = 0; s < kChunk / 8; s++) {
        const uint64_t ah = tc_desc(a0 + s * 4096), al = tc_desc(a0 + kPlaneBytes + s * 4096);
        const uint64_t bh = tc_desc(b0 + s * 4096), bl = tc_desc(b0 + kPlaneBytes + s * 4096);
        tc_mma(tmem, al, bh, (c | s) != 0);
        tc_mma(tmem, ah, bl, 1u);
        tc_mma(tmem, ah, bh, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&mbar[st])));
    }
  }
  asm volatile("cp.async.wait_all;");
  // the last commit tracks every MMA of the tile
  if (ok && nch > 0) ok = mbar_wait(smem_u32(&mbar[(nch - 1) & 1]), ((nch - 1) >> 1) & 1);
  ok = __syncthreads_and(ok);
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (ok) {
    double* A = Aall + d.aoff;
    double* bv = ball + d.boff;
    float* tile = reinterpret_cast<float*>(tc_smem);  // [128][kHalf + 1]
    for (int h = 0; h < 2; h++) {
      // accumulator rows 32 warp + lane, columns h kHalf ... -> shared tile
      for (int c0 = 0; c0 < kHalf; c0 += 8) {
        uint32_t r[8];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
              "=r"(r[7])
            : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(h * kHalf + c0)));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
        for (int j = 0; j < 8; j++)
          tile[(warp * 32 + lane) * (kHalf + 1) + c0 + j] = __uint_as_float(r[j]);
      }
      __syncthreads();
      // rows >= columns (and b, the augmented row n), threads along a row
      for (int r = warp; r < kTile; r += 4) {
        const int row = ti * kTile + r;
        for (int cc = lane; cc < kHalf; cc += 32) {
          const int col = tj * kTile + h * kHalf + cc;
          if (col >= d.n || row > d.n) continue;
          const double v = f2d_bits(tile[r * (kHalf + 1) + cc]);
          if (row == d.n)
            bv[col] = v;
          else if (row >= col)
            A[(long long)row * d.n + col] = v;
        }
      }
      // mirrored entries, threads along a row of the upper triangle
      for (int cc = warp; cc < kHalf; cc += 4) {
        const int col = tj * kTile + h * kHalf + cc;
        for (int r = lane; r < kTile; r += 32) {
          const int row = ti * kTile + r;
          if (row < d.n && col < d.n && row > col)
            A[(long long)col * d.n + row] = f2d_bits(tile[r * (kHalf + 1) + cc]);
        }
      }
      __syncthreads();
    }
  } else if (tid == 0) {
    atomicOr(&g_tc_err, 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTile));
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
    cudaFuncSetAttribute(k_normal_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
    const unsigned zero = 0;
    cudaMemcpyToSymbolAsync(g_tc_err, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, s);
    dim3 grid(maxtiles, 1, nsel);
    k_normal_tc<<<grid, 128, kTcSmem, s>>>(dd, xbuf, xbuf + xo, A, b);
    unsigned herr = 0;
    cudaMemcpyFromSymbolAsync(&herr, g_tc_err, sizeof(herr), 0, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || herr) return JGB_ERR_CUDA;
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
