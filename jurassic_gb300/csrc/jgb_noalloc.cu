// Allocation-free variant of the FP64 forward model on a device-resident
// batch.
//
// Why: some callers cannot allocate GPU memory while they run a forward
// model -- for example a host application that hands the library a fixed
// memory budget up front, a process whose allocator is owned by another
// runtime that must not see cudaMalloc/cudaFree traffic, or code that
// drives the GPU from a section where allocation is forbidden.  For them
// this entry point takes every scratch buffer (per-ray bookkeeping, the
// LOS arrays, the reflection scratch) from one file-scope device array
// instead of the context's grow-on-demand buffers.  The caller still owns
// all inputs and outputs.
//
// Limits and rules:
//  * the scratch array holds kNoAllocBytes (64 MiB); a batch whose rays and
//    LOS points do not fit is rejected with JGB_ERR_ARG and a message naming
//    the bytes it needs;
//  * the array is part of this file's device code, which CUDA loads onto a
//    device lazily; jgb_create loads it (and the kernels this entry point
//    launches) onto the context's device and resolves the array's address
//    there with cudaGetSymbolAddress, with that device current, so a call
//    itself loads and allocates nothing.  The array then stays on that
//    device until the process exits.  Should that set-up fail at
//    jgb_create, the first call retries it and returns JGB_ERR_CUDA if it
//    still fails;
//  * every call on a device shares the same array and it keeps the previous
//    call's contents; calls that overlap on the GPU (two contexts of one
//    device) race on it and must be serialised by the caller;
//  * nothing here calls cudaMalloc, cudaFree or an allocating library
//    routine; the cumulative sum over rays uses a kernel of this file instead
//    of a library scan with temporary storage.
#include <cstdio>
#include <mutex>

#include "../../include/jurassic_gb300.h"
#include "jgb_common.cuh"
#include "jgb_ctx.h"
#include "jgb_internal.h"

namespace jgb {

constexpr unsigned long long kNoAllocBytes = 64ull << 20;  // 64 MiB
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kNoAllocMaxDevices] = {};

// Device address of the scratch array on the current device (set up once).
int scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kNoAllocMaxDevices) return JGB_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return JGB_ERR_CUDA;
    g_scratch_ptr[device] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[device];
  return JGB_OK;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

__global__ void k_noalloc_ray_obs(int nobs, const int* ray_off, int* ray_obs) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nobs) return;
  for (int r = ray_off[o]; r < ray_off[o + 1]; r++) ray_obs[r] = o;
}

__global__ void k_noalloc_mask(long long n, const double* rad, unsigned char* mask) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) mask[i] = !isfinite(rad[i]);
}

// Exclusive prefix sum of the LOS point counts by one block: off[0] = 0,
// off[r+1] = off[r] + count[r].
__global__ void k_noalloc_scan(int n, const int* count, long long* off) {
  __shared__ long long part[1024];
  __shared__ long long carry;
  if (threadIdx.x == 0) {
    carry = 0;
    off[0] = 0;
  }
  __syncthreads();
  for (int base = 0; base < n; base += blockDim.x) {
    const int i = base + threadIdx.x;
    part[threadIdx.x] = i < n ? count[i] : 0;
    __syncthreads();
    for (int d = 1; d < (int)blockDim.x; d <<= 1) {
      const long long v = threadIdx.x >= (unsigned)d ? part[threadIdx.x - d] : 0;
      __syncthreads();
      part[threadIdx.x] += v;
      __syncthreads();
    }
    if (i < n) off[i + 1] = carry + part[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += part[threadIdx.x];
    __syncthreads();
  }
}

}  // namespace

int noalloc_prepare(int device) {
  unsigned char* p = nullptr;
  const int rc = scratch_address(device, &p);
  if (rc != JGB_OK) return rc;
  cudaFuncAttributes a;
  const void* fns[] = {(const void*)k_noalloc_ray_obs, (const void*)k_noalloc_mask,
                       (const void*)k_noalloc_scan};
  for (const void* f : fns)
    if (cudaFuncGetAttributes(&a, f) != cudaSuccess) return JGB_ERR_CUDA;
  return preload_fp64_kernels();
}

}  // namespace jgb

using namespace jgb;

extern "C" int jgb_formod_batch_dev_noalloc(jgb_ctx* x, const jgb_batch* db) {
  jgb::CtxLock lock(x);
  if (!x || !db || db->nobs <= 0) return ctx_fail(x, JGB_ERR_ARG, "empty batch");
  CtxView v;
  int rc = ctx_view(x, &v);
  if (rc) return rc;
  if (cudaSetDevice(v.device) != cudaSuccess) return ctx_fail(x, JGB_ERR_CUDA, "cudaSetDevice failed");
  unsigned char* base = nullptr;
  if (scratch_address(v.device, &base) != JGB_OK)
    return ctx_fail(x, JGB_ERR_CUDA, "cannot resolve the device address of the scratch array");
  const CtlDev& c = v.c;
  if (c.fov) return ctx_fail(x, JGB_ERR_UNSUPPORTED, "field of view not available without allocation");
  cudaStream_t s = v.stream;
  const int nobs = db->nobs;
  int nlev = 0, nray = 0;
  if (cudaMemcpy(&nlev, db->lev_off + nobs, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(&nray, db->ray_off + nobs, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return ctx_fail(x, JGB_ERR_CUDA, "cannot read batch offsets");
  if (nlev <= 0 || nray <= 0) return ctx_fail(x, JGB_ERR_ARG, "no levels or rays");

  // per-ray part of the scratch layout
  size_t o = 0;
  const size_t o_err = o;
  o = align256(o + sizeof(unsigned));
  const size_t o_rayobs = o;
  o = align256(o + sizeof(int) * (size_t)nray);
  const size_t o_count = o;
  o = align256(o + sizeof(int) * (size_t)nray);
  const size_t o_off = o;
  o = align256(o + sizeof(long long) * (size_t)(nray + 1));
  const size_t o_sft = o;
  o = align256(o + sizeof(double) * (size_t)nray);
  const size_t o_ends = o;
  o = align256(o + 6 * sizeof(double) * (size_t)nray);
  const size_t o_mask = o;
  o = align256(o + (size_t)c.nd * nray);
  const size_t o_planes = o;
  if (o_planes > kNoAllocBytes) {
    char msg[200];
    snprintf(msg, sizeof msg,
             "batch of %d rays needs more than %llu bytes of scratch; the allocation-free "
             "entry point holds %llu bytes", nray, (unsigned long long)o_planes, kNoAllocBytes);
    return ctx_fail(x, JGB_ERR_ARG, msg);
  }
  unsigned* d_err = reinterpret_cast<unsigned*>(base + o_err);
  BatchDev b{};
  b.nobs = nobs;
  b.nlev = nlev;
  b.nray = nray;
  b.nscal = 5 + c.ncl + c.nsf;
  b.lev_off = db->lev_off;
  b.ray_obs = reinterpret_cast<int*>(base + o_rayobs);
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
  b.mask = base + o_mask;
  LosDev L{};
  L.count = reinterpret_cast<int*>(base + o_count);
  L.off = reinterpret_cast<long long*>(base + o_off);
  L.sft = reinterpret_cast<double*>(base + o_sft);
  L.ends = reinterpret_cast<double*>(base + o_ends);
  L.ng = c.ng;
  L.nw = c.nw;
  L.cga = c.formod == 0;

  x->stats = jgb_stats{};
  cudaEventRecord(x->ev[0], s);
  // the error word must start at zero; everything else is written before read
  if (cudaMemsetAsync(d_err, 0, sizeof(unsigned), s) != cudaSuccess)
    return ctx_fail(x, JGB_ERR_CUDA, "cudaMemsetAsync failed");
  k_noalloc_ray_obs<<<(nobs + 127) / 128, 128, 0, s>>>(nobs, db->ray_off, const_cast<int*>(b.ray_obs));
  const long long nm = (long long)c.nd * nray;
  k_noalloc_mask<<<(unsigned)((nm + 255) / 256), 256, 0, s>>>(nm, b.rad, base + o_mask);
  if (c.hydz >= 0) launch_hydrostatic(c, b, const_cast<double*>(b.p), s);
  launch_trace_count(c, v.ch, b, L, d_err, s);
  k_noalloc_scan<<<1, 1024, 0, s>>>(nray, L.count, L.off);
  long long total = 0;
  unsigned h_err = 0;
  if (cudaMemcpyAsync(&total, L.off + nray, sizeof(long long), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&h_err, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return ctx_fail(x, JGB_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  if (h_err & kErrObserverBelowSurface) return ctx_fail(x, JGB_ERR_SURFACE, "Observer below surface!");
  if (h_err & kErrLosOverflow) return ctx_fail(x, JGB_ERR_LOS, "Too many LOS points!");

  // LOS planes (and the reflection scratch when a reflecting surface is on)
  const long long cap = total > 0 ? total : 1;
  const int nplanes = 8 + c.ng + c.nw + (c.formod == 0 ? 3 * c.ng : 0);
  const bool need_refl = c.sftype >= 2 && c.nsf > 0;
  size_t need = o_planes + align256(sizeof(double) * (size_t)cap * nplanes);
  const size_t o_refl = need;
  if (need_refl) need += align256(sizeof(double) * 2 * (size_t)cap * c.nd);
  if (need > kNoAllocBytes) {
    char msg[240];
    snprintf(msg, sizeof msg,
             "batch with %lld LOS points needs %llu bytes of scratch; the allocation-free "
             "entry point holds %llu bytes", (long long)total, (unsigned long long)need,
             kNoAllocBytes);
    return ctx_fail(x, JGB_ERR_ARG, msg);
  }
  double* P = reinterpret_cast<double*>(base + o_planes);
  L.cap = cap;
  L.z = P + 0 * cap;
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
  launch_trace_fill(c, v.ch, b, L, d_err, s);
  double* refl = need_refl ? reinterpret_cast<double*>(base + o_refl) : nullptr;
  launch_path_fp64(c, v.T, v.ch, b, L, refl, s);
  cudaEventRecord(x->ev[1], s);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
    return ctx_fail(x, JGB_ERR_CUDA, "forward-model kernels failed");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, x->ev[0], x->ev[1]);
  x->stats.total_ms = ms;
  x->stats.los_points = total;
  x->stats.trace_passes = 2;
  x->stats.path_launches = 6 + (c.hydz >= 0 ? 1 : 0);  // kernels of this call
  return JGB_OK;
}
