// Private definition of the library context shared by the translation
// units of libjurassic_gb300 (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/jurassic_gb300.h"
#include "jgb_common.cuh"

namespace jgb {

// Grow-only device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }  // a context's buffers go with it
  cudaError_t reserve(size_t bytes) {
    if (bytes <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    const size_t want = bytes + bytes / 8;  // headroom for slightly larger batches
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) n = want;
    return e;
  }
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};


}  // namespace jgb

// A batch of finite-difference perturbations whose path prefixes equal their
// base's (see fd_core): observations [0, nbase) are the unperturbed bases.
struct ResumeSpec {
  int nbase;
  const int4* pert;      // device, per observation: (array, index, level, step kind); x < 0: none
  const int* base_obs;   // device, per observation: its base observation
  const int* ray_off;    // device, ray offsets of the batch
  const int* h_ray_off;  // host copies
  const int* h_base_obs;
  const int4* h_pert;
};

struct jgb_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  jgb::CtlDev c{};
  std::vector<std::string> emitter;
  std::vector<double> nu, clnu, sfnu, retq_zmin, retq_zmax, retk_zmin, retk_zmax;
  std::vector<int> window;
  double retp_zmin = 0, retp_zmax = 0, rett_zmin = 0, rett_zmax = 0;
  int ret_flags[7] = {0, 0, 0, 0, 0, 0, 0};
  // device constants
  jgb::DevBuf d_nu, d_window, d_clnu, d_sfnu, d_ctm;
  // tables
  int tp = 0, tt = 0, tu = 0;
  bool tables_init = false;
  std::vector<int> h_np;
  // host copies of the float grids of the mixed path (padded like the device
  // arrays) and the emitters whose grids are the same for every channel
  std::vector<int> h_nt;
  std::vector<float> h_pf, h_tf;
  unsigned grid_mask = 0;
  // field of view: nfov samples (dz, w) on the device, pencil-beam scratch
  int nfov = 0;
  jgb::DevBuf d_fov, fov_raw;
  jgb::DevBuf t_np, t_p, t_nt, t_t, t_nu, t_u, t_eps, t_pf, t_tf, t_meta, t_ue;
  bool meta_stale = true;
  // source function
  jgb::DevBuf s_st, s_sr, s_srf;
  std::vector<char> src_set;
  bool srf_stale = true;
  // per-call scratch
  jgb::DevBuf b_levoff, b_rayoff, b_rayobs, b_lev, b_scal, b_geo, b_rad, b_tau, b_tp, b_mask, b_p;
  jgb::DevBuf los_off, los_cnt, los_cnt64, los_sft, los_ends, los_planes, scan_tmp, err_word;
  jgb::DevBuf tiles_perm, tiles_keys, tiles_keys2, tiles_vals, tiles_off, tiles_len, tiles_data;
  jgb::DevBuf refl;
  // finite-difference Jacobian: expanded batch and bookkeeping
  jgb::DevBuf kx_levoff, kx_rayoff, kx_rayobs, kx_src, kx_lev, kx_scal, kx_geo, kx_rad, kx_tau, kx_tp,
      kx_mask, kx_pert, kx_h, kx_ymap, kx_K, kx_base_rayoff, kx_base_levoff;
  cudaEvent_t ev[8] = {};
  // copies of the second chunk of a host batch overlap the first's compute
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t pev[3] = {};
  int path_variant = -1;  // mixed path kernel variant chosen by the autotuner
  double los_bound_scale = 1.0;  // factor on the per-ray LOS bound (0: count first)
  int path_split = -1;    // path split over emitters: -1 when latency-bound, 0 never, 1 always
  int fd_resume = 1;      // resume perturbed paths from their base's state: 0 never,
                          // 1 when the estimated schedule is shorter, 2 always,
                          // 3 always and with the emitters shared with the base
  const ResumeSpec* resume = nullptr;  // set by fd_core for the run_core call it makes
  jgb::DevBuf rs_start, rs_lists, rs_snap, rs_base, rs_seg;
  // resumed tracing: the base rays' walks and the perturbed rays' plan
  jgb::DevBuf rs_trace;
  // retrieval engines made from this context (detached by jgb_destroy)
  std::vector<jgb_engine*> engines;
  int sms = 152;          // multiprocessors of the device
  jgb::DevBuf seg;        // segment emissivities and flags of the split path
  std::vector<float> tune_ms;
  jgb_stats stats{};
  std::string err;
  // serialises the public entry points of the context (recursive: one entry
  // point may call another), so that host threads may share a context
  std::recursive_mutex mu;
};

namespace jgb {

// Forward model of a device-resident batch (ray tracing + path), shared by
// the batched forward model, the Jacobian and the retrieval.
int run_core(jgb_ctx* x, BatchDev& b, int precision, bool timed_h2d);
int ctx_error(jgb_ctx* x, int code, const std::string& msg);

// One retrieved state element (atm2x order, jurassic.c:29-83): the array it
// lives in (0 p, 1 t, 2 q, 3 k, 4 scal), the plane (q: emitter, k: window)
// or scal slot, the level within the observation (-1 for scal) and the step
// rule of kernel() (jurassic.c:4046-4068): 0 max(|0.01x|,1e-7), 1 1.0,
// 2 max(|0.01x|,1e-15), 3 1e-4, 4 0.1, 5 10.0, 6 1e-2.
struct Elem {
  int arr, idx, lev, hkind;
};
void state_layout(const jgb_ctx* x, const double* z, int nl, std::vector<Elem>& out);

// Host description of a batch for finite differences and retrievals.
struct FdLayout {
  int nobs = 0;
  std::vector<int> lev_off, ray_off;
  std::vector<std::vector<Elem>> lay;   // state layout per observation
  std::vector<int> mcnt, ncnt, yoff;    // measurement / state sizes, ymap offsets
  std::vector<int2> ymap;               // (ray within observation, channel), obs2y order
  std::vector<long long> kb;            // K block offsets
};
int fd_layout(jgb_ctx* x, int nobs, const int* lev_off, const int* ray_off, const double* z,
              const double* rad_mask, FdLayout& H);

// Device inputs of fd_core: the base batch after hydrostatic equilibrium.
struct FdInput {
  const double* lev;      // [6+ng+nw][nlev]: time z lon lat p t q[] k[]
  const double* scal;     // [nobs][nscal]
  const double* geo;      // [7][nray]
  const double* radmask;  // [nd][nray], NaN = masked
  const int* lev_off;     // [nobs+1]
  const int* ray_off;     // [nobs+1]
  const double* rad0;     // [nd][nray] forward model of the base
  const int* cnt;         // host: LOS points per ray of the base
};
int fd_core(jgb_ctx* x, const FdLayout& H, const FdInput& in, const std::vector<int>& list,
            double* K, int precision);
// observation index of every ray and the NaN mask of a device batch
void launch_ray_obs_mask(int nobs, const int* ray_off, int* ray_obs, long long n, const double* rad,
                         unsigned char* mask, cudaStream_t s);

}  // namespace jgb
