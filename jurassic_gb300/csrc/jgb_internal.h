// Launch wrappers shared between the translation units of libjurassic_gb300.
#pragma once

#include <cuda_runtime.h>

#include "jgb_common.cuh"

struct jgb_ctx;
struct jgb_engine;

namespace jgb {

// jgb_fp64.cu
void launch_trace_count(const CtlDev& c, const ChanDev& ch, const BatchDev& b, const LosDev& L,
                        unsigned* err, cudaStream_t s);
// jgb_fp64.cu: field-of-view convolution + BT + mask of pencil-beam results
void launch_fov(const CtlDev& c, const BatchDev& b, const double* prad, const double* ptau,
                int nfov, const double* fdz, const double* fw, const double* nu, unsigned* err,
                cudaStream_t s);
// jgb_trace_mixed.cu: ray tracing of the mixed-precision forward model
void launch_trace_count_mixed(const CtlDev& c, const BatchDev& b, const LosDev& L, unsigned* err,
                              cudaStream_t s);
void launch_trace_fill_mixed(const CtlDev& c, const BatchDev& b, const LosDev& L, const int* order,
                             unsigned* err, cudaStream_t s);
// Resumed tracing of finite-difference perturbations (EGA).  The fill of the
// base rays (the first nbase rays of the batch) keeps, per LOS point (indexed
// like the LOS planes, bpts points), the walk's FP64 position and direction,
// its raw segment length and its level interval.  A perturbed ray r then
// follows plan[r] = {base ray, m, mode}: mode 2 takes the base's geometry
// whole and recomputes the point values from its own profile (a perturbed
// mixing ratio or extinction: the step rule and refraction see z, p and T
// only; or a perturbed temperature whose levels the ray never comes near);
// mode 1 copies the base's points before m and walks on from the base's
// state at point m (a perturbed temperature, m before the first segment that
// comes near the perturbed levels); mode 0 walks from the start.  Every
// perturbed ray's LOS equals, bit for bit, what a walk from the start writes.
struct TraceResume {
  long long bpts;
  double* xs;        // [3][bpts] positions
  double* es;        // [3][bpts] directions
  float* dsr;        // [bpts] raw segment lengths
  int* lev;          // [bpts] level intervals
  const int4* plan;  // [nray] (perturbed rays)
};
// rays the fill kernel of the perturbed rays holds on the device at once
int trace_fill_resident(int sms);
// rays [r0, r0 + nr) (or order[0, nr)); role 1: the base rays (keep their
// walks in R), role 2: the perturbed rays (follow R.plan)
void launch_trace_fill_resumed(const CtlDev& c, const BatchDev& b, const LosDev& L,
                               const int* order, int r0, int nr, const TraceResume& R, int role,
                               unsigned* err, cudaStream_t s);
void launch_los_bound_mixed(const CtlDev& c, const BatchDev& b, double scale, int* cap,
                            cudaStream_t s);
void launch_trace_fill(const CtlDev& c, const ChanDev& ch, const BatchDev& b, const LosDev& L,
                       unsigned* err, cudaStream_t s);
void launch_path_fp64(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                      const LosDev& L, double* refl_scratch, cudaStream_t s);
void launch_srcfunc(int nd, int id0, int nch, const int* fn_off, const double* fnu,
                    const double* f, const double* st, double* sr, cudaStream_t s);
void launch_hydrostatic(const CtlDev& c, const BatchDev& b, double* p_out, cudaStream_t s);
// loads the kernels above onto the current device (JGB_OK or JGB_ERR_CUDA)
int preload_fp64_kernels();

// jgb_noalloc.cu: loads the allocation-free entry point's scratch array and
// kernels onto the device and resolves the array's address there (called by
// jgb_create with the device current; a failure is reported by the entry
// point's first call, which retries)
int noalloc_prepare(int device);

// jgb_mixed.cu
struct MixedPlan {
  int ntile;
  int* perm;            // [ntile*32]
  long long* toff;      // [ntile+1]
  int* tlen;            // [ntile]
  float* data;          // tile planes
  int nfield;
  unsigned brmask;      // emitters with p-T brackets precomputed per LOS point
  // split path (latency-bound batches): segment emissivity and saturation
  // flag of every (tile point, channel, emitter, lane), else nullptr
  float* seg_eps;
  unsigned char* seg_sat;
  // tiles [tile0, tile1) of this launch
  int tile0, tile1;
  // block shape of the path kernel: 0 = the 4 warps of a block take 4
  // channels of one tile (they share the tile's LOS data), 1 = one channel
  // of 4 consecutive tiles (they share the table rows: similar rays at
  // similar p-T)
  int tile_major;
  // resumed forward models (finite-difference perturbations): start[r] is
  // the LOS point ray r starts at (its state read from snap, slot r); ray r
  // saves the path state for the rays snap_ray[k] before its point
  // snap_ip[k], k in [snap_off[r], snap_off[r+1]); nullptr: no resume
  const int* start;
  const int* snap_off;
  const int* snap_ip;
  const int* snap_ray;
  float* snap;          // [nray][nd][kStateWords * ng + 3]
  // resumed launches, emitters shared with the base ray: a perturbation of
  // one emitter's mixing ratio (or of an extinction) leaves the other
  // emitters' inputs and path states equal to the base's.  The base launch
  // (reuse == nullptr) writes every emitter's segment emissivity at
  // seg_base[((L.off[rb] + ip) * nd + id) * ng + g] and the emitters'
  // saturation flags as bits of seg_satm[(L.off[rb] + ip) * nd + id], the
  // points it walked in seg_nvalid[rb * nd + id] and its final emitter states
  // at seg_final[(rb * nd + id) * kStateWords * ng]; a perturbed ray r with
  // reuse[r] = {rb, pg}, rb >= 0, takes every emitter but pg (pg < 0: all)
  // from there while ip < nvalid and continues from the base's final states
  // after that.  nullptr seg_base: nothing shared.
  float* seg_base;
  unsigned* seg_satm;
  int* seg_nvalid;
  unsigned* seg_final;
  const int2* reuse;
};
int mixed_nfield(const CtlDev& c, unsigned brmask);
void launch_pack_tiles_n(const CtlDev& c, const TblDev& T, const LosDev& L, const MixedPlan& P,
                         long long total_tile_points, cudaStream_t s);
// register-cap variants of the path kernel (each with both block shapes:
// variant v = cap + path_mixed_caps() * shape)
int path_mixed_caps();
int path_mixed_variants();
// the path split over emitters: one warp per (tile, channel, emitter) for the
// emitter path states, then the combination and radiance per (tile, channel)
void launch_path_split(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                       const LosDev& L, const MixedPlan& P, float* refl_scratch, cudaStream_t s);
// the path of tiles [P.tile0, P.tile1) with resume points and state snapshots
void launch_path_resume(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                        const LosDev& L, const MixedPlan& P, cudaStream_t s);
// words of one saved path state (per ray and channel)
int path_state_words(const CtlDev& c);
void launch_path_mixed(const CtlDev& c, const TblDev& T, const ChanDev& ch, const BatchDev& b,
                       const LosDev& L, const MixedPlan& P, float* refl_scratch, int variant,
                       cudaStream_t s);
void launch_src_to_float(int nd, const double* sr, float* srf, cudaStream_t s);
void launch_tables_to_float(long long n, const double* src, float* dst, cudaStream_t s);
void launch_rowmeta(long long nrow, int tu, const int* nu, const float* u, const float* e,
                    const float* tf, int cga, float4* meta, float2* ue, cudaStream_t s);

// jgb_retrieval.cu: frees an engine's device and pinned memory and unties
// it from its context (which is being destroyed); the handle then accepts
// only jgb_engine_destroy, every other call returns JGB_ERR_STATE
void engine_detach(jgb_engine* E);

// jgb_api.cu: read-only view of a context for entry points defined in other
// translation units.  Returns JGB_OK, or an error code with the context's
// message set when tables or source functions are missing.
struct CtxView {
  int device;
  cudaStream_t stream;
  CtlDev c;
  TblDev T;
  ChanDev ch;
};
int ctx_view(jgb_ctx* x, CtxView* out);  // fills *out; returns JGB_ERR_STATE if not ready

// jgb_normal.cu: batched normal-equation products on device buffers.
// Problems are concatenated (K blocks m_i x n_i, A blocks n_i x n_i, ...);
// sel (host, nullptr = all) picks the problems computed, the others' blocks
// are left untouched.  At most 65535 selected problems per call.
int normal_equations_dev(int nret, const int* m, const int* n, const double* K, const double* w,
                         const double* dy, double* A, double* b, int precision, const int* sel,
                         void* desc_dev, cudaStream_t s);
size_t normal_desc_bytes(int nret);
int ctx_fail(jgb_ctx* x, int code, const char* msg);

// The context's (recursive) lock for the duration of a public call: host
// threads may share a context, and their calls run one after another.
void ctx_lock(jgb_ctx* x);
void ctx_unlock(jgb_ctx* x);
struct CtxLock {
  jgb_ctx* x;
  explicit CtxLock(const jgb_ctx* c) : x(const_cast<jgb_ctx*>(c)) {
    if (x) ctx_lock(x);
  }
  ~CtxLock() {
    if (x) ctx_unlock(x);
  }
  CtxLock(const CtxLock&) = delete;
  CtxLock& operator=(const CtxLock&) = delete;
};

}  // namespace jgb
