// Host-side helpers shared by the librcv translation units: error reporting
// and workspace layout.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/rcv.h"

namespace rcv {

void set_error(const char* fmt, ...);

inline int cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return RCV_ERR_CUDA;
  }
  return RCV_OK;
}

// Counts one kernel launch of librcv (see rcv_kernel_launches) and reports a
// launch failure.
void count_launch();
// Adds delta (may be negative) to the launch count.
void add_launches(int64_t delta);
inline int launched(const char* what) {
  count_launch();
  return cuda_check(cudaGetLastError(), what);
}

#define RCV_TRY_CUDA(expr, what)                       \
  do {                                                   \
    int _rc = ::rcv::cuda_check((expr), (what));         \
    if (_rc != RCV_OK) return _rc;                       \
  } while (0)

#define RCV_REQUIRE(cond, ...)        \
  do {                                \
    if (!(cond)) {                    \
      ::rcv::set_error(__VA_ARGS__);  \
      return RCV_ERR_INVALID;         \
    }                                 \
  } while (0)

inline uint64_t align256(uint64_t v) { return (v + 255u) & ~uint64_t(255u); }

// Majorant supergrid cells along an axis of D voxels for factor f (0 = none).
inline int supergrid_cells(int D, int f) { return f > 0 ? (D + f - 1) / f : 0; }

// Layout of the medium workspace (all sections 256-byte aligned).  With a
// majorant supergrid: its cells for the two-state tracer (max of both
// states) and for the single-state tracers (new state).
struct MediumLayout {
  uint64_t cells, albedo, maxbits, grad_cells, grad_albedo, sg_two, sg_new, total;
};

// albedo_dims: resolution of the albedo grid (null = no albedo grid).  The
// albedo gradient is kept per albedo lookup cell like the density's: 8
// corners x RGB = 24 floats (96 B, six 16-byte vector reductions per event).
inline MediumLayout medium_layout(const int32_t dims[3], const int32_t* albedo_dims, int majorant_factor) {
  const uint64_t nc = uint64_t(dims[0] + 1) * uint64_t(dims[1] + 1) * uint64_t(dims[2] + 1);
  const bool has_albedo = albedo_dims != nullptr;
  const uint64_t nv = has_albedo ? uint64_t(albedo_dims[0]) * uint64_t(albedo_dims[1]) * uint64_t(albedo_dims[2]) : 0u;
  const uint64_t nca =
      has_albedo ? uint64_t(albedo_dims[0] + 1) * uint64_t(albedo_dims[1] + 1) * uint64_t(albedo_dims[2] + 1) : 0u;
  const uint64_t ns = uint64_t(supergrid_cells(dims[0], majorant_factor)) *
                      uint64_t(supergrid_cells(dims[1], majorant_factor)) *
                      uint64_t(supergrid_cells(dims[2], majorant_factor));
  MediumLayout l;
  uint64_t off = 0;
  l.cells = off;
  off = align256(off + nc * 64u);
  l.albedo = off;
  off = align256(off + nv * 32u);
  l.maxbits = off;
  off = align256(off + 16u);
  l.grad_cells = off;
  off = align256(off + nc * 32u);
  l.grad_albedo = off;
  off = align256(off + nca * 96u);
  l.sg_two = off;
  off = align256(off + ns * 4u);
  l.sg_new = off;
  off = align256(off + ns * 4u);
  l.total = off;
  return l;
}

// Bytes of the albedo gradient records of an albedo grid of the given
// resolution: one 96-byte record per lookup cell.
inline uint64_t albedo_grad_bytes(const int32_t ad[3]) {
  return uint64_t(ad[0] + 1) * uint64_t(ad[1] + 1) * uint64_t(ad[2] + 1) * 96u;
}

// Albedo grid resolution of a medium: its own when set, else the density's.
inline void albedo_dims_of(const rcv_medium* m, int32_t out[3]) {
  const bool own = m->albedo_dims[0] > 0 || m->albedo_dims[1] > 0 || m->albedo_dims[2] > 0;
  for (int a = 0; a < 3; ++a) out[a] = own ? m->albedo_dims[a] : m->dims[a];
}

inline uint64_t albedo_voxels_of(const rcv_medium* m) {
  if (m->albedo_old == nullptr) return 0;
  int32_t ad[3];
  albedo_dims_of(m, ad);
  return uint64_t(ad[0]) * uint64_t(ad[1]) * uint64_t(ad[2]);
}

inline MediumLayout medium_layout(const rcv_medium* m) {
  int32_t ad[3];
  albedo_dims_of(m, ad);
  return medium_layout(m->dims, m->albedo_old != nullptr ? ad : nullptr, m->majorant_factor);
}

// Scratch layout of one tracer call (all offsets 256-byte aligned):
// counters (queue, checkpoints / event records, tape slots, lost paths) |
// order bucket counts | pixel order | per-pixel cost | per-path radiance (32 B
// per path for two-state, 16 B single-state) | adjoint: per-path total
// radiance | scatter checkpoints (tape: event records, then their weights) |
// event tape | per-path camera-segment weight | lost-path list.
constexpr int kRenderOrderBuckets = 256;

struct RenderLayout {
  uint64_t counter, buckets, order, cost, path_out, ltot, ckpt, tape, cam_w, lost, total;
};

// Adjoint scatter checkpoints: 64 bytes each, room for 2 per path plus a
// margin; paths whose checkpoints do not fit are replayed whole.  The tape
// adjoint keeps its 32-byte event records in the first half of the same
// buffer and their 32-byte weights in the second.
inline int64_t ckpt_capacity(int64_t paths) { return 2 * paths + 65536; }

// Event tape of the adjoint: 16 bytes per event, kTapeSlotsPerPath per path
// (whole chunks of kTapeChunkSlots, the unit a warp claims), followed by one
// 4-byte extinction term per slot (volume tape).
constexpr int64_t kTapeSlotsPerPath = 16;
constexpr int64_t kTapeChunkSlots = 256;
inline int64_t tape_capacity(int64_t paths, int per_path) {
  const int64_t slots = paths * (int64_t)per_path;
  return (slots + kTapeChunkSlots - 1) / kTapeChunkSlots * kTapeChunkSlots;
}

inline uint64_t path_out_bytes(int64_t paths, int mode) {
  return mode == RCV_MODE_ADJOINT ? 0u : uint64_t(paths) * (mode == RCV_MODE_TWOSTATE ? 32u : 16u);
}

inline RenderLayout render_layout(int64_t npix, int64_t paths, int mode) {
  RenderLayout L;
  L.counter = 0;
  L.buckets = 256;
  L.order = align256(L.buckets + kRenderOrderBuckets * sizeof(uint32_t));
  L.cost = align256(L.order + uint64_t(npix) * sizeof(uint32_t));
  L.path_out = align256(L.cost + uint64_t(npix) * sizeof(uint32_t));
  const bool adj = mode == RCV_MODE_ADJOINT;
  L.ltot = align256(L.path_out + path_out_bytes(paths, mode));
  L.ckpt = align256(L.ltot + (adj ? uint64_t(paths) * 16u : 0u));
  L.tape = align256(L.ckpt + (adj ? uint64_t(ckpt_capacity(paths)) * 64u : 0u));
  L.cam_w = align256(L.tape + (adj ? uint64_t(tape_capacity(paths, kTapeSlotsPerPath)) * 20u : 0u));
  L.lost = align256(L.cam_w + (adj ? uint64_t(paths) * 8u : 0u));
  L.total = align256(L.lost + (adj ? uint64_t(paths) * 4u : 0u));
  return L;
}

// Per-pixel sum of per-path radiance slots in sample order (rcv_volume.cu).
int launch_reduce(bool two, const float4* po, int64_t path_begin, int64_t npix, int spp,
                  float* out_new, float* out_old, cudaStream_t st);

inline unsigned grid_for(int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  return (unsigned)g;
}

}  // namespace rcv
