// Two-state volumetric path tracer, single-state tracer and seed-replay
// adjoint for a heterogeneous medium in an axis-aligned box behind a null
// boundary, lit by a constant white environment (radiance 1).  The tracers
// work in box coordinates (the unit cube of the grid): a world direction d
// becomes d / box_size, so every distance along a ray stays a world distance
// and sigma_t keeps its world units.
//
// Restates the per-path algorithm of the reference:
//   plugins/twostatevolpath.py:141-385  sample_twostates (main loop)
//   plugins/twostatevolpath.py:387-479  sample_emitter_twostates (NEE with
//                                       two-state ratio tracking)
//   plugins/twostatemedium.py:15-107    sample_interaction_twostates
// and, for the adjoint, path replay backpropagation (Vicini et al. 2021) of
// the single-state estimator that a two-state integrator renders when its
// medium delegates every query to `new` (plugins/twostatemedium.py:125-151).
//
// Random-number order per path (one PCG32 stream per path):
//   film 2D, channel 1D, [camera iteration: RR 1D; on a cube hit the null
//   BSDF sample 1D + 2D], then per medium iteration: RR 1D, free flight 1D,
//   on a valid collision real/null 1D; on a real scattering event below
//   max_depth: phase 1D + 2D, NEE direction 2D, one 1D per ratio-tracking
//   step.  An escaping path draws the null BSDF sample (1D + 2D) and the RR
//   1D of the outside iteration before the environment is added.
//
// Execution shape (persistent): every warp pulls batches of path indices from
// one global counter and hands them to its idle lanes at the top of each loop
// iteration, so a lane starts a new path as soon as its path ends and a warp
// only drains at the end of the queue.  The main path and its NEE shadow walk
// share one loop body ("one free-flight step per iteration") so that lanes in
// different phases still execute the density lookup together.  Each path's
// radiance is written to a per-path slot; a separate pass sums a pixel's
// samples in sample order, so results do not depend on the schedule.
#pragma once
#include "../../include/rcv.h"
#include "rcv_common.h"
#include "rcv_device.cuh"
#include "rcv_env.cuh"

namespace rcv {

// Pinhole frame of one (sub-)sensor: origin in box coordinates, world-space
// forward / right / up (right and up scaled by the field of view).
struct CamFrame {
  V3 o, f, r, u;
};

// Packed lookup cell: 8 corners of the old and the new density, 64 bytes.
//   [0] old v000 v100 v010 v110   [1] old v001 v101 v011 v111
//   [2] new v000 ...              [3] new v001 ...
struct VolJob {
  // film / camera
  int32_t width, height, spp;
  int32_t n_cams;      // sub-sensors of a batch film (1 = a single sensor)
  float inv_w, inv_h;  // 1/width, 1/height
  // box transform: a world direction d moves by d * inv_box in box
  // coordinates, so distances along a ray stay world distances
  V3 inv_box;
  CamFrame cam[RCV_MAX_SENSORS];
  // integrator
  int32_t max_depth, rr_depth, hide_emitters;
  uint32_t seed;
  // medium
  int32_t dx, dy, dz;
  float scale;
  const float4* __restrict__ cells;   // (dz+1)(dy+1)(dx+1) * 4
  const float4* __restrict__ albedo;  // adz*ady*adx * 2 (old, new) or null
  int32_t adx, ady, adz;              // albedo grid resolution
  int32_t albedo_own_res;             // 1: differs from the density's
  float albedo_const[3];
  const uint32_t* maxbits;  // [0] max old density, [1] max new density (bits)
  // adjoint (forward mode: grad_cells / grad_albedo hold the packed tangent
  // field, out_img receives the image derivative)
  const float* grad_img;
  float4* grad_cells;   // (dz+1)(dy+1)(dx+1) * 2
  // albedo cell records ((adz+1)(ady+1)(adx+1) x 6 float4: 8 corners x RGB),
  // or in forward mode the tangent as one float4 per albedo voxel; or null
  float4* grad_albedo;
  float* out_img;
  int64_t path_begin;   // first global path index of this job (batched launches)
  int64_t path_count;   // width*height*spp
  const uint32_t* pixel_order;  // pixel handed out k-th (null = row-major)
  uint32_t* pixel_cost;         // per-pixel sum of path lengths (loop iterations), or null
  // majorant supergrid: cells per axis (0 = one global majorant) and the
  // cells' majorants for the two-state tracer / the single-state tracers
  int32_t sg[3];
  float sg_inv[3];  // 1 / sg (host-computed)
  const float* sg_two;
  const float* sg_new;
  // environment: a prepared map, or env.valid = 0 for the constant white
  // environment; box = the world size of the medium box (to turn a box
  // direction back into a world direction for the map)
  EnvMap env;
  V3 box;
};

// Work queue of a (possibly multi-job) persistent launch.
struct Queue {
  unsigned long long* counter;   // next unclaimed global path index (zeroed)
  float4* path_out;              // primal: per-path radiance [path][new, old]
  unsigned long long* counters;  // RCV_COUNTER_* totals of the launch or null
  const VolJob* jobs;            // device job table (batched launches) or null
  int64_t total;                 // paths in the launch (replay: camera tasks)
  int32_t batch;                 // paths claimed per warp fetch
  int32_t njobs;
  int32_t defer;                 // lanes that must wait before a deferred branch runs
  int32_t pad;
  // adjoint: scatter checkpoints (4 float4 each), how many were claimed (may
  // exceed the capacity) and per-path (total radiance, lost flag)
  float4* ckpt;
  unsigned long long* ckpt_count;
  int64_t ckpt_cap;
  float4* path_ltot;
  // kTape: the gradient-event tape (one float4 per event: position, reference)
  // with its claimed slots (whole chunks; may exceed the capacity), the
  // event records (2 float4 each, in the checkpoint buffer, counted by
  // ckpt_count) and the paths whose events did not fit.  kReplay with a lost
  // list replays only the paths on it.
  float4* tape;
  unsigned long long* tape_count;
  int64_t tape_cap;
  uint32_t* lost_list;
  unsigned long long* lost_count;
  // one float per tape slot: the event's sigma_n = majorant - sigma_t of
  // the new state (null collisions, shadow-walk steps) or sigma_t
  // (scattering events), so that the gradient pass needs no grid lookup
  float* tape_f;
};

// kForward: the replay tasks of kReplay, gathering a tangent field at every
// gradient event (forward-mode derivative of the image) instead of
// scattering the image gradient into the grids.
// kTape: the radiance pass of kAdjoint that, instead of checkpoints, records
// every gradient event of the path (main-walk null collisions, real
// scattering events, shadow-walk steps) on a tape; the gradient then comes
// from one flat pass over the tape (rcv_tape.cu) instead of replay tasks.
enum TraceMode { kTwoState = 0, kSingle = 1, kAdjoint = 2, kReplay = 3, kForward = 4, kTape = 5 };
constexpr int kTraceModes = 6;

// Tape events: float4 (x, y, z, ref) with ref = kind << 30 | index.  The
// index is the path (kEvCamera: null collisions before the first scattering
// event) or the event record of the last scattering event (kEvSegment: null
// collisions after its shadow walk; kEvScatter: the event itself; kEvShadow:
// steps of its shadow walk).  Event record (2 float4): [path, radiance
// gathered before the event's NEE contribution] [NEE contribution, 0].
enum TapeEvent : uint32_t { kEvCamera = 0, kEvSegment = 1, kEvScatter = 2, kEvShadow = 3 };
constexpr uint32_t kTapeIndexMask = 0x3fffffffu;
constexpr uint32_t kTapeEmpty = 0xffffffffu;  // unused slot at the end of a warp's last chunk
constexpr uint32_t kTapeChunk = 256;          // slots a warp claims at a time

// Slots [cur, end) of the tape chunk a warp fills (warp-uniform).
struct TapeCursor {
  uint32_t cur, end;
};

// Appends kWords consecutive float4 (a, then b) for each lane with `has` to
// the warp's tape chunk, in lane order, claiming a new chunk of kTapeChunk
// slots when the current one runs out; a chunk is only claimed whole inside
// the capacity.  A tape holds events of one size only (so an event never
// straddles two chunks).  Called by the whole warp.  Returns false on the
// lanes whose event did not fit.
template <int kWords>
__device__ __forceinline__ bool tape_append_n(const Queue& Q, TapeCursor& tc, bool has, const float4& a,
                                              const float4& b, float f = 0.0f) {
  const unsigned m = __ballot_sync(0xffffffffu, has);
  if (m == 0u) return true;
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t n = (uint32_t)__popc(m) * kWords, q = (uint32_t)__popc(m & ((1u << lane) - 1u)) * kWords;
  const uint32_t rem = tc.end - tc.cur;
  uint32_t nb = 0xffffffffu;  // start of the newly claimed chunk, if any
  if (n > rem) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(Q.tape_count, (unsigned long long)kTapeChunk);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c + kTapeChunk <= (unsigned long long)Q.tape_cap) nb = (uint32_t)c;
  }
  bool ok = true;
  if (has) {
    uint32_t slot = 0;
    if (q < rem) {
      slot = tc.cur + q;
    } else if (nb != 0xffffffffu) {
      slot = nb + (q - rem);
    } else {
      ok = false;
    }
    if (ok) {
      __stcs(Q.tape + slot, a);
      if (kWords == 2) __stcs(Q.tape + slot + 1, b);
      if (kWords == 1 && Q.tape_f != nullptr) __stcs(Q.tape_f + slot, f);
    }
  }
  if (n <= rem) {
    tc.cur += n;
  } else if (nb != 0xffffffffu) {
    tc.cur = nb + (n - rem);
    tc.end = nb + kTapeChunk;
  } else {
    tc.cur = tc.end;  // the tape is full: later events of this warp do not fit either
  }
  return ok;
}

// One-slot event (position, reference) of the volume tape, with its
// extinction term (sigma_n, or sigma_t at a scattering event).
__device__ __forceinline__ bool tape_append(const Queue& Q, TapeCursor& tc, bool has, const V3& x, uint32_t ref,
                                            float f) {
  const float4 a = make_float4(x.x, x.y, x.z, __uint_as_float(ref));
  return tape_append_n<1>(Q, tc, has, a, a, f);
}

// Marks the unused slots of the warp's last chunk empty (slot word .w =
// kTapeEmpty).  Called by the whole warp at exit.
__device__ __forceinline__ void tape_close(const Queue& Q, const TapeCursor& tc) {
  for (uint32_t i = tc.cur + (threadIdx.x & 31u); i < tc.end; i += 32u)
    __stcs(Q.tape + i, make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(kTapeEmpty)));
}

// Buffers of the two adjoint launches.
struct AdjBuffers {
  float4* ckpt;
  unsigned long long* ckpt_count;
  int64_t ckpt_cap;
  float4* path_ltot;
  float4* tape;  // null: checkpoints and replay tasks
  unsigned long long* tape_count;
  int64_t tape_cap;
  uint32_t* lost_list;
  unsigned long long* lost_count;
  float* tape_f;  // each event's sigma_n (sigma_t at scattering events)
};

struct Counts {
  uint32_t paths, lookups, nee_lookups, scatters;
  uint32_t grad_events, albedo_events;  // adjoint: density / albedo scatters
};

__device__ __forceinline__ float bits_to_float(uint32_t b) { return __uint_as_float(b); }

// A world direction in box coordinates (exact identity for the unit cube).
__device__ __forceinline__ V3 to_box(const VolJob& J, const V3& w) {
  return V3{w.x * J.inv_box.x, w.y * J.inv_box.y, w.z * J.inv_box.z};
}

// Camera ray of film position (px + u0, py + u1), origin and direction in box
// coordinates.  A batch film hands the position s = (px + u0) / width to
// sub-sensor k = min(floor(s n), n - 1) as s n - floor(s n) (Mitsuba's batch
// sensor, sensors/batch.cpp sample_ray).
__device__ __forceinline__ void camera_ray(const VolJob& J, int px, int py, float u0, float u1,
                                           V3& o, V3& d) {
  const float fx = (float)px + u0;
  const float fy = (float)py + u1;
  float nx = fx * J.inv_w;
  const float ny = fy * J.inv_h;
  int k = 0;
  if (J.n_cams > 1) {
    const float idx_f = nx * (float)J.n_cams;
    const int idx = (int)idx_f;
    k = idx < J.n_cams - 1 ? idx : J.n_cams - 1;
    nx = idx_f - (float)idx;
  }
  const CamFrame& C = J.cam[k];
  const float a = fmaf(2.0f, nx, -1.0f);
  const float b = fmaf(-2.0f, ny, 1.0f);
  V3 r;
  r.x = fmaf(b, C.u.x, fmaf(a, C.r.x, C.f.x));
  r.y = fmaf(b, C.u.y, fmaf(a, C.r.y, C.f.y));
  r.z = fmaf(b, C.u.z, fmaf(a, C.r.z, C.f.z));
  const float inv_len = 1.0f / sqrtf(fmaf(r.z, r.z, fmaf(r.y, r.y, r.x * r.x)));
  d = to_box(J, V3{r.x * inv_len, r.y * inv_len, r.z * inv_len});
  o = C.o;
}

struct Lookup {
  Axis ax, ay, az;
  uint32_t cell;  // (dx+1)(dy+1)(dz+1) * 4 < 2^32 is enforced on the host
};

__device__ __forceinline__ Lookup locate(const VolJob& J, const V3& x) {
  Lookup l;
  l.ax = axis_coord(x.x, J.dx);
  l.ay = axis_coord(x.y, J.dy);
  l.az = axis_coord(x.z, J.dz);
  l.cell = ((uint32_t)l.az.cell * (uint32_t)(J.dy + 1) + (uint32_t)l.ay.cell) * (uint32_t)(J.dx + 1) +
           (uint32_t)l.ax.cell;
  return l;
}

__device__ __forceinline__ void density2(const VolJob& J, const Lookup& l, float& rho_old,
                                         float& rho_new) {
  const float4* c = J.cells + l.cell * 4;
  const float4 o0 = __ldg(c + 0), o1 = __ldg(c + 1), n0 = __ldg(c + 2), n1 = __ldg(c + 3);
  rho_old = trilerp(o0, o1, l.ax.f, l.ay.f, l.az.f);
  rho_new = trilerp(n0, n1, l.ax.f, l.ay.f, l.az.f);
}

__device__ __forceinline__ float density_new(const VolJob& J, const Lookup& l) {
  const float4* c = J.cells + l.cell * 4;
  const float4 n0 = __ldg(c + 2), n1 = __ldg(c + 3);
  return trilerp(n0, n1, l.ax.f, l.ay.f, l.az.f);
}

__device__ __forceinline__ int clampi(int v, int hi) { return v < 0 ? 0 : (v > hi ? hi : v); }

// ------------------------------------------------------- majorant supergrid
// DDA set-up along one axis: cell of o, distance to the next cell face and
// between faces, step direction (inv_n = 1 / S; one division).
__device__ __forceinline__ void dda_axis(float o, float d, int S, float inv_n, int& c, float& tn, float& td,
                                         int& step) {
  c = clampi((int)floorf(o * (float)S), S - 1);
  if (d > 0.0f) {
    const float inv_d = 1.0f / d;
    tn = ((float)(c + 1) * inv_n - o) * inv_d;
    td = inv_n * inv_d;
    step = 1;
  } else if (d < 0.0f) {
    const float inv_d = 1.0f / d;
    tn = ((float)c * inv_n - o) * inv_d;
    td = -(inv_n * inv_d);
    step = -1;
  } else {
    tn = kInf;
    td = kInf;
    step = 0;
  }
}

// Free-flight distance of optical depth `tau` along o + t d, t in [0, tmax],
// through the majorant supergrid (plugins/twostatemedium.py:25-70): a DDA
// walk (Amanatides & Woo) accumulates majorant x segment length per cell and
// stops inside the cell where tau is reached.  The segment's majorant is the
// DDA's current cell (the reference looks the grid up at the segment's
// midpoint: the same cell up to floating-point ties on cell faces), and the
// sampled collision takes that cell's majorant, so sigma_n >= 0.  Returns
// kInf when the walk leaves the segment.
// The walk keeps its state in scalars (a dynamically indexed array would
// live in local memory).
__device__ __forceinline__ float supergrid_flight(const VolJob& J, const float* __restrict__ maj, const V3& o,
                                                  const V3& d, float tmax, float tau, float& mu_at) {
  int c0, c1, c2, s0, s1, s2;
  float tn0, tn1, tn2, td0, td1, td2;
  dda_axis(o.x, d.x, J.sg[0], J.sg_inv[0], c0, tn0, td0, s0);
  dda_axis(o.y, d.y, J.sg[1], J.sg_inv[1], c1, tn1, td1, s1);
  dda_axis(o.z, d.z, J.sg[2], J.sg_inv[2], c2, tn2, td2, s2);
  const int sx = J.sg[0], sxy = J.sg[0] * J.sg[1];
  float t = 0.0f, tau_acc = 0.0f;
  const int max_steps = J.sg[0] + J.sg[1] + J.sg[2] + 4;
  for (int s = 0; s < max_steps; ++s) {
    const float t_next = fminf(fminf(tn0, tn1), tn2);
    const float m = __ldg(maj + clampi(c2, J.sg[2] - 1) * sxy + clampi(c1, J.sg[1] - 1) * sx +
                          clampi(c0, J.sg[0] - 1));
    const float tau_next = tau_acc + m * (t_next - t);
    if (m > 0.0f && tau_next >= tau) {
      const float t_hit = t + (tau - tau_acc) / m;
      if (!(t_hit < tmax)) return kInf;
      mu_at = m;
      return t_hit;
    }
    if (!(t_next < tmax)) break;
    if (tn0 == t_next) {
      tn0 += td0;
      c0 += s0;
    } else if (tn1 == t_next) {
      tn1 += td1;
      c1 += s1;
    } else {
      tn2 += td2;
      c2 += s2;
    }
    t = t_next;
    tau_acc = tau_next;
  }
  return kInf;
}

// Albedo grid coordinates of a point: the density lookup's when both grids
// have one resolution, else its own (both grids span the unit cube).
struct AlbedoLookup {
  Axis ax, ay, az;
};

__device__ __forceinline__ AlbedoLookup albedo_lookup(const VolJob& J, const Lookup& l, const V3& x) {
  if (!J.albedo_own_res) return AlbedoLookup{l.ax, l.ay, l.az};
  return AlbedoLookup{axis_coord(x.x, J.adx), axis_coord(x.y, J.ady), axis_coord(x.z, J.adz)};
}

// Trilinear RGB albedo of one state (state 0 = old, 1 = new).
__device__ __forceinline__ V3 albedo_at(const VolJob& J, const AlbedoLookup& l, int state) {
  if (J.albedo == nullptr) return V3{J.albedo_const[0], J.albedo_const[1], J.albedo_const[2]};
  const int x0 = clampi(l.ax.cell - 1, J.adx - 1), x1 = clampi(l.ax.cell, J.adx - 1);
  const int y0 = clampi(l.ay.cell - 1, J.ady - 1), y1 = clampi(l.ay.cell, J.ady - 1);
  const int z0 = clampi(l.az.cell - 1, J.adz - 1), z1 = clampi(l.az.cell, J.adz - 1);
  auto at = [&](int x, int y, int z) {
    return __ldg(J.albedo + (((int64_t)z * J.ady + y) * J.adx + x) * 2 + state);
  };
  const float4 a000 = at(x0, y0, z0), a100 = at(x1, y0, z0), a010 = at(x0, y1, z0),
               a110 = at(x1, y1, z0), a001 = at(x0, y0, z1), a101 = at(x1, y0, z1),
               a011 = at(x0, y1, z1), a111 = at(x1, y1, z1);
  const float fx = l.ax.f, fy = l.ay.f, fz = l.az.f;
  V3 r;
  {
    const float c00 = lerpf(a000.x, a100.x, fx), c10 = lerpf(a010.x, a110.x, fx);
    const float c01 = lerpf(a001.x, a101.x, fx), c11 = lerpf(a011.x, a111.x, fx);
    r.x = lerpf(lerpf(c00, c10, fy), lerpf(c01, c11, fy), fz);
  }
  {
    const float c00 = lerpf(a000.y, a100.y, fx), c10 = lerpf(a010.y, a110.y, fx);
    const float c01 = lerpf(a001.y, a101.y, fx), c11 = lerpf(a011.y, a111.y, fx);
    r.y = lerpf(lerpf(c00, c10, fy), lerpf(c01, c11, fy), fz);
  }
  {
    const float c00 = lerpf(a000.z, a100.z, fx), c10 = lerpf(a010.z, a110.z, fx);
    const float c01 = lerpf(a001.z, a101.z, fx), c11 = lerpf(a011.z, a111.z, fx);
    r.z = lerpf(lerpf(c00, c10, fy), lerpf(c01, c11, fy), fz);
  }
  return r;
}

// Scatters g * (trilinear weight of each corner) into the cell gradient with
// two vector reductions (red.global.add.v4.f32).
__device__ __forceinline__ void scatter_density(const VolJob& J, const Lookup& l, float g) {
  const float fx = l.ax.f, fy = l.ay.f, fz = l.az.f;
  const float gx0 = 1.0f - fx, gy0 = 1.0f - fy, gz0 = 1.0f - fz;
  const float a = g * gz0, b = g * fz;
  const float a0 = a * gy0, a1 = a * fy, b0 = b * gy0, b1 = b * fy;
  float4* dst = J.grad_cells + l.cell * 2;
  red_add_v4(dst + 0, a0 * gx0, a0 * fx, a1 * gx0, a1 * fx);
  red_add_v4(dst + 1, b0 * gx0, b0 * fx, b1 * gx0, b1 * fx);
}

// Scatters g (RGB) * (trilinear weight of each corner) into the albedo
// cell's gradient record (8 corners x RGB = 24 floats, 96 bytes): six vector
// reductions of consecutive floats, none of them padding.  The fold resolves
// the clamping of edge cells to voxels.
__device__ __forceinline__ void scatter_albedo(const VolJob& J, const AlbedoLookup& l, const V3& g) {
  const float fx = l.ax.f, fy = l.ay.f, fz = l.az.f;
  const float gx0 = 1.0f - fx, gy0 = 1.0f - fy, gz0 = 1.0f - fz;
  const float w0 = gz0 * gy0, w1 = gz0 * fy, w2 = fz * gy0, w3 = fz * fy;
  const float w[8] = {w0 * gx0, w0 * fx, w1 * gx0, w1 * fx, w2 * gx0, w2 * fx, w3 * gx0, w3 * fx};
  const int64_t cell = ((int64_t)l.az.cell * (J.ady + 1) + l.ay.cell) * (J.adx + 1) + l.ax.cell;
  float4* dst = J.grad_albedo + cell * 6;
#pragma unroll
  for (int q = 0; q < 6; ++q) {
    float v[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int f = q * 4 + e;  // corner f / 3, channel f % 3
      const int c = f % 3;
      v[e] = (c == 0 ? g.x : (c == 1 ? g.y : g.z)) * w[f / 3];
    }
    red_add_v4(dst + q, v[0], v[1], v[2], v[3]);
  }
}

// Forward mode: the tangent of the density at a lookup (trilinear over the
// cell record in grad_cells, the layout scatter_density writes) and of the
// albedo (grad_albedo, one float4 per albedo voxel).
__device__ __forceinline__ float tangent_density(const VolJob& J, const Lookup& l) {
  const float4* c = J.grad_cells + l.cell * 2;
  return trilerp(__ldg(c), __ldg(c + 1), l.ax.f, l.ay.f, l.az.f);
}

__device__ __forceinline__ V3 tangent_albedo(const VolJob& J, const AlbedoLookup& l) {
  const int x0 = clampi(l.ax.cell - 1, J.adx - 1), x1 = clampi(l.ax.cell, J.adx - 1);
  const int y0 = clampi(l.ay.cell - 1, J.ady - 1), y1 = clampi(l.ay.cell, J.ady - 1);
  const int z0 = clampi(l.az.cell - 1, J.adz - 1), z1 = clampi(l.az.cell, J.adz - 1);
  auto at = [&](int x, int y, int z) { return __ldg(J.grad_albedo + ((int64_t)z * J.ady + y) * J.adx + x); };
  const float4 a000 = at(x0, y0, z0), a100 = at(x1, y0, z0), a010 = at(x0, y1, z0), a110 = at(x1, y1, z0),
               a001 = at(x0, y0, z1), a101 = at(x1, y0, z1), a011 = at(x0, y1, z1), a111 = at(x1, y1, z1);
  const float fx = l.ax.f, fy = l.ay.f, fz = l.az.f;
  auto tri = [&](float v000, float v100, float v010, float v110, float v001, float v101, float v011, float v111) {
    return lerpf(lerpf(lerpf(v000, v100, fx), lerpf(v010, v110, fx), fy),
                 lerpf(lerpf(v001, v101, fx), lerpf(v011, v111, fx), fy), fz);
  };
  return V3{tri(a000.x, a100.x, a010.x, a110.x, a001.x, a101.x, a011.x, a111.x),
            tri(a000.y, a100.y, a010.y, a110.y, a001.y, a101.y, a011.y, a111.y),
            tri(a000.z, a100.z, a010.z, a110.z, a001.z, a101.z, a011.z, a111.z)};
}

// Russian roulette at the top of an iteration (plugins/twostatevolpath.py:182-188).
// Returns false when the path terminates.
template <int kMode>
__device__ __forceinline__ bool roulette(const VolJob& J, Pcg32& rng, int depth, V3& bn, V3& bo) {
  bool alive = (bn.x != 0.0f || bn.y != 0.0f || bn.z != 0.0f);
  if (kMode == kTwoState) alive = alive || (bo.x != 0.0f || bo.y != 0.0f || bo.z != 0.0f);
  if (!alive) return false;
  float m = fmaxf(fmaxf(bn.x, bn.y), bn.z);
  if (kMode == kTwoState) m = fmaxf(fmaxf(fmaxf(bn.x, bo.x), fmaxf(bn.y, bo.y)), fmaxf(bn.z, bo.z));
  const float q = fminf(m, 0.99f);
  if (depth > J.rr_depth) {
    const float u = next1d(rng);
    if (!(u < q)) return false;
    const float inv = 1.0f / q;
    bn = V3{bn.x * inv, bn.y * inv, bn.z * inv};
    if (kMode == kTwoState) bo = V3{bo.x * inv, bo.y * inv, bo.z * inv};
  } else {
    pcg_skip1(rng);  // the draw is made but its value is unused
  }
  return true;
}

// ---------------------------------------- host launchers (rcv_volume.cu)
// Validates a medium + sensor + options and fills a job for one launch.
int make_volume_job(const rcv_medium* m, const rcv_sensor* s, const rcv_volpath_options* o, uint32_t seed,
                    int spp, VolJob* J);
// Writes the job's pixels into `order`, most expensive first: by `cost` (the
// per-pixel path lengths of the previous call, cleared here) or, when cost is
// null, by the chord length of the pixel's centre ray through the medium
// (buckets: 256 uint32 of scratch).
int order_pixels(const VolJob& J, uint32_t* buckets, uint32_t* order, uint32_t* cost, cudaStream_t st);
// Clears the medium workspace's cell (and albedo) gradient accumulators.
int reset_gradients(const rcv_medium* m, bool albedo, cudaStream_t st);
// Adds the folded voxel gradients of the medium workspace to grad_density
// (and grad_albedo when set and the medium has an albedo grid).
int launch_fold(const rcv_medium* m, float* grad_density, float* grad_albedo, cudaStream_t st);
// Bucket (0 = first handed out) of a pixel by the chord of its centre ray
// through the medium cube (misses last).
__device__ __forceinline__ int chord_key(const VolJob& J, int pix) {
  V3 o, d;
  camera_ray(J, pix % J.width, pix / J.width, 0.5f, 0.5f, o, d);
  float tn, tf;
  slab(o, recip(d), tn, tf);
  const float chord = (tn <= tf && tf > 0.0f) ? tf - fmaxf(tn, 0.0f) : 0.0f;
  int b = (int)(chord * (255.0f / 1.7320508f));
  b = b < 0 ? 0 : (b > 255 ? 255 : b);
  return 255 - b;
}

// Places the pixels of one block in their buckets: block-local ranks from a
// shared histogram, one global reservation per (block, bucket), so a popular
// bucket costs one global atomic per block instead of one per pixel.  Order
// within a bucket is arbitrary (it never changes results).
__device__ __forceinline__ void place_block(int key, bool valid, uint32_t pix, uint32_t* starts,
                                            uint32_t* order) {
  __shared__ uint32_t cnt[256], base[256];
  for (int k = threadIdx.x; k < 256; k += blockDim.x) cnt[k] = 0u;
  __syncthreads();
  const uint32_t rank = valid ? atomicAdd(&cnt[key], 1u) : 0u;
  __syncthreads();
  for (int k = threadIdx.x; k < 256; k += blockDim.x) base[k] = cnt[k] ? atomicAdd(starts + k, cnt[k]) : 0u;
  __syncthreads();
  if (valid) order[base[key] + rank] = pix;
}

// Bucket (0 = first handed out) of a pixel of cost c.
__device__ __forceinline__ int cost_bucket(uint32_t c) {
  if (c == 0u) return 255;
  const int b = (int)(log2f((float)c) * 16.0f);
  return 254 - (b < 254 ? b : 254);
}
// Persistent tracer launch (TraceMode `mode`) over `total` paths of one job
// (jobs == NULL) or of a device job table of njobs entries.
// supergrid: some job of the table has a majorant supergrid (the kernel
// variant that can traverse one is launched; single jobs decide from J.sg).
int launch_persistent(int mode, const VolJob& J, const VolJob* jobs, int njobs, int64_t total,
                      const rcv_volpath_options* o, unsigned long long* queue_counter, float4* path_out,
                      const AdjBuffers* adj, uint64_t* counters, cudaStream_t st, bool supergrid);
// Work queue of a persistent tracer launch (the arguments of
// launch_persistent); zeroes its hand-out counter on `st`.
int make_queue(int mode, const VolJob* jobs, int njobs, int64_t total, const rcv_volpath_options* o,
               unsigned long long* queue_counter, float4* path_out, const AdjBuffers* adj, uint64_t* counters,
               cudaStream_t st, Queue* out);
// One persistent launch of two tracers (rcv_pair.cu): the two-state primal
// over QA and the tape radiance pass over QB, each of a single job (JA, JB:
// the same medium and environment) or both of job tables (supergrid: some
// job of the tables has a majorant supergrid).
int launch_pair(const VolJob& JA, const Queue& QA, const VolJob& JB, const Queue& QB, const rcv_volpath_options* o,
                cudaStream_t st, bool supergrid);
void warm_pair_config();
// Queries the occupancy and SM count the launchers cache, so that later
// launches (e.g. under stream capture) make no device queries.
void warm_launch_config();
// The extinction terms follow the tape's slots in the tape region (16 B +
// 4 B per slot).
inline float* tape_terms(char* region, int64_t paths) {
  return reinterpret_cast<float*>(region + tape_capacity(paths, kTapeSlotsPerPath) * 16);
}

// Gradient from a kTape radiance pass (rcv_tape.cu) of one job (jobs ==
// NULL) or of a device job table: the per-record and per-path weights
// (`weights`: 2 float4 per record, `cam_w`: one float2 per path) and the
// scatter of every tape event into its job's gradient records.
int launch_tape_gradient(const VolJob& single, const VolJob* jobs, int njobs, const AdjBuffers& A, float4* weights,
                         float2* cam_w, int64_t paths, uint64_t* counters, int sms, cudaStream_t st);
int tracer_sm_count();

}  // namespace rcv
