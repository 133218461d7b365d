// Volumetric kernels of librcv and their C-ABI entry points:
// medium packing + majorants, two-state primal, single-state primal,
// seed-replay adjoint and the gradient fold back to voxel layout.
#include <cuda_runtime.h>

#include <cstring>

#include "rcv_common.h"
#include "rcv_volume.cuh"

namespace rcv {

// ------------------------------------------------------------------ packing
__global__ void pack_medium_kernel(int dx, int dy, int dz, const float* __restrict__ old_d,
                                   const float* __restrict__ new_d, float4* __restrict__ cells,
                                   const float* __restrict__ old_a, const float* __restrict__ new_a,
                                   float4* __restrict__ albedo, uint32_t* __restrict__ maxbits) {
  const int64_t nc = int64_t(dx + 1) * (dy + 1) * (dz + 1);
  const int64_t nv = int64_t(dx) * dy * dz;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  float mo = 0.0f, mn = 0.0f;
  if (i < nc) {
    const int cx = int(i % (dx + 1));
    const int cy = int((i / (dx + 1)) % (dy + 1));
    const int cz = int(i / (int64_t(dx + 1) * (dy + 1)));
    const int x0 = clampi(cx - 1, dx - 1), x1 = clampi(cx, dx - 1);
    const int y0 = clampi(cy - 1, dy - 1), y1 = clampi(cy, dy - 1);
    const int z0 = clampi(cz - 1, dz - 1), z1 = clampi(cz, dz - 1);
    auto idx = [&](int x, int y, int z) { return (int64_t(z) * dy + y) * dx + x; };
    const int64_t i000 = idx(x0, y0, z0), i100 = idx(x1, y0, z0), i010 = idx(x0, y1, z0),
                  i110 = idx(x1, y1, z0), i001 = idx(x0, y0, z1), i101 = idx(x1, y0, z1),
                  i011 = idx(x0, y1, z1), i111 = idx(x1, y1, z1);
    float4* c = cells + i * 4;
    c[0] = make_float4(old_d[i000], old_d[i100], old_d[i010], old_d[i110]);
    c[1] = make_float4(old_d[i001], old_d[i101], old_d[i011], old_d[i111]);
    c[2] = make_float4(new_d[i000], new_d[i100], new_d[i010], new_d[i110]);
    c[3] = make_float4(new_d[i001], new_d[i101], new_d[i011], new_d[i111]);
  }
  if (i < nv) {
    mo = old_d[i];
    mn = new_d[i];
    if (albedo != nullptr) {
      albedo[i * 2 + 0] = make_float4(old_a[i * 3 + 0], old_a[i * 3 + 1], old_a[i * 3 + 2], 0.0f);
      albedo[i * 2 + 1] = make_float4(new_a[i * 3 + 0], new_a[i * 3 + 1], new_a[i * 3 + 2], 0.0f);
    }
  }
  // majorant: maximum density of each state (non-negative part)
  mo = fmaxf(mo, 0.0f);
  mn = fmaxf(mn, 0.0f);
  uint32_t bo = __float_as_uint(mo), bn = __float_as_uint(mn);
  bo = __reduce_max_sync(0xffffffffu, bo);
  bn = __reduce_max_sync(0xffffffffu, bn);
  if ((threadIdx.x & 31) == 0) {
    if (bo) atomicMax(maxbits + 0, bo);
    if (bn) atomicMax(maxbits + 1, bn);
  }
}

// ----------------------------------------------------------------- tracing
__device__ __forceinline__ void add_counts(unsigned long long* counters, const Counts& c) {
  if (counters == nullptr) return;
  const unsigned p = __reduce_add_sync(0xffffffffu, c.paths);
  const unsigned l = __reduce_add_sync(0xffffffffu, c.lookups);
  const unsigned n = __reduce_add_sync(0xffffffffu, c.nee_lookups);
  const unsigned s = __reduce_add_sync(0xffffffffu, c.scatters);
  const unsigned ge = __reduce_add_sync(0xffffffffu, c.grad_events);
  const unsigned ae = __reduce_add_sync(0xffffffffu, c.albedo_events);
  if ((threadIdx.x & 31) == 0) {
    if (ge) atomicAdd(counters + RCV_COUNTER_GRAD_EVENTS, (unsigned long long)ge);
    if (ae) atomicAdd(counters + RCV_COUNTER_ALBEDO_EVENTS, (unsigned long long)ae);
    atomicAdd(counters + RCV_COUNTER_PATHS, (unsigned long long)p);
    atomicAdd(counters + RCV_COUNTER_LOOKUPS, (unsigned long long)l);
    atomicAdd(counters + RCV_COUNTER_NEE_LOOKUPS, (unsigned long long)n);
    atomicAdd(counters + RCV_COUNTER_SCATTERS, (unsigned long long)s);
  }
}

// One thread per (pixel, group of `chunk` samples); the spp/chunk threads of
// a pixel are adjacent lanes and combine their sums with a butterfly.
template <int kMode>
__device__ __forceinline__ void trace_thread(const VolJob& J, int64_t local, bool active) {
  const int T = J.spp / J.chunk;
  V3 ao{0, 0, 0}, an{0, 0, 0};
  Counts cnt{0, 0, 0, 0, 0, 0};
  int pix = 0, k = 0;
  if (active) {
    pix = int(local / T);
    k = int(local % T);
    trace_samples<kMode>(J, pix, k * J.chunk, (k + 1) * J.chunk, ao, an, cnt);
  }
  if (kMode != kAdjoint) {
    for (int off = 1; off < T; off <<= 1) {
      an.x += __shfl_xor_sync(0xffffffffu, an.x, off);
      an.y += __shfl_xor_sync(0xffffffffu, an.y, off);
      an.z += __shfl_xor_sync(0xffffffffu, an.z, off);
      if (kMode == kTwoState) {
        ao.x += __shfl_xor_sync(0xffffffffu, ao.x, off);
        ao.y += __shfl_xor_sync(0xffffffffu, ao.y, off);
        ao.z += __shfl_xor_sync(0xffffffffu, ao.z, off);
      }
    }
    if (active && k == 0) {
      const float fs = (float)J.spp;
      float* dn = J.out_new + int64_t(pix) * 3;
      dn[0] = an.x / fs;
      dn[1] = an.y / fs;
      dn[2] = an.z / fs;
      if (kMode == kTwoState) {
        float* d0 = J.out_old + int64_t(pix) * 3;
        d0[0] = ao.x / fs;
        d0[1] = ao.y / fs;
        d0[2] = ao.z / fs;
      }
    }
  }
  add_counts(J.counters, cnt);
}

template <int kMode>
__global__ void __launch_bounds__(128) trace_kernel(const __grid_constant__ VolJob J) {
  const int64_t gt = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  trace_thread<kMode>(J, gt, gt < J.thread_count);
}

// ------------------------------------------------------------ gradient fold
__device__ __forceinline__ int fold_candidates(int i, int D, int* cell, int* bit) {
  int n = 0;
  for (int c = i; c <= i + 1 && c <= D; ++c)
    for (int b = 0; b < 2; ++b) {
      const int v = clampi(c - 1 + b, D - 1);
      if (v == i) {
        cell[n] = c;
        bit[n] = b;
        ++n;
      }
    }
  return n;
}

__global__ void fold_density_kernel(int dx, int dy, int dz, const float* __restrict__ gcells,
                                    float* __restrict__ grad) {
  const int64_t nv = int64_t(dx) * dy * dz;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const int x = int(i % dx), y = int((i / dx) % dy), z = int(i / (int64_t(dx) * dy));
  int cxs[4], bxs[4], cys[4], bys[4], czs[4], bzs[4];
  const int nx = fold_candidates(x, dx, cxs, bxs);
  const int ny = fold_candidates(y, dy, cys, bys);
  const int nz = fold_candidates(z, dz, czs, bzs);
  float g = 0.0f;
  for (int a = 0; a < nz; ++a)
    for (int b = 0; b < ny; ++b)
      for (int c = 0; c < nx; ++c) {
        const int64_t cell = (int64_t(czs[a]) * (dy + 1) + cys[b]) * (dx + 1) + cxs[c];
        g += gcells[cell * 8 + bxs[c] + 2 * bys[b] + 4 * bzs[a]];
      }
  grad[i] += g;
}

__global__ void fold_albedo_kernel(int64_t nv, const float4* __restrict__ ga,
                                   float* __restrict__ grad) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const float4 g = ga[i];
  grad[i * 3 + 0] += g.x;
  grad[i * 3 + 1] += g.y;
  grad[i * 3 + 2] += g.z;
}

// ------------------------------------------------------------- host helpers
static int validate_medium(const rcv_medium* m) {
  RCV_REQUIRE(m != nullptr, "medium is NULL");
  RCV_REQUIRE(m->dims[0] > 0 && m->dims[1] > 0 && m->dims[2] > 0, "grid dims must be positive");
  RCV_REQUIRE(m->density_old != nullptr && m->density_new != nullptr, "density grids are NULL");
  RCV_REQUIRE((m->albedo_old == nullptr) == (m->albedo_new == nullptr),
              "albedo_old and albedo_new must both be set or both be NULL");
  RCV_REQUIRE(m->workspace != nullptr, "medium workspace is NULL");
  RCV_REQUIRE((reinterpret_cast<uintptr_t>(m->workspace) & 255u) == 0,
              "medium workspace must be 256-byte aligned");
  RCV_REQUIRE(m->scale >= 0.0f, "medium scale must be non-negative");
  return RCV_OK;
}

static int choose_chunk(int spp, int requested, int* chunk) {
  if (requested > 0) {
    RCV_REQUIRE(spp % requested == 0, "samples_per_thread (%d) must divide spp (%d)", requested, spp);
    const int T = spp / requested;
    RCV_REQUIRE(T <= 32 && (T & (T - 1)) == 0,
                "spp / samples_per_thread (%d) must be a power of two <= 32", T);
    *chunk = requested;
    return RCV_OK;
  }
  // default: as many threads per pixel as possible (<= 4), power of two
  int T = 1;
  while (T < 4 && spp % (T * 2) == 0) T *= 2;
  *chunk = spp / T;
  return RCV_OK;
}

static int make_job(const rcv_medium* m, const rcv_sensor* s, const rcv_volpath_options* o,
                    uint32_t seed, int spp, VolJob* J) {
  int rc = validate_medium(m);
  if (rc) return rc;
  RCV_REQUIRE(s != nullptr && o != nullptr, "sensor / options are NULL");
  RCV_REQUIRE(s->width > 0 && s->height > 0, "film size must be positive");
  RCV_REQUIRE(spp > 0, "spp must be positive");
  RCV_REQUIRE(o->max_depth >= 0 || o->max_depth == -1, "max_depth must be >= -1");
  std::memset(J, 0, sizeof(VolJob));
  J->width = s->width;
  J->height = s->height;
  J->spp = spp;
  rc = choose_chunk(spp, o->samples_per_thread, &J->chunk);
  if (rc) return rc;
  J->cam_o = V3{s->origin[0], s->origin[1], s->origin[2]};
  J->cam_f = V3{s->forward[0], s->forward[1], s->forward[2]};
  J->cam_r = V3{s->right[0], s->right[1], s->right[2]};
  J->cam_u = V3{s->up[0], s->up[1], s->up[2]};
  J->max_depth = o->max_depth < 0 ? 0x7fffffff : o->max_depth;
  J->rr_depth = o->rr_depth;
  J->hide_emitters = o->hide_emitters;
  J->seed = seed;
  J->dx = m->dims[0];
  J->dy = m->dims[1];
  J->dz = m->dims[2];
  J->scale = m->scale;
  const MediumLayout L = medium_layout(m->dims, m->albedo_old != nullptr);
  char* ws = static_cast<char*>(m->workspace);
  J->cells = reinterpret_cast<const float4*>(ws + L.cells);
  J->albedo = m->albedo_old ? reinterpret_cast<const float4*>(ws + L.albedo) : nullptr;
  J->albedo_const[0] = m->albedo_value[0];
  J->albedo_const[1] = m->albedo_value[1];
  J->albedo_const[2] = m->albedo_value[2];
  J->maxbits = reinterpret_cast<const uint32_t*>(ws + L.maxbits);
  J->grad_cells = reinterpret_cast<float4*>(ws + L.grad_cells);
  J->grad_albedo = m->albedo_old ? reinterpret_cast<float4*>(ws + L.grad_albedo) : nullptr;
  J->thread_begin = 0;
  J->thread_count = int64_t(s->width) * s->height * (spp / J->chunk);
  return RCV_OK;
}

template <int kMode>
static int launch_trace(const VolJob& J, cudaStream_t st) {
  const int block = 128;
  trace_kernel<kMode><<<grid_for(J.thread_count, block), block, 0, st>>>(J);
  return launched("trace kernel launch");
}

}  // namespace rcv

using namespace rcv;

extern "C" uint64_t rcv_medium_workspace_bytes(const int32_t dims[3], int32_t has_albedo_grid) {
  if (dims == nullptr || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0) return 0;
  return medium_layout(dims, has_albedo_grid != 0).total;
}

extern "C" int rcv_medium_prepare(const rcv_medium* m, void* stream) {
  int rc = validate_medium(m);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const MediumLayout L = medium_layout(m->dims, m->albedo_old != nullptr);
  char* ws = static_cast<char*>(m->workspace);
  RCV_TRY_CUDA(cudaMemsetAsync(ws + L.maxbits, 0, 16, st), "majorant reset");
  const int64_t nc = int64_t(m->dims[0] + 1) * (m->dims[1] + 1) * (m->dims[2] + 1);
  const int block = 256;
  pack_medium_kernel<<<grid_for(nc, block), block, 0, st>>>(
      m->dims[0], m->dims[1], m->dims[2], m->density_old, m->density_new,
      reinterpret_cast<float4*>(ws + L.cells), m->albedo_old, m->albedo_new,
      m->albedo_old ? reinterpret_cast<float4*>(ws + L.albedo) : nullptr,
      reinterpret_cast<uint32_t*>(ws + L.maxbits));
  return launched("pack_medium launch");
}

extern "C" int rcv_render_twostates_volume(const rcv_medium* m, const rcv_sensor* s,
                                           const rcv_volpath_options* o, uint32_t seed,
                                           int32_t spp, float* img_old, float* img_new,
                                           uint64_t* counters, void* stream) {
  VolJob J;
  int rc = make_job(m, s, o, seed, spp, &J);
  if (rc) return rc;
  RCV_REQUIRE(img_old != nullptr && img_new != nullptr, "output images are NULL");
  J.out_old = img_old;
  J.out_new = img_new;
  J.counters = reinterpret_cast<unsigned long long*>(counters);
  return launch_trace<kTwoState>(J, static_cast<cudaStream_t>(stream));
}

extern "C" int rcv_render_volume(const rcv_medium* m, const rcv_sensor* s,
                                 const rcv_volpath_options* o, uint32_t seed, int32_t spp,
                                 float* img, uint64_t* counters, void* stream) {
  VolJob J;
  int rc = make_job(m, s, o, seed, spp, &J);
  if (rc) return rc;
  RCV_REQUIRE(img != nullptr, "output image is NULL");
  J.out_new = img;
  J.counters = reinterpret_cast<unsigned long long*>(counters);
  return launch_trace<kSingle>(J, static_cast<cudaStream_t>(stream));
}

extern "C" int rcv_render_backward_volume(const rcv_medium* m, const rcv_sensor* s,
                                          const rcv_volpath_options* o, uint32_t seed,
                                          int32_t spp, const float* grad_img,
                                          float* grad_density, float* grad_albedo,
                                          uint64_t* counters, void* stream) {
  VolJob J;
  int rc = make_job(m, s, o, seed, spp, &J);
  if (rc) return rc;
  RCV_REQUIRE(grad_img != nullptr && grad_density != nullptr, "gradient buffers are NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const MediumLayout L = medium_layout(m->dims, m->albedo_old != nullptr);
  char* ws = static_cast<char*>(m->workspace);
  const int64_t nc = int64_t(m->dims[0] + 1) * (m->dims[1] + 1) * (m->dims[2] + 1);
  const int64_t nv = int64_t(m->dims[0]) * m->dims[1] * m->dims[2];
  RCV_TRY_CUDA(cudaMemsetAsync(ws + L.grad_cells, 0, nc * 32, st), "gradient reset");
  const bool want_albedo = grad_albedo != nullptr && m->albedo_old != nullptr;
  if (want_albedo) RCV_TRY_CUDA(cudaMemsetAsync(ws + L.grad_albedo, 0, nv * 16, st), "gradient reset");
  if (!want_albedo) J.grad_albedo = nullptr;
  J.grad_img = grad_img;
  J.counters = reinterpret_cast<unsigned long long*>(counters);
  rc = launch_trace<kAdjoint>(J, st);
  if (rc) return rc;
  const int block = 256;
  fold_density_kernel<<<grid_for(nv, block), block, 0, st>>>(
      m->dims[0], m->dims[1], m->dims[2], reinterpret_cast<const float*>(ws + L.grad_cells),
      grad_density);
  rc = launched("fold_density launch");
  if (rc) return rc;
  if (want_albedo) {
    fold_albedo_kernel<<<grid_for(nv, block), block, 0, st>>>(
        nv, reinterpret_cast<const float4*>(ws + L.grad_albedo), grad_albedo);
    rc = launched("fold_albedo launch");
  }
  return rc;
}
