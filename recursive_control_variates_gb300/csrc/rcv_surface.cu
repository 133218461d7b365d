// Surface two-state tracer kernels and their C-ABI entry points: texture
// packing, persistent two-state / single-state / adjoint launches and the
// texture-gradient fold.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "rcv_common.h"
#include "rcv_surface.cuh"

namespace rcv {

constexpr int kSurfBlock = 128;

__global__ void pack_texture_kernel(int64_t n, const float* __restrict__ old_t,
                                    const float* __restrict__ new_t, float4* __restrict__ pairs) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  pairs[i * 2 + 0] = make_float4(old_t[i * 3 + 0], old_t[i * 3 + 1], old_t[i * 3 + 2], 0.0f);
  pairs[i * 2 + 1] = make_float4(new_t[i * 3 + 0], new_t[i * 3 + 1], new_t[i * 3 + 2], 0.0f);
}

__global__ void fold_texture_kernel(int64_t n, const float4* __restrict__ g, float* __restrict__ out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 v = g[i];
  out[i * 3 + 0] += v.x;
  out[i * 3 + 1] += v.y;
  out[i * 3 + 2] += v.z;
}

template <int kMode>
__global__ void __launch_bounds__(kSurfBlock) trace_surface_kernel(const __grid_constant__ SurfJob S,
                                                                   const __grid_constant__ Queue Q) {
  SurfCounts cnt{0, 0, 0, 0, 0};
  trace_surface<kMode>(S, Q, cnt);
  if (Q.counters == nullptr) return;
  const unsigned p = __reduce_add_sync(0xffffffffu, cnt.paths);
  const unsigned b = __reduce_add_sync(0xffffffffu, cnt.bounces);
  const unsigned s = __reduce_add_sync(0xffffffffu, cnt.shadow_rays);
  const unsigned t = __reduce_add_sync(0xffffffffu, cnt.tex_vertices);
  const unsigned g = __reduce_add_sync(0xffffffffu, cnt.grad_events);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(Q.counters + RCV_COUNTER_PATHS, (unsigned long long)p);
    atomicAdd(Q.counters + RCV_COUNTER_LOOKUPS, (unsigned long long)b);
    atomicAdd(Q.counters + RCV_COUNTER_NEE_LOOKUPS, (unsigned long long)s);
    atomicAdd(Q.counters + RCV_COUNTER_SCATTERS, (unsigned long long)t);
    if (g) atomicAdd(Q.counters + RCV_COUNTER_GRAD_EVENTS, (unsigned long long)g);
  }
}

struct SurfLayout {
  uint64_t pairs, grad, total;
};

static SurfLayout surf_layout(int tw, int th) {
  const uint64_t n = uint64_t(tw) * uint64_t(th);
  SurfLayout L;
  L.pairs = 0;
  L.grad = align256(n * 32u);
  L.total = align256(L.grad + n * 16u);
  return L;
}

static int validate_scene(const rcv_surface_scene* sc) {
  RCV_REQUIRE(sc != nullptr, "surface scene is NULL");
  RCV_REQUIRE(sc->tex_width > 0 && sc->tex_height > 0, "texture size must be positive");
  RCV_REQUIRE(uint64_t(sc->tex_width) * uint64_t(sc->tex_height) < (uint64_t(1) << 30),
              "texture too large");
  RCV_REQUIRE(sc->tex_old != nullptr && sc->tex_new != nullptr, "textures are NULL");
  RCV_REQUIRE(sc->num_spheres >= 0 && sc->num_spheres <= RCV_MAX_SPHERES, "num_spheres must be in [0, %d]",
              RCV_MAX_SPHERES);
  RCV_REQUIRE(sc->plane_half > 0.0f, "plane_half must be positive");
  RCV_REQUIRE(sc->light_half[0] > 0.0f && sc->light_half[1] > 0.0f, "light extents must be positive");
  RCV_REQUIRE(sc->workspace != nullptr && (reinterpret_cast<uintptr_t>(sc->workspace) & 255u) == 0,
              "surface workspace must be non-NULL and 256-byte aligned");
  for (int k = 0; k < sc->num_spheres; ++k)
    RCV_REQUIRE(sc->spheres[k].radius > 0.0f, "sphere radius must be positive");
  return RCV_OK;
}

static int make_surf_job(const rcv_surface_scene* sc, const rcv_sensor* s, const rcv_volpath_options* o,
                         uint32_t seed, int spp, SurfJob* S) {
  int rc = validate_scene(sc);
  if (rc) return rc;
  RCV_REQUIRE(s != nullptr && o != nullptr, "sensor / options are NULL");
  RCV_REQUIRE(s->width > 0 && s->height > 0, "film size must be positive");
  RCV_REQUIRE(s->count <= 1, "the surface tracer renders a single sensor (batch sensors: media only)");
  RCV_REQUIRE(spp > 0, "spp must be positive");
  RCV_REQUIRE(o->max_depth >= -1, "max_depth must be >= -1");
  RCV_REQUIRE(int64_t(s->width) * s->height * spp < (int64_t(1) << 32),
              "width * height * spp must be below 2^32 (one random stream per path)");
  std::memset(S, 0, sizeof(SurfJob));
  S->width = s->width;
  S->height = s->height;
  S->spp = spp;
  S->max_depth = o->max_depth < 0 ? 0x7fffffff : o->max_depth;
  S->rr_depth = o->rr_depth;
  S->hide_emitters = o->hide_emitters;
  S->seed = seed;
  S->cam_o = V3{s->origin[0], s->origin[1], s->origin[2]};
  S->cam_f = V3{s->forward[0], s->forward[1], s->forward[2]};
  S->cam_r = V3{s->right[0], s->right[1], s->right[2]};
  S->cam_u = V3{s->up[0], s->up[1], s->up[2]};
  S->inv_w = 1.0f / (float)s->width;
  S->inv_h = 1.0f / (float)s->height;
  S->plane_half = sc->plane_half;
  S->tex_w = sc->tex_width;
  S->tex_h = sc->tex_height;
  const SurfLayout L = surf_layout(sc->tex_width, sc->tex_height);
  char* ws = static_cast<char*>(sc->workspace);
  S->tex = reinterpret_cast<const float4*>(ws + L.pairs);
  S->nspheres = sc->num_spheres;
  for (int k = 0; k < sc->num_spheres; ++k) {
    const rcv_sphere& q = sc->spheres[k];
    S->sph[k] = Sphere{V3{q.center[0], q.center[1], q.center[2]}, q.radius,
                       V3{q.albedo[0], q.albedo[1], q.albedo[2]}};
  }
  S->light_c = V3{sc->light_center[0], sc->light_center[1], sc->light_center[2]};
  S->light_hx = sc->light_half[0];
  S->light_hz = sc->light_half[1];
  S->light_area = (2.0f * sc->light_half[0]) * (2.0f * sc->light_half[1]);
  S->light_le = V3{sc->light_radiance[0], sc->light_radiance[1], sc->light_radiance[2]};
  S->path_count = int64_t(s->width) * s->height * spp;
  return RCV_OK;
}

__global__ void pack_texture_tangent_kernel(int64_t n, const float* __restrict__ t, float4* __restrict__ out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = make_float4(t[i * 3 + 0], t[i * 3 + 1], t[i * 3 + 2], 0.0f);
}

// Gradient from the surface tape: per recorded texture vertex (2 float4:
// [x, z, path, 0] [radiance gathered before the vertex]),
// dL * (L - gathered) / albedo scattered bilinearly into the texels, as the
// replay pass of kAdjoint does at the same vertex.  Vertices of paths that
// lost one are skipped (the replay takes those paths).
__global__ void __launch_bounds__(256) surface_tape_scatter_kernel(const __grid_constant__ SurfJob S,
                                                                   const float4* __restrict__ tape,
                                                                   const unsigned long long* __restrict__ tape_count,
                                                                   int64_t tape_cap,
                                                                   const float4* __restrict__ ltot) {
  const int64_t n = min((int64_t)*tape_count, tape_cap) / 2;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float4 a = __ldcs(tape + 2 * i);
    if (__float_as_uint(a.w) == kTapeEmpty) continue;
    const float4 b = __ldcs(tape + 2 * i + 1);
    const uint32_t path = __float_as_uint(a.z);
    const float4 lt = __ldg(ltot + path);
    if (lt.w != 0.0f) continue;
    const int pix = (int)(path / (uint32_t)S.spp);
    const float fs = (float)S.spp;
    const float* g = S.grad_img + (int64_t)pix * 3;
    const V3 dL{g[0] / fs, g[1] / fs, g[2] / fs};
    const TexLookup tl = tex_locate(S, V3{a.x, 0.0f, a.y});
    const V3 an = tex_eval(S, tl, 1);
    const V3 lr{lt.x - b.x, lt.y - b.y, lt.z - b.z};
    tex_scatter(S, tl,
                V3{(dL.x * lr.x) / fmaxf(an.x, 1e-8f), (dL.y * lr.y) / fmaxf(an.y, 1e-8f),
                   (dL.z * lr.z) / fmaxf(an.z, 1e-8f)});
  }
}

static int surf_resident_blocks(int mode) {
  static std::once_flag once;
  static int blocks[5] = {1, 1, 1, 1, 1};
  std::call_once(once, [] {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[0], trace_surface_kernel<kTwoState>, kSurfBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[1], trace_surface_kernel<kSingle>, kSurfBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[2], trace_surface_kernel<kAdjoint>, kSurfBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[3], trace_surface_kernel<kForward>, kSurfBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[4], trace_surface_kernel<kTape>, kSurfBlock, 0);
    for (int& b : blocks) b = b < 1 ? 1 : b;
  });
  return blocks[mode == kForward ? 3 : (mode == kTape ? 4 : mode)];
}

static int launch_surface(int mode, const SurfJob& S, const Queue& Q, const rcv_volpath_options* o,
                          cudaStream_t st) {
  RCV_TRY_CUDA(cudaMemsetAsync(Q.counter, 0, sizeof(unsigned long long), st), "queue reset");
  const int sms = tracer_sm_count();
  int per_sm = surf_resident_blocks(mode);
  if (o != nullptr && o->blocks_per_sm > 0 && o->blocks_per_sm < per_sm) per_sm = o->blocks_per_sm;
  int64_t blocks = ((S.path_count + Q.batch - 1) / Q.batch + (kSurfBlock / 32) - 1) / (kSurfBlock / 32);
  if (blocks > int64_t(sms) * per_sm) blocks = int64_t(sms) * per_sm;
  if (blocks < 1) blocks = 1;
  switch (mode) {
    case kTwoState: trace_surface_kernel<kTwoState><<<(unsigned)blocks, kSurfBlock, 0, st>>>(S, Q); break;
    case kSingle: trace_surface_kernel<kSingle><<<(unsigned)blocks, kSurfBlock, 0, st>>>(S, Q); break;
    case kForward: trace_surface_kernel<kForward><<<(unsigned)blocks, kSurfBlock, 0, st>>>(S, Q); break;
    case kTape: trace_surface_kernel<kTape><<<(unsigned)blocks, kSurfBlock, 0, st>>>(S, Q); break;
    default: trace_surface_kernel<kAdjoint><<<(unsigned)blocks, kSurfBlock, 0, st>>>(S, Q); break;
  }
  return launched("trace_surface launch");
}

static int run_surface(int mode, const SurfJob& S, const rcv_volpath_options* o, void* workspace,
                       uint64_t* counters, float* img_new, float* img_old, cudaStream_t st) {
  RCV_REQUIRE(workspace != nullptr && (reinterpret_cast<uintptr_t>(workspace) & 255u) == 0,
              "render workspace must be non-NULL and 256-byte aligned");
  const int64_t npix = int64_t(S.width) * S.height;
  const RenderLayout L = render_layout(npix, S.path_count, mode);
  char* ws = static_cast<char*>(workspace);
  Queue Q;
  std::memset(&Q, 0, sizeof(Q));
  Q.counter = reinterpret_cast<unsigned long long*>(ws + L.counter);
  const bool adj = mode == kAdjoint || mode == kForward;
  Q.path_out = adj ? nullptr : reinterpret_cast<float4*>(ws + L.path_out);
  Q.counters = reinterpret_cast<unsigned long long*>(counters);
  Q.total = S.path_count;
  Q.batch = (o != nullptr && o->batch > 0) ? o->batch : 64;
  RCV_REQUIRE(Q.batch <= (1 << 20), "batch must be <= 2^20");
  Q.defer = 1;
  const int adjoint = o == nullptr ? RCV_ADJOINT_TAPE : o->adjoint;
  RCV_REQUIRE(adjoint == RCV_ADJOINT_TAPE || adjoint == RCV_ADJOINT_REPLAY, "unknown adjoint %d", adjoint);
  if (mode == kAdjoint && adjoint == RCV_ADJOINT_TAPE && S.path_count < (int64_t(1) << 28)) {
    // one pass records the texture vertices, one flat pass scatters them, and
    // the replay takes the paths whose vertices did not fit (2 slots each)
    const int per_path = (o == nullptr || o->tape_events_per_path == 0) ? int(kTapeSlotsPerPath)
                                                                      : o->tape_events_per_path;
    RCV_REQUIRE(per_path >= 1 && per_path <= kTapeSlotsPerPath, "tape_events_per_path must be in [0, %d]",
                int(kTapeSlotsPerPath));
    unsigned long long* qc = Q.counter;
    Q.tape = reinterpret_cast<float4*>(ws + L.tape);
    Q.tape_count = qc + 2;
    Q.tape_cap = tape_capacity(S.path_count, per_path) & ~int64_t(1);
    Q.lost_list = reinterpret_cast<uint32_t*>(ws + L.lost);
    Q.lost_count = qc + 3;
    Q.path_ltot = reinterpret_cast<float4*>(ws + L.ltot);
    RCV_TRY_CUDA(cudaMemsetAsync(qc + 2, 0, 2 * sizeof(unsigned long long), st), "tape counters reset");
    int rc = launch_surface(kTape, S, Q, o, st);
    if (rc) return rc;
    const int block = 256;
    const int sms = tracer_sm_count();
    surface_tape_scatter_kernel<<<(unsigned)sms * 8u, block, 0, st>>>(S, Q.tape, Q.tape_count, Q.tape_cap,
                                                                       Q.path_ltot);
    rc = launched("surface_tape_scatter launch");
    if (rc) return rc;
    return launch_surface(kAdjoint, S, Q, o, st);  // the lost-path list only
  }
  int rc = launch_surface(mode, S, Q, o, st);
  if (rc || adj) return rc;
  return launch_reduce(mode == kTwoState, reinterpret_cast<const float4*>(ws + L.path_out), 0, npix, S.spp,
                       img_new, img_old, st);
}

}  // namespace rcv

using namespace rcv;

extern "C" uint64_t rcv_surface_workspace_bytes(int32_t tex_width, int32_t tex_height) {
  if (tex_width <= 0 || tex_height <= 0) return 0;
  return surf_layout(tex_width, tex_height).total;
}

extern "C" int rcv_surface_prepare(const rcv_surface_scene* sc, void* stream) {
  int rc = validate_scene(sc);
  if (rc) return rc;
  const SurfLayout L = surf_layout(sc->tex_width, sc->tex_height);
  const int64_t n = int64_t(sc->tex_width) * sc->tex_height;
  const int block = 256;
  pack_texture_kernel<<<grid_for(n, block), block, 0, static_cast<cudaStream_t>(stream)>>>(
      n, sc->tex_old, sc->tex_new, reinterpret_cast<float4*>(static_cast<char*>(sc->workspace) + L.pairs));
  return launched("pack_texture launch");
}

extern "C" int rcv_render_twostates_surface(const rcv_surface_scene* sc, const rcv_sensor* s,
                                            const rcv_volpath_options* o, uint32_t seed, int32_t spp,
                                            float* img_old, float* img_new, void* workspace,
                                            uint64_t* counters, void* stream) {
  SurfJob S;
  int rc = make_surf_job(sc, s, o, seed, spp, &S);
  if (rc) return rc;
  RCV_REQUIRE(img_old != nullptr && img_new != nullptr, "output images are NULL");
  return run_surface(kTwoState, S, o, workspace, counters, img_new, img_old, static_cast<cudaStream_t>(stream));
}

extern "C" int rcv_render_surface(const rcv_surface_scene* sc, const rcv_sensor* s,
                                  const rcv_volpath_options* o, uint32_t seed, int32_t spp, float* img,
                                  void* workspace, uint64_t* counters, void* stream) {
  SurfJob S;
  int rc = make_surf_job(sc, s, o, seed, spp, &S);
  if (rc) return rc;
  RCV_REQUIRE(img != nullptr, "output image is NULL");
  return run_surface(kSingle, S, o, workspace, counters, img, nullptr, static_cast<cudaStream_t>(stream));
}

extern "C" int rcv_render_backward_surface(const rcv_surface_scene* sc, const rcv_sensor* s,
                                           const rcv_volpath_options* o, uint32_t seed, int32_t spp,
                                           const float* grad_img, float* grad_texture, void* workspace,
                                           uint64_t* counters, void* stream) {
  SurfJob S;
  int rc = make_surf_job(sc, s, o, seed, spp, &S);
  if (rc) return rc;
  RCV_REQUIRE(grad_img != nullptr && grad_texture != nullptr, "gradient buffers are NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const SurfLayout L = surf_layout(sc->tex_width, sc->tex_height);
  char* ws = static_cast<char*>(sc->workspace);
  const int64_t n = int64_t(sc->tex_width) * sc->tex_height;
  RCV_TRY_CUDA(cudaMemsetAsync(ws + L.grad, 0, n * 16, st), "texture gradient reset");
  S.grad_img = grad_img;
  S.grad_tex = reinterpret_cast<float4*>(ws + L.grad);
  rc = run_surface(kAdjoint, S, o, workspace, counters, nullptr, nullptr, st);
  if (rc) return rc;
  const int block = 256;
  fold_texture_kernel<<<grid_for(n, block), block, 0, st>>>(n, reinterpret_cast<const float4*>(ws + L.grad),
                                                           grad_texture);
  return launched("fold_texture launch");
}

// Forward mode of the surface path replay along a texture tangent
// ([tex_h][tex_w][3], device): dimg ([height][width][3], overwritten).
extern "C" int rcv_render_forward_surface(const rcv_surface_scene* sc, const rcv_sensor* s,
                                          const rcv_volpath_options* o, uint32_t seed, int32_t spp,
                                          const float* tangent_texture, float* dimg, void* workspace,
                                          uint64_t* counters, void* stream) {
  SurfJob S;
  int rc = make_surf_job(sc, s, o, seed, spp, &S);
  if (rc) return rc;
  RCV_REQUIRE(tangent_texture != nullptr && dimg != nullptr, "tangent / output buffers are NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const SurfLayout L = surf_layout(sc->tex_width, sc->tex_height);
  char* ws = static_cast<char*>(sc->workspace);
  const int64_t n = int64_t(sc->tex_width) * sc->tex_height;
  // the texture gradient record holds the tangent during the call
  const int block = 256;
  pack_texture_tangent_kernel<<<grid_for(n, block), block, 0, st>>>(n, tangent_texture,
                                                                   reinterpret_cast<float4*>(ws + L.grad));
  rc = launched("pack_texture_tangent launch");
  if (rc) return rc;
  RCV_TRY_CUDA(cudaMemsetAsync(dimg, 0, size_t(S.width) * S.height * 3 * sizeof(float), st), "derivative reset");
  S.grad_tex = reinterpret_cast<float4*>(ws + L.grad);
  S.out_img = dimg;
  return run_surface(kForward, S, o, workspace, counters, nullptr, nullptr, st);
}
