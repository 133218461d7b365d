// Volumetric kernels of librcv and their C-ABI entry points:
// medium packing + majorants, persistent two-state primal, single-state
// primal and seed-replay adjoint, the per-pixel sample reduction and the
// gradient fold back to voxel layout.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "rcv_common.h"
#include "rcv_pack.cuh"
#include "rcv_trace.cuh"

namespace rcv {

// ------------------------------------------------------------------ packing
// One thread per cell / voxel / albedo voxel (na: albedo grid voxels).
__global__ void pack_medium_kernel(int dx, int dy, int dz, const float* __restrict__ old_d,
                                   const float* __restrict__ new_d, float4* __restrict__ cells,
                                   const float* __restrict__ old_a, const float* __restrict__ new_a,
                                   float4* __restrict__ albedo, int64_t na, uint32_t* __restrict__ maxbits) {
  const int64_t nc = int64_t(dx + 1) * (dy + 1) * (dz + 1);
  const int64_t nv = int64_t(dx) * dy * dz;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  float mo = 0.0f, mn = 0.0f;
  if (i < nc) pack_cell(i, dx, dy, dz, old_d, new_d, cells);
  if (i < nv) {
    mo = old_d[i];
    mn = new_d[i];
  }
  if (albedo != nullptr && i < na) pack_albedo(i, old_a, new_a, albedo);
  // majorant: maximum density of each state (non-negative part)
  reduce_majorants(mo, mn, maxbits);
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
    atomicAdd(counters + RCV_COUNTER_PATHS, (unsigned long long)p);
    atomicAdd(counters + RCV_COUNTER_LOOKUPS, (unsigned long long)l);
    atomicAdd(counters + RCV_COUNTER_NEE_LOOKUPS, (unsigned long long)n);
    atomicAdd(counters + RCV_COUNTER_SCATTERS, (unsigned long long)s);
    if (ge) atomicAdd(counters + RCV_COUNTER_GRAD_EVENTS, (unsigned long long)ge);
    if (ae) atomicAdd(counters + RCV_COUNTER_ALBEDO_EVENTS, (unsigned long long)ae);
  }
}

template <int kMode, bool kSG, bool kCount, bool kEnv>
__global__ void __launch_bounds__(kTraceBlock, 5) trace_kernel(const __grid_constant__ VolJob J,
                                                            const __grid_constant__ Queue Q) {
  Counts cnt{0, 0, 0, 0, 0, 0};
  trace_persistent<kMode, kSG, kCount, kEnv>(J, Q, cnt);
  if (kCount) add_counts(Q.counters, cnt);
}

// Tracer variants by index mode + kTraceModes * (supergrid + 2 * counting +
// 4 * environment map).
using TraceKernel = void (*)(VolJob, Queue);
template <bool kSG, bool kCount, bool kEnv>
struct TraceVariants {
  static constexpr TraceKernel k[kTraceModes] = {
      trace_kernel<kTwoState, kSG, kCount, kEnv>, trace_kernel<kSingle, kSG, kCount, kEnv>,
      trace_kernel<kAdjoint, kSG, kCount, kEnv>, trace_kernel<kReplay, kSG, kCount, kEnv>,
      trace_kernel<kForward, kSG, kCount, kEnv>, trace_kernel<kTape, kSG, kCount, kEnv>};
};
static const TraceKernel* const kTraceTables[8] = {
    TraceVariants<false, false, false>::k, TraceVariants<true, false, false>::k,
    TraceVariants<false, true, false>::k,  TraceVariants<true, true, false>::k,
    TraceVariants<false, false, true>::k,  TraceVariants<true, false, true>::k,
    TraceVariants<false, true, true>::k,   TraceVariants<true, true, true>::k};
constexpr int kTraceVariants = 8 * kTraceModes;

static int trace_variant(int mode, bool sg, bool count, bool env) {
  return mode + kTraceModes * ((sg ? 1 : 0) + (count ? 2 : 0) + (env ? 4 : 0));
}
static TraceKernel trace_kernel_of(int variant) { return kTraceTables[variant / kTraceModes][variant % kTraceModes]; }

// Majorant supergrid of a medium (both states' cells and the new state's).
__global__ void supergrid_kernel(int sx, int sy, int sz, int dx, int dy, int dz, float scale,
                                 const float* __restrict__ old_d, const float* __restrict__ new_d,
                                 float* __restrict__ sg_two, float* __restrict__ sg_new) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= int64_t(sx) * sy * sz) return;
  const int sg[3] = {sx, sy, sz};
  supergrid_cell(i, sg, dx, dy, dz, scale, old_d, new_d, sg_two, sg_new);
}

// ------------------------------------------------------ hand-out ordering
// Pixels are handed to the persistent tracer most-expensive first, so that
// the queue ends on cheap paths instead of on a few long ones: by the
// measured path lengths of the previous call (cost_bucket), or by the length
// of the pixel-centre ray's chord through the medium cube, in 256 buckets
// (bucket 0 = longest; misses last).
constexpr int kOrderBuckets = 256;

__device__ __forceinline__ int order_key(const VolJob& J, int pix, const uint32_t* cost) {
  return cost != nullptr ? cost_bucket(cost[pix]) : chord_key(J, pix);
}

__global__ void order_count_kernel(const __grid_constant__ VolJob J, int npix, uint32_t* counts,
                                   const uint32_t* cost) {
  __shared__ uint32_t hist[kOrderBuckets];
  for (int k = threadIdx.x; k < kOrderBuckets; k += blockDim.x) hist[k] = 0;
  __syncthreads();
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix < npix) atomicAdd(&hist[order_key(J, pix, cost)], 1u);
  __syncthreads();
  for (int k = threadIdx.x; k < kOrderBuckets; k += blockDim.x)
    if (hist[k]) atomicAdd(counts + k, hist[k]);
}

__global__ void order_scan_kernel(uint32_t* counts) {
  // exclusive prefix sum of the 256 bucket counts, in place (one block)
  __shared__ uint32_t s[kOrderBuckets];
  const int t = threadIdx.x;
  s[t] = counts[t];
  __syncthreads();
  for (int off = 1; off < kOrderBuckets; off <<= 1) {
    const uint32_t v = t >= off ? s[t - off] : 0u;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  counts[t] = t == 0 ? 0u : s[t - 1];
}

__global__ void order_place_kernel(const __grid_constant__ VolJob J, int npix, uint32_t* starts,
                                   uint32_t* order, uint32_t* cost) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = pix < npix;
  place_block(valid ? order_key(J, pix, cost) : 0, valid, (uint32_t)pix, starts, order);
  if (valid && cost != nullptr) cost[pix] = 0u;  // the next tracer call accumulates afresh
}

// Sum of a pixel's samples in sample order, divided by spp (the box-filter
// film develop of plugins/twostatevolpath.py:80-89).
template <bool kTwo>
__global__ void reduce_paths_kernel(const float4* __restrict__ path_out, int64_t path_begin,
                                    int64_t npix, int spp, float* __restrict__ out_new,
                                    float* __restrict__ out_old) {
  const int64_t pix = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (pix >= npix) return;
  V3 n, o;
  reduce_pixel<kTwo>(path_out, path_begin, pix, spp, n, o);
  out_new[pix * 3 + 0] = n.x;
  out_new[pix * 3 + 1] = n.y;
  out_new[pix * 3 + 2] = n.z;
  if (kTwo) {
    out_old[pix * 3 + 0] = o.x;
    out_old[pix * 3 + 1] = o.y;
    out_old[pix * 3 + 2] = o.z;
  }
}

// ------------------------------------------------------------ gradient fold
__global__ void fold_density_kernel(int dx, int dy, int dz, const float* __restrict__ gcells,
                                    float* __restrict__ grad) {
  const int64_t nv = int64_t(dx) * dy * dz;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  grad[i] += fold_voxel(i, dx, dy, dz, gcells);
}

__global__ void fold_albedo_kernel(int adx, int ady, int adz, const float* __restrict__ gcells,
                                   float* __restrict__ grad) {
  const int64_t nv = int64_t(adx) * ady * adz;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nv) return;
  const V3 g = fold_voxel_rgb(i, adx, ady, adz, gcells);
  grad[i * 3 + 0] += g.x;
  grad[i * 3 + 1] += g.y;
  grad[i * 3 + 2] += g.z;
}

// Forward mode: the tangent of the density packed like a cell gradient
// record (8 corners, the layout tangent_density reads), and the albedo
// tangent as one float4 per albedo voxel.
__global__ void pack_tangent_kernel(int dx, int dy, int dz, const float* __restrict__ t,
                                    float4* __restrict__ cells) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= int64_t(dx + 1) * (dy + 1) * (dz + 1)) return;
  const uint32_t ex = (uint32_t)(dx + 1), ey = (uint32_t)(dy + 1);
  const uint32_t row = (uint32_t)i / ex;
  const int cx = int((uint32_t)i - row * ex);
  const uint32_t cz_u = row / ey;
  const int cy = int(row - cz_u * ey), cz = int(cz_u);
  const int x0 = clampi(cx - 1, dx - 1), x1 = clampi(cx, dx - 1);
  const int y0 = clampi(cy - 1, dy - 1), y1 = clampi(cy, dy - 1);
  const int z0 = clampi(cz - 1, dz - 1), z1 = clampi(cz, dz - 1);
  auto v = [&](int x, int y, int z) { return t[(int64_t(z) * dy + y) * dx + x]; };
  cells[i * 2 + 0] = make_float4(v(x0, y0, z0), v(x1, y0, z0), v(x0, y1, z0), v(x1, y1, z0));
  cells[i * 2 + 1] = make_float4(v(x0, y0, z1), v(x1, y0, z1), v(x0, y1, z1), v(x1, y1, z1));
}

__global__ void pack_tangent_albedo_kernel(int64_t na, const float* __restrict__ t, float4* __restrict__ out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= na) return;
  out[i] = make_float4(t[i * 3 + 0], t[i * 3 + 1], t[i * 3 + 2], 0.0f);
}

// ------------------------------------------------------------- host helpers
static int validate_medium(const rcv_medium* m) {
  RCV_REQUIRE(m != nullptr, "medium is NULL");
  RCV_REQUIRE(m->dims[0] > 0 && m->dims[1] > 0 && m->dims[2] > 0, "grid dims must be positive");
  RCV_REQUIRE(uint64_t(m->dims[0] + 1) * uint64_t(m->dims[1] + 1) * uint64_t(m->dims[2] + 1) * 4u <
                  (uint64_t(1) << 32),
              "grid too large: (Dx+1)(Dy+1)(Dz+1) must be below 2^30");
  RCV_REQUIRE(m->density_old != nullptr && m->density_new != nullptr, "density grids are NULL");
  RCV_REQUIRE((m->albedo_old == nullptr) == (m->albedo_new == nullptr),
              "albedo_old and albedo_new must both be set or both be NULL");
  RCV_REQUIRE(m->workspace != nullptr, "medium workspace is NULL");
  RCV_REQUIRE((reinterpret_cast<uintptr_t>(m->workspace) & 255u) == 0,
              "medium workspace must be 256-byte aligned");
  RCV_REQUIRE(m->scale >= 0.0f, "medium scale must be non-negative");
  RCV_REQUIRE(m->majorant_factor >= 0, "majorant_factor must be >= 0");
  const bool own = m->albedo_dims[0] != 0 || m->albedo_dims[1] != 0 || m->albedo_dims[2] != 0;
  RCV_REQUIRE(!own || (m->albedo_dims[0] > 0 && m->albedo_dims[1] > 0 && m->albedo_dims[2] > 0),
              "albedo_dims must be all positive or all 0");
  return RCV_OK;
}

int make_volume_job(const rcv_medium* m, const rcv_sensor* s, const rcv_volpath_options* o,
                    uint32_t seed, int spp, VolJob* J) {
  int rc = validate_medium(m);
  if (rc) return rc;
  RCV_REQUIRE(s != nullptr && o != nullptr, "sensor / options are NULL");
  RCV_REQUIRE(s->width > 0 && s->height > 0, "film size must be positive");
  RCV_REQUIRE(spp > 0, "spp must be positive");
  RCV_REQUIRE(o->max_depth >= -1, "max_depth must be >= -1");
  RCV_REQUIRE(int64_t(s->width) * s->height * spp < (int64_t(1) << 32),
              "width * height * spp must be below 2^32 (one random stream per path)");
  const int n_cams = s->count > 1 ? s->count : 1;
  RCV_REQUIRE(n_cams <= RCV_MAX_SENSORS, "a batch sensor has at most %d sub-sensors", RCV_MAX_SENSORS);
  RCV_REQUIRE(s->width % n_cams == 0, "batch film width %d is not a multiple of its %d sensors", s->width,
              n_cams);
  float inv_box[3];
  for (int a = 0; a < 3; ++a) {
    RCV_REQUIRE(m->box_size[a] >= 0.0f && std::isfinite(m->box_size[a]) && std::isfinite(m->box_min[a]),
                "medium box must have a finite, non-negative size");
    inv_box[a] = m->box_size[a] > 0.0f ? 1.0f / m->box_size[a] : 1.0f;
  }
  std::memset(J, 0, sizeof(VolJob));
  J->width = s->width;
  J->height = s->height;
  J->spp = spp;
  J->n_cams = n_cams;
  J->inv_box = V3{inv_box[0], inv_box[1], inv_box[2]};
  J->box = V3{m->box_size[0] > 0.0f ? m->box_size[0] : 1.0f, m->box_size[1] > 0.0f ? m->box_size[1] : 1.0f,
              m->box_size[2] > 0.0f ? m->box_size[2] : 1.0f};
  if (o->envmap != nullptr) {
    const rcv_envmap* e = o->envmap;
    RCV_REQUIRE(e->width > 0 && e->height > 0 && e->workspace != nullptr &&
                    (reinterpret_cast<uintptr_t>(e->workspace) & 255u) == 0,
                "environment map: positive size and a 256-byte aligned workspace are required");
    RCV_REQUIRE(std::isfinite(e->scale) && e->scale >= 0.0f, "environment map scale must be finite and >= 0");
    const EnvLayout EL = env_layout(e->width, e->height);
    const char* ew = static_cast<const char*>(e->workspace);
    J->env.valid = 1;
    J->env.w = e->width;
    J->env.h = e->height;
    J->env.inv_w = 1.0f / (float)e->width;
    J->env.inv_h = 1.0f / (float)e->height;
    J->env.scale = e->scale;
    J->env.tex = reinterpret_cast<const float4*>(ew + EL.tex);
    J->env.cond = reinterpret_cast<const float*>(ew + EL.cond);
    J->env.marg = reinterpret_cast<const float*>(ew + EL.marg);
    J->env.hdr = reinterpret_cast<const float*>(ew + EL.hdr);
  }
  for (int k = 0; k < n_cams; ++k) {
    const float* o = k == 0 ? s->origin : s->more[k - 1].origin;
    const float* f = k == 0 ? s->forward : s->more[k - 1].forward;
    const float* r = k == 0 ? s->right : s->more[k - 1].right;
    const float* u = k == 0 ? s->up : s->more[k - 1].up;
    // camera origin in box coordinates; the directions stay in world space
    J->cam[k].o = V3{(o[0] - m->box_min[0]) * inv_box[0], (o[1] - m->box_min[1]) * inv_box[1],
                     (o[2] - m->box_min[2]) * inv_box[2]};
    J->cam[k].f = V3{f[0], f[1], f[2]};
    J->cam[k].r = V3{r[0], r[1], r[2]};
    J->cam[k].u = V3{u[0], u[1], u[2]};
  }
  J->inv_w = 1.0f / (float)s->width;
  J->inv_h = 1.0f / (float)s->height;
  J->max_depth = o->max_depth < 0 ? 0x7fffffff : o->max_depth;
  J->rr_depth = o->rr_depth;
  J->hide_emitters = o->hide_emitters;
  J->seed = seed;
  J->dx = m->dims[0];
  J->dy = m->dims[1];
  J->dz = m->dims[2];
  J->scale = m->scale;
  const MediumLayout L = medium_layout(m);
  char* ws = static_cast<char*>(m->workspace);
  J->cells = reinterpret_cast<const float4*>(ws + L.cells);
  J->albedo = m->albedo_old ? reinterpret_cast<const float4*>(ws + L.albedo) : nullptr;
  int32_t ad[3];
  albedo_dims_of(m, ad);
  J->adx = ad[0];
  J->ady = ad[1];
  J->adz = ad[2];
  J->albedo_own_res = (ad[0] != m->dims[0] || ad[1] != m->dims[1] || ad[2] != m->dims[2]) ? 1 : 0;
  J->albedo_const[0] = m->albedo_value[0];
  J->albedo_const[1] = m->albedo_value[1];
  J->albedo_const[2] = m->albedo_value[2];
  J->maxbits = reinterpret_cast<const uint32_t*>(ws + L.maxbits);
  J->sg[0] = supergrid_cells(m->dims[0], m->majorant_factor);
  J->sg[1] = supergrid_cells(m->dims[1], m->majorant_factor);
  J->sg[2] = supergrid_cells(m->dims[2], m->majorant_factor);
  for (int a = 0; a < 3; ++a) J->sg_inv[a] = J->sg[a] > 0 ? 1.0f / (float)J->sg[a] : 0.0f;
  J->sg_two = J->sg[0] > 0 ? reinterpret_cast<const float*>(ws + L.sg_two) : nullptr;
  J->sg_new = J->sg[0] > 0 ? reinterpret_cast<const float*>(ws + L.sg_new) : nullptr;
  J->grad_cells = reinterpret_cast<float4*>(ws + L.grad_cells);
  J->grad_albedo = m->albedo_old ? reinterpret_cast<float4*>(ws + L.grad_albedo) : nullptr;
  J->path_begin = 0;
  J->path_count = int64_t(s->width) * s->height * spp;
  return RCV_OK;
}

// Resident blocks per SM of each tracer variant (queried once per process).
static int resident_blocks(int variant) {
  static std::once_flag once;
  static int blocks[kTraceVariants];
  std::call_once(once, [] {
    for (int v = 0; v < kTraceVariants; ++v) {
      blocks[v] = 1;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[v], trace_kernel_of(v), kTraceBlock, 0);
      if (blocks[v] < 1) blocks[v] = 1;
    }
  });
  return blocks[variant];
}

static int sm_count() {
  static std::once_flag once;
  static int n = 1;
  std::call_once(once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n < 1) n = 1;
  });
  return n;
}

int tracer_sm_count() { return sm_count(); }

void warm_launch_config() {
  (void)resident_blocks(0);
  (void)sm_count();
  warm_pair_config();
}

static_assert(kOrderBuckets == kRenderOrderBuckets, "order bucket count mismatch");
static_assert(int64_t(kTapeChunk) == kTapeChunkSlots, "tape chunk mismatch");

// Fills `order` with the job's pixels, longest expected path first.
int order_pixels(const VolJob& J, uint32_t* buckets, uint32_t* order, uint32_t* cost, cudaStream_t st) {
  const int npix = J.width * J.height;
  RCV_TRY_CUDA(cudaMemsetAsync(buckets, 0, kOrderBuckets * sizeof(uint32_t), st), "order reset");
  const int block = 256;
  order_count_kernel<<<grid_for(npix, block), block, 0, st>>>(J, npix, buckets, cost);
  int rc = launched("order_count launch");
  if (rc) return rc;
  order_scan_kernel<<<1, kOrderBuckets, 0, st>>>(buckets);
  rc = launched("order_scan launch");
  if (rc) return rc;
  order_place_kernel<<<grid_for(npix, block), block, 0, st>>>(J, npix, buckets, order, cost);
  return launched("order_place launch");
}

// Work queue of a persistent launch over `total` paths of one job (jobs ==
// null) or of a device job table; zeroes its hand-out counter on `st`.
int make_queue(int mode, const VolJob* jobs, int njobs, int64_t total, const rcv_volpath_options* o,
               unsigned long long* queue_counter, float4* path_out, const AdjBuffers* adj, uint64_t* counters,
               cudaStream_t st, Queue* out) {
  Queue& Q = *out;
  std::memset(&Q, 0, sizeof(Q));
  Q.counter = queue_counter;
  Q.path_out = (mode == kTwoState || mode == kSingle) ? path_out : nullptr;
  if (mode == kAdjoint || mode == kReplay || mode == kForward || mode == kTape) {
    RCV_REQUIRE(adj != nullptr && adj->ckpt && adj->ckpt_count && adj->path_ltot, "adjoint buffers missing");
    RCV_REQUIRE(total < (int64_t(1) << 32), "an adjoint launch must have fewer than 2^32 paths");
    Q.ckpt = adj->ckpt;
    Q.ckpt_count = adj->ckpt_count;
    Q.ckpt_cap = adj->ckpt_cap;
    Q.path_ltot = adj->path_ltot;
    if (adj->tape != nullptr) {
      // tape pass, or the replay of the paths it lost
      RCV_REQUIRE(mode == kTape || mode == kReplay, "the tape serves the gradient only");
      RCV_REQUIRE(total < (int64_t(1) << 30) && adj->ckpt_cap < (int64_t(1) << 30) &&
                      adj->tape_cap <= (int64_t(1) << 32) - int64_t(kTapeChunk),
                  "too many paths for the tape adjoint");
      RCV_REQUIRE(adj->tape_f != nullptr, "the tape needs its extinction terms");
      Q.tape = adj->tape;
      Q.tape_f = adj->tape_f;
      Q.tape_count = adj->tape_count;
      Q.tape_cap = adj->tape_cap;
      Q.lost_list = adj->lost_list;
      Q.lost_count = adj->lost_count;
    }
  }
  RCV_REQUIRE(mode != kTape || Q.tape != nullptr, "the tape pass needs a tape");
  Q.counters = reinterpret_cast<unsigned long long*>(counters);
  Q.jobs = jobs;
  Q.njobs = njobs;
  Q.total = total;
  Q.batch = (o != nullptr && o->batch > 0) ? o->batch : 64;
  RCV_REQUIRE(Q.batch <= (1 << 20), "batch must be <= 2^20");
  Q.defer = (o != nullptr && o->defer > 0) ? o->defer : 8;
  RCV_REQUIRE(Q.defer <= 32, "defer must be in [1, 32]");
  RCV_TRY_CUDA(cudaMemsetAsync(Q.counter, 0, sizeof(unsigned long long), st), "queue reset");
  return RCV_OK;
}

// Persistent launch over `total` paths of one job (jobs == null) or of a
// device job table.
int launch_persistent(int mode, const VolJob& J, const VolJob* jobs, int njobs, int64_t total,
                      const rcv_volpath_options* o, unsigned long long* queue_counter,
                      float4* path_out, const AdjBuffers* adj, uint64_t* counters, cudaStream_t st,
                      bool supergrid) {
  Queue Q;
  int rc = make_queue(mode, jobs, njobs, total, o, queue_counter, path_out, adj, counters, st, &Q);
  if (rc) return rc;
  const bool sg = supergrid || (jobs == nullptr && J.sg[0] > 0);
  // an environment map belongs to a single job (batched tables take the constant environment)
  const int variant = trace_variant(mode, sg, counters != nullptr, jobs == nullptr && J.env.valid != 0);
  int per_sm = resident_blocks(variant);
  if (o != nullptr && o->blocks_per_sm > 0 && o->blocks_per_sm < per_sm) per_sm = o->blocks_per_sm;
  // replay: the checkpoint tasks come on top of one camera task per path
  const int64_t tasks = (mode == kReplay || mode == kForward) ? 2 * total : total;
  const int64_t warps_needed = (tasks + Q.batch - 1) / Q.batch;
  int64_t blocks = (warps_needed + (kTraceBlock / 32) - 1) / (kTraceBlock / 32);
  const int64_t cap = int64_t(sm_count()) * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  const unsigned g = (unsigned)blocks;
  trace_kernel_of(variant)<<<g, kTraceBlock, 0, st>>>(J, Q);
  return launched("trace kernel launch");
}

int launch_reduce(bool two, const float4* po, int64_t path_begin, int64_t npix, int spp,
                  float* out_new, float* out_old, cudaStream_t st) {
  const int block = 256;
  if (two)
    reduce_paths_kernel<true><<<grid_for(npix, block), block, 0, st>>>(po, path_begin, npix, spp,
                                                                     out_new, out_old);
  else
    reduce_paths_kernel<false><<<grid_for(npix, block), block, 0, st>>>(po, path_begin, npix, spp,
                                                                      out_new, nullptr);
  return launched("reduce_paths launch");
}

int launch_fold(const rcv_medium* m, float* grad_density, float* grad_albedo, cudaStream_t st) {
  const MediumLayout L = medium_layout(m);
  const char* ws = static_cast<const char*>(m->workspace);
  const int64_t nv = int64_t(m->dims[0]) * m->dims[1] * m->dims[2];
  const int block = 256;
  fold_density_kernel<<<grid_for(nv, block), block, 0, st>>>(
      m->dims[0], m->dims[1], m->dims[2], reinterpret_cast<const float*>(ws + L.grad_cells),
      grad_density);
  int rc = launched("fold_density launch");
  if (rc) return rc;
  if (grad_albedo != nullptr && m->albedo_old != nullptr) {
    int32_t ad[3];
    albedo_dims_of(m, ad);
    const int64_t na = (int64_t)albedo_voxels_of(m);
    fold_albedo_kernel<<<grid_for(na, block), block, 0, st>>>(
        ad[0], ad[1], ad[2], reinterpret_cast<const float*>(ws + L.grad_albedo), grad_albedo);
    rc = launched("fold_albedo launch");
  }
  return rc;
}

int reset_gradients(const rcv_medium* m, bool albedo, cudaStream_t st) {
  const MediumLayout L = medium_layout(m);
  char* ws = static_cast<char*>(m->workspace);
  const int64_t nc = int64_t(m->dims[0] + 1) * (m->dims[1] + 1) * (m->dims[2] + 1);
  RCV_TRY_CUDA(cudaMemsetAsync(ws + L.grad_cells, 0, nc * 32, st), "gradient reset");
  if (albedo && m->albedo_old != nullptr) {
    int32_t ad[3];
    albedo_dims_of(m, ad);
    RCV_TRY_CUDA(cudaMemsetAsync(ws + L.grad_albedo, 0, albedo_grad_bytes(ad), st), "gradient reset");
  }
  return RCV_OK;
}

}  // namespace rcv

using namespace rcv;

extern "C" uint64_t rcv_medium_workspace_bytes(const int32_t dims[3], int32_t has_albedo_grid,
                                               int32_t majorant_factor) {
  if (dims == nullptr || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0 || majorant_factor < 0) return 0;
  return medium_layout(dims, has_albedo_grid ? dims : nullptr, majorant_factor).total;
}

extern "C" uint64_t rcv_medium_workspace_bytes_for(const rcv_medium* m) {
  if (m == nullptr || m->dims[0] <= 0 || m->dims[1] <= 0 || m->dims[2] <= 0 || m->majorant_factor < 0) return 0;
  for (int a = 0; a < 3; ++a)
    if (m->albedo_dims[a] < 0) return 0;
  return medium_layout(m).total;
}

// Environment-map tables: one thread per row packs its texels with their
// sampling weight f = luminance * sin(theta of the row centre) and writes the
// row's conditional CDF from double prefix sums taken in order; then one
// thread writes the marginal CDF over the rows and the normalisation.
__global__ void env_rows_kernel(int w, int h, float inv_h, const float* __restrict__ texels, float4* __restrict__ tex,
                                float* __restrict__ cond, double* __restrict__ rows) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= h) return;
  const float sin_i = env_row_sin(i, inv_h);
  double sum = 0.0;
  for (int j = 0; j < w; ++j) {
    const float* t = texels + (int64_t(i) * w + j) * 3;
    const float f = env_luminance(t[0], t[1], t[2]) * sin_i;
    tex[int64_t(i) * w + j] = make_float4(t[0], t[1], t[2], f);
    sum += (double)f;
  }
  rows[i] = sum;
  float* c = cond + int64_t(i) * (w + 1);
  double acc = 0.0;
  for (int j = 0; j < w; ++j) {
    c[j] = sum > 0.0 ? (float)(acc / sum) : (float)((double)j / (double)w);
    acc += (double)tex[int64_t(i) * w + j].w;
  }
  c[w] = 1.0f;
}

__global__ void env_marginal_kernel(int w, int h, const double* __restrict__ rows, float* __restrict__ marg,
                                    float* __restrict__ hdr) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double total = 0.0;
  for (int i = 0; i < h; ++i) total += rows[i];
  double acc = 0.0;
  for (int i = 0; i < h; ++i) {
    marg[i] = total > 0.0 ? (float)(acc / total) : (float)((double)i / (double)h);
    acc += rows[i];
  }
  marg[h] = 1.0f;
  hdr[0] = total > 0.0 ? (float)((double)w * (double)h / total) : 0.0f;
  hdr[1] = total > 0.0 ? 1.0f : 0.0f;
}

extern "C" uint64_t rcv_envmap_workspace_bytes(int32_t width, int32_t height) {
  if (width <= 0 || height <= 0) return 0;
  return env_layout(width, height).total;
}

extern "C" int rcv_envmap_prepare(const rcv_envmap* e, void* stream) {
  RCV_REQUIRE(e != nullptr && e->texels != nullptr, "environment map or its texels are NULL");
  RCV_REQUIRE(e->width > 0 && e->height > 0 && int64_t(e->width) * e->height < (int64_t(1) << 30),
              "environment map size must be positive and below 2^30 texels");
  RCV_REQUIRE(e->workspace != nullptr && (reinterpret_cast<uintptr_t>(e->workspace) & 255u) == 0,
              "environment map workspace must be non-NULL and 256-byte aligned");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const EnvLayout L = env_layout(e->width, e->height);
  char* ws = static_cast<char*>(e->workspace);
  env_rows_kernel<<<grid_for(e->height, 128), 128, 0, st>>>(
      e->width, e->height, 1.0f / (float)e->height, e->texels, reinterpret_cast<float4*>(ws + L.tex),
      reinterpret_cast<float*>(ws + L.cond), reinterpret_cast<double*>(ws + L.rows));
  int rc = launched("envmap rows launch");
  if (rc) return rc;
  env_marginal_kernel<<<1, 1, 0, st>>>(e->width, e->height, reinterpret_cast<const double*>(ws + L.rows),
                                       reinterpret_cast<float*>(ws + L.marg), reinterpret_cast<float*>(ws + L.hdr));
  return launched("envmap marginal launch");
}

extern "C" uint64_t rcv_render_workspace_bytes(int32_t width, int32_t height, int32_t spp,
                                               int32_t mode) {
  if (width <= 0 || height <= 0 || spp <= 0 || mode < 0 || mode > 2) return 0;
  const int64_t npix = int64_t(width) * height;
  return render_layout(npix, npix * spp, mode).total;
}

extern "C" int rcv_medium_prepare(const rcv_medium* m, void* stream) {
  int rc = validate_medium(m);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const MediumLayout L = medium_layout(m);
  char* ws = static_cast<char*>(m->workspace);
  RCV_TRY_CUDA(cudaMemsetAsync(ws + L.maxbits, 0, 16, st), "majorant reset");
  const int64_t nc = int64_t(m->dims[0] + 1) * (m->dims[1] + 1) * (m->dims[2] + 1);
  const int64_t na = (int64_t)albedo_voxels_of(m);
  const int block = 256;
  pack_medium_kernel<<<grid_for(nc > na ? nc : na, block), block, 0, st>>>(
      m->dims[0], m->dims[1], m->dims[2], m->density_old, m->density_new,
      reinterpret_cast<float4*>(ws + L.cells), m->albedo_old, m->albedo_new,
      m->albedo_old ? reinterpret_cast<float4*>(ws + L.albedo) : nullptr, na,
      reinterpret_cast<uint32_t*>(ws + L.maxbits));
  rc = launched("pack_medium launch");
  if (rc || m->majorant_factor == 0) return rc;
  const int sx = supergrid_cells(m->dims[0], m->majorant_factor);
  const int sy = supergrid_cells(m->dims[1], m->majorant_factor);
  const int sz = supergrid_cells(m->dims[2], m->majorant_factor);
  supergrid_kernel<<<grid_for(int64_t(sx) * sy * sz, 128), 128, 0, st>>>(
      sx, sy, sz, m->dims[0], m->dims[1], m->dims[2], m->scale, m->density_old, m->density_new,
      reinterpret_cast<float*>(ws + L.sg_two), reinterpret_cast<float*>(ws + L.sg_new));
  return launched("supergrid launch");
}

// Adjoint stages: both launches, the radiance pass alone, or the replay alone
// (which reuses the pixel order, checkpoints and total radiance the radiance
// pass left in the same workspace).
enum AdjStage { kAdjBoth = 0, kAdjRadiance = 1, kAdjReplay = 2, kAdjForward = 3 };

static int check_workspace(const void* workspace) {
  RCV_REQUIRE(workspace != nullptr && (reinterpret_cast<uintptr_t>(workspace) & 255u) == 0,
              "render workspace must be non-NULL and 256-byte aligned");
  return RCV_OK;
}

// Pixel hand-out order of a job (RCV_ORDER_*), in its workspace; `sort`
// false reuses the order an earlier stage left there.
static int order_job(VolJob& J, const rcv_volpath_options* o, char* ws, const RenderLayout& L, bool sort,
                     cudaStream_t st) {
  J.pixel_order = nullptr;
  J.pixel_cost = nullptr;
  const int order = o == nullptr ? RCV_ORDER_COST : o->order;
  RCV_REQUIRE(order == RCV_ORDER_COST || order == RCV_ORDER_ROW_MAJOR || order == RCV_ORDER_LONGEST_FIRST,
              "unknown pixel order %d", order);
  if (order == RCV_ORDER_ROW_MAJOR) return RCV_OK;
  uint32_t* cost = order == RCV_ORDER_COST ? reinterpret_cast<uint32_t*>(ws + L.cost) : nullptr;
  if (sort) {
    const int rc = order_pixels(J, reinterpret_cast<uint32_t*>(ws + L.buckets),
                                reinterpret_cast<uint32_t*>(ws + L.order), cost, st);
    if (rc) return rc;
  }
  J.pixel_order = reinterpret_cast<const uint32_t*>(ws + L.order);
  J.pixel_cost = cost;
  return RCV_OK;
}

// Adjoint buffers of a job in its workspace (queue counters at qc: hand-out,
// records, tape slots, lost paths).  *tape: the gradient comes from the
// event tape (RCV_ADJOINT_TAPE, except in forward mode and for jobs of 2^28
// paths or more, whose tape slots would not fit 32-bit indices).
static int adjoint_buffers(const VolJob& J, const rcv_volpath_options* o, char* ws, const RenderLayout& L,
                           unsigned long long* qc, int stage, AdjBuffers* out, bool* tape_out) {
  AdjBuffers& A = *out;
  std::memset(&A, 0, sizeof(A));
  A.ckpt = reinterpret_cast<float4*>(ws + L.ckpt);
  A.ckpt_count = qc + 1;
  A.ckpt_cap = ckpt_capacity(J.path_count);
  A.path_ltot = reinterpret_cast<float4*>(ws + L.ltot);
  const int adjoint = o == nullptr ? RCV_ADJOINT_TAPE : o->adjoint;
  const int per_path = (o == nullptr || o->tape_events_per_path == 0) ? int(kTapeSlotsPerPath)
                                                                    : o->tape_events_per_path;
  RCV_REQUIRE(adjoint == RCV_ADJOINT_TAPE || adjoint == RCV_ADJOINT_REPLAY, "unknown adjoint %d", adjoint);
  RCV_REQUIRE(per_path >= 1 && per_path <= kTapeSlotsPerPath, "tape_events_per_path must be in [0, %d]",
              int(kTapeSlotsPerPath));
  const bool tape = adjoint == RCV_ADJOINT_TAPE && stage != kAdjForward && J.path_count < (int64_t(1) << 28);
  if (tape) {
    A.tape = reinterpret_cast<float4*>(ws + L.tape);
    A.tape_count = qc + 2;
    A.tape_cap = tape_capacity(J.path_count, per_path);
    A.lost_list = reinterpret_cast<uint32_t*>(ws + L.lost);
    A.lost_count = qc + 3;
    A.tape_f = tape_terms(ws + L.tape, J.path_count);
  }
  *tape_out = tape;
  return RCV_OK;
}

// Orders the pixels, runs the persistent tracer of one job and, for the
// primal tracers, reduces the per-path radiance into the output image(s).
static int run_single_job(int mode, VolJob& J, const rcv_volpath_options* o, void* workspace,
                          uint64_t* counters, float* img_new, float* img_old, cudaStream_t st,
                          int stage = kAdjBoth) {
  int rc = check_workspace(workspace);
  if (rc) return rc;
  const int64_t npix = int64_t(J.width) * J.height;
  const RenderLayout L = render_layout(npix, J.path_count, mode);
  char* ws = static_cast<char*>(workspace);
  rc = order_job(J, o, ws, L, stage != kAdjReplay, st);
  if (rc) return rc;
  float4* po = reinterpret_cast<float4*>(ws + L.path_out);
  unsigned long long* qc = reinterpret_cast<unsigned long long*>(ws + L.counter);
  if (mode == kAdjoint) {
    AdjBuffers A;
    bool tape = false;
    rc = adjoint_buffers(J, o, ws, L, qc, stage, &A, &tape);
    if (rc) return rc;
    if (stage != kAdjReplay) {
      RCV_TRY_CUDA(cudaMemsetAsync(A.ckpt_count, 0, 3 * sizeof(unsigned long long), st), "adjoint counters reset");
      rc = launch_persistent(tape ? kTape : kAdjoint, J, nullptr, 0, J.path_count, o, qc, nullptr, &A, counters,
                             st, false);
      if (rc || stage == kAdjRadiance) return rc;
    }
    if (tape) {
      // weights of the event records: the second half of the checkpoint buffer
      float4* weights = reinterpret_cast<float4*>(ws + L.ckpt + uint64_t(A.ckpt_cap) * 32u);
      rc = launch_tape_gradient(J, nullptr, 0, A, weights, reinterpret_cast<float2*>(ws + L.cam_w), J.path_count,
                                counters, sm_count(), st);
      if (rc) return rc;
      // the paths whose events did not fit, replayed whole
    }
    return launch_persistent(stage == kAdjForward ? kForward : kReplay, J, nullptr, 0, J.path_count, o, qc,
                             nullptr, &A, counters, st, false);
  }
  rc = launch_persistent(mode, J, nullptr, 0, J.path_count, o, qc, po, nullptr, counters, st, false);
  if (rc) return rc;
  return launch_reduce(mode == kTwoState, po, 0, npix, J.spp, img_new, img_old, st);
}

extern "C" int rcv_render_twostates_volume(const rcv_medium* m, const rcv_sensor* s,
                                           const rcv_volpath_options* o, uint32_t seed,
                                           int32_t spp, float* img_old, float* img_new,
                                           void* workspace, uint64_t* counters, void* stream) {
  VolJob J;
  int rc = make_volume_job(m, s, o, seed, spp, &J);
  if (rc) return rc;
  RCV_REQUIRE(img_old != nullptr && img_new != nullptr, "output images are NULL");
  return run_single_job(kTwoState, J, o, workspace, counters, img_new, img_old,
                        static_cast<cudaStream_t>(stream));
}

extern "C" int rcv_render_volume(const rcv_medium* m, const rcv_sensor* s,
                                 const rcv_volpath_options* o, uint32_t seed, int32_t spp,
                                 float* img, void* workspace, uint64_t* counters, void* stream) {
  VolJob J;
  int rc = make_volume_job(m, s, o, seed, spp, &J);
  if (rc) return rc;
  RCV_REQUIRE(img != nullptr, "output image is NULL");
  return run_single_job(kSingle, J, o, workspace, counters, img, nullptr, static_cast<cudaStream_t>(stream));
}

// The two-state primal of (seed, spp) and the adjoint's radiance pass of
// (seed_grad, spp_grad) on the same medium: one persistent launch that runs
// both (rcv_pair.cu), where the two launches in a row would each end on
// their longest paths.  With event counting, the replay adjoint or
// separate_tracers the two run as separate launches.
extern "C" int rcv_render_twostates_volume_and_adjoint_radiance(
    const rcv_medium* m, const rcv_sensor* s, const rcv_volpath_options* o, uint32_t seed, int32_t spp,
    float* img_old, float* img_new, void* workspace, uint32_t seed_grad, int32_t spp_grad, void* adjoint_workspace,
    uint64_t* counters, void* stream) {
  VolJob JA, JB;
  int rc = make_volume_job(m, s, o, seed, spp, &JA);
  if (rc) return rc;
  rc = make_volume_job(m, s, o, seed_grad, spp_grad, &JB);
  if (rc) return rc;
  RCV_REQUIRE(img_old != nullptr && img_new != nullptr, "output images are NULL");
  RCV_REQUIRE(workspace != adjoint_workspace, "the render and the adjoint need separate workspaces");
  RCV_REQUIRE(o == nullptr || o->separate_tracers == 0 || o->separate_tracers == 1,
              "separate_tracers must be 0 or 1");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rc = check_workspace(workspace);
  if (rc == RCV_OK) rc = check_workspace(adjoint_workspace);
  if (rc) return rc;
  const int64_t npix = int64_t(JA.width) * JA.height;
  const RenderLayout LA = render_layout(npix, JA.path_count, kTwoState);
  const RenderLayout LB = render_layout(npix, JB.path_count, kAdjoint);
  char* wa = static_cast<char*>(workspace);
  char* wb = static_cast<char*>(adjoint_workspace);
  unsigned long long* qa = reinterpret_cast<unsigned long long*>(wa + LA.counter);
  unsigned long long* qb = reinterpret_cast<unsigned long long*>(wb + LB.counter);
  AdjBuffers A;
  bool tape = false;
  rc = adjoint_buffers(JB, o, wb, LB, qb, kAdjRadiance, &A, &tape);
  if (rc) return rc;
  if (counters != nullptr || !tape || (o != nullptr && o->separate_tracers)) {
    rc = run_single_job(kTwoState, JA, o, workspace, counters, img_new, img_old, st);
    if (rc) return rc;
    return run_single_job(kAdjoint, JB, o, adjoint_workspace, counters, nullptr, nullptr, st, kAdjRadiance);
  }
  rc = order_job(JA, o, wa, LA, true, st);
  if (rc == RCV_OK) rc = order_job(JB, o, wb, LB, true, st);
  if (rc) return rc;
  RCV_TRY_CUDA(cudaMemsetAsync(A.ckpt_count, 0, 3 * sizeof(unsigned long long), st), "adjoint counters reset");
  float4* po = reinterpret_cast<float4*>(wa + LA.path_out);
  Queue QA, QB;
  rc = make_queue(kTwoState, nullptr, 0, JA.path_count, o, qa, po, nullptr, nullptr, st, &QA);
  if (rc == RCV_OK) rc = make_queue(kTape, nullptr, 0, JB.path_count, o, qb, nullptr, &A, nullptr, st, &QB);
  if (rc == RCV_OK) rc = launch_pair(JA, QA, JB, QB, o, st, false);
  if (rc) return rc;
  return launch_reduce(true, po, 0, npix, JA.spp, img_new, img_old, st);
}

static int backward_volume(const rcv_medium* m, const rcv_sensor* s, const rcv_volpath_options* o, uint32_t seed,
                           int32_t spp, const float* grad_img, float* grad_density, float* grad_albedo,
                           void* workspace, uint64_t* counters, void* stream, int stage) {
  VolJob J;
  int rc = make_volume_job(m, s, o, seed, spp, &J);
  if (rc) return rc;
  RCV_REQUIRE(grad_img != nullptr && grad_density != nullptr, "gradient buffers are NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool want_albedo = grad_albedo != nullptr && m->albedo_old != nullptr;
  rc = reset_gradients(m, want_albedo, st);
  if (rc) return rc;
  if (!want_albedo) J.grad_albedo = nullptr;
  J.grad_img = grad_img;
  rc = run_single_job(kAdjoint, J, o, workspace, counters, nullptr, nullptr, st, stage);
  if (rc) return rc;
  return launch_fold(m, grad_density, want_albedo ? grad_albedo : nullptr, st);
}

extern "C" int rcv_render_backward_volume(const rcv_medium* m, const rcv_sensor* s,
                                          const rcv_volpath_options* o, uint32_t seed,
                                          int32_t spp, const float* grad_img,
                                          float* grad_density, float* grad_albedo,
                                          void* workspace, uint64_t* counters, void* stream) {
  return backward_volume(m, s, o, seed, spp, grad_img, grad_density, grad_albedo, workspace, counters, stream,
                         kAdjBoth);
}

extern "C" int rcv_render_forward_volume(const rcv_medium* m, const rcv_sensor* s,
                                         const rcv_volpath_options* o, uint32_t seed, int32_t spp,
                                         const float* tangent_density, const float* tangent_albedo,
                                         float* dimg, void* workspace, uint64_t* counters, void* stream) {
  VolJob J;
  int rc = make_volume_job(m, s, o, seed, spp, &J);
  if (rc) return rc;
  RCV_REQUIRE(dimg != nullptr, "output derivative image is NULL");
  RCV_REQUIRE(tangent_density != nullptr || tangent_albedo != nullptr, "no tangent given");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the medium's gradient records hold the packed tangent during the call
  const MediumLayout L = medium_layout(m);
  char* ws = static_cast<char*>(m->workspace);
  const int64_t nc = int64_t(m->dims[0] + 1) * (m->dims[1] + 1) * (m->dims[2] + 1);
  const int block = 256;
  if (tangent_density != nullptr) {
    pack_tangent_kernel<<<grid_for(nc, block), block, 0, st>>>(m->dims[0], m->dims[1], m->dims[2],
                                                               tangent_density,
                                                               reinterpret_cast<float4*>(ws + L.grad_cells));
    rc = launched("pack_tangent launch");
    if (rc) return rc;
  } else {
    RCV_TRY_CUDA(cudaMemsetAsync(ws + L.grad_cells, 0, nc * 32, st), "tangent reset");
  }
  const bool albedo = tangent_albedo != nullptr && m->albedo_old != nullptr;
  if (albedo) {
    const int64_t na = (int64_t)albedo_voxels_of(m);
    pack_tangent_albedo_kernel<<<grid_for(na, block), block, 0, st>>>(
        na, tangent_albedo, reinterpret_cast<float4*>(ws + L.grad_albedo));
    rc = launched("pack_tangent_albedo launch");
    if (rc) return rc;
  } else {
    J.grad_albedo = nullptr;
  }
  RCV_TRY_CUDA(cudaMemsetAsync(dimg, 0, size_t(J.width) * J.height * 3 * sizeof(float), st), "derivative reset");
  J.out_img = dimg;
  return run_single_job(kAdjoint, J, o, workspace, counters, nullptr, nullptr, st, kAdjForward);
}

extern "C" int rcv_render_adjoint_radiance(const rcv_medium* m, const rcv_sensor* s,
                                           const rcv_volpath_options* o, uint32_t seed, int32_t spp,
                                           void* workspace, uint64_t* counters, void* stream) {
  VolJob J;
  int rc = make_volume_job(m, s, o, seed, spp, &J);
  if (rc) return rc;
  return run_single_job(kAdjoint, J, o, workspace, counters, nullptr, nullptr, static_cast<cudaStream_t>(stream),
                        kAdjRadiance);
}

extern "C" int rcv_render_backward_replay(const rcv_medium* m, const rcv_sensor* s,
                                          const rcv_volpath_options* o, uint32_t seed, int32_t spp,
                                          const float* grad_img, float* grad_density, float* grad_albedo,
                                          void* workspace, uint64_t* counters, void* stream) {
  return backward_volume(m, s, o, seed, spp, grad_img, grad_density, grad_albedo, workspace, counters, stream,
                         kAdjReplay);
}

// ------------------------------------------------- allocation-free render
// Single-state render for callers that cannot allocate device memory: code
// running where cudaMalloc is unavailable or forbidden, such as a host that
// owns a fixed memory pool and hands this library only its inputs and
// outputs, or a real-time loop that may not allocate between frames.  Its
// scratch (work-queue counter, pixel order, per-path radiance) lives in this
// file-scope array instead of a caller buffer.  Every GPU that loads librcv
// holds the array until the process exits.
namespace rcv {

constexpr uint64_t kNoAllocScratchBytes = uint64_t(16) << 20;  // 16 MiB
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch on the current device.  In host code the
// symbol is only a host-side stand-in, so the address is looked up once per
// device (with that device current) and cached.  The cached address belongs to
// the device's primary context; a cudaDeviceReset ends its validity, which is
// why callers may not use the entry point on that device afterwards.
static int noalloc_scratch(void** out) {
  static std::mutex mu;
  static void* addr[kNoAllocMaxDevices] = {};
  int dev = 0;
  RCV_TRY_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  RCV_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices, "device ordinal %d is not supported", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (addr[dev] == nullptr) {
    void* p = nullptr;
    RCV_TRY_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
    addr[dev] = p;
  }
  *out = addr[dev];
  return RCV_OK;
}

}  // namespace rcv

extern "C" int rcv_render_volume_noalloc(const rcv_medium* m, const rcv_sensor* s,
                                         const rcv_volpath_options* o, uint32_t seed, int32_t spp,
                                         float* img, uint64_t* counters, void* stream) {
  VolJob J;
  int rc = make_volume_job(m, s, o, seed, spp, &J);
  if (rc) return rc;
  RCV_REQUIRE(img != nullptr, "output image is NULL");
  const uint64_t need = render_layout(int64_t(J.width) * J.height, J.path_count, kSingle).total;
  RCV_REQUIRE(need <= kNoAllocScratchBytes,
              "rcv_render_volume_noalloc: width*height*spp = %lld needs %llu bytes of scratch, "
              "more than its static %llu bytes (16 MiB); use rcv_render_volume with caller scratch",
              (long long)J.path_count, (unsigned long long)need,
              (unsigned long long)kNoAllocScratchBytes);
  void* ws = nullptr;
  rc = noalloc_scratch(&ws);
  if (rc) return rc;
  return run_single_job(kSingle, J, o, ws, counters, img, nullptr, static_cast<cudaStream_t>(stream));
}
