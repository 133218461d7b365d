// Batched cv_ps steps: many optimisation jobs of uneven grid, film and
// sample counts advanced by one step in six kernel launches.
//
//   prologue   1 block: per job, seeds, CV scalars and Adam step size from the
//              job's device counters and bias-correction tables; counters++
//   pack       medium packing of every job (old = theta_{it-1}, new =
//              theta_it from the parameter double buffer), majorants, and
//              zeroed gradient cells
//   trace 2S   ONE persistent two-state launch over the paths of all jobs;
//              with the tape adjoint the same launch runs the adjoint's
//              radiance pass over the gradient paths of all jobs
//              (rcv_pair.cu; separate_tracers: a second launch on a side
//              stream)
//   image      per pixel of every job: sample reduction (H, F), control
//              variate blend + statistics, loss gradient and loss sum
//   trace adj  the adjoint's gradient: from the tape (weights + scatter),
//              then ONE persistent replay launch over the paths the tape
//              lost (or over all gradient paths, after a checkpoint
//              radiance launch, with the replay adjoint)
//   update     per voxel of every job: cell-gradient fold, Adam + clamp into
//              the other half of the parameter double buffer
//
// The elementwise kernels give each job a whole number of blocks (a block
// never spans two jobs) and find their job by binary search over the block
// prefix table.  Nothing the host passes changes between steps, so a step can
// be captured once into a CUDA graph and replayed.
//
// Per job, every stage performs the arithmetic of the single-job entry points
// it replaces (rcv_medium_prepare, rcv_render_twostates_volume, rcv_cv_step,
// rcv_loss, rcv_render_backward_volume, rcv_adam_step) through the same
// element functions, so images are identical to the single-job path and
// gradients differ only by the order of float atomics.
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <vector>

#include "rcv_common.h"
#include "rcv_cvmath.cuh"
#include "rcv_pack.cuh"
#include "rcv_volume.cuh"

namespace rcv {

constexpr int kBatchBlock = 256;
constexpr int kBatchKernels = 7;
constexpr int kMaxBatchJobs = 1 << 16;

// Per-step values of a job, written by the prologue.
struct StepParams {
  CvScalars S;
  float lr_t;        // Adam step size with both bias corrections
  int32_t cur;       // density[cur] = theta_it (new), density[cur ^ 1] = theta_{it-1}
  uint32_t seed, seed_grad;
};

struct JobHeader {
  rcv_batch_job_status status;
  StepParams step;
};
static_assert(sizeof(rcv_batch_job_status) == 32, "status layout");

// Job workspace: header | medium (cells, albedo pairs, majorants, gradient
// cells) | order buckets | pixel order | per-pixel cost | dL/dimage.
struct JobLayout {
  uint64_t header, medium, buckets, order, cost, grad_img, total;
};

static JobLayout job_layout(const rcv_batch_job& j) {
  JobLayout L;
  const uint64_t npix = uint64_t(j.sensor.width) * uint64_t(j.sensor.height);
  uint64_t off = 0;
  L.header = off;
  off = align256(off + sizeof(JobHeader));
  L.medium = off;
  off = align256(off + medium_layout(j.dims, j.albedo[0] != nullptr ? j.dims : nullptr, j.majorant_factor).total);
  L.buckets = off;
  off = align256(off + kRenderOrderBuckets * sizeof(uint32_t));
  L.order = off;
  off = align256(off + npix * sizeof(uint32_t));
  L.cost = off;
  off = align256(off + npix * sizeof(uint32_t));
  L.grad_img = off;
  off = align256(off + npix * 3 * sizeof(float));
  L.total = off;
  return L;
}

// Device view of one job.
struct BatchEntry {
  rcv_batch_job d;
  JobHeader* hdr;
  float4* cells;
  float4* albedo;  // packed (old, new) pairs or null
  uint32_t* maxbits;
  float4* grad_cells;
  float4* grad_albedo;  // albedo cell records (6 float4 per cell) or null
  float* grad_img;
  uint32_t* buckets;  // 256 order buckets
  uint32_t* order;    // pixel hand-out order
  uint32_t* cost;     // per-pixel path lengths of the last step
  int64_t npix, nv, nc;
  int64_t two_begin;  // first path of the job in the two-state launch
  double inv_n;       // 1 / (npix * 3)
  float gscale;       // float32(1 / (npix * 3))
  int32_t has_albedo;  // albedo grid (else albedo_value)
  int32_t opt_albedo;  // albedo is optimised (moments given)
};

__device__ __forceinline__ int job_of_block(const int32_t* __restrict__ bp, int n, int block) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(bp + mid) <= block)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// d[k] = 1 - beta^k from a table that saturates at 1.0f.
__device__ __forceinline__ float table_d(const float* __restrict__ tab, int len, int k) {
  return k < len ? __ldg(tab + k) : 1.0f;
}

__global__ void batch_prologue_kernel(BatchEntry* __restrict__ E, VolJob* __restrict__ two,
                                      VolJob* __restrict__ adj, int n) {
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const rcv_batch_job& d = E[j].d;
    JobHeader* h = E[j].hdr;
    const int it = h->status.it, cnt = h->status.welford_count, t = h->status.adam_t + 1;
    StepParams P;
    // seed = seed_base + it; seed_grad = sample_tea_32(seed, 1)[0]
    // (plugins/twostatepath.py:84-92)
    P.seed = d.seed_base + (uint32_t)it;
    uint32_t a, b;
    tea(P.seed, 1u, 4, a, b);
    P.seed_grad = a;
    P.cur = it & 1;
    // control-variate scalars, as rcv_cv_step derives them on the host
    CvScalars& S = P.S;
    S.b1 = d.cv_beta1;
    S.b2 = d.cv_beta2;
    S.omb1 = 1.0f - d.cv_beta1;
    S.omb2 = 1.0f - d.cv_beta2;
    S.has_prev = cnt > 0;
    S.d1_prev = cnt > 0 ? table_d(d.cv_table1, d.cv_table1_len, cnt) : 1.0f;
    S.d1_next = table_d(d.cv_table1, d.cv_table1_len, cnt + 1);
    const bool update = it > 0;
    S.do_pre = update && d.pre_update;
    S.do_post = update && !d.pre_update;
    S.do_weight = it > d.warmup;
    S.d2_get = table_d(d.cv_table2, d.cv_table2_len, cnt + (S.do_pre ? 1 : 0));
    // lr_t = lr * sqrt(1 - beta2^t) / (1 - beta1^t) in double, as rcv_adam_step
    double s2 = 1.0, bc1 = 1.0;
    if (t < d.adam_table_len) {
      s2 = d.adam_table[2 * t];
      bc1 = d.adam_table[2 * t + 1];
    }
    P.lr_t = (float)(((double)d.lr * s2) / bc1);
    h->step = P;
    h->status.it = it + 1;
    h->status.welford_count = cnt + (update ? 1 : 0);
    h->status.adam_t = t;
    h->status.loss_sum = 0.0;
    E[j].maxbits[0] = 0u;
    E[j].maxbits[1] = 0u;
    two[j].seed = P.seed;
    adj[j].seed = P.seed_grad;
  }
}

__global__ void batch_pack_kernel(const BatchEntry* __restrict__ E, const int32_t* __restrict__ bp, int n) {
  const int j = job_of_block(bp, n, blockIdx.x);
  const BatchEntry& B = E[j];
  const int64_t i = int64_t(blockIdx.x - __ldg(bp + j)) * blockDim.x + threadIdx.x;
  if (i < kRenderOrderBuckets) B.buckets[i] = 0u;  // for this step's pixel order
  const int cur = B.hdr->step.cur;
  const float* nd = B.d.density[cur];
  const float* od = B.d.density[cur ^ 1];
  const int dx = B.d.dims[0], dy = B.d.dims[1], dz = B.d.dims[2];
  float mo = 0.0f, mn = 0.0f;
  if (i < B.nc) {
    pack_cell(i, dx, dy, dz, od, nd, B.cells);
    B.grad_cells[i * 2 + 0] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    B.grad_cells[i * 2 + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (B.opt_albedo) {
      // the albedo grid has the density's resolution: one 6-float4 record per cell
#pragma unroll
      for (int q = 0; q < 6; ++q) B.grad_albedo[i * 6 + q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
  }
  if (i < B.nv) {
    mo = od[i];
    mn = nd[i];
    if (B.has_albedo) pack_albedo(i, B.d.albedo[cur ^ 1], B.d.albedo[cur], B.albedo);
  }
  reduce_majorants(mo, mn, B.maxbits);
}

// Pixel order of every job by the path lengths of its last step (most
// expensive first): bucket counts, per-job exclusive scan, placement.
__global__ void batch_order_count_kernel(const BatchEntry* __restrict__ E, const int32_t* __restrict__ bp,
                                         int n) {
  const int j = job_of_block(bp, n, blockIdx.x);
  const BatchEntry& B = E[j];
  const int64_t pix = int64_t(blockIdx.x - __ldg(bp + j)) * blockDim.x + threadIdx.x;
  __shared__ uint32_t hist[kRenderOrderBuckets];
  for (int k = threadIdx.x; k < kRenderOrderBuckets; k += blockDim.x) hist[k] = 0u;
  __syncthreads();
  if (pix < B.npix) atomicAdd(&hist[cost_bucket(B.cost[pix])], 1u);
  __syncthreads();
  for (int k = threadIdx.x; k < kRenderOrderBuckets; k += blockDim.x)
    if (hist[k]) atomicAdd(B.buckets + k, hist[k]);
}

__global__ void batch_order_scan_kernel(const BatchEntry* __restrict__ E) {
  uint32_t* counts = E[blockIdx.x].buckets;
  __shared__ uint32_t sh[kRenderOrderBuckets];
  const int t = threadIdx.x;
  sh[t] = counts[t];
  __syncthreads();
  for (int off = 1; off < kRenderOrderBuckets; off <<= 1) {
    const uint32_t v = t >= off ? sh[t - off] : 0u;
    __syncthreads();
    sh[t] += v;
    __syncthreads();
  }
  counts[t] = t == 0 ? 0u : sh[t - 1];
}

__global__ void batch_order_place_kernel(const BatchEntry* __restrict__ E, const int32_t* __restrict__ bp,
                                         int n) {
  const int j = job_of_block(bp, n, blockIdx.x);
  const BatchEntry& B = E[j];
  const int64_t pix = int64_t(blockIdx.x - __ldg(bp + j)) * blockDim.x + threadIdx.x;
  const bool valid = pix < B.npix;
  place_block(valid ? cost_bucket(B.cost[pix]) : 0, valid, (uint32_t)pix, B.buckets, B.order);
  if (valid) B.cost[pix] = 0u;
}

// Majorant supergrids of the jobs that have one (old = the other half of the
// parameter double buffer, new = the current half).
__global__ void batch_supergrid_kernel(const BatchEntry* __restrict__ E, const VolJob* __restrict__ two,
                                       const int32_t* __restrict__ bp, int n) {
  const int j = job_of_block(bp, n, blockIdx.x);
  const BatchEntry& B = E[j];
  const VolJob& J = two[j];
  const int64_t i = int64_t(blockIdx.x - __ldg(bp + j)) * blockDim.x + threadIdx.x;
  if (J.sg[0] == 0 || i >= int64_t(J.sg[0]) * J.sg[1] * J.sg[2]) return;
  const int cur = B.hdr->step.cur;
  supergrid_cell(i, J.sg, B.d.dims[0], B.d.dims[1], B.d.dims[2], B.d.scale, B.d.density[cur ^ 1],
                 B.d.density[cur], const_cast<float*>(J.sg_two), const_cast<float*>(J.sg_new));
}

// Initial per-pixel cost of a job: its chord order (longest chord first).
__global__ void cost_from_chord_kernel(const __grid_constant__ VolJob J, int npix, uint32_t* cost) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix < npix) cost[pix] = 4u * uint32_t(255 - chord_key(J, pix));
}

__global__ void batch_image_kernel(const BatchEntry* __restrict__ E, const int32_t* __restrict__ bp, int n,
                                   const float4* __restrict__ path_out) {
  const int j = job_of_block(bp, n, blockIdx.x);
  const BatchEntry& B = E[j];
  const int64_t pix = int64_t(blockIdx.x - __ldg(bp + j)) * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (pix < B.npix) {
    const CvScalars S = B.hdr->step.S;
    V3 F, H;
    reduce_pixel<true>(path_out, B.two_begin, pix, B.d.spp, F, H);
    if (B.d.img_new != nullptr) {
      B.d.img_new[pix * 3 + 0] = F.x;
      B.d.img_new[pix * 3 + 1] = F.y;
      B.d.img_new[pix * 3 + 2] = F.z;
    }
    if (B.d.img_old != nullptr) {
      B.d.img_old[pix * 3 + 0] = H.x;
      B.d.img_old[pix * 3 + 1] = H.y;
      B.d.img_old[pix * 3 + 2] = H.z;
    }
    const float hs[3] = {H.x, H.y, H.z}, fs[3] = {F.x, F.y, F.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t i = pix * 3 + c;
      const float g = cv_element(B.d.cv, i, hs[c], fs[c], S);
      B.grad_img[i] = loss_grad(B.d.loss, g - __ldg(B.d.target + i), B.gscale, acc);
    }
  }
  // block sum of the loss terms, one atomic per block
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  __shared__ double warp_sums[kBatchBlock / 32];
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kBatchBlock / 32; ++k) s += warp_sums[k];
    atomicAdd(&B.hdr->status.loss_sum, s);
  }
}

__global__ void batch_update_kernel(const BatchEntry* __restrict__ E, const int32_t* __restrict__ bp, int n) {
  const int j = job_of_block(bp, n, blockIdx.x);
  const BatchEntry& B = E[j];
  const int64_t i = int64_t(blockIdx.x - __ldg(bp + j)) * blockDim.x + threadIdx.x;
  if (i == 0) B.hdr->status.loss = float(B.hdr->status.loss_sum * B.inv_n);
  if (i >= B.nv) return;
  const int cur = B.hdr->step.cur;
  const float lr_t = B.hdr->step.lr_t;
  const float b1 = B.d.adam_beta1, b2 = B.d.adam_beta2, eps = B.d.adam_eps;
  const float omb1 = 1.0f - b1, omb2 = 1.0f - b2;
  // the single-job path accumulates the fold into a zeroed gradient: 0 + g
  const float g = 0.0f + fold_voxel(i, B.d.dims[0], B.d.dims[1], B.d.dims[2],
                                    reinterpret_cast<const float*>(B.grad_cells));
  {
    float m = B.d.density_m[i], v = B.d.density_v[i];
    B.d.density[cur ^ 1][i] =
        adam_value(B.d.density[cur][i], g, m, v, lr_t, b1, b2, omb1, omb2, eps, B.d.density_lo, B.d.density_hi);
    B.d.density_m[i] = m;
    B.d.density_v[i] = v;
  }
  if (B.opt_albedo) {
    const V3 ga = fold_voxel_rgb(i, B.d.dims[0], B.d.dims[1], B.d.dims[2],
                                 reinterpret_cast<const float*>(B.grad_albedo));
    const float gs[3] = {0.0f + ga.x, 0.0f + ga.y, 0.0f + ga.z};
    const float* pin = B.d.albedo[cur];
    float* pout = B.d.albedo[cur ^ 1];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t k = i * 3 + c;
      float m = B.d.albedo_m[k], v = B.d.albedo_v[k];
      pout[k] = adam_value(pin[k], gs[c], m, v, lr_t, b1, b2, omb1, omb2, eps, B.d.albedo_lo, B.d.albedo_hi);
      B.d.albedo_m[k] = m;
      B.d.albedo_v[k] = v;
    }
  }
}

// ------------------------------------------------------------------ host
static int validate_job(const rcv_batch_job* j, int idx) {
  RCV_REQUIRE(j != nullptr, "job %d is NULL", idx);
  RCV_REQUIRE(j->dims[0] > 0 && j->dims[1] > 0 && j->dims[2] > 0, "job %d: grid dims must be positive", idx);
  RCV_REQUIRE(uint64_t(j->dims[0] + 1) * uint64_t(j->dims[1] + 1) * uint64_t(j->dims[2] + 1) * 4u <
                  (uint64_t(1) << 32),
              "job %d: grid too large: (Dx+1)(Dy+1)(Dz+1) must be below 2^30", idx);
  RCV_REQUIRE(j->sensor.width > 0 && j->sensor.height > 0, "job %d: film size must be positive", idx);
  RCV_REQUIRE(j->spp > 0 && j->spp_grad > 0, "job %d: spp and spp_grad must be positive", idx);
  const int64_t npix = int64_t(j->sensor.width) * j->sensor.height;
  RCV_REQUIRE(npix * j->spp < (int64_t(1) << 32) && npix * j->spp_grad < (int64_t(1) << 32),
              "job %d: width * height * spp must be below 2^32", idx);
  RCV_REQUIRE(j->max_depth >= -1, "job %d: max_depth must be >= -1", idx);
  RCV_REQUIRE(j->scale >= 0.0f, "job %d: scale must be non-negative", idx);
  RCV_REQUIRE(j->density[0] && j->density[1] && j->density_m && j->density_v,
              "job %d: density buffers / moments are NULL", idx);
  RCV_REQUIRE(j->density[0] != j->density[1], "job %d: the two density buffers must differ", idx);
  const bool alb = j->albedo[0] != nullptr, opt_alb = j->albedo_m != nullptr;
  RCV_REQUIRE(alb == (j->albedo[1] != nullptr), "job %d: albedo[0] and albedo[1] must both be set or both be NULL",
              idx);
  RCV_REQUIRE(opt_alb == (j->albedo_v != nullptr), "job %d: albedo_m and albedo_v must both be set or both be NULL",
              idx);
  RCV_REQUIRE(!opt_alb || alb, "job %d: albedo moments without an albedo grid", idx);
  RCV_REQUIRE(!opt_alb || j->albedo[0] != j->albedo[1], "job %d: the two albedo buffers must differ", idx);
  RCV_REQUIRE(j->target != nullptr, "job %d: target is NULL", idx);
  const rcv_cv_state& s = j->cv;
  RCV_REQUIRE(s.img && s.w_s && s.v_n && s.mean_x && s.mean_y && s.var_x && s.var_y && s.cov,
              "job %d: a control-variate state array is NULL", idx);
  RCV_REQUIRE(j->cv_beta1 >= 0.0f && j->cv_beta1 < 1.0f && j->cv_beta2 >= 0.0f && j->cv_beta2 < 1.0f,
              "job %d: cv betas must be in [0, 1)", idx);
  RCV_REQUIRE(j->adam_beta1 >= 0.0f && j->adam_beta1 < 1.0f && j->adam_beta2 >= 0.0f && j->adam_beta2 < 1.0f,
              "job %d: Adam betas must be in [0, 1)", idx);
  RCV_REQUIRE(j->cv_table1 && j->cv_table2 && j->cv_table1_len > 0 && j->cv_table2_len > 0,
              "job %d: CV bias-correction tables are missing", idx);
  RCV_REQUIRE(j->adam_table && j->adam_table_len > 0, "job %d: Adam bias-correction table is missing", idx);
  RCV_REQUIRE(j->loss == RCV_LOSS_L2 || j->loss == RCV_LOSS_L1, "job %d: unknown loss kind %d", idx, j->loss);
  RCV_REQUIRE(j->majorant_factor >= 0, "job %d: majorant_factor must be >= 0", idx);
  RCV_REQUIRE(j->workspace != nullptr && (reinterpret_cast<uintptr_t>(j->workspace) & 255u) == 0,
              "job %d: workspace must be non-NULL and 256-byte aligned", idx);
  return RCV_OK;
}

// Plan workspace: entries | two-state jobs | adjoint jobs | block prefixes |
// queue counters (two-state, adjoint radiance, replay, checkpoints / event
// records, tape slots, lost paths) | tracer counters | per-path radiance |
// adjoint per-path total radiance | scatter checkpoints (tape: event records
// and their weights) | event tape | per-path camera-segment weights |
// lost-path list.
struct PlanLayout {
  uint64_t entries, two, adj, prefix, queue, counters, path_out, ltot, ckpt, tape, cam_w, lost, total;
};

static PlanLayout plan_layout(int n, int64_t total_two_paths, int64_t total_adj_paths) {
  PlanLayout L;
  uint64_t off = 0;
  L.entries = off;
  off = align256(off + uint64_t(n) * sizeof(BatchEntry));
  L.two = off;
  off = align256(off + uint64_t(n) * sizeof(VolJob));
  L.adj = off;
  off = align256(off + uint64_t(n) * sizeof(VolJob));
  L.prefix = off;
  off = align256(off + 4u * uint64_t(n + 1) * sizeof(int32_t));
  L.queue = off;
  off = align256(off + 8u * sizeof(unsigned long long));
  L.counters = off;
  off = align256(off + 2u * RCV_COUNTER_COUNT * sizeof(uint64_t));
  L.path_out = off;
  off = align256(off + uint64_t(total_two_paths) * 32u);
  L.ltot = off;
  off = align256(off + uint64_t(total_adj_paths) * 16u);
  L.ckpt = off;
  off = align256(off + uint64_t(ckpt_capacity(total_adj_paths)) * 64u);
  L.tape = off;
  off = align256(off + uint64_t(tape_capacity(total_adj_paths, kTapeSlotsPerPath)) * 20u);
  L.cam_w = off;
  off = align256(off + uint64_t(total_adj_paths) * 8u);
  L.lost = off;
  off = align256(off + uint64_t(total_adj_paths) * 4u);
  L.total = off;
  return L;
}

static int64_t primal_paths(const rcv_batch_job& j) { return int64_t(j.sensor.width) * j.sensor.height * j.spp; }

static rcv_medium job_medium(const rcv_batch_job& j, const JobLayout& L) {
  rcv_medium m;
  std::memset(&m, 0, sizeof(m));
  std::memcpy(m.dims, j.dims, sizeof(m.dims));
  m.scale = j.scale;
  m.density_old = j.density[0];
  m.density_new = j.density[1];
  m.albedo_old = j.albedo[0];
  m.albedo_new = j.albedo[1];
  std::memcpy(m.albedo_value, j.albedo_value, sizeof(m.albedo_value));
  m.majorant_factor = j.majorant_factor;
  std::memcpy(m.box_min, j.box_min, sizeof(m.box_min));
  std::memcpy(m.box_size, j.box_size, sizeof(m.box_size));
  m.workspace = static_cast<char*>(j.workspace) + L.medium;
  return m;
}

static rcv_volpath_options job_options(const rcv_batch_job& j, const rcv_volpath_options* o) {
  rcv_volpath_options r;
  std::memset(&r, 0, sizeof(r));
  if (o != nullptr) r = *o;
  r.max_depth = j.max_depth;
  r.rr_depth = j.rr_depth;
  r.hide_emitters = j.hide_emitters;
  r.envmap = nullptr;  // batched jobs see the constant environment
  return r;
}

}  // namespace rcv

using namespace rcv;

struct rcv_batch {
  int n = 0;
  int device = 0;
  rcv_volpath_options opt{};
  BatchEntry* entries = nullptr;
  VolJob* two = nullptr;
  VolJob* adj = nullptr;
  int32_t* prefix = nullptr;  // pack | image | update | supergrid block prefixes, n + 1 each
  unsigned long long* queue = nullptr;
  uint64_t* counters = nullptr;
  float4* path_out = nullptr;
  AdjBuffers adjbuf{};
  bool tape = false;  // gradient from the event tape (else replay tasks)
  // the two-state and tape radiance passes in one launch (rcv_pair.cu), else
  // two launches on two streams
  bool paired = false;
  float4* tape_weights = nullptr;
  float2* cam_w = nullptr;
  int64_t total_two = 0, total_adj = 0;
  int32_t pack_blocks = 0, pix_blocks = 0, vox_blocks = 0, sg_blocks = 0;
  // host copies of the tables (kept until destroy: the upload reads them)
  std::vector<BatchEntry> h_entries;
  std::vector<VolJob> h_two, h_adj;
  std::vector<int32_t> h_prefix;
  cudaStream_t capture_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // the adjoint radiance launch runs beside the two-state launch
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

extern "C" uint64_t rcv_batch_job_workspace_bytes(const rcv_batch_job* job) {
  if (job == nullptr || job->dims[0] <= 0 || job->dims[1] <= 0 || job->dims[2] <= 0 || job->sensor.width <= 0 ||
      job->sensor.height <= 0)
    return 0;
  return job_layout(*job).total;
}

extern "C" int rcv_batch_job_init(const rcv_batch_job* job, void* stream) {
  int rc = validate_job(job, 0);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const JobLayout L = job_layout(*job);
  char* ws = static_cast<char*>(job->workspace);
  RCV_TRY_CUDA(cudaMemsetAsync(ws + L.header, 0, sizeof(JobHeader), st), "job status reset");
  const rcv_medium m = job_medium(*job, L);
  const rcv_volpath_options o = job_options(*job, nullptr);
  VolJob J;
  rc = make_volume_job(&m, &job->sensor, &o, 0u, job->spp, &J);
  if (rc) return rc;
  rc = order_pixels(J, reinterpret_cast<uint32_t*>(ws + L.buckets), reinterpret_cast<uint32_t*>(ws + L.order),
                    nullptr, st);
  if (rc) return rc;
  const int npix = J.width * J.height;
  cost_from_chord_kernel<<<grid_for(npix, kBatchBlock), kBatchBlock, 0, st>>>(
      J, npix, reinterpret_cast<uint32_t*>(ws + L.cost));
  return launched("batch cost init launch");
}

extern "C" uint64_t rcv_batch_workspace_bytes(const rcv_batch_job* jobs, int32_t n) {
  if (jobs == nullptr || n < 1 || n > kMaxBatchJobs) return 0;
  int64_t total = 0, total_adj = 0;
  for (int j = 0; j < n; ++j) {
    if (jobs[j].sensor.width <= 0 || jobs[j].sensor.height <= 0 || jobs[j].spp <= 0 || jobs[j].spp_grad <= 0)
      return 0;
    total += primal_paths(jobs[j]);
    total_adj += int64_t(jobs[j].sensor.width) * jobs[j].sensor.height * jobs[j].spp_grad;
  }
  return plan_layout(n, total, total_adj).total;
}

extern "C" int rcv_batch_create(const rcv_batch_job* jobs, int32_t n, const rcv_volpath_options* opts,
                                void* workspace, uint64_t workspace_bytes, rcv_batch** out, void* stream) {
  RCV_REQUIRE(opts == nullptr || opts->envmap == nullptr,
              "the batched engine renders under the constant environment only (no environment map)");
  RCV_REQUIRE(out != nullptr, "out is NULL");
  *out = nullptr;
  RCV_REQUIRE(jobs != nullptr && n >= 1 && n <= kMaxBatchJobs, "need 1..%d jobs", kMaxBatchJobs);
  for (int j = 0; j < n; ++j) {
    int rc = validate_job(&jobs[j], j);
    if (rc) return rc;
  }
  if (opts != nullptr) {
    RCV_REQUIRE(opts->order == RCV_ORDER_COST || opts->order == RCV_ORDER_LONGEST_FIRST ||
                    opts->order == RCV_ORDER_ROW_MAJOR,
                "unknown pixel order %d", opts->order);
    RCV_REQUIRE(opts->batch >= 0 && opts->batch <= (1 << 20), "batch must be in [0, 2^20]");
    RCV_REQUIRE(opts->defer >= 0 && opts->defer <= 32, "defer must be in [0, 32]");
    RCV_REQUIRE(opts->blocks_per_sm >= 0, "blocks_per_sm must be >= 0");
    RCV_REQUIRE(opts->adjoint == RCV_ADJOINT_TAPE || opts->adjoint == RCV_ADJOINT_REPLAY, "unknown adjoint %d",
                opts->adjoint);
    RCV_REQUIRE(opts->tape_events_per_path >= 0 && opts->tape_events_per_path <= kTapeSlotsPerPath,
                "tape_events_per_path must be in [0, %d]", int(kTapeSlotsPerPath));
    RCV_REQUIRE(opts->separate_tracers == 0 || opts->separate_tracers == 1, "separate_tracers must be 0 or 1");
  }
  const uint64_t need = rcv_batch_workspace_bytes(jobs, n);
  RCV_REQUIRE(need > 0 && workspace_bytes >= need, "batch workspace too small: %llu bytes, need %llu",
              (unsigned long long)workspace_bytes, (unsigned long long)need);
  RCV_REQUIRE(workspace != nullptr && (reinterpret_cast<uintptr_t>(workspace) & 255u) == 0,
              "batch workspace must be non-NULL and 256-byte aligned");

  int device = 0;
  RCV_TRY_CUDA(cudaGetDevice(&device), "cudaGetDevice");
  rcv_batch* b = new (std::nothrow) rcv_batch();
  RCV_REQUIRE(b != nullptr, "out of host memory");
  b->n = n;
  b->device = device;
  if (opts != nullptr) b->opt = *opts;
  b->h_entries.resize(n);
  b->h_two.resize(n);
  b->h_adj.resize(n);
  b->h_prefix.assign(4 * size_t(n + 1), 0);
  int32_t* pp = b->h_prefix.data();
  int32_t* pi = pp + (n + 1);
  int32_t* pv = pi + (n + 1);
  int32_t* ps = pv + (n + 1);
  int64_t two_total = 0, adj_total = 0, pack_blocks = 0, pix_blocks = 0, vox_blocks = 0, sg_blocks = 0;
  for (int j = 0; j < n; ++j) {
    const rcv_batch_job& d = jobs[j];
    const JobLayout L = job_layout(d);
    char* ws = static_cast<char*>(d.workspace);
    const rcv_medium m = job_medium(d, L);
    const rcv_volpath_options o = job_options(d, opts);
    VolJob T, A;
    int rc = make_volume_job(&m, &d.sensor, &o, 0u, d.spp, &T);
    if (rc == RCV_OK) rc = make_volume_job(&m, &d.sensor, &o, 0u, d.spp_grad, &A);
    if (rc) {
      delete b;
      return rc;
    }
    const uint32_t* order = reinterpret_cast<const uint32_t*>(ws + L.order);
    const int policy = opts == nullptr ? RCV_ORDER_COST : opts->order;
    uint32_t* cost = policy == RCV_ORDER_COST ? reinterpret_cast<uint32_t*>(ws + L.cost) : nullptr;
    T.pixel_order = policy != RCV_ORDER_ROW_MAJOR ? order : nullptr;
    A.pixel_order = T.pixel_order;
    T.pixel_cost = cost;
    A.pixel_cost = cost;
    T.path_begin = two_total;
    A.path_begin = adj_total;
    A.grad_img = reinterpret_cast<const float*>(ws + L.grad_img);
    if (d.albedo_m == nullptr) A.grad_albedo = nullptr;  // a fixed albedo grid gets no gradient
    b->h_two[j] = T;
    b->h_adj[j] = A;

    BatchEntry& e = b->h_entries[j];
    std::memset(&e, 0, sizeof(e));
    e.d = d;
    e.hdr = reinterpret_cast<JobHeader*>(ws + L.header);
    const MediumLayout M = medium_layout(d.dims, d.albedo[0] != nullptr ? d.dims : nullptr, d.majorant_factor);
    char* mw = ws + L.medium;
    e.cells = reinterpret_cast<float4*>(mw + M.cells);
    e.has_albedo = d.albedo[0] != nullptr;
    e.albedo = e.has_albedo ? reinterpret_cast<float4*>(mw + M.albedo) : nullptr;
    e.maxbits = reinterpret_cast<uint32_t*>(mw + M.maxbits);
    e.grad_cells = reinterpret_cast<float4*>(mw + M.grad_cells);
    e.opt_albedo = d.albedo_m != nullptr;
    e.grad_albedo = e.opt_albedo ? reinterpret_cast<float4*>(mw + M.grad_albedo) : nullptr;
    e.grad_img = reinterpret_cast<float*>(ws + L.grad_img);
    e.buckets = reinterpret_cast<uint32_t*>(ws + L.buckets);
    e.order = reinterpret_cast<uint32_t*>(ws + L.order);
    e.cost = reinterpret_cast<uint32_t*>(ws + L.cost);
    e.npix = int64_t(d.sensor.width) * d.sensor.height;
    e.nv = int64_t(d.dims[0]) * d.dims[1] * d.dims[2];
    e.nc = int64_t(d.dims[0] + 1) * (d.dims[1] + 1) * (d.dims[2] + 1);
    e.two_begin = two_total;
    const int64_t nelem = e.npix * 3;
    e.inv_n = 1.0 / (double)nelem;
    e.gscale = (float)(1.0 / (double)nelem);

    pp[j] = (int32_t)pack_blocks;
    pi[j] = (int32_t)pix_blocks;
    pv[j] = (int32_t)vox_blocks;
    ps[j] = (int32_t)sg_blocks;
    pack_blocks += grid_for(e.nc, kBatchBlock);
    pix_blocks += grid_for(e.npix, kBatchBlock);
    vox_blocks += grid_for(e.nv, kBatchBlock);
    if (T.sg[0] > 0) sg_blocks += grid_for(int64_t(T.sg[0]) * T.sg[1] * T.sg[2], kBatchBlock);
    two_total += T.path_count;
    adj_total += A.path_count;
    if (pack_blocks >= INT32_MAX || pix_blocks >= INT32_MAX || vox_blocks >= INT32_MAX) {
      delete b;
      set_error("batch too large: more than 2^31 blocks in an elementwise kernel");
      return RCV_ERR_INVALID;
    }
  }
  pp[n] = (int32_t)pack_blocks;
  pi[n] = (int32_t)pix_blocks;
  pv[n] = (int32_t)vox_blocks;
  ps[n] = (int32_t)sg_blocks;
  b->sg_blocks = (int32_t)sg_blocks;
  b->total_two = two_total;
  b->total_adj = adj_total;
  b->pack_blocks = (int32_t)pack_blocks;
  b->pix_blocks = (int32_t)pix_blocks;
  b->vox_blocks = (int32_t)vox_blocks;

  RCV_REQUIRE(adj_total < (int64_t(1) << 32), "a batch must have fewer than 2^32 gradient paths");
  const PlanLayout P = plan_layout(n, two_total, adj_total);
  char* w = static_cast<char*>(workspace);
  b->entries = reinterpret_cast<BatchEntry*>(w + P.entries);
  b->two = reinterpret_cast<VolJob*>(w + P.two);
  b->adj = reinterpret_cast<VolJob*>(w + P.adj);
  b->prefix = reinterpret_cast<int32_t*>(w + P.prefix);
  b->queue = reinterpret_cast<unsigned long long*>(w + P.queue);
  b->counters = reinterpret_cast<uint64_t*>(w + P.counters);
  b->path_out = reinterpret_cast<float4*>(w + P.path_out);
  b->adjbuf.ckpt = reinterpret_cast<float4*>(w + P.ckpt);
  b->adjbuf.ckpt_count = b->queue + 3;
  b->adjbuf.ckpt_cap = ckpt_capacity(adj_total);
  b->adjbuf.path_ltot = reinterpret_cast<float4*>(w + P.ltot);
  // (tape slots are 32-bit indices: batches of 2^28 gradient paths or more replay)
  b->tape = b->opt.adjoint == RCV_ADJOINT_TAPE && adj_total < (int64_t(1) << 28);
  b->paired = b->tape && !b->opt.count_events && !b->opt.separate_tracers;
  if (b->tape) {
    const int per_path = b->opt.tape_events_per_path > 0 ? b->opt.tape_events_per_path : int(kTapeSlotsPerPath);
    b->adjbuf.tape = reinterpret_cast<float4*>(w + P.tape);
    b->adjbuf.tape_count = b->queue + 4;
    b->adjbuf.tape_cap = tape_capacity(adj_total, per_path);
    b->adjbuf.lost_list = reinterpret_cast<uint32_t*>(w + P.lost);
    b->adjbuf.lost_count = b->queue + 5;
    b->adjbuf.tape_f = tape_terms(w + P.tape, adj_total);
    b->tape_weights = reinterpret_cast<float4*>(w + P.ckpt + uint64_t(b->adjbuf.ckpt_cap) * 32u);
    b->cam_w = reinterpret_cast<float2*>(w + P.cam_w);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(b->entries, b->h_entries.data(), sizeof(BatchEntry) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->two, b->h_two.data(), sizeof(VolJob) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->adj, b->h_adj.data(), sizeof(VolJob) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->prefix, b->h_prefix.data(), sizeof(int32_t) * b->h_prefix.size(),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->counters, 0, 2 * RCV_COUNTER_COUNT * sizeof(uint64_t), st);
  if (e != cudaSuccess) {
    delete b;
    return cuda_check(e, "batch table upload");
  }
  warm_launch_config();
  if (cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess) {
    rcv_batch_destroy(b);
    return cuda_check(cudaGetLastError(), "batch stream / event creation");
  }
  *out = b;
  return RCV_OK;
}

namespace rcv {
static int enqueue_step(rcv_batch* b, cudaStream_t st) {
  const int n = b->n;
  const int32_t* pp = b->prefix;
  const int32_t* pi = pp + (n + 1);
  const int32_t* pv = pi + (n + 1);
  const int32_t* ps = pv + (n + 1);
  const bool sg = b->sg_blocks > 0;
  batch_prologue_kernel<<<1, kBatchBlock, 0, st>>>(b->entries, b->two, b->adj, n);
  int rc = launched("batch prologue launch");
  if (rc) return rc;
  batch_pack_kernel<<<(unsigned)b->pack_blocks, kBatchBlock, 0, st>>>(b->entries, pp, n);
  rc = launched("batch pack launch");
  if (rc) return rc;
  if (sg) {
    batch_supergrid_kernel<<<(unsigned)b->sg_blocks, kBatchBlock, 0, st>>>(b->entries, b->two, ps, n);
    rc = launched("batch supergrid launch");
    if (rc) return rc;
  }
  if (b->opt.order == RCV_ORDER_COST) {
    batch_order_count_kernel<<<(unsigned)b->pix_blocks, kBatchBlock, 0, st>>>(b->entries, pi, n);
    rc = launched("batch order count launch");
    if (rc) return rc;
    batch_order_scan_kernel<<<(unsigned)n, kRenderOrderBuckets, 0, st>>>(b->entries);
    rc = launched("batch order scan launch");
    if (rc) return rc;
    batch_order_place_kernel<<<(unsigned)b->pix_blocks, kBatchBlock, 0, st>>>(b->entries, pi, n);
    rc = launched("batch order place launch");
    if (rc) return rc;
  }
  VolJob none;
  std::memset(&none, 0, sizeof(none));
  // event counts only when asked for: the counting tracers hold the counts in registers
  uint64_t* cnt = b->opt.count_events ? b->counters : nullptr;
  if (b->paired) {
    // the adjoint radiance pass needs no image gradient: it runs in the
    // launch of the two-state pass
    RCV_TRY_CUDA(cudaMemsetAsync(b->adjbuf.ckpt_count, 0, 3 * sizeof(unsigned long long), st),
                 "adjoint counters reset");
    Queue QA, QB;
    rc = make_queue(kTwoState, b->two, n, b->total_two, &b->opt, b->queue + 0, b->path_out, nullptr, nullptr, st,
                    &QA);
    if (rc == RCV_OK)
      rc = make_queue(kTape, b->adj, n, b->total_adj, &b->opt, b->queue + 1, nullptr, &b->adjbuf, nullptr, st, &QB);
    if (rc == RCV_OK) rc = launch_pair(none, QA, none, QB, &b->opt, st, sg);
    if (rc) return rc;
    batch_image_kernel<<<(unsigned)b->pix_blocks, kBatchBlock, 0, st>>>(b->entries, pi, n, b->path_out);
    rc = launched("batch image launch");
    if (rc) return rc;
  } else {
    // ... or on the side stream beside the two-state pass and the image kernel
    RCV_TRY_CUDA(cudaEventRecord(b->fork, st), "fork record");
    RCV_TRY_CUDA(cudaStreamWaitEvent(b->side, b->fork, 0), "fork wait");
    // checkpoint / event-record, tape-slot and lost-path counters
    RCV_TRY_CUDA(cudaMemsetAsync(b->adjbuf.ckpt_count, 0, 3 * sizeof(unsigned long long), b->side),
                 "adjoint counters reset");
    rc = launch_persistent(b->tape ? kTape : kAdjoint, none, b->adj, n, b->total_adj, &b->opt, b->queue + 1,
                           nullptr, &b->adjbuf, cnt ? cnt + RCV_COUNTER_COUNT : nullptr, b->side, sg);
    if (rc) return rc;
    RCV_TRY_CUDA(cudaEventRecord(b->join, b->side), "join record");
    rc = launch_persistent(kTwoState, none, b->two, n, b->total_two, &b->opt, b->queue + 0, b->path_out, nullptr,
                           cnt, st, sg);
    if (rc) return rc;
    batch_image_kernel<<<(unsigned)b->pix_blocks, kBatchBlock, 0, st>>>(b->entries, pi, n, b->path_out);
    rc = launched("batch image launch");
    if (rc) return rc;
    RCV_TRY_CUDA(cudaStreamWaitEvent(st, b->join, 0), "join wait");
  }
  if (b->tape) {
    // the gradient from the tape; the replay then takes only the lost paths
    rc = launch_tape_gradient(none, b->adj, n, b->adjbuf, b->tape_weights, b->cam_w, b->total_adj,
                              cnt ? cnt + RCV_COUNTER_COUNT : nullptr, tracer_sm_count(), st);
    if (rc) return rc;
  }
  rc = launch_persistent(kReplay, none, b->adj, n, b->total_adj, &b->opt, b->queue + 2, nullptr, &b->adjbuf,
                         cnt ? cnt + RCV_COUNTER_COUNT : nullptr, st, sg);
  if (rc) return rc;
  batch_update_kernel<<<(unsigned)b->vox_blocks, kBatchBlock, 0, st>>>(b->entries, pv, n);
  return launched("batch update launch");
}
}  // namespace rcv

extern "C" int rcv_batch_step(rcv_batch* b, int32_t use_graph, void* stream) {
  RCV_REQUIRE(b != nullptr, "batch is NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!use_graph) return enqueue_step(b, st);
  if (b->exec == nullptr) {
    if (b->capture_stream == nullptr)
      RCV_TRY_CUDA(cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking), "capture stream");
    RCV_TRY_CUDA(cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    const uint64_t before = rcv_kernel_launches();
    const int rc = enqueue_step(b, b->capture_stream);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->capture_stream, &g);
    // captured launches did not run: take them out of the launch count
    add_launches(-int64_t(rcv_kernel_launches() - before));
    if (rc != RCV_OK || e != cudaSuccess) {
      if (g != nullptr) cudaGraphDestroy(g);
      return rc != RCV_OK ? rc : cuda_check(e, "end capture");
    }
    const cudaError_t ie = cudaGraphInstantiate(&b->exec, g, 0);
    if (ie != cudaSuccess) {
      cudaGraphDestroy(g);
      b->exec = nullptr;
      return cuda_check(ie, "graph instantiate");
    }
    b->graph = g;
  }
  RCV_TRY_CUDA(cudaGraphLaunch(b->exec, st), "graph launch");
  add_launches(rcv_batch_kernels_per_step(b));
  return RCV_OK;
}

extern "C" uint64_t* rcv_batch_counters(rcv_batch* b) { return b != nullptr ? b->counters : nullptr; }

extern "C" int32_t rcv_batch_kernels_per_step(const rcv_batch* b) {
  if (b == nullptr) return RCV_ERR_INVALID;
  return kBatchKernels + (b->opt.order == RCV_ORDER_COST ? 3 : 0) + (b->sg_blocks > 0 ? 1 : 0) + (b->tape ? 2 : 0) -
         (b->paired ? 1 : 0);
}

extern "C" int rcv_batch_destroy(rcv_batch* b) {
  if (b == nullptr) return RCV_OK;
  if (b->exec != nullptr) cudaGraphExecDestroy(b->exec);
  if (b->graph != nullptr) cudaGraphDestroy(b->graph);
  if (b->capture_stream != nullptr) cudaStreamDestroy(b->capture_stream);
  if (b->side != nullptr) cudaStreamDestroy(b->side);
  if (b->fork != nullptr) cudaEventDestroy(b->fork);
  if (b->join != nullptr) cudaEventDestroy(b->join);
  delete b;
  return RCV_OK;
}
