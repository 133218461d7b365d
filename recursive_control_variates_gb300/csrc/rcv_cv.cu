// Per-pixel recursive control variate (blend + EMA-Welford statistics),
// image losses and the Adam/clamp step of librcv, with their C-ABI entry
// points.  All arithmetic follows the float32 operation order of the
// reference (plugins/cv_integrator.py:58-77, plugins/welford.py:4-78,
// utils.py:21-25) with no contraction (the library builds with -fmad=false).
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>

#include "rcv_common.h"
#include "rcv_cvmath.cuh"
#include "rcv_device.cuh"

namespace rcv {

static thread_local char g_error[512] = {0};
static std::atomic<uint64_t> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void add_launches(int64_t delta) { g_launches.fetch_add(uint64_t(delta), std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_error, sizeof(g_error), fmt, ap);
  va_end(ap);
}

static float pow_f32(float b, int n) { return (float)std::pow((double)b, (double)n); }

__global__ void cv_step_kernel(rcv_cv_state st, int64_t n, const float* __restrict__ H,
                               const float* __restrict__ F, CvScalars S) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  cv_element(st, i, H[i], F[i], S);
}

__global__ void stats_update_kernel(rcv_cv_state st, int64_t n, const float* __restrict__ X,
                                    const float* __restrict__ Y, CvScalars S) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float mx = st.mean_x[i], my = st.mean_y[i], vx = st.var_x[i], vy = st.var_y[i], cv = st.cov[i];
  welford2(S, X[i], Y[i], mx, my, vx, vy, cv);
  st.mean_x[i] = mx;
  st.mean_y[i] = my;
  st.var_x[i] = vx;
  st.var_y[i] = vy;
  st.cov[i] = cv;
}

__global__ void clamp_kernel(float* __restrict__ x, int64_t n, float lo, float hi) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) x[i] = fminf(fmaxf(x[i], lo), hi);
}

__global__ void stats_get_kernel(const float* __restrict__ vx, const float* __restrict__ vy,
                                 const float* __restrict__ cv, int64_t n, float d2,
                                 float* __restrict__ ox, float* __restrict__ oy,
                                 float* __restrict__ oc) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  ox[i] = vx[i] / d2;
  oy[i] = vy[i] / d2;
  oc[i] = cv[i] / d2;
}

__global__ void welford1_kernel(float* __restrict__ mean, float* __restrict__ var, int64_t n,
                                const float* __restrict__ xs, CvScalars S) {
  // plugins/welford.py:25-31
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = xs[i];
  float m = mean[i], v = var[i];
  const float dx1 = S.has_prev ? x - m / S.d1_prev : x;
  m = S.b1 * m + S.omb1 * x;
  const float dx2 = x - m / S.d1_next;
  v = S.b2 * v + (S.omb2 * dx1) * dx2;
  mean[i] = m;
  var[i] = v;
}

__global__ void div_kernel(const float* __restrict__ a, int64_t n, float d, float* __restrict__ o) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) o[i] = a[i] / d;
}

// ------------------------------------------------------------------- losses
constexpr int kLossBlock = 256;
constexpr int kLossMaxBlocks = 1024;

__global__ void loss_partial_kernel(int kind, const float* __restrict__ img,
                                    const float* __restrict__ ref, int64_t n, float gscale,
                                    float* __restrict__ grad, double* __restrict__ partials) {
  double acc = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += int64_t(gridDim.x) * blockDim.x) {
    const float gi = loss_grad(kind, img[i] - ref[i], gscale, acc);
    if (grad) grad[i] = gi;
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  __shared__ double warp_sums[kLossBlock / 32];
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kLossBlock / 32; ++k) s += warp_sums[k];
    partials[blockIdx.x] = s;
  }
}

__global__ void loss_final_kernel(const double* __restrict__ partials, int nblocks, double inv_n,
                                  float* __restrict__ loss) {
  __shared__ double sh[kLossMaxBlocks];
  for (int k = threadIdx.x; k < kLossMaxBlocks; k += blockDim.x) sh[k] = k < nblocks ? partials[k] : 0.0;
  __syncthreads();
  for (int w = kLossMaxBlocks / 2; w > 0; w >>= 1) {
    for (int k = threadIdx.x; k < w; k += blockDim.x) sh[k] += sh[k + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = float(sh[0] * inv_n);
}

// --------------------------------------------------------------------- Adam
__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr_t, float b1, float b2,
                            float omb1, float omb2, float eps, float lo, float hi, int zero_grad) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  adam_element(p, g, m, v, i, lr_t, b1, b2, omb1, omb2, eps, lo, hi, zero_grad != 0);
}

static CvScalars make_scalars(float beta1, float beta2, int n) {
  CvScalars S;
  std::memset(&S, 0, sizeof(S));
  S.b1 = beta1;
  S.b2 = beta2;
  S.omb1 = 1.0f - beta1;
  S.omb2 = 1.0f - beta2;
  S.has_prev = n > 0;
  S.d1_prev = n > 0 ? 1.0f - pow_f32(beta1, n) : 1.0f;
  S.d1_next = 1.0f - pow_f32(beta1, n + 1);
  return S;
}

}  // namespace rcv

using namespace rcv;

extern "C" const char* rcv_last_error(void) { return g_error; }

extern "C" uint64_t rcv_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" int rcv_device_info(int32_t* major, int32_t* minor, int32_t* sm_count) {
  int dev = 0;
  RCV_TRY_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  int a = 0, b = 0, c = 0;
  RCV_TRY_CUDA(cudaDeviceGetAttribute(&a, cudaDevAttrComputeCapabilityMajor, dev), "attr");
  RCV_TRY_CUDA(cudaDeviceGetAttribute(&b, cudaDevAttrComputeCapabilityMinor, dev), "attr");
  RCV_TRY_CUDA(cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev), "attr");
  if (major) *major = a;
  if (minor) *minor = b;
  if (sm_count) *sm_count = c;
  return RCV_OK;
}

extern "C" uint64_t rcv_struct_size(const char* name) {
  if (name == nullptr) return 0;
  struct Entry {
    const char* name;
    uint64_t size;
  };
  static const Entry table[] = {
      {"rcv_camera_frame", sizeof(rcv_camera_frame)}, {"rcv_sensor", sizeof(rcv_sensor)},
      {"rcv_medium", sizeof(rcv_medium)},             {"rcv_volpath_options", sizeof(rcv_volpath_options)},
      {"rcv_sphere", sizeof(rcv_sphere)},             {"rcv_surface_scene", sizeof(rcv_surface_scene)},
      {"rcv_cv_state", sizeof(rcv_cv_state)},         {"rcv_batch_job", sizeof(rcv_batch_job)},
      {"rcv_batch_job_status", sizeof(rcv_batch_job_status)},
      {"rcv_volpathsimple_flags", sizeof(rcv_volpathsimple_flags)}, {"rcv_envmap", sizeof(rcv_envmap)},
  };
  for (const Entry& e : table)
    if (std::strcmp(e.name, name) == 0) return e.size;
  return 0;
}

extern "C" void rcv_sample_tea_32(uint32_t v0, uint32_t v1, uint32_t out[2]) {
  uint32_t a, b;
  tea(v0, v1, 4, a, b);
  out[0] = a;
  out[1] = b;
}

static int check_state(const rcv_cv_state* s) {
  RCV_REQUIRE(s != nullptr, "state is NULL");
  RCV_REQUIRE(s->img && s->w_s && s->v_n && s->mean_x && s->mean_y && s->var_x && s->var_y && s->cov,
              "a control-variate state array is NULL");
  return RCV_OK;
}

extern "C" int rcv_cv_step(const rcv_cv_state* state, int64_t n, const float* H, const float* F,
                           int32_t it, int32_t warmup, int32_t* welford_count, float beta1,
                           float beta2, int32_t pre_update, void* stream) {
  int rc = check_state(state);
  if (rc) return rc;
  RCV_REQUIRE(n > 0, "n must be positive");
  RCV_REQUIRE(H != nullptr && F != nullptr, "H / F are NULL");
  RCV_REQUIRE(welford_count != nullptr && *welford_count >= 0, "welford_count is invalid");
  RCV_REQUIRE(it >= 0, "it must be non-negative");
  int count = *welford_count;
  CvScalars S = make_scalars(beta1, beta2, count);
  const bool update = it > 0;
  S.do_pre = update && pre_update;
  S.do_post = update && !pre_update;
  S.do_weight = it > warmup;
  // get() sees the count after a pre-update, before a post-update
  const int n_get = count + (S.do_pre ? 1 : 0);
  S.d2_get = 1.0f - pow_f32(beta2, n_get);
  const int block = 256;
  cv_step_kernel<<<grid_for(n, block), block, 0, static_cast<cudaStream_t>(stream)>>>(*state, n, H,
                                                                                       F, S);
  rc = launched("cv_step launch");
  if (rc) return rc;
  if (update) *welford_count = count + 1;
  return RCV_OK;
}

extern "C" int rcv_statistics_get(const rcv_cv_state* state, int64_t n, int32_t welford_count,
                                  float beta2, float* out_vx, float* out_vy, float* out_cov,
                                  void* stream) {
  int rc = check_state(state);
  if (rc) return rc;
  RCV_REQUIRE(out_vx && out_vy && out_cov, "outputs are NULL");
  const float d2 = 1.0f - pow_f32(beta2, welford_count);
  const int block = 256;
  stats_get_kernel<<<grid_for(n, block), block, 0, static_cast<cudaStream_t>(stream)>>>(
      state->var_x, state->var_y, state->cov, n, d2, out_vx, out_vy, out_cov);
  return launched("stats_get launch");
}

extern "C" int rcv_statistics_update(const rcv_cv_state* state, int64_t n, const float* x,
                                     const float* y, int32_t* welford_count, float beta1,
                                     float beta2, void* stream) {
  int rc = check_state(state);
  if (rc) return rc;
  RCV_REQUIRE(n > 0, "n must be positive");
  RCV_REQUIRE(x != nullptr && y != nullptr, "x / y are NULL");
  RCV_REQUIRE(welford_count != nullptr && *welford_count >= 0, "welford_count is invalid");
  CvScalars S = make_scalars(beta1, beta2, *welford_count);
  const int block = 256;
  stats_update_kernel<<<grid_for(n, block), block, 0, static_cast<cudaStream_t>(stream)>>>(*state, n,
                                                                                           x, y, S);
  rc = launched("stats_update launch");
  if (rc) return rc;
  *welford_count += 1;
  return RCV_OK;
}

extern "C" int rcv_clamp(float* x, int64_t n, float lo, float hi, void* stream) {
  RCV_REQUIRE(x != nullptr, "x is NULL");
  RCV_REQUIRE(n > 0, "n must be positive");
  const int block = 256;
  clamp_kernel<<<grid_for(n, block), block, 0, static_cast<cudaStream_t>(stream)>>>(x, n, lo, hi);
  return launched("clamp launch");
}

extern "C" int rcv_welford_update(float* mean, float* var, int64_t n, const float* x,
                                  int32_t* count, float beta1, float beta2, void* stream) {
  RCV_REQUIRE(mean && var && x, "welford buffers are NULL");
  RCV_REQUIRE(count != nullptr && *count >= 0, "count is invalid");
  RCV_REQUIRE(n > 0, "n must be positive");
  CvScalars S = make_scalars(beta1, beta2, *count);
  const int block = 256;
  welford1_kernel<<<grid_for(n, block), block, 0, static_cast<cudaStream_t>(stream)>>>(mean, var, n,
                                                                                        x, S);
  int rc = launched("welford launch");
  if (rc) return rc;
  *count += 1;
  return RCV_OK;
}

extern "C" int rcv_welford_get(const float* var, int64_t n, int32_t count, float beta2, float* out,
                               void* stream) {
  RCV_REQUIRE(var && out, "welford buffers are NULL");
  const float d2 = 1.0f - pow_f32(beta2, count);
  const int block = 256;
  div_kernel<<<grid_for(n, block), block, 0, static_cast<cudaStream_t>(stream)>>>(var, n, d2, out);
  return launched("welford_get launch");
}

extern "C" uint64_t rcv_loss_workspace_bytes(int64_t n) {
  (void)n;
  return align256(sizeof(double) * kLossMaxBlocks);
}

extern "C" int rcv_loss(int32_t kind, const float* img, const float* ref, int64_t n, float* loss,
                        float* grad, void* workspace, void* stream) {
  RCV_REQUIRE(kind == RCV_LOSS_L2 || kind == RCV_LOSS_L1, "unknown loss kind %d", kind);
  RCV_REQUIRE(img && ref && loss && workspace, "loss buffers are NULL");
  RCV_REQUIRE(n > 0, "n must be positive");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int64_t nb = (n + kLossBlock * 4 - 1) / (kLossBlock * 4);
  if (nb > kLossMaxBlocks) nb = kLossMaxBlocks;
  if (nb < 1) nb = 1;
  const float gscale = (float)(1.0 / (double)n);
  double* partials = static_cast<double*>(workspace);
  loss_partial_kernel<<<(unsigned)nb, kLossBlock, 0, st>>>(kind, img, ref, n, gscale, grad, partials);
  int rc = launched("loss launch");
  if (rc) return rc;
  loss_final_kernel<<<1, 256, 0, st>>>(partials, (int)nb, 1.0 / (double)n, loss);
  return launched("loss final launch");
}

extern "C" int rcv_adam_step(float* param, float* grad, float* m, float* v, int64_t n, int32_t t,
                             float lr, float beta1, float beta2, float eps, float lo, float hi,
                             int32_t zero_grad, void* stream) {
  RCV_REQUIRE(param && grad && m && v, "adam buffers are NULL");
  RCV_REQUIRE(t >= 1, "adam step count must be >= 1");
  RCV_REQUIRE(n > 0, "n must be positive");
  // lr_t = lr * sqrt(1 - beta2^t) / (1 - beta1^t)
  const double bc2 = 1.0 - std::pow((double)beta2, (double)t);
  const double bc1 = 1.0 - std::pow((double)beta1, (double)t);
  const float lr_t = (float)((double)lr * std::sqrt(bc2) / bc1);
  const int block = 256;
  adam_kernel<<<grid_for(n, block), block, 0, static_cast<cudaStream_t>(stream)>>>(
      param, grad, m, v, n, lr_t, beta1, beta2, 1.0f - beta1, 1.0f - beta2, eps, lo, hi, zero_grad);
  return launched("adam launch");
}

// ------------------------------------------------- bias-correction tables
namespace rcv {
constexpr int64_t kMaxPowerTable = int64_t(1) << 22;
}

extern "C" int64_t rcv_cv_table_len(float beta) {
  RCV_REQUIRE(beta >= 0.0f && beta < 1.0f, "beta must be in [0, 1), got %g", (double)beta);
  for (int64_t k = 0; k < kMaxPowerTable; ++k)
    if (1.0f - pow_f32(beta, (int)k) == 1.0f) return k + 1;
  set_error("beta = %.9g: 1 - beta^k does not reach 1.0f within %lld steps", (double)beta,
            (long long)kMaxPowerTable);
  return RCV_ERR_UNSUPPORTED;
}

extern "C" int rcv_cv_table_fill(float beta, float* out, int64_t len) {
  RCV_REQUIRE(beta >= 0.0f && beta < 1.0f, "beta must be in [0, 1), got %g", (double)beta);
  RCV_REQUIRE(out != nullptr && len > 0 && len <= kMaxPowerTable, "invalid table buffer / length");
  for (int64_t k = 0; k < len; ++k) out[k] = 1.0f - pow_f32(beta, (int)k);
  return RCV_OK;
}

namespace rcv {
// (sqrt(1 - beta2^t), 1 - beta1^t) with the arithmetic of rcv_adam_step.
static void adam_corrections(float beta1, float beta2, int64_t t, double& s2, double& bc1) {
  const double bc2 = 1.0 - std::pow((double)beta2, (double)t);
  bc1 = 1.0 - std::pow((double)beta1, (double)t);
  s2 = std::sqrt(bc2);
}
}  // namespace rcv

extern "C" int64_t rcv_adam_table_len(float beta1, float beta2) {
  RCV_REQUIRE(beta1 >= 0.0f && beta1 < 1.0f && beta2 >= 0.0f && beta2 < 1.0f,
              "Adam betas must be in [0, 1)");
  for (int64_t t = 0; t < kMaxPowerTable; ++t) {
    double s2, bc1;
    adam_corrections(beta1, beta2, t, s2, bc1);
    if (s2 == 1.0 && bc1 == 1.0) return t + 1;
  }
  set_error("Adam betas (%.9g, %.9g): bias corrections do not reach 1.0 within %lld steps", (double)beta1,
            (double)beta2, (long long)kMaxPowerTable);
  return RCV_ERR_UNSUPPORTED;
}

extern "C" int rcv_adam_table_fill(float beta1, float beta2, double* out, int64_t len) {
  RCV_REQUIRE(beta1 >= 0.0f && beta1 < 1.0f && beta2 >= 0.0f && beta2 < 1.0f,
              "Adam betas must be in [0, 1)");
  RCV_REQUIRE(out != nullptr && len > 0 && len <= kMaxPowerTable, "invalid table buffer / length");
  for (int64_t t = 0; t < len; ++t) adam_corrections(beta1, beta2, t, out[2 * t], out[2 * t + 1]);
  return RCV_OK;
}
