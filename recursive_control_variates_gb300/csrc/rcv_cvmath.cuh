// Per-element arithmetic of the recursive control variate, shared by the
// single-job and the batched kernels: EMA-Welford update (plugins/welford.py:
// 59-75), weight update (plugins/cv_integrator.py:60-67) and blend (:69), in
// the reference's float32 operation order (built with -fmad=false).
#pragma once
#include <cstdint>

#include "../../include/rcv.h"

namespace rcv {

// Scalars of one control-variate step.  Bias corrections are the float32
// values the reference's float32 tensors produce: beta^n rounded to float32,
// then 1 - that in float32.
struct CvScalars {
  float b1, b2, omb1, omb2;  // beta1, beta2, 1-beta1, 1-beta2 (float32)
  float d1_prev;             // 1 - beta1^n       (n = count before the update)
  float d1_next;             // 1 - beta1^(n+1)
  float d2_get;              // 1 - beta2^n_get   (count seen by get())
  int32_t has_prev;          // n > 0
  int32_t do_pre, do_weight, do_post;
};

__host__ __device__ __forceinline__ void welford2(const CvScalars& S, float x, float y, float& mean_x,
                                                  float& mean_y, float& var_x, float& var_y, float& cov) {
  const float dx1 = S.has_prev ? x - mean_x / S.d1_prev : x;
  const float dy1 = S.has_prev ? y - mean_y / S.d1_prev : y;
  mean_y = S.b1 * mean_y + S.omb1 * y;
  mean_x = S.b1 * mean_x + S.omb1 * x;
  const float dx2 = x - mean_x / S.d1_next;
  const float dy2 = y - mean_y / S.d1_next;
  var_x = S.b2 * var_x + (S.omb2 * dx1) * dx2;
  var_y = S.b2 * var_y + (S.omb2 * dy1) * dy2;
  cov = S.b2 * cov + (S.omb2 * dx1) * dy2;
}

// One element of a control-variate step, in place on the state arrays;
// returns the blended image value.
__device__ __forceinline__ float cv_element(const rcv_cv_state& st, int64_t i, float x, float y,
                                            const CvScalars& S) {
  float img = st.img[i], w = st.w_s[i], vn = st.v_n[i];
  float mx = st.mean_x[i], my = st.mean_y[i], vx = st.var_x[i], vy = st.var_y[i], cv = st.cov[i];
  if (S.do_pre) welford2(S, x, y, mx, my, vx, vy, cv);
  if (S.do_weight) {
    const float v0 = vx / S.d2_get, v1 = vy / S.d2_get, c = cv / S.d2_get;
    vn = ((w * w) * (vn + v0) + v1) - (2.0f * w) * c;
    w = c / (v0 + vn);
    if (isnan(w) || isinf(w)) w = 0.0f;
    w = fminf(fmaxf(w, 0.0f), 1.0f);
  }
  img = w * (img - x) + y;
  if (S.do_post) welford2(S, x, y, mx, my, vx, vy, cv);
  st.img[i] = img;
  st.w_s[i] = w;
  st.v_n[i] = vn;
  st.mean_x[i] = mx;
  st.mean_y[i] = my;
  st.var_x[i] = vx;
  st.var_y[i] = vy;
  st.cov[i] = cv;
  return img;
}

// Adam update of one parameter value (bias correction folded into lr_t) +
// clamp; updates the moments in place and returns the new value.
__device__ __forceinline__ float adam_value(float p, float g, float& m, float& v, float lr_t, float b1, float b2,
                                            float omb1, float omb2, float eps, float lo, float hi) {
  m = b1 * m + omb1 * g;
  v = b2 * v + omb2 * (g * g);
  const float q = p - (lr_t * m) / (sqrtf(v) + eps);
  return fminf(fmaxf(q, lo), hi);
}

__device__ __forceinline__ void adam_element(float* p, float* g, float* m, float* v, int64_t i, float lr_t,
                                             float b1, float b2, float omb1, float omb2, float eps, float lo,
                                             float hi, bool zero_grad) {
  float mi = m[i], vi = v[i];
  const float pi = adam_value(p[i], g[i], mi, vi, lr_t, b1, b2, omb1, omb2, eps, lo, hi);
  m[i] = mi;
  v[i] = vi;
  p[i] = pi;
  if (zero_grad) g[i] = 0.0f;
}

// Derivative of the image loss for one element (utils.py:21-25): L2
// 2 diff / n, L1 sign(diff) / n with gscale = float32(1 / n); adds the
// element's loss term to acc.
__device__ __forceinline__ float loss_grad(int kind, float diff, float gscale, double& acc) {
  if (kind == RCV_LOSS_L2) {
    acc += double(diff * diff);
    return (2.0f * diff) * gscale;
  }
  acc += double(fabsf(diff));
  return (diff > 0.0f ? 1.0f : (diff < 0.0f ? -1.0f : 0.0f)) * gscale;
}

}  // namespace rcv
