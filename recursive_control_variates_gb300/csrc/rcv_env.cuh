// Environment map emitter (the reference's `envmap`, experiments.py:81-85,
// 195-199, 315-319): latitude-longitude RGB radiance with bilinear lookup and
// importance sampling from a piecewise-constant density over the texels.
//
// Conventions (include/rcv.h, rcv_envmap): a world direction (x, y, z) maps
// to u = atan2(x, -z) / (2 pi) wrapped into [0, 1) and v = acos(y) / pi; row 0
// is the +y pole.  The sampling density of texel (i, j) is proportional to
// f_ij = luminance_ij * sin(theta_i) at the row centre; in (u, v) it is
// p = f_ij * W * H / sum(f), in solid angle p / (2 pi^2 sin(theta)) (the
// piecewise-constant 2D distribution of Pharr, Jakob & Humphreys, Physically
// Based Rendering, "infinite area lights").  Sampling inverts the marginal CDF
// over rows and the conditional CDF of the chosen row by binary search and
// places the sample linearly inside the texel.
//
// atan2 is evaluated by octant reduction, a pi/4 shift for arguments above
// tan(pi/8) and the arctangent Taylor series through x^19 (error below 1e-9
// relative on the reduced range); sin / cos by sincos_2pi.  The CPU oracle
// restates the same operations, so both give the same bits.
#pragma once
#include "rcv_device.cuh"

namespace rcv {

constexpr float kInvTwoPi = 0.159154943091895335769f;
constexpr float kEnvInvPi = 0.318309886183790671538f;
constexpr float kInv2PiSq = 0.0506605918211688965f;  // 1 / (2 pi^2)
constexpr float kPiF = 3.14159265358979323846f;
constexpr float kQuarterPi = 0.785398163397448309616f;

// Device view of a prepared environment map (valid = 0: the constant white
// environment of radiance 1).
struct EnvMap {
  int32_t valid, w, h, pad;
  float inv_w, inv_h, scale, pad2;
  const float4* tex;  // [h][w] (r, g, b, f)
  const float* cond;  // [h][w + 1] conditional CDF of each row
  const float* marg;  // [h + 1] marginal CDF over rows
  const float* hdr;   // [0] W * H / sum(f), [1] 1 when sum(f) > 0 (else no NEE samples)
};

// Workspace layout of an environment map (256-byte aligned sections):
// header, texels with their sampling weights, conditional CDFs, marginal
// CDF, row sums (double).
struct EnvLayout {
  uint64_t hdr, tex, cond, marg, rows, total;
};

inline uint64_t env_align(uint64_t v) { return (v + 255u) & ~uint64_t(255u); }

inline EnvLayout env_layout(int w, int h) {
  EnvLayout L;
  L.hdr = 0;
  L.tex = 256;
  L.cond = L.tex + env_align(uint64_t(w) * uint64_t(h) * 16u);
  L.marg = L.cond + env_align(uint64_t(w + 1) * uint64_t(h) * 4u);
  L.rows = L.marg + env_align(uint64_t(h + 1) * 4u);
  L.total = L.rows + env_align(uint64_t(h) * 8u);
  return L;
}

RCV_HD float ldf(const float* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

RCV_HD float4 ldf4(const float4* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

// Sampling weight f of texel (row i) and luminance of an RGB value.
RCV_HD float env_luminance(float r, float g, float b) { return (0.2126f * r + 0.7152f * g) + 0.0722f * b; }

RCV_HD float env_row_sin(int i, float inv_h) {
  float s, c;
  sincos_2pi((((float)i + 0.5f) * inv_h) * 0.5f, s, c);
  return s;
}

// arctan of a in [0, 1].
RCV_HD float atan_unit(float a) {
  const bool big = a > 0.414213562373095f;  // tan(pi/8)
  const float x = big ? (a - 1.0f) / (a + 1.0f) : a;
  const float x2 = x * x;
  float p = fmaf(x2, -1.0f / 19.0f, 1.0f / 17.0f);
  p = fmaf(x2, p, -1.0f / 15.0f);
  p = fmaf(x2, p, 1.0f / 13.0f);
  p = fmaf(x2, p, -1.0f / 11.0f);
  p = fmaf(x2, p, 1.0f / 9.0f);
  p = fmaf(x2, p, -1.0f / 7.0f);
  p = fmaf(x2, p, 1.0f / 5.0f);
  p = fmaf(x2, p, -1.0f / 3.0f);
  const float r = fmaf(x * x2, p, x);
  return big ? r + kQuarterPi : r;
}

// atan2(y, x) in (-pi, pi].
RCV_HD float atan2_own(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  const float a = mx > 0.0f ? mn / mx : 0.0f;
  float r = atan_unit(a);
  if (ay > ax) r = 2.0f * kQuarterPi - r;
  if (x < 0.0f) r = kPiF - r;
  return y < 0.0f ? -r : r;
}

// (u, v) and sin(theta) of a unit world direction.
RCV_HD void env_uv(const V3& d, float& u, float& v, float& sin_t) {
  u = atan2_own(d.x, -d.z) * kInvTwoPi;
  if (u < 0.0f) u = u + 1.0f;
  if (!(u < 1.0f)) u = 0.0f;
  sin_t = sqrtf(fmaxf(0.0f, fmaf(-d.y, d.y, 1.0f)));
  v = atan2_own(sin_t, d.y) * kEnvInvPi;
}

// Unit world direction of (u, v) and its sin(theta).
RCV_HD V3 env_dir(float u, float v, float& sin_t) {
  float st, ct, sp, cp;
  sincos_2pi(v * 0.5f, st, ct);  // theta = pi v
  sincos_2pi(u, sp, cp);         // phi = 2 pi u
  sin_t = st;
  return V3{st * sp, ct, -(st * cp)};
}

RCV_HD int wrapi(int x, int n) {
  const int r = x % n;
  return r < 0 ? r + n : r;
}

// Bilinear radiance at (u, v), times the map's scale.
RCV_HD V3 env_eval_uv(const EnvMap& E, float u, float v) {
  const float fx = fmaf(u, (float)E.w, -0.5f), fy = fmaf(v, (float)E.h, -0.5f);
  const float x0f = floorf(fx), y0f = floorf(fy);
  const float tx = fx - x0f, ty = fy - y0f;
  const int x0 = (int)fmaxf(fminf(x0f, (float)E.w), -1.0f);
  const int y0 = (int)fmaxf(fminf(y0f, (float)E.h), -1.0f);
  const int ix0 = wrapi(x0, E.w), ix1 = wrapi(x0 + 1, E.w);
  const int iy0 = y0 < 0 ? 0 : (y0 > E.h - 1 ? E.h - 1 : y0);
  const int iy1 = y0 + 1 < 0 ? 0 : (y0 + 1 > E.h - 1 ? E.h - 1 : y0 + 1);
  const float4 a = ldf4(E.tex + (int64_t)iy0 * E.w + ix0), b = ldf4(E.tex + (int64_t)iy0 * E.w + ix1);
  const float4 c = ldf4(E.tex + (int64_t)iy1 * E.w + ix0), d = ldf4(E.tex + (int64_t)iy1 * E.w + ix1);
  const V3 r{lerpf(lerpf(a.x, b.x, tx), lerpf(c.x, d.x, tx), ty), lerpf(lerpf(a.y, b.y, tx), lerpf(c.y, d.y, tx), ty),
             lerpf(lerpf(a.z, b.z, tx), lerpf(c.z, d.z, tx), ty)};
  return V3{r.x * E.scale, r.y * E.scale, r.z * E.scale};
}

// Solid-angle pdf of sampling a unit world direction (0 for a black map).
RCV_HD float env_pdf(const EnvMap& E, float u, float v, float sin_t) {
  if (ldf(E.hdr + 1) == 0.0f || !(sin_t > 0.0f)) return 0.0f;
  int i = (int)(v * (float)E.h), j = (int)(u * (float)E.w);
  i = i < 0 ? 0 : (i > E.h - 1 ? E.h - 1 : i);
  j = j < 0 ? 0 : (j > E.w - 1 ? E.w - 1 : j);
  const float f = ldf4(E.tex + (int64_t)i * E.w + j).w;
  return ((f * ldf(E.hdr)) * kInv2PiSq) / sin_t;
}

// Index k in [0, n - 1] with cdf[k] <= x < cdf[k + 1] (cdf[0] = 0 <= x < 1 = cdf[n]).
RCV_HD int cdf_find(const float* cdf, int n, float x) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (ldf(cdf + mid) <= x)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Samples a unit world direction from (u0, u1): its radiance Le and pdf
// (pdf 0 when nothing can be sampled: a black map, or the pole of the
// parametrisation).
RCV_HD V3 env_sample(const EnvMap& E, float u0, float u1, V3& Le, float& pdf) {
  Le = V3{0.0f, 0.0f, 0.0f};
  pdf = 0.0f;
  if (ldf(E.hdr + 1) == 0.0f) return V3{0.0f, 1.0f, 0.0f};
  const int i = cdf_find(E.marg, E.h, u1);
  const float m0 = ldf(E.marg + i), m1 = ldf(E.marg + i + 1);
  const float dv = (u1 - m0) / (m1 - m0);
  const float* row = E.cond + (int64_t)i * (E.w + 1);
  const int j = cdf_find(row, E.w, u0);
  const float c0 = ldf(row + j), c1 = ldf(row + j + 1);
  const float du = (u0 - c0) / (c1 - c0);
  const float u = ((float)j + du) * E.inv_w, v = ((float)i + dv) * E.inv_h;
  float sin_t;
  const V3 d = env_dir(u, v, sin_t);
  const float f = ldf4(E.tex + (int64_t)i * E.w + j).w;
  if (sin_t > 0.0f) {
    pdf = ((f * ldf(E.hdr)) * kInv2PiSq) / sin_t;
    Le = env_eval_uv(E, u, v);
  }
  return d;
}

// Power heuristic of a strategy of pdf a against one of pdf b
// (mis_weight of mitsuba.ad.common, used at plugins/twostatevolpath.py:302,341).
RCV_HD float env_mis(float a, float b) {
  const float a2 = a * a, b2 = b * b;
  const float s = a2 + b2;
  return s > 0.0f ? a2 / s : 0.0f;
}

}  // namespace rcv
