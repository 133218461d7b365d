// Device-side arithmetic shared by every volumetric kernel of librcv.
//
// Everything here is written so that a CPU restatement that performs the same
// IEEE-754 single-precision operations in the same order (no contraction,
// explicit fmaf) produces bit-identical results: the library is compiled with
// -fmad=false, transcendental functions are evaluated by the project's own
// polynomial kernels below instead of CUDA's libm, and division / sqrt use the
// default IEEE-rounded forms.
//
// Behaviour restated (not copied) from the reference path:
//   - per-lane PCG32 streams seeded by TEA (Mitsuba's `independent` sampler,
//     used by plugins/twostatevolpath.py:104-112 via `self.prepare`);
//   - trilinear `gridvolume` lookups at voxel centres with clamp-to-edge
//     (plugins/twostatemedium.py:93-94 `get_scattering_coefficients`);
//   - uniform sphere sampling for the isotropic phase function and for the
//     constant environment emitter (plugins/twostatevolpath.py:275, 393).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#ifndef RCV_HD
#define RCV_HD __host__ __device__ __forceinline__
#endif

namespace rcv {

// 1/(4*pi) rounded to float: pdf of a uniform direction on the sphere.
constexpr float kInvFourPi = 0.0795774715459476678844f;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kHalfPi = 1.57079632679489661923f;
constexpr float kInf = __builtin_huge_valf();

// ---------------------------------------------------------------- sampler --
// TEA block cipher with the key schedule of Zafar, Olano & Curtis, "GPU random
// numbers via the tiny encryption algorithm" (HPG 2010).  The reference uses
// it as `mi.sample_tea_32` for the default gradient seed
// (plugins/twostatepath.py:87-89).
RCV_HD void tea(uint32_t v0, uint32_t v1, int rounds, uint32_t& o0, uint32_t& o1) {
  uint32_t sum = 0;
  for (int i = 0; i < rounds; ++i) {
    sum += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + sum) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + sum) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  o0 = v0;
  o1 = v1;
}

// PCG32 (O'Neill 2014, pcg32_random_r / pcg32_srandom_r).
struct Pcg32 {
  uint64_t state;
  uint64_t inc;
};

RCV_HD uint32_t pcg_next(Pcg32& r) {
  const uint64_t old = r.state;
  r.state = old * 6364136223846793005ull + r.inc;
  const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  const uint32_t rot = (uint32_t)(old >> 59u);
  return (xs >> rot) | (xs << ((32u - rot) & 31u));
}

RCV_HD void pcg_seed(Pcg32& r, uint64_t initstate, uint64_t initseq) {
  r.state = 0ull;
  r.inc = (initseq << 1u) | 1ull;
  pcg_next(r);
  r.state += initstate;
  pcg_next(r);
}

// One independent stream per (render seed, path index).  A lane's stream only
// advances on that lane's own draws, which is what masked draws of the
// reference's vectorised sampler amount to.
RCV_HD void seed_lane(Pcg32& r, uint32_t seed, uint32_t lane) {
  uint32_t a, b, c, d;
  tea(seed, lane, 4, a, b);
  tea(lane, seed, 4, c, d);
  pcg_seed(r, ((uint64_t)a << 32) | b, ((uint64_t)c << 32) | d);
}

// Advances the stream by one draw without producing the output (for draws
// whose value the algorithm discards): same state sequence as pcg_next.
RCV_HD void pcg_skip1(Pcg32& r) { r.state = r.state * 6364136223846793005ull + r.inc; }

// Advances by three draws: state <- A^3 state + (A^2 + A + 1) inc (mod 2^64).
RCV_HD void pcg_skip3(Pcg32& r) {
  constexpr uint64_t A = 6364136223846793005ull;
  constexpr uint64_t A3 = A * A * A;
  constexpr uint64_t K3 = A * A + A + 1ull;
  r.state = r.state * A3 + r.inc * K3;
}

// State after n more draws, by the LCG jump-ahead of O'Neill 2014 (section
// on pcg32_advance): n = sum of powers of two, each applied as
// state <- A^(2^i) state + C_(2^i) inc with C_m = 1 + A + ... + A^(m-1).
RCV_HD uint64_t pcg_jump(uint64_t state, uint64_t inc, uint32_t n) {
  uint64_t acc_a = 1ull, acc_c = 0ull;
  uint64_t a = 6364136223846793005ull, c = 1ull;
  while (n != 0u) {
    if (n & 1u) {
      acc_a *= a;
      acc_c = acc_c * a + c;
    }
    c *= a + 1ull;
    a *= a;
    n >>= 1u;
  }
  return acc_a * state + acc_c * inc;
}

RCV_HD float u32_to_unit(uint32_t v) {
  // 23 random mantissa bits -> [1, 2) -> [0, 1)
  union { uint32_t u; float f; } x;
  x.u = (v >> 9) | 0x3f800000u;
  return x.f - 1.0f;
}

RCV_HD float next1d(Pcg32& r) { return u32_to_unit(pcg_next(r)); }

// next1d of the stream (state, inc), advancing the state in place.
RCV_HD float next1d_state(uint64_t& state, uint64_t inc) {
  Pcg32 r{state, inc};
  const float u = next1d(r);
  state = r.state;
  return u;
}

#ifdef __CUDACC__
// Vector reduction without a returned value (red.global.add.v4.f32): the
// float4 atomicAdd overload returns the old value, which the L1 must wait
// for and write back even when it is unused.
__device__ __forceinline__ void red_add_v4(float4* dst, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

__device__ __forceinline__ void red_add_u32(uint32_t* dst, uint32_t v) {
  asm volatile("red.global.add.u32 [%0], %1;" ::"l"(dst), "r"(v) : "memory");
}
#endif

// ------------------------------------------------------------- float math --
struct V3 {
  float x, y, z;
};

RCV_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }

// Natural logarithm for x in (0, 1]: x = m * 2^e with m in [sqrt(1/2), sqrt(2)),
// log(m) = 2 atanh(s), s = (m-1)/(m+1), evaluated by the atanh power series
// truncated after s^11 (|s| <= 0.1716, truncation error < 2^-30 relative).
RCV_HD float log_unit(float x) {
  union { float f; uint32_t u; } b;
  b.f = x;
  int e = (int)((b.u >> 23) & 0xffu) - 127;
  b.u = (b.u & 0x007fffffu) | 0x3f800000u;  // m in [1, 2)
  float m = b.f;
  if (m > 1.41421356237f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = fmaf(s2, 1.0f / 11.0f, 1.0f / 9.0f);
  p = fmaf(s2, p, 1.0f / 7.0f);
  p = fmaf(s2, p, 1.0f / 5.0f);
  p = fmaf(s2, p, 1.0f / 3.0f);
  p = fmaf(s2, p, 1.0f);
  const float lm = (2.0f * s) * p;
  const float fe = (float)e;
  // ln 2 split in a part exact for |e| < 2^8 and a correction.
  return fmaf(fe, 0.693145751953125f, fmaf(fe, 1.4286068203094172e-06f, lm));
}

// e^x for x <= 0: n = round(x log2 e), r = x - n ln2 (ln 2 split as in
// log_unit, so n * the first part is exact), Taylor polynomial of degree 8 on
// |r| <= ln2/2 (truncation < 2^-28 relative), times 2^n.  0 below -87.
RCV_HD float exp_nonpos(float x) {
  if (!(x > -87.0f)) return 0.0f;
  const float n = rintf(x * 1.44269504088896341f);
  float r = fmaf(n, -0.693145751953125f, x);
  r = fmaf(n, -1.4286068203094172e-06f, r);
  float p = 1.0f / 40320.0f;
  p = fmaf(r, p, 1.0f / 5040.0f);
  p = fmaf(r, p, 1.0f / 720.0f);
  p = fmaf(r, p, 1.0f / 120.0f);
  p = fmaf(r, p, 1.0f / 24.0f);
  p = fmaf(r, p, 1.0f / 6.0f);
  p = fmaf(r, p, 0.5f);
  p = fmaf(r, p, 1.0f);
  p = fmaf(r, p, 1.0f);
  union { float f; uint32_t u; } s;
  s.u = (uint32_t)((int)n + 127) << 23;
  return p * s.f;
}

// sin and cos of 2*pi*u for u in [0, 1).  Exact quadrant reduction on u, then
// Taylor series of sin / cos on [0, pi/4].
RCV_HD void sincos_2pi(float u, float& s, float& c) {
  const float u4 = u * 4.0f;         // exact
  const float qf = floorf(u4);
  const int q = (int)qf & 3;
  float f = u4 - qf;                 // exact, in [0, 1)
  const bool swap = f > 0.5f;
  if (swap) f = 1.0f - f;            // exact
  const float x = f * kHalfPi;       // [0, pi/4]
  const float x2 = x * x;
  float ps = fmaf(x2, 1.0f / 362880.0f, -1.0f / 5040.0f);
  ps = fmaf(x2, ps, 1.0f / 120.0f);
  ps = fmaf(x2, ps, -1.0f / 6.0f);
  const float sn = fmaf(x * x2, ps, x);
  float pc = fmaf(x2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
  pc = fmaf(x2, pc, -1.0f / 720.0f);
  pc = fmaf(x2, pc, 1.0f / 24.0f);
  pc = fmaf(x2, pc, -0.5f);
  const float cs = fmaf(x2, pc, 1.0f);
  const float s0 = swap ? cs : sn;   // sin of the first-quadrant angle
  const float c0 = swap ? sn : cs;
  switch (q) {
    case 0: s = s0; c = c0; break;
    case 1: s = c0; c = -s0; break;
    case 2: s = -s0; c = -c0; break;
    default: s = -c0; c = s0; break;
  }
}

// Uniform direction on the unit sphere from two uniforms (azimuth from u0,
// z from u1); pdf = 1/(4 pi).
RCV_HD V3 uniform_sphere(float u0, float u1) {
  const float z = fmaf(-2.0f, u1, 1.0f);
  const float r = sqrtf(fmaxf(0.0f, fmaf(-z, z, 1.0f)));
  float s, c;
  sincos_2pi(u0, s, c);
  return V3{r * c, r * s, z};
}

// Slab test against the unit cube [0,1]^3.  Returns entry / exit distances.
RCV_HD void slab(const V3& o, const V3& inv, float& tn, float& tf) {
  const float ax = (0.0f - o.x) * inv.x, bx = (1.0f - o.x) * inv.x;
  const float ay = (0.0f - o.y) * inv.y, by = (1.0f - o.y) * inv.y;
  const float az = (0.0f - o.z) * inv.z, bz = (1.0f - o.z) * inv.z;
  tn = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fminf(az, bz));
  tf = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fmaxf(az, bz));
}

RCV_HD V3 recip(const V3& d) { return V3{1.0f / d.x, 1.0f / d.y, 1.0f / d.z}; }

RCV_HD V3 advance(const V3& p, float t, const V3& d) {
  return V3{fmaf(t, d.x, p.x), fmaf(t, d.y, p.y), fmaf(t, d.z, p.z)};
}

RCV_HD float lerpf(float a, float b, float t) { return fmaf(t, b - a, a); }

// Free-flight distance for optical depth -log(1-u) under majorant mu
// (inv_mu = 1/mu, computed once per path).
RCV_HD float free_flight(float u, float mu, float inv_mu) {
  const float tau = -log_unit(1.0f - u);
  return mu > 0.0f ? tau * inv_mu : kInf;
}

// Grid coordinate of a point along one axis: voxel centres at (i + 1/2)/D.
struct Axis {
  int cell;  // cell index in [0, D]; corners are clamp(cell-1), clamp(cell)
  float f;   // interpolation weight of the upper corner
};

RCV_HD Axis axis_coord(float p, int D) {
  const float g = fmaf(p, (float)D, -0.5f);
  const float fl = floorf(g);
  Axis a;
  a.f = g - fl;
  // clamp before the integer conversion so that no float -> int overflow occurs
  const float flc = fminf(fmaxf(fl, -1.0f), (float)D);
  int c = (int)flc + 1;
  c = c < 0 ? 0 : (c > D ? D : c);
  a.cell = c;
  return a;
}

// Trilinear interpolation of 8 corner values ordered (x fastest)
// v000 v100 v010 v110 v001 v101 v011 v111.
RCV_HD float trilerp(const float4& lo, const float4& hi, float fx, float fy, float fz) {
  const float c00 = lerpf(lo.x, lo.y, fx);
  const float c10 = lerpf(lo.z, lo.w, fx);
  const float c01 = lerpf(hi.x, hi.y, fx);
  const float c11 = lerpf(hi.z, hi.w, fx);
  const float c0 = lerpf(c00, c10, fy);
  const float c1 = lerpf(c01, c11, fy);
  return lerpf(c0, c1, fz);
}

RCV_HD V3 lerp3(const float4& a, const float4& b, float t) {
  return V3{lerpf(a.x, b.x, t), lerpf(a.y, b.y, t), lerpf(a.z, b.z, t)};
}

}  // namespace rcv
