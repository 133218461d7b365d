// CPU oracle for the recursive-control-variate gradient step — TEST
// INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file; the
// tests, the smoke check and the CPU-baseline leg of bench.py load it to
// check results against.
//
// It restates, as plain sequential C++ (one path at a time, nested loops),
// the per-path algorithm of the reference for its grid-scene family
// (heterogeneous medium in an axis-aligned box behind a null boundary,
// constant white environment, isotropic phase function, box film, one
// perspective sensor or a batch of them):
//   plugins/twostatevolpath.py:141-385  TwoStatePRBVolpathIntegrator.sample_twostates
//   plugins/twostatevolpath.py:387-479  sample_emitter_twostates
//   plugins/twostatemedium.py:15-107    TwoStateMedium.sample_interaction_twostates
//   plugins/twostatevolpath.py:80-138   render_twostates + develop (box filter)
// plus the single-state estimator a two-state integrator renders on `new`
// (plugins/twostatemedium.py:125-151), its path-replay adjoint (the default
// adjoint of the cv integrator, plugins/cv_integrator.py:87-94) and forward
// mode (cv_integrator.py:79-85), the majorant supergrid
// (plugins/twostatemedium.py:25-70) and the volpathsimple integrator
// (plugins/volpathsimple.py).
// Mitsuba primitives the reference calls (sampler, gridvolume, warps) are
// restated from their documented behaviour.
//
// Floating point: every float32 operation is written out in the same order
// as the GPU kernels, compiled with -ffp-contract=off, so that paths agree
// bit for bit; gradients accumulate in double.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

constexpr float kInvFourPi = 0.0795774715459476678844f;
constexpr float kHalfPi = 1.57079632679489661923f;
constexpr float kInf = __builtin_huge_valf();

// ------------------------------------------------------------ sampler
// TEA with the GPU-random-number key schedule (Zafar, Olano, Curtis 2010).
void tea(uint32_t v0, uint32_t v1, int rounds, uint32_t& o0, uint32_t& o1) {
  uint32_t sum = 0;
  for (int i = 0; i < rounds; ++i) {
    sum += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + sum) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + sum) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  o0 = v0;
  o1 = v1;
}

// PCG32 (O'Neill 2014).
struct Rng {
  uint64_t state = 0, inc = 1;
  uint32_t next() {
    uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  void seed(uint64_t initstate, uint64_t initseq) {
    state = 0;
    inc = (initseq << 1u) | 1u;
    next();
    state += initstate;
    next();
  }
  float next1d() {
    uint32_t bits = (next() >> 9) | 0x3f800000u;
    float f;
    std::memcpy(&f, &bits, 4);
    return f - 1.0f;
  }
};

Rng lane_rng(uint32_t seed, uint32_t lane) {
  uint32_t a, b, c, d;
  tea(seed, lane, 4, a, b);
  tea(lane, seed, 4, c, d);
  Rng r;
  r.seed(((uint64_t)a << 32) | b, ((uint64_t)c << 32) | d);
  return r;
}

// ------------------------------------------------------------ float math
struct V3 {
  float x, y, z;
};

// ln(x), x in (0,1]: atanh series of the reduced mantissa (see the GPU notes).
float log_unit(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  int e = (int)((u >> 23) & 0xffu) - 127;
  u = (u & 0x007fffffu) | 0x3f800000u;
  float m;
  std::memcpy(&m, &u, 4);
  if (m > 1.41421356237f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float s2 = s * s;
  float p = std::fmaf(s2, 1.0f / 11.0f, 1.0f / 9.0f);
  p = std::fmaf(s2, p, 1.0f / 7.0f);
  p = std::fmaf(s2, p, 1.0f / 5.0f);
  p = std::fmaf(s2, p, 1.0f / 3.0f);
  p = std::fmaf(s2, p, 1.0f);
  const float lm = (2.0f * s) * p;
  const float fe = (float)e;
  return std::fmaf(fe, 0.693145751953125f, std::fmaf(fe, 1.4286068203094172e-06f, lm));
}

void sincos_2pi(float u, float& s, float& c) {
  const float u4 = u * 4.0f;
  const float qf = std::floor(u4);
  const int q = (int)qf & 3;
  float f = u4 - qf;
  const bool swap = f > 0.5f;
  if (swap) f = 1.0f - f;
  const float x = f * kHalfPi;
  const float x2 = x * x;
  float ps = std::fmaf(x2, 1.0f / 362880.0f, -1.0f / 5040.0f);
  ps = std::fmaf(x2, ps, 1.0f / 120.0f);
  ps = std::fmaf(x2, ps, -1.0f / 6.0f);
  const float sn = std::fmaf(x * x2, ps, x);
  float pc = std::fmaf(x2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
  pc = std::fmaf(x2, pc, -1.0f / 720.0f);
  pc = std::fmaf(x2, pc, 1.0f / 24.0f);
  pc = std::fmaf(x2, pc, -0.5f);
  const float cs = std::fmaf(x2, pc, 1.0f);
  const float s0 = swap ? cs : sn, c0 = swap ? sn : cs;
  switch (q) {
    case 0: s = s0; c = c0; break;
    case 1: s = c0; c = -s0; break;
    case 2: s = -s0; c = -c0; break;
    default: s = -c0; c = s0; break;
  }
}

V3 square_to_uniform_sphere(float u0, float u1) {
  const float z = std::fmaf(-2.0f, u1, 1.0f);
  const float r = std::sqrt(std::fmax(0.0f, std::fmaf(-z, z, 1.0f)));
  float s, c;
  sincos_2pi(u0, s, c);
  return V3{r * c, r * s, z};
}

// unit cube [0,1]^3: returns (t_near, t_far)
void cube_hit(const V3& o, const V3& d, float& tn, float& tf) {
  const V3 inv{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
  const float ax = (0.0f - o.x) * inv.x, bx = (1.0f - o.x) * inv.x;
  const float ay = (0.0f - o.y) * inv.y, by = (1.0f - o.y) * inv.y;
  const float az = (0.0f - o.z) * inv.z, bz = (1.0f - o.z) * inv.z;
  tn = std::fmax(std::fmax(std::fmin(ax, bx), std::fmin(ay, by)), std::fmin(az, bz));
  tf = std::fmin(std::fmin(std::fmax(ax, bx), std::fmax(ay, by)), std::fmax(az, bz));
}

V3 ray_at(const V3& o, float t, const V3& d) {
  return V3{std::fmaf(t, d.x, o.x), std::fmaf(t, d.y, o.y), std::fmaf(t, d.z, o.z)};
}

float lerp(float a, float b, float t) { return std::fmaf(t, b - a, a); }

}  // namespace

extern "C" {

// Scene description shared by every oracle entry point.
struct oracle_scene {
  int32_t width, height;
  float cam_o[3], cam_f[3], cam_r[3], cam_u[3];
  int32_t max_depth, rr_depth, hide_emitters;
  int32_t dx, dy, dz;
  float scale;
  const float* dens_old;
  const float* dens_new;
  const float* alb_old;  // [dz][dy][dx][3] or null
  const float* alb_new;
  float albedo_const[3];
  int32_t majorant_factor;  // 0: global majorant; f: supergrid of ceil(D/f) cells per axis
  // medium box: to_world = translate(box_min) * scale(box_size), size 0 = 1
  float box_min[3], box_size[3];
  // batch film: n_cams sub-sensors side by side (<= 1: the camera above);
  // sub-sensor k >= 1 is cams[k-1] = origin, forward, right, up (world space)
  int32_t n_cams;
  float cams[15][12];
  // albedo grid resolution when it differs from the density's (0 = same)
  int32_t adx, ady, adz;
  // environment map (env_w = 0: the constant white environment): RGB texels
  // [env_h][env_w][3], row 0 at the +y pole, radiance times env_scale
  int32_t env_w, env_h;
  float env_scale;
  const float* env_texels;
};
}

namespace {

// Voxel grid corner interpolation of Mitsuba's gridvolume (voxel centres at
// (i+1/2)/D, clamp to edge).
struct Corners {
  int x0, x1, y0, y1, z0, z1;
  float fx, fy, fz;
};

void axis(float p, int D, int& i0, int& i1, float& f) {
  const float g = std::fmaf(p, (float)D, -0.5f);
  const float fl = std::floor(g);
  f = g - fl;
  const float flc = std::fmin(std::fmax(fl, -1.0f), (float)D);
  const int ix = (int)flc;
  i0 = std::min(std::max(ix, 0), D - 1);
  i1 = std::min(std::max(ix + 1, 0), D - 1);
}

Corners corners(const oracle_scene& S, const V3& x) {
  Corners c;
  axis(x.x, S.dx, c.x0, c.x1, c.fx);
  axis(x.y, S.dy, c.y0, c.y1, c.fy);
  axis(x.z, S.dz, c.z0, c.z1, c.fz);
  return c;
}

inline int64_t vidx(const oracle_scene& S, int x, int y, int z) {
  return ((int64_t)z * S.dy + y) * S.dx + x;
}

float trilinear(const oracle_scene& S, const float* g, int stride, int ch, const Corners& c) {
  auto v = [&](int x, int y, int z) { return g[vidx(S, x, y, z) * stride + ch]; };
  const float c00 = lerp(v(c.x0, c.y0, c.z0), v(c.x1, c.y0, c.z0), c.fx);
  const float c10 = lerp(v(c.x0, c.y1, c.z0), v(c.x1, c.y1, c.z0), c.fx);
  const float c01 = lerp(v(c.x0, c.y0, c.z1), v(c.x1, c.y0, c.z1), c.fx);
  const float c11 = lerp(v(c.x0, c.y1, c.z1), v(c.x1, c.y1, c.z1), c.fx);
  const float c0 = lerp(c00, c10, c.fy);
  const float c1 = lerp(c01, c11, c.fy);
  return lerp(c0, c1, c.fz);
}

// Albedo grid resolution (the density's unless set).
void albedo_dims(const oracle_scene& S, int& ax, int& ay, int& az) {
  const bool own = S.adx > 0;
  ax = own ? S.adx : S.dx;
  ay = own ? S.ady : S.dy;
  az = own ? S.adz : S.dz;
}

// Corners of the albedo grid at x: the density's when both have one
// resolution (both grids span the unit cube).
Corners albedo_corners(const oracle_scene& S, const V3& x, const Corners& c) {
  int ax, ay, az;
  albedo_dims(S, ax, ay, az);
  if (ax == S.dx && ay == S.dy && az == S.dz) return c;
  Corners a;
  axis(x.x, ax, a.x0, a.x1, a.fx);
  axis(x.y, ay, a.y0, a.y1, a.fy);
  axis(x.z, az, a.z0, a.z1, a.fz);
  return a;
}

inline int64_t avidx(const oracle_scene& S, int x, int y, int z) {
  int ax, ay, az;
  albedo_dims(S, ax, ay, az);
  return ((int64_t)z * ay + y) * ax + x;
}

float albedo_channel(const oracle_scene& S, const float* g, int ch, const Corners& c) {
  auto v = [&](int x, int y, int z) { return g[avidx(S, x, y, z) * 3 + ch]; };
  const float c00 = lerp(v(c.x0, c.y0, c.z0), v(c.x1, c.y0, c.z0), c.fx);
  const float c10 = lerp(v(c.x0, c.y1, c.z0), v(c.x1, c.y1, c.z0), c.fx);
  const float c01 = lerp(v(c.x0, c.y0, c.z1), v(c.x1, c.y0, c.z1), c.fx);
  const float c11 = lerp(v(c.x0, c.y1, c.z1), v(c.x1, c.y1, c.z1), c.fx);
  const float c0 = lerp(c00, c10, c.fy);
  const float c1 = lerp(c01, c11, c.fy);
  return lerp(c0, c1, c.fz);
}

// Trilinear RGB albedo at x (c: the density corners at x).
V3 albedo(const oracle_scene& S, const float* grid, const V3& x, const Corners& c) {
  if (grid == nullptr) return V3{S.albedo_const[0], S.albedo_const[1], S.albedo_const[2]};
  const Corners a = albedo_corners(S, x, c);
  return V3{albedo_channel(S, grid, 0, a), albedo_channel(S, grid, 1, a), albedo_channel(S, grid, 2, a)};
}

float grid_max(const oracle_scene& S, const float* g) {
  float m = 0.0f;
  const int64_t n = (int64_t)S.dx * S.dy * S.dz;
  for (int64_t i = 0; i < n; ++i) m = std::fmax(m, g[i]);
  return m;
}

// Inverse box size (1 for a zero or unit size).
V3 inv_box(const oracle_scene& S) {
  V3 r;
  r.x = S.box_size[0] > 0.0f ? 1.0f / S.box_size[0] : 1.0f;
  r.y = S.box_size[1] > 0.0f ? 1.0f / S.box_size[1] : 1.0f;
  r.z = S.box_size[2] > 0.0f ? 1.0f / S.box_size[2] : 1.0f;
  return r;
}

// A world direction in box coordinates: distances along the ray stay world
// distances.
V3 to_box(const oracle_scene& S, const V3& w) {
  const V3 ib = inv_box(S);
  return V3{w.x * ib.x, w.y * ib.y, w.z * ib.z};
}

// Camera ray of film position (px + u0, py + u1) in box coordinates.  A batch
// film (Mitsuba's batch sensor) gives the position s = (px + u0) / width to
// sub-sensor k = min(floor(s n), n - 1) as s n - floor(s n).
void camera_ray(const oracle_scene& S, int px, int py, float u0, float u1, V3& o, V3& d) {
  const float fx = (float)px + u0, fy = (float)py + u1;
  const float inv_w = 1.0f / (float)S.width, inv_h = 1.0f / (float)S.height;
  float nx = fx * inv_w;
  const float ny = fy * inv_h;
  int k = 0;
  if (S.n_cams > 1) {
    const float idx_f = nx * (float)S.n_cams;
    const int idx = (int)idx_f;
    k = std::min(idx, S.n_cams - 1);
    nx = idx_f - (float)idx;
  }
  const float* co = k == 0 ? S.cam_o : S.cams[k - 1];
  const float* cf = k == 0 ? S.cam_f : S.cams[k - 1] + 3;
  const float* cr = k == 0 ? S.cam_r : S.cams[k - 1] + 6;
  const float* cu = k == 0 ? S.cam_u : S.cams[k - 1] + 9;
  const float a = std::fmaf(2.0f, nx, -1.0f), b = std::fmaf(-2.0f, ny, 1.0f);
  V3 r;
  r.x = std::fmaf(b, cu[0], std::fmaf(a, cr[0], cf[0]));
  r.y = std::fmaf(b, cu[1], std::fmaf(a, cr[1], cf[1]));
  r.z = std::fmaf(b, cu[2], std::fmaf(a, cr[2], cf[2]));
  const float inv_len = 1.0f / std::sqrt(std::fmaf(r.z, r.z, std::fmaf(r.y, r.y, r.x * r.x)));
  d = to_box(S, V3{r.x * inv_len, r.y * inv_len, r.z * inv_len});
  const V3 ib = inv_box(S);
  o = V3{(co[0] - S.box_min[0]) * ib.x, (co[1] - S.box_min[1]) * ib.y, (co[2] - S.box_min[2]) * ib.z};
}

// Majorant supergrid (plugins/twostatemedium.py:25-70): ceil(D/f) cells per
// axis covering the unit cube; a cell bounds sigma_t over every point inside
// it, i.e. scale * the largest density among the voxels trilinear
// interpolation reads there.  `two` bounds both states, `nw` the new one.
struct Supergrid {
  int s[3] = {0, 0, 0};
  float inv[3] = {0.0f, 0.0f, 0.0f};  // 1 / s
  std::vector<float> two, nw;

  static int64_t floordiv(int64_t a, int64_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

  // voxels read by trilinear interpolation for x in [c/S, (c+1)/S)
  static void span(int c, int S, int D, int& lo, int& hi) {
    const int64_t den = 2 * int64_t(S);
    lo = (int)floordiv(2 * int64_t(c) * D - S, den);
    hi = (int)floordiv(2 * int64_t(c + 1) * D - S, den) + 1;
    lo = std::min(std::max(lo, 0), D - 1);
    hi = std::min(std::max(hi, 0), D - 1);
  }

  void build(const oracle_scene& S) {
    const int f = S.majorant_factor;
    if (f <= 0) return;
    const int D[3] = {S.dx, S.dy, S.dz};
    for (int a = 0; a < 3; ++a) {
      s[a] = (D[a] + f - 1) / f;
      inv[a] = 1.0f / (float)s[a];
    }
    two.assign((size_t)s[0] * s[1] * s[2], 0.0f);
    nw.assign(two.size(), 0.0f);
    for (int cz = 0; cz < s[2]; ++cz)
      for (int cy = 0; cy < s[1]; ++cy)
        for (int cx = 0; cx < s[0]; ++cx) {
          int x0, x1, y0, y1, z0, z1;
          span(cx, s[0], S.dx, x0, x1);
          span(cy, s[1], S.dy, y0, y1);
          span(cz, s[2], S.dz, z0, z1);
          float mo = 0.0f, mn = 0.0f;
          for (int z = z0; z <= z1; ++z)
            for (int y = y0; y <= y1; ++y)
              for (int x = x0; x <= x1; ++x) {
                const int64_t v = ((int64_t)z * S.dy + y) * S.dx + x;
                mo = std::fmax(mo, S.dens_old[v]);
                mn = std::fmax(mn, S.dens_new[v]);
              }
          const size_t i = ((size_t)cz * s[1] + cy) * s[0] + cx;
          two[i] = S.scale * std::fmax(mo, mn);
          nw[i] = S.scale * mn;
        }
  }

  bool active() const { return s[0] > 0; }

  // Distance at which the optical depth along o + t d reaches tau, walking the
  // cells along the ray and accumulating majorant x length; infinity when t
  // would exceed tmax.  mu_at: the majorant of the cell the collision lies in.
  float flight(const std::vector<float>& g, const V3& o, const V3& d, float tmax, float tau, float& mu_at) const {
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    float tn[3], td[3];
    int c[3], st[3];
    for (int a = 0; a < 3; ++a) {
      const float n = (float)s[a];
      c[a] = std::min(std::max((int)std::floor(oo[a] * n), 0), s[a] - 1);
      st[a] = dd[a] > 0.0f ? 1 : (dd[a] < 0.0f ? -1 : 0);
      // cell faces at c / s = c * (1 / s); one division per axis
      if (st[a] > 0) {
        const float inv_d = 1.0f / dd[a];
        tn[a] = ((float)(c[a] + 1) * inv[a] - oo[a]) * inv_d;
        td[a] = inv[a] * inv_d;
      } else if (st[a] < 0) {
        const float inv_d = 1.0f / dd[a];
        tn[a] = ((float)c[a] * inv[a] - oo[a]) * inv_d;
        td[a] = -(inv[a] * inv_d);
      } else {
        tn[a] = kInf;
        td[a] = kInf;
      }
    }
    auto clampc = [&](int v, int a) { return std::min(std::max(v, 0), s[a] - 1); };
    float t = 0.0f, acc = 0.0f;
    for (int step = 0; step < s[0] + s[1] + s[2] + 4; ++step) {
      const float t_next = std::fmin(std::fmin(tn[0], tn[1]), tn[2]);
      const int k = tn[0] == t_next ? 0 : (tn[1] == t_next ? 1 : 2);
      const float m = g[((size_t)clampc(c[2], 2) * s[1] + clampc(c[1], 1)) * s[0] + clampc(c[0], 0)];
      const float acc_next = acc + m * (t_next - t);
      if (m > 0.0f && acc_next >= tau) {
        const float t_hit = t + (tau - acc) / m;
        if (!(t_hit < tmax)) return kInf;
        mu_at = m;
        return t_hit;
      }
      if (!(t_next < tmax)) break;
      tn[k] += td[k];
      c[k] += st[k];
      t = t_next;
      acc = acc_next;
    }
    return kInf;
  }
};

// Gradient sink of the adjoint (double accumulators, one per worker).
// Where the adjoint's gradient terms go: scattered into voxel gradients, or
// (forward mode, tan_d / tan_a set) gathered against a tangent field into
// `acc`, the derivative of the path's contribution along the tangent.
struct GradSink {
  std::vector<double> dens, alb;
  const float* tan_d = nullptr;  // [dz][dy][dx] density tangent
  const float* tan_a = nullptr;  // [adz][ady][adx][3] albedo tangent
  double acc = 0.0;
  void density(const oracle_scene& S, const Corners& c, float g) {
    if (tan_d != nullptr || tan_a != nullptr) {
      if (tan_d != nullptr) acc += (double)g * (double)trilinear(S, tan_d, 1, 0, c);
      return;
    }
    const float gx0 = 1.0f - c.fx, gy0 = 1.0f - c.fy, gz0 = 1.0f - c.fz;
    const float a = g * gz0, b = g * c.fz;
    const float a0 = a * gy0, a1 = a * c.fy, b0 = b * gy0, b1 = b * c.fy;
    dens[vidx(S, c.x0, c.y0, c.z0)] += a0 * gx0;
    dens[vidx(S, c.x1, c.y0, c.z0)] += a0 * c.fx;
    dens[vidx(S, c.x0, c.y1, c.z0)] += a1 * gx0;
    dens[vidx(S, c.x1, c.y1, c.z0)] += a1 * c.fx;
    dens[vidx(S, c.x0, c.y0, c.z1)] += b0 * gx0;
    dens[vidx(S, c.x1, c.y0, c.z1)] += b0 * c.fx;
    dens[vidx(S, c.x0, c.y1, c.z1)] += b1 * gx0;
    dens[vidx(S, c.x1, c.y1, c.z1)] += b1 * c.fx;
  }
  void albedo(const oracle_scene& S, const V3& x, const Corners& dc, const V3& g) {
    if (tan_d != nullptr || tan_a != nullptr) {
      if (tan_a != nullptr) {
        const Corners a = albedo_corners(S, x, dc);
        acc += (double)g.x * albedo_channel(S, tan_a, 0, a) + (double)g.y * albedo_channel(S, tan_a, 1, a) +
               (double)g.z * albedo_channel(S, tan_a, 2, a);
      }
      return;
    }
    if (alb.empty()) return;
    const Corners c = albedo_corners(S, x, dc);
    const float wx[2] = {1.0f - c.fx, c.fx}, wy[2] = {1.0f - c.fy, c.fy}, wz[2] = {1.0f - c.fz, c.fz};
    const int xs[2] = {c.x0, c.x1}, ys[2] = {c.y0, c.y1}, zs[2] = {c.z0, c.z1};
    for (int k = 0; k < 8; ++k) {
      const int i = k & 1, j = (k >> 1) & 1, m = k >> 2;
      const float w = (wz[m] * wy[j]) * wx[i];
      const int64_t v = avidx(S, xs[i], ys[j], zs[m]);
      alb[v * 3 + 0] += g.x * w;
      alb[v * 3 + 1] += g.y * w;
      alb[v * 3 + 2] += g.z * w;
    }
  }
};

enum Mode { kTwoState = 0, kSingle = 1 };

// ------------------------------------------------------ environment map
// The `envmap` emitter of the reference's grid scenes (experiments.py:81-85):
// latitude-longitude radiance, bilinear between texel centres (wrap in u,
// clamp in v), importance-sampled from a piecewise-constant density
// proportional to luminance x sin(theta) of the row centre (Pharr, Jakob &
// Humphreys, PBR, infinite area lights).  Direction (x, y, z) <-> (u, v):
// u = atan2(x, -z) / (2 pi) in [0, 1), v = acos(y) / pi.  atan2 by octant
// reduction, a pi/4 shift above tan(pi/8) and the arctangent series through
// x^19; sin / cos by sincos_2pi.
constexpr float kEnvInvTwoPi = 0.159154943091895335769f;
constexpr float kEnvInvPi = 0.318309886183790671538f;
constexpr float kEnvInv2PiSq = 0.0506605918211688965f;
constexpr float kEnvPi = 3.14159265358979323846f;
constexpr float kEnvQuarterPi = 0.785398163397448309616f;

float arctan01(float a) {
  const bool big = a > 0.414213562373095f;
  const float x = big ? (a - 1.0f) / (a + 1.0f) : a;
  const float x2 = x * x;
  // (-1)^k / (2k + 1), k = 9 .. 1, Horner in x^2
  static const float c[9] = {-1.0f / 19.0f, 1.0f / 17.0f, -1.0f / 15.0f, 1.0f / 13.0f, -1.0f / 11.0f,
                             1.0f / 9.0f,   -1.0f / 7.0f, 1.0f / 5.0f,   -1.0f / 3.0f};
  float p = std::fmaf(x2, c[0], c[1]);
  for (int k = 2; k < 9; ++k) p = std::fmaf(x2, p, c[k]);
  const float r = std::fmaf(x * x2, p, x);
  return big ? r + kEnvQuarterPi : r;
}

float arctan2(float y, float x) {
  const float ax = std::fabs(x), ay = std::fabs(y);
  const float mx = std::fmax(ax, ay), mn = std::fmin(ax, ay);
  const float a = mx > 0.0f ? mn / mx : 0.0f;
  float r = arctan01(a);
  if (ay > ax) r = 2.0f * kEnvQuarterPi - r;
  if (x < 0.0f) r = kEnvPi - r;
  return y < 0.0f ? -r : r;
}

struct Env {
  int w = 0, h = 0;
  float scale = 1.0f, inv_w = 0.0f, inv_h = 0.0f, inv_norm = 0.0f;
  bool sample = false;
  std::vector<float> rgb, f, cond, marg;  // texels, weights, CDFs

  explicit Env(const oracle_scene& S) {
    if (S.env_w <= 0 || S.env_h <= 0 || S.env_texels == nullptr) return;
    w = S.env_w;
    h = S.env_h;
    scale = S.env_scale;
    inv_w = 1.0f / (float)w;
    inv_h = 1.0f / (float)h;
    rgb.assign(S.env_texels, S.env_texels + (size_t)w * h * 3);
    f.resize((size_t)w * h);
    cond.resize((size_t)(w + 1) * h);
    marg.resize((size_t)h + 1);
    std::vector<double> rows(h);
    for (int i = 0; i < h; ++i) {
      float s_, c_;
      sincos_2pi((((float)i + 0.5f) * inv_h) * 0.5f, s_, c_);
      double sum = 0.0;
      for (int j = 0; j < w; ++j) {
        const float* t = &rgb[((size_t)i * w + j) * 3];
        const float lum = (0.2126f * t[0] + 0.7152f * t[1]) + 0.0722f * t[2];
        f[(size_t)i * w + j] = lum * s_;
        sum += (double)f[(size_t)i * w + j];
      }
      rows[i] = sum;
      double acc = 0.0;
      for (int j = 0; j < w; ++j) {
        cond[(size_t)i * (w + 1) + j] = sum > 0.0 ? (float)(acc / sum) : (float)((double)j / (double)w);
        acc += (double)f[(size_t)i * w + j];
      }
      cond[(size_t)i * (w + 1) + w] = 1.0f;
    }
    double total = 0.0;
    for (int i = 0; i < h; ++i) total += rows[i];
    double acc = 0.0;
    for (int i = 0; i < h; ++i) {
      marg[i] = total > 0.0 ? (float)(acc / total) : (float)((double)i / (double)h);
      acc += rows[i];
    }
    marg[h] = 1.0f;
    inv_norm = total > 0.0 ? (float)((double)w * (double)h / total) : 0.0f;
    sample = total > 0.0;
  }

  bool valid() const { return w > 0; }

  static void uv(const V3& d, float& u, float& v, float& sin_t) {
    u = arctan2(d.x, -d.z) * kEnvInvTwoPi;
    if (u < 0.0f) u = u + 1.0f;
    if (!(u < 1.0f)) u = 0.0f;
    sin_t = std::sqrt(std::fmax(0.0f, std::fmaf(-d.y, d.y, 1.0f)));
    v = arctan2(sin_t, d.y) * kEnvInvPi;
  }

  V3 eval(float u, float v) const {
    const float fx = std::fmaf(u, (float)w, -0.5f), fy = std::fmaf(v, (float)h, -0.5f);
    const float x0f = std::floor(fx), y0f = std::floor(fy);
    const float tx = fx - x0f, ty = fy - y0f;
    const int x0 = (int)std::fmax(std::fmin(x0f, (float)w), -1.0f);
    const int y0 = (int)std::fmax(std::fmin(y0f, (float)h), -1.0f);
    auto wrap = [&](int x) { const int r = x % w; return r < 0 ? r + w : r; };
    auto clampy = [&](int y) { return y < 0 ? 0 : (y > h - 1 ? h - 1 : y); };
    const int c0 = wrap(x0), c1 = wrap(x0 + 1), r0 = clampy(y0), r1 = clampy(y0 + 1);
    float out[3];
    for (int k = 0; k < 3; ++k) {
      const float a = rgb[((size_t)r0 * w + c0) * 3 + k], b = rgb[((size_t)r0 * w + c1) * 3 + k];
      const float c = rgb[((size_t)r1 * w + c0) * 3 + k], d = rgb[((size_t)r1 * w + c1) * 3 + k];
      out[k] = lerp(lerp(a, b, tx), lerp(c, d, tx), ty) * scale;
    }
    return V3{out[0], out[1], out[2]};
  }

  float pdf(float u, float v, float sin_t) const {
    if (!sample || !(sin_t > 0.0f)) return 0.0f;
    int i = (int)(v * (float)h), j = (int)(u * (float)w);
    i = std::min(std::max(i, 0), h - 1);
    j = std::min(std::max(j, 0), w - 1);
    return ((f[(size_t)i * w + j] * inv_norm) * kEnvInv2PiSq) / sin_t;
  }

  static int find(const float* cdf, int n, float x) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (cdf[mid] <= x)
        lo = mid;
      else
        hi = mid;
    }
    return lo;
  }

  // sampled unit world direction, its radiance and pdf
  V3 sample_dir(float u0, float u1, V3& Le, float& p) const {
    Le = V3{0.0f, 0.0f, 0.0f};
    p = 0.0f;
    if (!sample) return V3{0.0f, 1.0f, 0.0f};
    const int i = find(marg.data(), h, u1);
    const float dv = (u1 - marg[i]) / (marg[i + 1] - marg[i]);
    const float* row = &cond[(size_t)i * (w + 1)];
    const int j = find(row, w, u0);
    const float du = (u0 - row[j]) / (row[j + 1] - row[j]);
    const float u = ((float)j + du) * inv_w, v = ((float)i + dv) * inv_h;
    float st, ct, sp, cp;
    sincos_2pi(v * 0.5f, st, ct);
    sincos_2pi(u, sp, cp);
    const V3 d{st * sp, ct, -(st * cp)};
    if (st > 0.0f) {
      p = ((f[(size_t)i * w + j] * inv_norm) * kEnvInv2PiSq) / st;
      Le = eval(u, v);
    }
    return d;
  }

  // radiance along a box-space direction and the pdf of sampling it
  V3 along(const oracle_scene& S, const V3& d, float& p) const {
    const float bx = S.box_size[0] > 0.0f ? S.box_size[0] : 1.0f;
    const float by = S.box_size[1] > 0.0f ? S.box_size[1] : 1.0f;
    const float bz = S.box_size[2] > 0.0f ? S.box_size[2] : 1.0f;
    V3 wd{d.x * bx, d.y * by, d.z * bz};
    const float inv_len = 1.0f / std::sqrt(std::fmaf(wd.z, wd.z, std::fmaf(wd.y, wd.y, wd.x * wd.x)));
    wd = V3{wd.x * inv_len, wd.y * inv_len, wd.z * inv_len};
    float u, v, st;
    uv(wd, u, v, st);
    p = pdf(u, v, st);
    return eval(u, v);
  }
};

// Power heuristic (mitsuba.ad.common.mis_weight).
float mis2(float a, float b) {
  const float a2 = a * a, b2 = b * b;
  const float s = a2 + b2;
  return s > 0.0f ? a2 / s : 0.0f;
}

struct PathOut {
  V3 L_old{0, 0, 0}, L_new{0, 0, 0};
  uint64_t lookups = 0, nee_lookups = 0, scatters = 0;
};

struct Tracer {
  const oracle_scene& S;
  int mode;         // kTwoState or kSingle
  float mu;         // global majorant used for free-flight sampling
  GradSink* sink;   // non-null: adjoint replay
  V3 dL{0, 0, 0};   // adjoint: dLoss/dL for this path
  V3 Ltot{0, 0, 0}; // adjoint: the path's total radiance (radiance pass)
  const Supergrid* sg = nullptr;  // majorant supergrid, if the medium has one
  const Env* env = nullptr;       // environment map, if the scene has one

  // Radiance the path still gathers after the contributions in `got`:
  // L_rem = L - got, one rounding per channel.
  V3 remaining(const V3& got) const { return V3{Ltot.x - got.x, Ltot.y - got.y, Ltot.z - got.z}; }

  float sigma_t(const float* g, const Corners& c) const { return S.scale * trilinear(S, g, 1, 0, c); }

  bool roulette(Rng& rng, int depth, V3& bn, V3& bo) const {
    bool alive = bn.x != 0.0f || bn.y != 0.0f || bn.z != 0.0f;
    if (mode == kTwoState) alive = alive || bo.x != 0.0f || bo.y != 0.0f || bo.z != 0.0f;
    if (!alive) return false;
    float m = std::fmax(std::fmax(bn.x, bn.y), bn.z);
    if (mode == kTwoState)
      m = std::fmax(std::fmax(std::fmax(bn.x, bo.x), std::fmax(bn.y, bo.y)), std::fmax(bn.z, bo.z));
    const float q = std::fmin(m, 0.99f);
    const float u = rng.next1d();
    if (depth > S.rr_depth) {
      if (!(u < q)) return false;
      const float inv = 1.0f / q;
      bn = V3{bn.x * inv, bn.y * inv, bn.z * inv};
      if (mode == kTwoState) bo = V3{bo.x * inv, bo.y * inv, bo.z * inv};
    }
    return true;
  }

  // Free-flight distance from o along d within [0, tmax]; m = the majorant
  // of the sampled collision (global, or its supergrid cell's).
  float free_flight(Rng& rng, const V3& o, const V3& d, float tmax, float& m) const {
    const float u = rng.next1d();
    const float tau = -log_unit(1.0f - u);
    m = mu;
    if (sg != nullptr && sg->active())
      return sg->flight(mode == kTwoState ? sg->two : sg->nw, o, d, tmax, tau, m);
    return mu > 0.0f ? tau * (1.0f / mu) : kInf;
  }

  // Ratio-tracking transmittance from p along w to the cube boundary
  // (plugins/twostatevolpath.py:408-477).  With `grad_scale` set, instead
  // back-propagates grad_scale * dlog(T) into the density.
  void transmittance(Rng& rng, const V3& p, const V3& w, float& tro, float& trn, PathOut& out,
                     const float* grad_scale) const {
    float tn, tf;
    cube_hit(p, w, tn, tf);
    float tr_rem = tf;
    V3 q = p;
    tro = 1.0f;
    trn = 1.0f;
    for (;;) {
      float m;
      const float t = free_flight(rng, q, w, tr_rem, m);
      if (!(t <= tr_rem)) break;
      const float inv_m = 1.0f / m;
      const V3 x = ray_at(q, t, w);
      const Corners c = corners(S, x);
      ++out.nee_lookups;
      const float st_n = sigma_t(S.dens_new, c);
      if (grad_scale) {
        const float sn = m - st_n;
        if (sn > 0.0f) sink->density(S, c, -(S.scale * *grad_scale) / sn);
      }
      trn = trn * ((m - st_n) * inv_m);
      if (mode == kTwoState) {
        const float st_o = sigma_t(S.dens_old, c);
        tro = tro * ((m - st_o) * inv_m);
      }
      q = x;
      tr_rem = tr_rem - t;
      const bool dead = mode == kTwoState ? (trn == 0.0f && tro == 0.0f) : trn == 0.0f;
      if (dead) break;
    }
  }

  PathOut trace(uint32_t seed, uint32_t lane, int px, int py) const {
    PathOut out;
    Rng rng = lane_rng(seed, lane);
    // camera ray from the film sample (box filter: the sample stays in its pixel)
    const float u0 = rng.next1d(), u1 = rng.next1d();
    V3 o, d;
    camera_ray(S, px, py, u0, u1, o, d);
    (void)rng.next1d();  // colour channel (grey extinction: unused)

    V3 bo{1, 1, 1}, bn{1, 1, 1};
    V3& Lo = out.L_old;
    V3& Ln = out.L_new;
    int depth = 0;
    const float mis = 0.5f;
    const float emit_weight = 1.0f / kInvFourPi;

    // camera iteration: Russian roulette draw, then the cube boundary
    if (!roulette(rng, depth, bn, bo)) return out;
    float tn, tf;
    cube_hit(o, d, tn, tf);
    if (!(tn <= tf && tf > 0.0f)) {
      if (!S.hide_emitters) {
        if (env && env->valid()) {
          float pe;
          const V3 Le = env->along(S, d, pe);
          Ln = V3{Ln.x + bn.x * Le.x, Ln.y + bn.y * Le.y, Ln.z + bn.z * Le.z};
          if (mode == kTwoState) Lo = V3{Lo.x + bo.x * Le.x, Lo.y + bo.y * Le.y, Lo.z + bo.z * Le.z};
        } else {
          Ln = V3{Ln.x + bn.x, Ln.y + bn.y, Ln.z + bn.z};
          if (mode == kTwoState) Lo = V3{Lo.x + bo.x, Lo.y + bo.y, Lo.z + bo.z};
        }
      }
      return out;
    }
    rng.next1d();  // null BSDF sample (1D + 2D)
    rng.next1d();
    rng.next1d();
    V3 p = ray_at(o, std::fmax(tn, 0.0f), d);
    float t_rem;
    {
      float a0, b0;
      cube_hit(p, d, a0, b0);
      t_rem = b0;
    }

    for (;;) {
      if (!roulette(rng, depth, bn, bo)) return out;
      float m;
      const float t = free_flight(rng, p, d, t_rem, m);
      const float inv_m = 1.0f / m;
      if (!(t <= t_rem)) {
        // leaves the medium through the null boundary, then escapes
        rng.next1d();
        rng.next1d();
        rng.next1d();
        if (!roulette(rng, depth, bn, bo)) return out;
        if (!(S.hide_emitters && depth == 0)) {
          if (env && env->valid()) {
            // map hit after a phase sample: power heuristic against NEE
            // (plugins/twostatevolpath.py:288-308)
            float pe;
            const V3 Le = env->along(S, d, pe);
            const float k = depth == 0 ? 1.0f : mis2(kInvFourPi, pe);
            Ln = V3{Ln.x + (bn.x * Le.x) * k, Ln.y + (bn.y * Le.y) * k, Ln.z + (bn.z * Le.z) * k};
            if (mode == kTwoState)
              Lo = V3{Lo.x + (bo.x * Le.x) * k, Lo.y + (bo.y * Le.y) * k, Lo.z + (bo.z * Le.z) * k};
          } else {
            const float k = depth == 0 ? 1.0f : mis;
            const V3 cn{bn.x * k, bn.y * k, bn.z * k};
            Ln = V3{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
            if (mode == kTwoState) Lo = V3{Lo.x + bo.x * k, Lo.y + bo.y * k, Lo.z + bo.z * k};
          }
        }
        return out;
      }
      const V3 x = ray_at(p, t, d);
      const Corners c = corners(S, x);
      ++out.lookups;
      const float st_n = sigma_t(S.dens_new, c);
      const float st_o = mode == kTwoState ? sigma_t(S.dens_old, c) : 0.0f;
      const float ur = rng.next1d();
      // mean of both states' sigma_t / mu (plugins/twostatevolpath.py:222-225)
      const float prob = mode == kTwoState ? (st_n + st_o) * (0.5f * inv_m) : st_n * inv_m;
      if (ur >= prob) {
        // null collision
        if (mode == kTwoState) {
          const float sn_o = m - st_o, sn_n = m - st_n;
          const float den = sn_n + sn_o;
          const float wn = (2.0f * sn_n) / den, wo = 2.0f - wn;  // weights sum to 2
          bn = V3{bn.x * wn, bn.y * wn, bn.z * wn};
          bo = V3{bo.x * wo, bo.y * wo, bo.z * wo};
        } else if (sink) {
          const float sn = m - st_n;
          const V3 Lr = remaining(Ln);
          const float sd = (dL.x * Lr.x + dL.y * Lr.y) + dL.z * Lr.z;
          sink->density(S, c, -(S.scale * sd) / sn);
        }
        p = x;
        t_rem = t_rem - t;
        continue;
      }
      // real scattering
      depth += 1;
      if (depth >= S.max_depth) return out;
      ++out.scatters;
      const V3 an = albedo(S, S.alb_new, x, c);
      const V3 ssn{st_n * an.x, st_n * an.y, st_n * an.z};
      if (mode == kTwoState) {
        const V3 ao = albedo(S, S.alb_old, x, c);
        const V3 sso{st_o * ao.x, st_o * ao.y, st_o * ao.z};
        // sigma_s / mean sigma_t as ss * (2 / (st_n + st_o)): for equal
        // states 2 / (2 st) == 1 / st exactly, the single-state weight below
        const float k2 = 2.0f / (st_n + st_o);
        bn = V3{bn.x * (ssn.x * k2), bn.y * (ssn.y * k2), bn.z * (ssn.z * k2)};
        bo = V3{bo.x * (sso.x * k2), bo.y * (sso.y * k2), bo.z * (sso.z * k2)};
      } else {
        const float k1 = 1.0f / st_n;
        bn = V3{bn.x * (ssn.x * k1), bn.y * (ssn.y * k1), bn.z * (ssn.z * k1)};
        if (sink) {
          const V3 Lr = remaining(Ln);
          const float sd = (dL.x * Lr.x + dL.y * Lr.y) + dL.z * Lr.z;
          sink->density(S, c, (S.scale * sd) / st_n);
          sink->albedo(S, x, c, V3{(dL.x * Lr.x) / std::fmax(an.x, 1e-8f), (dL.y * Lr.y) / std::fmax(an.y, 1e-8f),
                                (dL.z * Lr.z) / std::fmax(an.z, 1e-8f)});
        }
      }
      // phase function sample: isotropic, 1D (unused) + 2D
      rng.next1d();
      const float pu0 = rng.next1d(), pu1 = rng.next1d();
      const V3 wo = to_box(S, square_to_uniform_sphere(pu0, pu1));
      // next event estimation towards the environment (constant, or the map
      // by importance with a power-heuristic weight against the phase pdf,
      // plugins/twostatevolpath.py:315-344)
      const float nu0 = rng.next1d(), nu1 = rng.next1d();
      V3 w, e{0.0f, 0.0f, 0.0f};
      const bool use_env = env && env->valid();
      if (use_env) {
        V3 Le;
        float pe;
        w = to_box(S, env->sample_dir(nu0, nu1, Le, pe));
        float k = 0.0f;
        if (pe > 0.0f && pe < std::numeric_limits<float>::infinity()) k = (kInvFourPi * mis2(pe, kInvFourPi)) / pe;
        e = V3{Le.x * k, Le.y * k, Le.z * k};
      } else {
        w = to_box(S, square_to_uniform_sphere(nu0, nu1));
      }
      const Rng rng_before = rng;
      float tro, trn;
      transmittance(rng, x, w, tro, trn, out, nullptr);
      V3 cn;
      if (use_env) {
        cn = V3{(bn.x * e.x) * trn, (bn.y * e.y) * trn, (bn.z * e.z) * trn};
      } else {
        const float en = emit_weight * trn;
        cn = V3{((bn.x * kInvFourPi) * mis) * en, ((bn.y * kInvFourPi) * mis) * en,
                ((bn.z * kInvFourPi) * mis) * en};
      }
      Ln = V3{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
      if (mode == kTwoState) {
        if (use_env) {
          Lo = V3{Lo.x + (bo.x * e.x) * tro, Lo.y + (bo.y * e.y) * tro, Lo.z + (bo.z * e.z) * tro};
        } else {
          const float eo = emit_weight * tro;
          Lo = V3{Lo.x + ((bo.x * kInvFourPi) * mis) * eo, Lo.y + ((bo.y * kInvFourPi) * mis) * eo,
                  Lo.z + ((bo.z * kInvFourPi) * mis) * eo};
        }
      }
      if (sink) {
        // replay the shadow walk with the same numbers to differentiate it
        float gs = (dL.x * cn.x + dL.y * cn.y) + dL.z * cn.z;
        Rng replay = rng_before;
        float a0, b0;
        PathOut scratch;
        transmittance(replay, x, w, a0, b0, scratch, &gs);
      }
      p = x;
      d = wo;
      {
        float a0, b0;
        cube_hit(p, d, a0, b0);
        t_rem = b0;
      }
    }
  }
};

// Butterfly combination of T partial sums (T a power of two), the order in
// which adjacent GPU lanes combine them with xor-shuffles.
V3 butterfly(std::vector<V3> v) {
  const size_t T = v.size();
  for (size_t off = 1; off < T; off <<= 1) {
    std::vector<V3> n(T);
    for (size_t i = 0; i < T; ++i)
      n[i] = V3{v[i].x + v[i ^ off].x, v[i].y + v[i ^ off].y, v[i].z + v[i ^ off].z};
    v.swap(n);
  }
  return v[0];
}

// Rows row0, row0 + stride, ... < row1 split over `threads` workers,
// interleaved for load balance.
template <class F>
void parallel_rows(int row0, int row1, int stride, int threads, F&& f) {
  if (stride < 1) stride = 1;
  if (threads <= 1) {
    for (int y = row0; y < row1; y += stride) f(0, y, y + 1);
    return;
  }
  std::vector<std::thread> pool;
  for (int k = 0; k < threads; ++k) {
    pool.emplace_back([&, k] {
      for (int y = row0 + k * stride; y < row1; y += threads * stride) f(k, y, y + 1);
    });
  }
  for (auto& t : pool) t.join();
}

}  // namespace

extern "C" {
// Environment-map primitives for the tests: (u, v, sin theta) of unit
// directions, the map's radiance and pdf there, and sampled directions with
// their radiance and pdf.
void oracle_env_uv(const float* d, int n, float* uvs) {
  for (int i = 0; i < n; ++i) Env::uv(V3{d[3 * i], d[3 * i + 1], d[3 * i + 2]}, uvs[3 * i], uvs[3 * i + 1], uvs[3 * i + 2]);
}

float oracle_atan2(float y, float x) { return arctan2(y, x); }

int oracle_env_sample(const oracle_scene* S, const float* u, int n, float* dirs, float* le, float* pdf) {
  if (!S || S->env_w <= 0) return -1;
  const Env env(*S);
  for (int i = 0; i < n; ++i) {
    V3 L;
    const V3 d = env.sample_dir(u[2 * i], u[2 * i + 1], L, pdf[i]);
    dirs[3 * i] = d.x;
    dirs[3 * i + 1] = d.y;
    dirs[3 * i + 2] = d.z;
    le[3 * i] = L.x;
    le[3 * i + 1] = L.y;
    le[3 * i + 2] = L.z;
  }
  return 0;
}

int oracle_env_eval(const oracle_scene* S, const float* d, int n, float* le, float* pdf) {
  if (!S || S->env_w <= 0) return -1;
  const Env env(*S);
  for (int i = 0; i < n; ++i) {
    float u, v, st;
    Env::uv(V3{d[3 * i], d[3 * i + 1], d[3 * i + 2]}, u, v, st);
    const V3 L = env.eval(u, v);
    le[3 * i] = L.x;
    le[3 * i + 1] = L.y;
    le[3 * i + 2] = L.z;
    pdf[i] = env.pdf(u, v, st);
  }
  return 0;
}
}

extern "C" {

// Primal render.  mode 0 = two-state (out_old = H, out_new = F), 1 = single
// state on `new` (out_new).  `chunk` = samples per GPU thread, which fixes the
// summation order of a pixel's samples (sequential per chunk, butterfly across
// chunks).  counters (optional) = [paths, lookups, nee lookups, scatters].
// Rows [row0, row1) of the image only (row1 <= 0: all rows); other pixels of
// the outputs are left untouched.
int oracle_render(const oracle_scene* S, int mode, uint32_t seed, int spp, int chunk, float* out_old,
                  float* out_new, uint64_t* counters, int threads, int row0, int row1, int row_stride) {
  if (S && row1 <= 0) row1 = S->height;
  if (!S || row0 < 0 || row1 > S->height || row0 > row1) return -1;
  if (!S || spp <= 0 || chunk <= 0 || spp % chunk) return -1;
  const float mu_o = S->scale * grid_max(*S, S->dens_old);
  const float mu_n = S->scale * grid_max(*S, S->dens_new);
  const float mu = mode == kTwoState ? std::fmax(mu_o, mu_n) : mu_n;
  Supergrid sg;
  sg.build(*S);
  const Env env(*S);
  const int T = spp / chunk;
  std::vector<uint64_t> cnt((size_t)std::max(threads, 1) * 4, 0);
  parallel_rows(row0, row1, row_stride, threads, [&](int k, int y0, int y1) {
    Tracer tr{*S, mode, mu, nullptr};
    tr.sg = &sg;
    tr.env = &env;
    for (int py = y0; py < y1; ++py)
      for (int px = 0; px < S->width; ++px) {
        const int pix = py * S->width + px;
        std::vector<V3> so(T), sn(T);
        for (int g = 0; g < T; ++g) {
          V3 ao{0, 0, 0}, an{0, 0, 0};
          for (int s = g * chunk; s < (g + 1) * chunk; ++s) {
            const PathOut o = tr.trace(seed, (uint32_t)((int64_t)pix * spp + s), px, py);
            an = V3{an.x + o.L_new.x, an.y + o.L_new.y, an.z + o.L_new.z};
            ao = V3{ao.x + o.L_old.x, ao.y + o.L_old.y, ao.z + o.L_old.z};
            cnt[k * 4 + 0] += 1;
            cnt[k * 4 + 1] += o.lookups;
            cnt[k * 4 + 2] += o.nee_lookups;
            cnt[k * 4 + 3] += o.scatters;
          }
          so[g] = ao;
          sn[g] = an;
        }
        const V3 Fv = butterfly(sn), Hv = butterfly(so);
        const float fs = (float)spp;
        if (out_new) {
          out_new[pix * 3 + 0] = Fv.x / fs;
          out_new[pix * 3 + 1] = Fv.y / fs;
          out_new[pix * 3 + 2] = Fv.z / fs;
        }
        if (out_old && mode == kTwoState) {
          out_old[pix * 3 + 0] = Hv.x / fs;
          out_old[pix * 3 + 1] = Hv.y / fs;
          out_old[pix * 3 + 2] = Hv.z / fs;
        }
      }
  });
  if (counters)
    for (int k = 0; k < std::max(threads, 1); ++k)
      for (int j = 0; j < 4; ++j) counters[j] += cnt[k * 4 + j];
  return 0;
}

// Path-replay adjoint on `new`: gradients (double) are ADDED to grad_density
// [dz][dy][dx] and, when the scene has an albedo grid and grad_albedo is not
// null, to grad_albedo [dz][dy][dx][3].
int oracle_backward(const oracle_scene* S, uint32_t seed, int spp, const float* grad_img,
                    double* grad_density, double* grad_albedo, int threads, int row0, int row1,
                    int row_stride) {
  if (S && row1 <= 0) row1 = S->height;
  if (!S || row0 < 0 || row1 > S->height || row0 > row1) return -1;
  if (!S || spp <= 0 || !grad_img || !grad_density) return -1;
  const float mu = S->scale * grid_max(*S, S->dens_new);
  Supergrid sg;
  sg.build(*S);
  const Env env(*S);
  const int64_t nv = (int64_t)S->dx * S->dy * S->dz;
  int adx, ady, adz;
  albedo_dims(*S, adx, ady, adz);
  const int64_t na = (int64_t)adx * ady * adz;
  const int nt = std::max(threads, 1);
  std::vector<GradSink> sinks(nt);
  const bool alb = grad_albedo != nullptr && S->alb_new != nullptr;
  for (auto& s : sinks) {
    s.dens.assign(nv, 0.0);
    if (alb) s.alb.assign(na * 3, 0.0);
  }
  parallel_rows(row0, row1, row_stride, threads, [&](int k, int y0, int y1) {
    for (int py = y0; py < y1; ++py)
      for (int px = 0; px < S->width; ++px) {
        const int pix = py * S->width + px;
        const float fs = (float)spp;
        const V3 dL{grad_img[pix * 3 + 0] / fs, grad_img[pix * 3 + 1] / fs, grad_img[pix * 3 + 2] / fs};
        for (int s = 0; s < spp; ++s) {
          const uint32_t lane = (uint32_t)((int64_t)pix * spp + s);
          Tracer primal{*S, kSingle, mu, nullptr};
          primal.sg = &sg;
          primal.env = &env;
          const PathOut o = primal.trace(seed, lane, px, py);
          Tracer adj{*S, kSingle, mu, &sinks[k], dL, o.L_new};
          adj.sg = &sg;
          adj.env = &env;
          adj.trace(seed, lane, px, py);
        }
      }
  });
  for (auto& s : sinks) {
    for (int64_t i = 0; i < nv; ++i) grad_density[i] += s.dens[i];
    if (alb)
      for (int64_t i = 0; i < na * 3; ++i) grad_albedo[i] += s.alb[i];
  }
  return 0;
}

// Forward-mode derivative image [height][width][3] of the single-state
// render along a density tangent [dz][dy][dx] and / or an albedo tangent
// [adz][ady][adx][3] (either may be null): per sample and channel k, the
// adjoint replay with dL = e_k gathers the tangent where it would scatter.
int oracle_forward(const oracle_scene* S, uint32_t seed, int spp, const float* tan_d, const float* tan_a,
                   float* out, int threads) {
  if (!S || spp <= 0 || !out || (!tan_d && !tan_a)) return -1;
  const float mu = S->scale * grid_max(*S, S->dens_new);
  Supergrid sg;
  sg.build(*S);
  const Env env(*S);
  const float* ta = S->alb_new != nullptr ? tan_a : nullptr;
  parallel_rows(0, S->height, 1, threads, [&](int, int y0, int y1) {
    for (int py = y0; py < y1; ++py)
      for (int px = 0; px < S->width; ++px) {
        const int pix = py * S->width + px;
        double d[3] = {0.0, 0.0, 0.0};
        for (int s = 0; s < spp; ++s) {
          const uint32_t lane = (uint32_t)((int64_t)pix * spp + s);
          Tracer primal{*S, kSingle, mu, nullptr};
          primal.sg = &sg;
          primal.env = &env;
          const PathOut o = primal.trace(seed, lane, px, py);
          for (int k = 0; k < 3; ++k) {
            GradSink g;
            g.tan_d = tan_d;
            g.tan_a = ta;
            const V3 e{k == 0 ? 1.0f : 0.0f, k == 1 ? 1.0f : 0.0f, k == 2 ? 1.0f : 0.0f};
            Tracer adj{*S, kSingle, mu, &g, e, o.L_new};
            adj.sg = &sg;
            adj.env = &env;
            adj.trace(seed, lane, px, py);
            d[k] += g.acc;
          }
        }
        for (int k = 0; k < 3; ++k) out[pix * 3 + k] = (float)(d[k] / spp);
      }
  });
  return 0;
}

// Default gradient seed of the reference (plugins/twostatepath.py:87-89).
uint32_t oracle_sample_tea_32(uint32_t v0, uint32_t v1) {
  uint32_t a, b;
  tea(v0, v1, 4, a, b);
  return a;
}

// Raw PCG32 outputs for (initstate, initseq) (known-answer checks).
void oracle_pcg32(uint64_t initstate, uint64_t initseq, int n, uint32_t* out) {
  Rng r;
  r.seed(initstate, initseq);
  for (int i = 0; i < n; ++i) out[i] = r.next();
}

// Draws `n` consecutive uniforms of the stream of (seed, lane).
void oracle_rng_stream(uint32_t seed, uint32_t lane, int n, float* out) {
  Rng r = lane_rng(seed, lane);
  for (int i = 0; i < n; ++i) out[i] = r.next1d();
}

void oracle_log_unit(const float* x, int n, float* out) {
  for (int i = 0; i < n; ++i) out[i] = log_unit(x[i]);
}

void oracle_uniform_sphere(const float* u, int n, float* out) {
  for (int i = 0; i < n; ++i) {
    const V3 d = square_to_uniform_sphere(u[2 * i], u[2 * i + 1]);
    out[3 * i] = d.x;
    out[3 * i + 1] = d.y;
    out[3 * i + 2] = d.z;
  }
}

}  // extern "C"

// ===================================================================
// volpathsimple (plugins/volpathsimple.py): the reference's simplified
// volumetric path tracer and its adjoint, used as `adjoint_integrator` in
// every grid experiment (experiments.py:131,245,364).
//
// Primal (VolpathSimpleIntegrator.sample, :53-327): per loop iteration
//   Russian roulette (1D), a *real* interaction by delta tracking
//   (sample_real_interaction :349-395: per collision a free-flight 1D and, if
//   inside the segment, a real/null 1D), NEE towards the environment (2D +
//   one 1D per ratio-tracking step, :398-491), then the phase sample (1D + 2D).
//   A path that leaves the cube sees the environment with the MIS weight of
//   its last scattering event (:296-321).  After reaching the medium one 1D is
//   drawn to seed the adjoint's second stream (:103-113).
// Adjoint (render_backward of the path-replay base integrator): the primal
//   pass gives L; a second pass replays the same draws with L_rem = L minus
//   the NEE contributions so far and back-propagates:
//   - at each real interaction, the scattering term with MIS weight
//     s^2/(1+s^2), s = sigma_t (:160-186);
//   - at each real interaction or escape, the transmittance of the last
//     segment through 4 uniform samples (:597-620);
//   - each NEE shadow ray by replaying its ratio tracking (:412-422, :481-505);
//   - one differential-ratio-tracking term per path: a reservoir picks one
//     scattering event (:743-778, weight = throughput), and after the path a
//     distance is resampled on that event's segment in proportion to the
//     transmittance, with a recursive path estimating the in-scattered
//     radiance there, MIS weight 1/(1+s^2) (:508-594, :623-668).
//   The adjoint's extra random numbers come from a second stream whose seed
//   is sample_tea_32(bits of lane 0's seeding draw, 1) (:108-113).
// sample_interaction_drt lives in the Mitsuba fork the reference depends on
// (not in the reference tree); it is restated as: distance t' on [0, tmax]
// from the majorant's exponential truncated to the segment, pdf
// mu e^{-mu t'} / (1 - e^{-mu tmax}), weight T^(t') / pdf with T^ a ratio-
// tracking estimate on [0, t'], so weight x f(t') estimates the integral of
// T(t) f(t) over the segment.
// ===================================================================
namespace {

// e^x for x <= 0: n = round(x log2 e), r = x - n ln2 (ln 2 split as in
// log_unit), Taylor polynomial of degree 8 on |r| <= ln2/2, times 2^n.
float exp_nonpos(float x) {
  if (!(x > -87.0f)) return 0.0f;
  const float n = std::rint(x * 1.44269504088896341f);
  float r = std::fmaf(n, -0.693145751953125f, x);
  r = std::fmaf(n, -1.4286068203094172e-06f, r);
  float p = 1.0f / 40320.0f;
  p = std::fmaf(r, p, 1.0f / 5040.0f);
  p = std::fmaf(r, p, 1.0f / 720.0f);
  p = std::fmaf(r, p, 1.0f / 120.0f);
  p = std::fmaf(r, p, 1.0f / 24.0f);
  p = std::fmaf(r, p, 1.0f / 6.0f);
  p = std::fmaf(r, p, 0.5f);
  p = std::fmaf(r, p, 1.0f);
  p = std::fmaf(r, p, 1.0f);
  union { float f; uint32_t u; } s;
  s.u = (uint32_t)((int)n + 127) << 23;
  return p * s.f;
}

struct VpsFlags {
  int32_t use_nee, use_drt, use_drt_subsampling, use_drt_mis;
};

struct VpsSegment {
  V3 o, d;
  float tmax;  // distance to the cube boundary
};

struct Vps {
  const oracle_scene& S;
  VpsFlags F;
  float mu;  // majorant of `new`
  const Supergrid* sg;
  GradSink* sink = nullptr;
  const Env* env = nullptr;  // environment map, if the scene has one

  bool use_env() const { return env != nullptr && env->valid(); }

  float flight(Rng& r, const V3& o, const V3& d, float tmax, float& m) const {
    const float tau = -log_unit(1.0f - r.next1d());
    m = mu;
    if (sg != nullptr && sg->active()) return sg->flight(sg->nw, o, d, tmax, tau, m);
    return mu > 0.0f ? tau * (1.0f / mu) : kInf;
  }

  float sigma_t(const Corners& c) const { return S.scale * trilinear(S, S.dens_new, 1, 0, c); }

  // Delta tracking to the next real interaction; returns its distance from
  // seg.o (the sum of the free-flight distances) or kInf on escape.
  float real_interaction(Rng& r, const VpsSegment& seg) const {
    V3 p = seg.o;
    float rem = seg.tmax, t_acc = 0.0f;
    for (;;) {
      float m;
      const float t = flight(r, p, seg.d, rem, m);
      if (!(t <= rem)) return kInf;
      const V3 x = ray_at(p, t, seg.d);
      const float st = sigma_t(corners(S, x));
      const float ratio = m != 0.0f ? st / m : 0.0f;
      const float u = r.next1d();
      t_acc = t_acc + t;
      if (u < ratio) return t_acc;
      p = x;
      rem = rem - t;
    }
  }

  // Ratio-tracking transmittance from o along w to distance tmax.  With
  // `adj`, back-propagates adj . d log(T).
  float transmittance(Rng& r, const V3& o, const V3& w, float tmax, const V3* adj) const {
    V3 q = o;
    float rem = tmax, tr = 1.0f;
    for (;;) {
      float m;
      const float t = flight(r, q, w, rem, m);
      if (!(t <= rem)) break;
      const V3 x = ray_at(q, t, w);
      const Corners c = corners(S, x);
      const float sn = m - sigma_t(c);
      const float contrib = m != 0.0f ? sn / m : sn;
      if (adj != nullptr && contrib > 0.0f) {
        const float wn = (adj->x + adj->y) + adj->z;  // adj already carries dL
        sink->density(S, c, -(S.scale * wn) / sn);
      }
      tr = tr * contrib;
      q = x;
      rem = rem - t;
      if (tr == 0.0f) break;
    }
    return tr;
  }

  // NEE towards the environment from x with throughput thr (:398-446).
  V3 nee(Rng& r, const V3& x, const V3& thr, const V3* dL) const {
    Rng replay = r;
    const float u0 = r.next1d(), u1 = r.next1d();
    V3 w, e{0.0f, 0.0f, 0.0f};
    if (use_env()) {
      V3 Le;
      float pe;
      w = to_box(S, env->sample_dir(u0, u1, Le, pe));
      float k = 0.0f;
      if (pe > 0.0f && pe < std::numeric_limits<float>::infinity()) k = (kInvFourPi * mis2(pe, kInvFourPi)) / pe;
      e = V3{Le.x * k, Le.y * k, Le.z * k};
    } else {
      w = to_box(S, square_to_uniform_sphere(u0, u1));
    }
    float tn, tf;
    cube_hit(x, w, tn, tf);
    const float tr = transmittance(r, x, w, tf, nullptr);
    V3 c;
    if (use_env()) {
      c = V3{(thr.x * e.x) * tr, (thr.y * e.y) * tr, (thr.z * e.z) * tr};
    } else {
      const float mis = 0.5f;
      const float en = (1.0f / kInvFourPi) * tr;
      c = V3{((thr.x * kInvFourPi) * mis) * en, ((thr.y * kInvFourPi) * mis) * en,
             ((thr.z * kInvFourPi) * mis) * en};
    }
    if (dL != nullptr) {
      // replay the shadow walk with the same numbers (:412-422)
      const V3 adj{dL->x * c.x, dL->y * c.y, dL->z * c.z};
      replay.next1d();
      replay.next1d();
      transmittance(replay, x, w, tf, &adj);
    }
    return c;
  }

  // Primal path from a segment (the loop of sample(), :126-290 and the
  // environment term :296-321).  depth / has_scattered / last pdf as the
  // path state of a recursive call (:73-99).
  V3 primal_from(Rng& r, VpsSegment seg, int depth, bool has_scattered, bool active) const {
    V3 L{0, 0, 0}, thr{1, 1, 1};
    bool escaped = false;
    while (active) {
      const float q = std::fmin(std::fmax(std::fmax(thr.x, thr.y), thr.z), 0.99f);
      const bool rr = depth > S.rr_depth;
      const bool alive = thr.x != 0.0f || thr.y != 0.0f || thr.z != 0.0f;
      const float u = r.next1d();
      if (!alive || (rr && !(u < q))) break;
      if (rr) {
        const float iq = 1.0f / q;
        thr = V3{thr.x * iq, thr.y * iq, thr.z * iq};
      }
      const float t = real_interaction(r, seg);
      if (!(t < kInf)) {
        escaped = true;
        break;
      }
      const V3 x = ray_at(seg.o, t, seg.d);
      const V3 a = albedo(S, S.alb_new, x, corners(S, x));
      has_scattered = true;
      thr = V3{thr.x * a.x, thr.y * a.y, thr.z * a.z};
      depth += 1;
      if (depth >= S.max_depth) break;
      if (F.use_nee) {
        const V3 c = nee(r, x, thr, nullptr);
        L = V3{L.x + c.x, L.y + c.y, L.z + c.z};
      }
      r.next1d();
      const float pu0 = r.next1d(), pu1 = r.next1d();
      seg.o = x;
      seg.d = to_box(S, square_to_uniform_sphere(pu0, pu1));
      float tn, tf;
      cube_hit(seg.o, seg.d, tn, tf);
      if (!(tf > 0.0f)) break;  // accidental escape (:279-283)
      seg.tmax = tf;
    }
    if (escaped && !(depth <= 0 && S.hide_emitters)) {
      if (use_env()) {
        float pe;
        const V3 Le = env->along(S, seg.d, pe);
        const float k = (F.use_nee && has_scattered) ? mis2(kInvFourPi, pe) : 1.0f;
        L = V3{L.x + (thr.x * Le.x) * k, L.y + (thr.y * Le.y) * k, L.z + (thr.z * Le.z) * k};
      } else {
        const float k = (F.use_nee && has_scattered) ? 0.5f : 1.0f;
        L = V3{L.x + thr.x * k, L.y + thr.y * k, L.z + thr.z * k};
      }
    }
    return L;
  }

  // Camera ray of sample `lane`, then the medium entry (reach_medium,
  // :329-346).  Returns false when the ray misses the cube.
  bool camera(Rng& r, int px, int py, V3& o, V3& d, VpsSegment& seg) const {
    const float u0 = r.next1d(), u1 = r.next1d();
    camera_ray(S, px, py, u0, u1, o, d);
    r.next1d();  // colour channel
    float tn, tf;
    cube_hit(o, d, tn, tf);
    if (!(tn <= tf && tf > 0.0f)) return false;
    seg.o = ray_at(o, std::fmax(tn, 0.0f), d);
    seg.d = d;
    cube_hit(seg.o, d, tn, tf);
    seg.tmax = tf;
    return true;
  }

  V3 render_path(uint32_t seed, uint32_t lane, int px, int py) const {
    Rng r = lane_rng(seed, lane);
    V3 o, d;
    VpsSegment seg;
    if (!camera(r, px, py, o, d, seg)) {
      if (S.hide_emitters) return V3{0.0f, 0.0f, 0.0f};
      if (use_env()) {
        float pe;
        return env->along(S, d, pe);
      }
      return V3{1.0f, 1.0f, 1.0f};
    }
    r.next1d();  // seeds the adjoint's second stream
    return primal_from(r, seg, 0, false, true);
  }

  // Differential ratio tracking on `seg` (restated sample_interaction_drt,
  // :540-594) with adjoint `adj` (dL x sampling weight).
  void drt(Rng& alt, const VpsSegment& seg, int depth, const V3& adj) const {
    if (!(mu > 0.0f)) return;
    const float e = exp_nonpos(-(mu * seg.tmax));
    const float u = alt.next1d();
    const float tp = -log_unit(1.0f - u * (1.0f - e)) / mu;
    const float pdf = (mu * exp_nonpos(-(mu * tp))) / (1.0f - e);
    const float tr = transmittance(alt, seg.o, seg.d, tp, nullptr);
    const float wdrt = tr / pdf;
    const V3 x = ray_at(seg.o, tp, seg.d);
    const Corners c = corners(S, x);
    const float st = sigma_t(c);
    const V3 a = albedo(S, S.alb_new, x, c);
    // in-scattered radiance at x: NEE + a recursive path (sample_recursive, :623-668)
    V3 Li{0, 0, 0};
    if (F.use_nee) Li = nee(alt, x, V3{1, 1, 1}, nullptr);
    alt.next1d();
    const float pu0 = alt.next1d(), pu1 = alt.next1d();
    VpsSegment next{x, to_box(S, square_to_uniform_sphere(pu0, pu1)), 0.0f};
    float tn, tf;
    cube_hit(next.o, next.d, tn, tf);
    const bool ok = tf > 0.0f;
    next.tmax = tf;
    const int next_depth = depth + 1;
    const bool active = ok && next_depth < S.max_depth;
    if (active) alt.next1d();  // the recursive call's seeding draw (:103)
    const V3 Lr = primal_from(alt, next, next_depth, true, active);
    Li = V3{Li.x + Lr.x, Li.y + Lr.y, Li.z + Lr.z};
    const float mis = F.use_drt_mis ? 1.0f / (1.0f + st * st) : 1.0f;
    const float k0 = mis * wdrt;
    const V3 k{(k0 * adj.x) * Li.x, (k0 * adj.y) * Li.y, (k0 * adj.z) * Li.z};
    sink->density(S, c, S.scale * ((k.x * a.x + k.y * a.y) + k.z * a.z));
    sink->albedo(S, x, c, V3{k.x * st, k.y * st, k.z * st});
  }

  // Adjoint pass of one sample: replays the primal's draws with L_rem.
  void backward_path(uint32_t seed, uint32_t alt_seed, uint32_t lane, int px, int py, const V3& dL) const {
    const V3 Ltot = render_path(seed, lane, px, py);
    Rng r = lane_rng(seed, lane);
    Rng alt = lane_rng(alt_seed, lane);
    V3 o, d;
    VpsSegment seg;
    if (!camera(r, px, py, o, d, seg)) return;
    r.next1d();
    V3 res = Ltot, thr{1, 1, 1};
    int depth = 0;
    // reservoir of one scattering event for DRT (:743-778)
    V3 wsum{0, 0, 0}, cur{0, 0, 0};
    bool have = false;
    VpsSegment keep{};
    int keep_depth = 0;
    for (;;) {
      const float q = std::fmin(std::fmax(std::fmax(thr.x, thr.y), thr.z), 0.99f);
      const bool rr = depth > S.rr_depth;
      const bool alive = thr.x != 0.0f || thr.y != 0.0f || thr.z != 0.0f;
      const float u = r.next1d();
      if (!alive || (rr && !(u < q))) break;
      if (rr) {
        const float iq = 1.0f / q;
        thr = V3{thr.x * iq, thr.y * iq, thr.z * iq};
      }
      const float t = real_interaction(r, seg);
      const bool escape = !(t < kInf);
      // DRT estimates the in-scattering integral over the whole segment, so
      // it runs for every segment the path traverses, escaping or not (the
      // loop's `active` mask, :158-163)
      if (F.use_drt) {
        if (F.use_drt_subsampling) {
          wsum = V3{wsum.x + thr.x, wsum.y + thr.y, wsum.z + thr.z};
          const float pick = alt.next1d();
          const float ratio = ((thr.x / wsum.x + thr.y / wsum.y) + thr.z / wsum.z) / 3.0f;
          if (pick <= ratio) {
            cur = thr;
            keep = seg;
            keep_depth = depth;
            have = true;
          }
        } else {
          drt(alt, seg, depth, V3{dL.x * thr.x, dL.y * thr.y, dL.z * thr.z});
        }
      }
      if (!escape) {
        const V3 x = ray_at(seg.o, t, seg.d);
        const Corners c = corners(S, x);
        const float st = sigma_t(c);
        const V3 a = albedo(S, S.alb_new, x, c);
        if (!F.use_drt || F.use_drt_mis) {
          const float mis = F.use_drt ? (st * st) / (1.0f + st * st) : 1.0f;
          const float inv_pdf = 1.0f / st;
          const V3 k{((mis * dL.x) * (res.x / std::fmax(1e-8f, a.x))) * inv_pdf,
                     ((mis * dL.y) * (res.y / std::fmax(1e-8f, a.y))) * inv_pdf,
                     ((mis * dL.z) * (res.z / std::fmax(1e-8f, a.z))) * inv_pdf};
          sink->density(S, c, S.scale * ((k.x * a.x + k.y * a.y) + k.z * a.z));
          sink->albedo(S, x, c, V3{k.x * st, k.y * st, k.z * st});
        }
      }
      {
        // transmittance of the last segment: 4 uniform samples (:597-620)
        const float interval = escape ? seg.tmax : t;
        const float w = (dL.x * res.x + dL.y * res.y) + dL.z * res.z;
        const float coef = -(w * (interval * 0.25f));
        for (int j = 0; j < 4; ++j) {
          const float tj = alt.next1d() * interval;
          sink->density(S, corners(S, ray_at(seg.o, tj, seg.d)), S.scale * coef);
        }
      }
      if (escape) break;
      const V3 x = ray_at(seg.o, t, seg.d);
      const V3 a = albedo(S, S.alb_new, x, corners(S, x));
      thr = V3{thr.x * a.x, thr.y * a.y, thr.z * a.z};
      depth += 1;
      if (depth >= S.max_depth) break;
      if (F.use_nee) {
        const V3 c = nee(r, x, thr, &dL);
        res = V3{res.x - c.x, res.y - c.y, res.z - c.z};
      }
      r.next1d();
      const float pu0 = r.next1d(), pu1 = r.next1d();
      seg.o = x;
      seg.d = to_box(S, square_to_uniform_sphere(pu0, pu1));
      float tn, tf;
      cube_hit(seg.o, seg.d, tn, tf);
      if (!(tf > 0.0f)) break;
      seg.tmax = tf;
    }
    if (F.use_drt && F.use_drt_subsampling && have) {
      const float dmean = ((cur.x + cur.y) + cur.z) / 3.0f;
      if (dmean != 0.0f) {
        const float wmean = ((wsum.x + wsum.y) + wsum.z) / 3.0f;
        const V3 sw{(wmean * cur.x) / dmean, (wmean * cur.y) / dmean, (wmean * cur.z) / dmean};
        drt(alt, keep, keep_depth, V3{sw.x * dL.x, sw.y * dL.y, sw.z * dL.z});
      }
    }
  }
};

// Seed of the adjoint's second stream: sample_tea_32(bits of the seeding
// draw of lane 0, 1)[0] (:108-113); lane 0's fourth draw (film 2D, channel).
uint32_t vps_alt_seed(uint32_t seed) {
  Rng r = lane_rng(seed, 0);
  r.next1d();
  r.next1d();
  r.next1d();
  const float u = r.next1d();
  uint32_t bits;
  std::memcpy(&bits, &u, 4);
  uint32_t a, b;
  tea(bits, 1u, 4, a, b);
  return a;
}

}  // namespace

extern "C" {

uint32_t oracle_vps_alt_seed(uint32_t seed) { return vps_alt_seed(seed); }

float oracle_exp_nonpos(float x) { return exp_nonpos(x); }

// volpathsimple primal image [height][width][3] (box film, sample order).
int oracle_vps_render(const oracle_scene* S, const int32_t flags[4], uint32_t seed, int spp, float* out, int threads,
                      int row0, int row1, int row_stride) {
  if (S && row1 <= 0) row1 = S->height;
  if (!S || !flags || !out || spp <= 0 || row0 < 0 || row1 > S->height || row0 > row1) return -1;
  Supergrid sg;
  sg.build(*S);
  const Env env(*S);
  Vps vps{*S, VpsFlags{flags[0], flags[1], flags[2], flags[3]}, S->scale * grid_max(*S, S->dens_new), &sg};
  vps.env = &env;
  parallel_rows(row0, row1, row_stride, threads, [&](int, int y0, int y1) {
    for (int py = y0; py < y1; ++py)
      for (int px = 0; px < S->width; ++px) {
        const int pix = py * S->width + px;
        V3 acc{0, 0, 0};
        for (int s = 0; s < spp; ++s) {
          const V3 L = vps.render_path(seed, (uint32_t)((int64_t)pix * spp + s), px, py);
          acc = V3{acc.x + L.x, acc.y + L.y, acc.z + L.z};
        }
        const float fs = (float)spp;
        out[pix * 3 + 0] = acc.x / fs;
        out[pix * 3 + 1] = acc.y / fs;
        out[pix * 3 + 2] = acc.z / fs;
      }
  });
  return 0;
}

// volpathsimple adjoint: gradients (double) ADDED to grad_density and, when
// the scene has an albedo grid and grad_albedo is set, to grad_albedo.
int oracle_vps_backward(const oracle_scene* S, const int32_t flags[4], uint32_t seed, int spp, const float* grad_img,
                        double* grad_density, double* grad_albedo, int threads) {
  if (!S || !flags || spp <= 0 || !grad_img || !grad_density) return -1;
  Supergrid sg;
  sg.build(*S);
  const Env env(*S);
  const float mu = S->scale * grid_max(*S, S->dens_new);
  const uint32_t alt_seed = vps_alt_seed(seed);
  const int64_t nv = (int64_t)S->dx * S->dy * S->dz;
  int adx, ady, adz;
  albedo_dims(*S, adx, ady, adz);
  const int64_t na = (int64_t)adx * ady * adz;
  const int nt = std::max(threads, 1);
  std::vector<GradSink> sinks(nt);
  const bool alb = grad_albedo != nullptr && S->alb_new != nullptr;
  for (auto& s : sinks) {
    s.dens.assign(nv, 0.0);
    if (alb) s.alb.assign(na * 3, 0.0);
  }
  parallel_rows(0, S->height, 1, threads, [&](int k, int y0, int y1) {
    Vps vps{*S, VpsFlags{flags[0], flags[1], flags[2], flags[3]}, mu, &sg};
    vps.sink = &sinks[k];
    vps.env = &env;
    for (int py = y0; py < y1; ++py)
      for (int px = 0; px < S->width; ++px) {
        const int pix = py * S->width + px;
        const float fs = (float)spp;
        const V3 dL{grad_img[pix * 3 + 0] / fs, grad_img[pix * 3 + 1] / fs, grad_img[pix * 3 + 2] / fs};
        for (int s = 0; s < spp; ++s)
          vps.backward_path(seed, alt_seed, (uint32_t)((int64_t)pix * spp + s), px, py, dL);
      }
  });
  for (auto& s : sinks) {
    for (int64_t i = 0; i < nv; ++i) grad_density[i] += s.dens[i];
    if (alb)
      for (int64_t i = 0; i < na * 3; ++i) grad_albedo[i] += s.alb[i];
  }
  return 0;
}

}  // extern "C"
