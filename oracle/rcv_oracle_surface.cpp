// CPU oracle of the surface two-state tracer — TEST INFRASTRUCTURE ONLY.
//
// Restates, one path at a time, TwoStatePRBIntegrator.sample_twostates
// (plugins/twostatepath.py:225-364) with the two-state BSDF of
// plugins/twostatebsdf.py for the synthetic surface scene: a ground
// rectangle y = 0 with a two-state diffuse RGB texture (bilinear, repeat),
// diffuse spheres and one rectangular area light facing -y.  Also the
// path-replay adjoint on `new` into the texture.  Float operations follow the
// GPU kernels one for one (explicit fmaf, -ffp-contract=off).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kInvFourPiS = 0.0795774715459476678844f;
constexpr float kHalfPiS = 1.57079632679489661923f;
constexpr float kShadowEps = 1e-3f;
constexpr float kInfS = __builtin_huge_valf();

void tea_s(uint32_t v0, uint32_t v1, uint32_t& o0, uint32_t& o1) {
  uint32_t sum = 0;
  for (int i = 0; i < 4; ++i) {
    sum += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + sum) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + sum) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  o0 = v0;
  o1 = v1;
}

struct Pcg {
  uint64_t state = 0, inc = 1;
  uint32_t next() {
    const uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  float u() {
    uint32_t b = (next() >> 9) | 0x3f800000u;
    float f;
    std::memcpy(&f, &b, 4);
    return f - 1.0f;
  }
};

Pcg make_rng(uint32_t seed, uint32_t lane) {
  uint32_t a, b, c, d;
  tea_s(seed, lane, a, b);
  tea_s(lane, seed, c, d);
  Pcg r;
  r.inc = ((((uint64_t)c << 32) | d) << 1u) | 1u;
  r.next();
  r.state += ((uint64_t)a << 32) | b;
  r.next();
  return r;
}

void sincos2pi(float u, float& s, float& c) {
  const float u4 = u * 4.0f;
  const float qf = std::floor(u4);
  const int q = (int)qf & 3;
  float f = u4 - qf;
  const bool swap = f > 0.5f;
  if (swap) f = 1.0f - f;
  const float x = f * kHalfPiS;
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

struct V {
  float x, y, z;
};

float dot(const V& a, const V& b) { return std::fmaf(a.z, b.z, std::fmaf(a.y, b.y, a.x * b.x)); }

}  // namespace

extern "C" {
struct oracle_surface {
  int32_t width, height;
  float cam_o[3], cam_f[3], cam_r[3], cam_u[3];
  int32_t max_depth, rr_depth, hide_emitters;
  float plane_half;
  int32_t tex_w, tex_h;
  const float* tex_old;  // [tex_h][tex_w][3]
  const float* tex_new;
  int32_t nspheres;
  float spheres[8][7];  // cx, cy, cz, r, albedo rgb
  float light_c[3], light_h[2], light_le[3];
};
}

namespace {

struct Tex {
  int i00, i10, i01, i11;
  float fx, fy;
};

struct Surf {
  const oracle_surface& S;
  int mode;  // 0 two-state, 1 new only
  std::vector<double>* grad = nullptr;
  V dL{0, 0, 0}, Lrem{0, 0, 0};
  // forward mode: texture tangent [tex_h][tex_w][3] gathered into acc
  const float* tan = nullptr;
  double acc[3] = {0.0, 0.0, 0.0};

  float light_area() const { return (2.0f * S.light_h[0]) * (2.0f * S.light_h[1]); }

  int hit(const V& o, const V& d, float tmax, float& th) const {
    int id = -1;
    th = tmax;
    if (d.y != 0.0f) {
      const float t = (0.0f - o.y) / d.y;
      if (t > 1e-6f && t < th) {
        const float x = std::fmaf(t, d.x, o.x), z = std::fmaf(t, d.z, o.z);
        if (std::fabs(x) <= S.plane_half && std::fabs(z) <= S.plane_half) {
          th = t;
          id = 0;
        }
      }
      const float tl = (S.light_c[1] - o.y) / d.y;
      if (tl > 1e-6f && tl < th) {
        const float x = std::fmaf(tl, d.x, o.x) - S.light_c[0], z = std::fmaf(tl, d.z, o.z) - S.light_c[2];
        if (std::fabs(x) <= S.light_h[0] && std::fabs(z) <= S.light_h[1]) {
          th = tl;
          id = 100;
        }
      }
    }
    for (int k = 0; k < S.nspheres; ++k) {
      const float* s = S.spheres[k];
      const V oc{o.x - s[0], o.y - s[1], o.z - s[2]};
      const float b = dot(oc, d);
      const float c = std::fmaf(-s[3], s[3], dot(oc, oc));
      const float disc = std::fmaf(b, b, -c);
      if (disc < 0.0f) continue;
      const float sq = std::sqrt(disc);
      float t = -b - sq;
      if (!(t > 1e-6f)) t = -b + sq;
      if (t > 1e-6f && t < th) {
        th = t;
        id = k + 1;
      }
    }
    return id;
  }

  V normal(int id, const V& p) const {
    if (id == 0) return V{0.0f, 1.0f, 0.0f};
    if (id == 100) return V{0.0f, -1.0f, 0.0f};
    const float* s = S.spheres[id - 1];
    const float inv = 1.0f / s[3];
    return V{(p.x - s[0]) * inv, (p.y - s[1]) * inv, (p.z - s[2]) * inv};
  }

  static V offset(const V& p, const V& n, const V& w) {
    const float m = std::fmax(std::fmax(std::fabs(p.x), std::fabs(p.y)), std::fabs(p.z));
    const float e = 1e-4f * (1.0f + m);
    const float s = dot(n, w) >= 0.0f ? e : -e;
    return V{std::fmaf(s, n.x, p.x), std::fmaf(s, n.y, p.y), std::fmaf(s, n.z, p.z)};
  }

  Tex locate(const V& p) const {
    const float inv = 0.5f / S.plane_half;
    const float u = (p.x + S.plane_half) * inv, v = (p.z + S.plane_half) * inv;
    const float px = std::fmaf(u, (float)S.tex_w, -0.5f), py = std::fmaf(v, (float)S.tex_h, -0.5f);
    const float flx = std::floor(px), fly = std::floor(py);
    Tex t;
    t.fx = px - flx;
    t.fy = py - fly;
    int x0 = (int)std::fmin(std::fmax(flx, -1.0f), (float)S.tex_w) % S.tex_w;
    int y0 = (int)std::fmin(std::fmax(fly, -1.0f), (float)S.tex_h) % S.tex_h;
    if (x0 < 0) x0 += S.tex_w;
    if (y0 < 0) y0 += S.tex_h;
    const int x1 = x0 + 1 == S.tex_w ? 0 : x0 + 1;
    const int y1 = y0 + 1 == S.tex_h ? 0 : y0 + 1;
    t.i00 = y0 * S.tex_w + x0;
    t.i10 = y0 * S.tex_w + x1;
    t.i01 = y1 * S.tex_w + x0;
    t.i11 = y1 * S.tex_w + x1;
    return t;
  }

  V tex(const float* img, const Tex& t) const {
    auto lerp = [](float a, float b, float f) { return std::fmaf(f, b - a, a); };
    V r;
    float* out[3] = {&r.x, &r.y, &r.z};
    for (int c = 0; c < 3; ++c) {
      const float lo = lerp(img[t.i00 * 3 + c], img[t.i10 * 3 + c], t.fx);
      const float hi = lerp(img[t.i01 * 3 + c], img[t.i11 * 3 + c], t.fx);
      *out[c] = lerp(lo, hi, t.fy);
    }
    return r;
  }

  static float mis(float a, float b) {
    const float a2 = a * a, b2 = b * b;
    const float w = a2 / (a2 + b2);
    return std::isfinite(w) ? w : 0.0f;
  }

  // Returns (L_old, L_new) of one path.
  void trace(uint32_t seed, uint32_t lane, int px, int py, V& Lo, V& Ln) {
    Pcg rng = make_rng(seed, lane);
    const float u0 = rng.u(), u1 = rng.u();
    const float inv_w = 1.0f / (float)S.width, inv_h = 1.0f / (float)S.height;
    const float nx = ((float)px + u0) * inv_w, ny = ((float)py + u1) * inv_h;
    const float a = std::fmaf(2.0f, nx, -1.0f), b = std::fmaf(-2.0f, ny, 1.0f);
    V r{std::fmaf(b, S.cam_u[0], std::fmaf(a, S.cam_r[0], S.cam_f[0])),
        std::fmaf(b, S.cam_u[1], std::fmaf(a, S.cam_r[1], S.cam_f[1])),
        std::fmaf(b, S.cam_u[2], std::fmaf(a, S.cam_r[2], S.cam_f[2]))};
    const float inv_len = 1.0f / std::sqrt(std::fmaf(r.z, r.z, std::fmaf(r.y, r.y, r.x * r.x)));
    V d{r.x * inv_len, r.y * inv_len, r.z * inv_len};
    V o{S.cam_o[0], S.cam_o[1], S.cam_o[2]};
    V bo{1, 1, 1}, bn{1, 1, 1};
    Lo = V{0, 0, 0};
    Ln = V{0, 0, 0};
    float prev_pdf = 1.0f;
    bool prev_delta = true;
    const float area = light_area();
    const V le{S.light_le[0], S.light_le[1], S.light_le[2]};
    for (int depth = 0;; ++depth) {
      float t;
      const int id = hit(o, d, kInfS, t);
      if (id < 0) return;
      const V p{std::fmaf(t, d.x, o.x), std::fmaf(t, d.y, o.y), std::fmaf(t, d.z, o.z)};
      const V n = normal(id, p);
      const V wi{-d.x, -d.y, -d.z};
      // emission with MIS against the previous BSDF sample
      if (id == 100 && d.y > 0.0f && !(S.hide_emitters && depth == 0)) {
        float pdf_em = 0.0f;
        if (!prev_delta) pdf_em = (t * t) / (d.y * area);
        const float w = mis(prev_pdf, pdf_em);
        const V cn{(bn.x * w) * le.x, (bn.y * w) * le.y, (bn.z * w) * le.z};
        Ln = V{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
        Lo = V{Lo.x + (bo.x * w) * le.x, Lo.y + (bo.y * w) * le.y, Lo.z + (bo.z * w) * le.z};
        Lrem = V{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
      }
      V an, ao;
      Tex tl{};
      if (id == 0) {
        tl = locate(p);
        an = tex(S.tex_new, tl);
        ao = mode == 0 ? tex(S.tex_old, tl) : an;
      } else if (id == 100) {
        an = V{0, 0, 0};
        ao = an;
      } else {
        an = V{S.spheres[id - 1][4], S.spheres[id - 1][5], S.spheres[id - 1][6]};
        ao = an;
      }
      const float cos_i = dot(n, wi);
      const bool active_next = depth + 1 < S.max_depth;
      if (tan && id == 0 && active_next) {
        const int idx[4] = {tl.i00, tl.i10, tl.i01, tl.i11};
        const float gx = 1.0f - tl.fx, gy = 1.0f - tl.fy;
        const float ws[4] = {gx * gy, tl.fx * gy, gx * tl.fy, tl.fx * tl.fy};
        const float an_c[3] = {an.x, an.y, an.z}, lr[3] = {Lrem.x, Lrem.y, Lrem.z};
        for (int c = 0; c < 3; ++c) {
          double t = 0.0;
          for (int k = 0; k < 4; ++k) t += (double)ws[k] * tan[idx[k] * 3 + c];
          acc[c] += (double)lr[c] * t / std::fmax(an_c[c], 1e-8f);
        }
      }
      if (grad && id == 0 && active_next) {
        const V g{(dL.x * Lrem.x) / std::fmax(an.x, 1e-8f), (dL.y * Lrem.y) / std::fmax(an.y, 1e-8f),
                  (dL.z * Lrem.z) / std::fmax(an.z, 1e-8f)};
        const float gx = 1.0f - tl.fx, gy = 1.0f - tl.fy;
        const float w00 = gx * gy, w10 = tl.fx * gy, w01 = gx * tl.fy, w11 = tl.fx * tl.fy;
        const int idx[4] = {tl.i00, tl.i10, tl.i01, tl.i11};
        const float ws[4] = {w00, w10, w01, w11};
        for (int k = 0; k < 4; ++k) {
          (*grad)[idx[k] * 3 + 0] += g.x * ws[k];
          (*grad)[idx[k] * 3 + 1] += g.y * ws[k];
          (*grad)[idx[k] * 3 + 2] += g.z * ws[k];
        }
      }
      // next event estimation on the area light
      const float e0 = rng.u(), e1 = rng.u();
      if (active_next && cos_i > 0.0f) {
        const V lp{S.light_c[0] + std::fmaf(2.0f, e0, -1.0f) * S.light_h[0], S.light_c[1],
                   S.light_c[2] + std::fmaf(2.0f, e1, -1.0f) * S.light_h[1]};
        const V v{lp.x - p.x, lp.y - p.y, lp.z - p.z};
        const float dist2 = dot(v, v);
        const float dist = std::sqrt(dist2);
        const float inv_dist = 1.0f / dist;
        const V wl{v.x * inv_dist, v.y * inv_dist, v.z * inv_dist};
        const float cos_l = wl.y;
        const float cos_o = dot(n, wl);
        if (cos_l > 0.0f && cos_o > 0.0f) {
          const float pdf_l = dist2 / (cos_l * area);
          const V org = offset(p, n, wl);
          float ts;
          const int sid = hit(org, wl, dist * (1.0f - kShadowEps), ts);
          if (sid == -1 || sid == 100) {
            const float w = mis(pdf_l, kInvPi * cos_o);
            const V ew{le.x / pdf_l, le.y / pdf_l, le.z / pdf_l};
            const V vn{(an.x * kInvPi) * cos_o, (an.y * kInvPi) * cos_o, (an.z * kInvPi) * cos_o};
            const V cn{((bn.x * w) * vn.x) * ew.x, ((bn.y * w) * vn.y) * ew.y, ((bn.z * w) * vn.z) * ew.z};
            Ln = V{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
            const V vo{(ao.x * kInvPi) * cos_o, (ao.y * kInvPi) * cos_o, (ao.z * kInvPi) * cos_o};
            Lo = V{Lo.x + ((bo.x * w) * vo.x) * ew.x, Lo.y + ((bo.y * w) * vo.y) * ew.y,
                   Lo.z + ((bo.z * w) * vo.z) * ew.z};
            Lrem = V{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
          }
        }
      }
      // BSDF sample of `new`: cosine-weighted hemisphere
      (void)rng.u();
      const float s0 = rng.u(), s1 = rng.u();
      bool alive = active_next && cos_i > 0.0f;
      if (alive) {
        const float rr = std::sqrt(s0);
        float sn, cs;
        sincos2pi(s1, sn, cs);
        const float lz = std::sqrt(std::fmax(0.0f, 1.0f - s0));
        const float sign = std::copysign(1.0f, n.z);
        const float aa = -1.0f / (sign + n.z);
        const float bb = n.x * n.y * aa;
        const V ts{std::fmaf(sign * n.x * n.x, aa, 1.0f), sign * bb, -sign * n.x};
        const V tt{bb, std::fmaf(n.y * n.y, aa, sign), -n.y};
        const float lx = rr * cs, ly = rr * sn;
        const V wo{std::fmaf(lz, n.x, std::fmaf(ly, tt.x, lx * ts.x)),
                   std::fmaf(lz, n.y, std::fmaf(ly, tt.y, lx * ts.y)),
                   std::fmaf(lz, n.z, std::fmaf(ly, tt.z, lx * ts.z))};
        const float pdf = kInvPi * lz;
        if (pdf > 0.0f) {
          if (mode == 0) {
            const V vold{(ao.x * kInvPi) * lz, (ao.y * kInvPi) * lz, (ao.z * kInvPi) * lz};
            bo = V{bo.x * (vold.x / pdf), bo.y * (vold.y / pdf), bo.z * (vold.z / pdf)};
          }
          bn = V{bn.x * an.x, bn.y * an.y, bn.z * an.z};
          prev_pdf = pdf;
          prev_delta = false;
          o = offset(p, n, wo);
          d = wo;
        } else {
          alive = false;
        }
      }
      if (!alive) {
        bn = V{0, 0, 0};
        bo = V{0, 0, 0};
      }
      const float bmax = std::fmax(std::fmax(bn.x, bn.y), bn.z);
      alive = alive && bmax != 0.0f;
      const float rr_prob = std::fmin(bmax, 0.95f);
      const float ur = rng.u();
      if (depth >= S.rr_depth) {
        const float inv = 1.0f / rr_prob;
        bn = V{bn.x * inv, bn.y * inv, bn.z * inv};
        bo = V{bo.x * inv, bo.y * inv, bo.z * inv};
        alive = alive && ur < rr_prob;
      }
      if (!alive) return;
    }
  }
};

// Rows row0, row0 + stride, ... < row1 (row1 <= 0: the image's height)
// split over `threads` workers; f(worker, row).
template <class F>
void for_rows(int h, int threads, F&& f, int row0 = 0, int row1 = 0, int stride = 1) {
  const int nt = std::max(1, threads);
  const int end = row1 > 0 ? std::min(row1, h) : h;
  const int st = std::max(1, stride);
  std::vector<std::thread> pool;
  for (int k = 0; k < nt; ++k)
    pool.emplace_back([&, k] {
      for (int y = row0 + k * st; y < end; y += nt * st) f(k, y);
    });
  for (auto& t : pool) t.join();
}

}  // namespace

extern "C" {

// mode 0: two-state (out_old = H, out_new = F); 1: single state (out_new).
// Samples of a pixel are summed in sample order.  Only rows row0, row0 +
// stride, ... < row1 are rendered (row1 <= 0: all rows); other pixels of
// the outputs are left untouched.
int oracle_surface_render(const oracle_surface* S, int mode, uint32_t seed, int spp, float* out_old,
                          float* out_new, int threads, int row0, int row1, int row_stride) {
  if (!S || spp <= 0 || S->nspheres < 0 || S->nspheres > 8 || row0 < 0 || row1 > S->height) return -1;
  for_rows(S->height, threads, [&](int, int py) {
    Surf tr{*S, mode};
    for (int px = 0; px < S->width; ++px) {
      const int pix = py * S->width + px;
      V ao{0, 0, 0}, an{0, 0, 0};
      for (int s = 0; s < spp; ++s) {
        V Lo, Ln;
        tr.trace(seed, (uint32_t)((int64_t)pix * spp + s), px, py, Lo, Ln);
        an = V{an.x + Ln.x, an.y + Ln.y, an.z + Ln.z};
        ao = V{ao.x + Lo.x, ao.y + Lo.y, ao.z + Lo.z};
      }
      const float fs = (float)spp;
      out_new[pix * 3 + 0] = an.x / fs;
      out_new[pix * 3 + 1] = an.y / fs;
      out_new[pix * 3 + 2] = an.z / fs;
      if (mode == 0 && out_old) {
        out_old[pix * 3 + 0] = ao.x / fs;
        out_old[pix * 3 + 1] = ao.y / fs;
        out_old[pix * 3 + 2] = ao.z / fs;
      }
    }
  }, row0, row1, row_stride);
  return 0;
}

// Forward-mode derivative image [height][width][3] of the render on `new`
// along a texture tangent [tex_h][tex_w][3].
int oracle_surface_forward(const oracle_surface* S, uint32_t seed, int spp, const float* tangent, float* out,
                           int threads) {
  if (!S || spp <= 0 || !tangent || !out) return -1;
  const int nt = std::max(1, threads);
  for_rows(S->height, nt, [&](int, int py) {
    for (int px = 0; px < S->width; ++px) {
      const int pix = py * S->width + px;
      double d[3] = {0.0, 0.0, 0.0};
      for (int s = 0; s < spp; ++s) {
        const uint32_t lane = (uint32_t)((int64_t)pix * spp + s);
        Surf primal{*S, 1};
        V Lo, Ln;
        primal.trace(seed, lane, px, py, Lo, Ln);
        Surf fw{*S, 1, nullptr, V{0, 0, 0}, Ln};
        fw.tan = tangent;
        fw.trace(seed, lane, px, py, Lo, Ln);
        for (int c = 0; c < 3; ++c) d[c] += fw.acc[c];
      }
      for (int c = 0; c < 3; ++c) out[pix * 3 + c] = (float)(d[c] / spp);
    }
  });
  return 0;
}

// Path-replay adjoint on `new`: ADDS dLoss/dtexture (double) to grad_tex,
// from the paths of rows row0, row0 + stride, ... < row1 (row1 <= 0: all).
int oracle_surface_backward(const oracle_surface* S, uint32_t seed, int spp, const float* grad_img,
                            double* grad_tex, int threads, int row0, int row1, int row_stride) {
  if (!S || spp <= 0 || !grad_img || !grad_tex || row0 < 0 || row1 > S->height) return -1;
  const int nt = std::max(1, threads);
  const size_t n = (size_t)S->tex_w * S->tex_h * 3;
  std::vector<std::vector<double>> sinks(nt, std::vector<double>(n, 0.0));
  for_rows(S->height, nt, [&](int k, int py) {
    for (int px = 0; px < S->width; ++px) {
      const int pix = py * S->width + px;
      const float fs = (float)spp;
      const V dL{grad_img[pix * 3 + 0] / fs, grad_img[pix * 3 + 1] / fs, grad_img[pix * 3 + 2] / fs};
      for (int s = 0; s < spp; ++s) {
        const uint32_t lane = (uint32_t)((int64_t)pix * spp + s);
        Surf primal{*S, 1};
        V Lo, Ln;
        primal.trace(seed, lane, px, py, Lo, Ln);
        Surf adj{*S, 1, &sinks[k], dL, Ln};
        adj.trace(seed, lane, px, py, Lo, Ln);
      }
    }
  }, row0, row1, row_stride);
  for (auto& s : sinks)
    for (size_t i = 0; i < n; ++i) grad_tex[i] += s[i];
  return 0;
}

}  // extern "C"
