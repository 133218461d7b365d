// Surface two-state path tracer (twostateprb) and its path-replay adjoint.
//
// Restates plugins/twostatepath.py:225-364 (TwoStatePRBIntegrator.
// sample_twostates) with plugins/twostatebsdf.py (sampling / pdf / eval on
// `new`, eval_old on `old`) for this scene family: a ground rectangle y = 0
// whose diffuse reflectance is a two-state RGB texture, diffuse spheres and
// one rectangular area light facing down.  Per bounce:
//   intersect; emission with MIS against the previous BSDF pdf; NEE (2D
//   sample, visibility-tested) weighted by eval_pdf (new) / eval_old (old);
//   BSDF sample (1D + 2D) of `new`: beta_new *= weight,
//   beta_old *= eval_old / pdf; Russian roulette with an unconditional 1D
//   draw, probability min(max(beta_new), 0.95) once depth >= rr_depth.
// Random numbers per path: film 2D, then per bounce NEE 2D, BSDF 1D + 2D,
// RR 1D.  The adjoint (Mitsuba's PRBIntegrator.render_backward on `new`)
// scatters at every texture vertex dL * L_rem / albedo bilinearly into the
// four texels, L_rem = L - (radiance gathered before the vertex's
// reflectance acts).  kAdjoint traces each path twice (L, then the replay);
// kTape traces it once and records each texture vertex (its position, the
// path and the radiance gathered so far) on a tape that
// surface_tape_scatter_kernel (rcv_surface.cu) turns into the gradient once
// L is known; paths whose vertices did not fit are replayed by kAdjoint over
// the lost-path list.
#pragma once
#include "rcv_volume.cuh"

namespace rcv {

constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kShadowEps = 1e-3f;
constexpr int kMaxSpheres = 8;

struct Sphere {
  V3 c;
  float r;
  V3 albedo;
};

struct SurfJob {
  int32_t width, height, spp, max_depth, rr_depth, hide_emitters;
  uint32_t seed;
  V3 cam_o, cam_f, cam_r, cam_u;
  float inv_w, inv_h;
  float plane_half;
  int32_t tex_w, tex_h;
  const float4* __restrict__ tex;  // [tex_h * tex_w][2] (old, new) rgb + pad
  int32_t nspheres;
  Sphere sph[kMaxSpheres];
  V3 light_c;  // rectangle at y = light_c.y, facing -y
  float light_hx, light_hz, light_area;
  V3 light_le;
  const float* grad_img;
  float4* grad_tex;  // [tex_h * tex_w] rgb + pad (forward mode: the texture tangent)
  float* out_img;    // forward mode: image derivative
  int64_t path_count;
};

enum Hit { kMiss = -1, kPlane = 0, kLight = 100 };

__device__ __forceinline__ float dot3(const V3& a, const V3& b) {
  return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x));
}

// Closest hit; returns the shape id (kPlane, sphere index + 1, kLight, kMiss).
__device__ __forceinline__ int intersect(const SurfJob& S, const V3& o, const V3& d, float tmax,
                                         float& t_hit) {
  int id = kMiss;
  t_hit = tmax;
  if (d.y != 0.0f) {
    const float t = (0.0f - o.y) / d.y;
    if (t > 1e-6f && t < t_hit) {
      const float x = fmaf(t, d.x, o.x), z = fmaf(t, d.z, o.z);
      if (fabsf(x) <= S.plane_half && fabsf(z) <= S.plane_half) {
        t_hit = t;
        id = kPlane;
      }
    }
    const float tl = (S.light_c.y - o.y) / d.y;
    if (tl > 1e-6f && tl < t_hit) {
      const float x = fmaf(tl, d.x, o.x) - S.light_c.x, z = fmaf(tl, d.z, o.z) - S.light_c.z;
      if (fabsf(x) <= S.light_hx && fabsf(z) <= S.light_hz) {
        t_hit = tl;
        id = kLight;
      }
    }
  }
  for (int k = 0; k < S.nspheres; ++k) {
    const V3 oc{o.x - S.sph[k].c.x, o.y - S.sph[k].c.y, o.z - S.sph[k].c.z};
    const float b = dot3(oc, d);
    const float c = fmaf(-S.sph[k].r, S.sph[k].r, dot3(oc, oc));
    const float disc = fmaf(b, b, -c);
    if (disc < 0.0f) continue;
    const float sq = sqrtf(disc);
    float t = -b - sq;
    if (!(t > 1e-6f)) t = -b + sq;
    if (t > 1e-6f && t < t_hit) {
      t_hit = t;
      id = k + 1;
    }
  }
  return id;
}

// Shadow test: is anything but the light between o and o + dist * d?
__device__ __forceinline__ bool occluded(const SurfJob& S, const V3& o, const V3& d, float dist) {
  float t;
  const int id = intersect(S, o, d, dist * (1.0f - kShadowEps), t);
  return id != kMiss && id != kLight;
}

__device__ __forceinline__ V3 shape_normal(const SurfJob& S, int id, const V3& p) {
  if (id == kPlane) return V3{0.0f, 1.0f, 0.0f};
  if (id == kLight) return V3{0.0f, -1.0f, 0.0f};
  const Sphere& s = S.sph[id - 1];
  const float inv = 1.0f / s.r;
  return V3{(p.x - s.c.x) * inv, (p.y - s.c.y) * inv, (p.z - s.c.z) * inv};
}

// Orthonormal basis around n (Duff et al. 2017, "Building an Orthonormal
// Basis, Revisited").
__device__ __forceinline__ void onb(const V3& n, V3& s, V3& t) {
  const float sign = copysignf(1.0f, n.z);
  const float a = -1.0f / (sign + n.z);
  const float b = n.x * n.y * a;
  s = V3{fmaf(sign * n.x * n.x, a, 1.0f), sign * b, -sign * n.x};
  t = V3{b, fmaf(n.y * n.y, a, sign), -n.y};
}

// Origin offset off the surface, on the side of direction w.
__device__ __forceinline__ V3 offset_origin(const V3& p, const V3& n, const V3& w) {
  const float m = fmaxf(fmaxf(fabsf(p.x), fabsf(p.y)), fabsf(p.z));
  const float e = 1e-4f * (1.0f + m);
  const float s = dot3(n, w) >= 0.0f ? e : -e;
  return V3{fmaf(s, n.x, p.x), fmaf(s, n.y, p.y), fmaf(s, n.z, p.z)};
}

struct TexLookup {
  int i00, i10, i01, i11;  // texel indices
  float fx, fy;
};

__device__ __forceinline__ TexLookup tex_locate(const SurfJob& S, const V3& p) {
  const float inv = 0.5f / S.plane_half;
  const float u = (p.x + S.plane_half) * inv, v = (p.z + S.plane_half) * inv;
  const float px = fmaf(u, (float)S.tex_w, -0.5f), py = fmaf(v, (float)S.tex_h, -0.5f);
  const float flx = floorf(px), fly = floorf(py);
  TexLookup l;
  l.fx = px - flx;
  l.fy = py - fly;
  int x0 = (int)fminf(fmaxf(flx, -1.0f), (float)S.tex_w) % S.tex_w;
  int y0 = (int)fminf(fmaxf(fly, -1.0f), (float)S.tex_h) % S.tex_h;
  if (x0 < 0) x0 += S.tex_w;
  if (y0 < 0) y0 += S.tex_h;
  const int x1 = x0 + 1 == S.tex_w ? 0 : x0 + 1;
  const int y1 = y0 + 1 == S.tex_h ? 0 : y0 + 1;
  l.i00 = y0 * S.tex_w + x0;
  l.i10 = y0 * S.tex_w + x1;
  l.i01 = y1 * S.tex_w + x0;
  l.i11 = y1 * S.tex_w + x1;
  return l;
}

// Bilinear RGB of one state (0 = old, 1 = new), repeat wrap.
__device__ __forceinline__ V3 tex_eval(const SurfJob& S, const TexLookup& l, int state) {
  const float4 a = __ldg(S.tex + l.i00 * 2 + state), b = __ldg(S.tex + l.i10 * 2 + state);
  const float4 c = __ldg(S.tex + l.i01 * 2 + state), d = __ldg(S.tex + l.i11 * 2 + state);
  const V3 lo = lerp3(a, b, l.fx), hi = lerp3(c, d, l.fx);
  return V3{lerpf(lo.x, hi.x, l.fy), lerpf(lo.y, hi.y, l.fy), lerpf(lo.z, hi.z, l.fy)};
}

__device__ __forceinline__ void tex_scatter(const SurfJob& S, const TexLookup& l, const V3& g) {
  const float gx = 1.0f - l.fx, gy = 1.0f - l.fy;
  const float w00 = gx * gy, w10 = l.fx * gy, w01 = gx * l.fy, w11 = l.fx * l.fy;
  red_add_v4(S.grad_tex + l.i00, g.x * w00, g.y * w00, g.z * w00, 0.0f);
  red_add_v4(S.grad_tex + l.i10, g.x * w10, g.y * w10, g.z * w10, 0.0f);
  red_add_v4(S.grad_tex + l.i01, g.x * w01, g.y * w01, g.z * w01, 0.0f);
  red_add_v4(S.grad_tex + l.i11, g.x * w11, g.y * w11, g.z * w11, 0.0f);
}

// Forward mode: bilinear tangent of the texture (grad_tex holds it).
__device__ __forceinline__ V3 tex_tangent(const SurfJob& S, const TexLookup& l) {
  const float4 a = __ldg(S.grad_tex + l.i00), b = __ldg(S.grad_tex + l.i10);
  const float4 c = __ldg(S.grad_tex + l.i01), d = __ldg(S.grad_tex + l.i11);
  const V3 lo = lerp3(a, b, l.fx), hi = lerp3(c, d, l.fx);
  return V3{lerpf(lo.x, hi.x, l.fy), lerpf(lo.y, hi.y, l.fy), lerpf(lo.z, hi.z, l.fy)};
}

__device__ __forceinline__ float mis_power(float a, float b) {
  const float a2 = a * a, b2 = b * b;
  const float w = a2 / (a2 + b2);
  return isfinite(w) ? w : 0.0f;
}

__device__ __forceinline__ void surf_camera(const SurfJob& S, int px, int py, float u0, float u1,
                                            V3& d) {
  const float nx = ((float)px + u0) * S.inv_w, ny = ((float)py + u1) * S.inv_h;
  const float a = fmaf(2.0f, nx, -1.0f), b = fmaf(-2.0f, ny, 1.0f);
  V3 r;
  r.x = fmaf(b, S.cam_u.x, fmaf(a, S.cam_r.x, S.cam_f.x));
  r.y = fmaf(b, S.cam_u.y, fmaf(a, S.cam_r.y, S.cam_f.y));
  r.z = fmaf(b, S.cam_u.z, fmaf(a, S.cam_r.z, S.cam_f.z));
  const float inv_len = 1.0f / sqrtf(fmaf(r.z, r.z, fmaf(r.y, r.y, r.x * r.x)));
  d = V3{r.x * inv_len, r.y * inv_len, r.z * inv_len};
}

struct SurfCounts {
  uint32_t paths, bounces, shadow_rays, tex_vertices, grad_events;
};

enum SurfPhase { kSIdle = 0, kSStart = 1, kSBounce = 2 };

template <int kMode>
__device__ void trace_surface(const SurfJob& S, const Queue& Q, SurfCounts& cnt) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  // kAdjoint after a tape pass: only the paths on the lost list
  const bool lost_only = kMode == kAdjoint && Q.lost_list != nullptr;
  const int64_t total = lost_only ? (int64_t)*Q.lost_count : Q.total;
  TapeCursor tc{0u, 0u};  // kTape: the warp's tape chunk
  bool lost = false;      // kTape: a vertex of this path did not fit
  int64_t batch_next = 0, batch_end = 0;
  bool queue_empty = false;
  int64_t path = 0;
  int phase = kSIdle, pass = 0;
  Pcg32 rng;
  V3 o, d;
  V3 bo{1, 1, 1}, bn{1, 1, 1}, Lo{0, 0, 0}, Ln{0, 0, 0}, Lrem{0, 0, 0}, Ltot{0, 0, 0}, dL{0, 0, 0};
  float prev_pdf = 1.0f;
  bool prev_delta = true;
  int depth = 0;

  while (true) {
    unsigned need = __ballot_sync(0xffffffffu, phase == kSIdle);
    while (need != 0u && !queue_empty) {
      if (batch_next == batch_end) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(Q.counter, (unsigned long long)Q.batch);
        b = __shfl_sync(0xffffffffu, b, 0);
        if ((int64_t)b >= total) {
          queue_empty = true;
          break;
        }
        batch_next = (int64_t)b;
        batch_end = min((int64_t)b + Q.batch, total);
      }
      const unsigned avail = (unsigned)(batch_end - batch_next);
      const unsigned take = min((unsigned)__popc(need), avail);
      const unsigned rank = (unsigned)__popc(need & lt_mask);
      if (((need >> lane) & 1u) && rank < take) {
        path = lost_only ? (int64_t)Q.lost_list[batch_next + rank] : batch_next + rank;
        phase = kSStart;
        pass = 0;
      }
      batch_next += take;
      need = __ballot_sync(0xffffffffu, phase == kSIdle);
    }
    if (queue_empty && __all_sync(0xffffffffu, phase == kSIdle)) break;
    // kTape: idle lanes stay for the warp-wide tape append below
    if (kMode != kTape && phase == kSIdle) continue;

    const int pix = (int)(path / S.spp);
    bool finished = false;
    bool ev = false;  // kTape: this bounce's texture vertex, recorded below
    V3 ev_p{0.0f, 0.0f, 0.0f}, ev_l{0.0f, 0.0f, 0.0f};
    if (phase == kSStart) {
      seed_lane(rng, S.seed, (uint32_t)path);
      const float u0 = next1d(rng), u1 = next1d(rng);
      surf_camera(S, pix % S.width, pix / S.width, u0, u1, d);
      o = S.cam_o;
      bo = V3{1, 1, 1};
      bn = V3{1, 1, 1};
      Lo = V3{0, 0, 0};
      Ln = V3{0, 0, 0};
      prev_pdf = 1.0f;
      prev_delta = true;
      depth = 0;
      lost = false;
      if (kMode == kAdjoint || kMode == kForward) {
        if (pass == 0) {
          if (kMode == kAdjoint) {
            const float fs = (float)S.spp;
            const float* g = S.grad_img + (int64_t)pix * 3;
            dL = V3{g[0] / fs, g[1] / fs, g[2] / fs};
          } else {
            dL = V3{0.0f, 0.0f, 0.0f};  // forward mode: the path's image derivative
          }
        }
        Lrem = Ltot;
      }
      phase = kSBounce;
    }

    // ------------------------------------------------------------ one bounce
    if (kMode != kTape || phase == kSBounce) {
      ++cnt.bounces;
      float t;
      const int id = intersect(S, o, d, kInf, t);
      if (id == kMiss) {
        finished = true;  // no environment light
      } else {
        const V3 p = advance(o, t, d);
        const V3 n = shape_normal(S, id, p);
        const V3 wi{-d.x, -d.y, -d.z};
        // emission with MIS (plugins/twostatepath.py:282-290)
        if (id == kLight && d.y > 0.0f && !(S.hide_emitters && depth == 0)) {
          float pdf_em = 0.0f;
          if (!prev_delta) {
            const float dist2 = t * t;
            pdf_em = dist2 / (d.y * S.light_area);
          }
          const float mis = mis_power(prev_pdf, pdf_em);
          const V3 cn{(bn.x * mis) * S.light_le.x, (bn.y * mis) * S.light_le.y, (bn.z * mis) * S.light_le.z};
          Ln = V3{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
          if (kMode == kTwoState)
            Lo = V3{Lo.x + (bo.x * mis) * S.light_le.x, Lo.y + (bo.y * mis) * S.light_le.y,
                    Lo.z + (bo.z * mis) * S.light_le.z};
          if (kMode == kAdjoint || kMode == kForward) Lrem = V3{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
        }
        // reflectance of both states at p
        V3 an, ao;
        TexLookup tl;
        if (id == kPlane) {
          tl = tex_locate(S, p);
          an = tex_eval(S, tl, 1);
          if (kMode == kTwoState) ao = tex_eval(S, tl, 0);
          ++cnt.tex_vertices;
        } else if (id == kLight) {
          an = V3{0.0f, 0.0f, 0.0f};
          ao = an;
        } else {
          an = S.sph[id - 1].albedo;
          ao = an;
        }
        const float cos_i = dot3(n, wi);
        const bool active_next = depth + 1 < S.max_depth;
        // adjoint: texture gradient at this vertex (everything after the
        // emission above carries this vertex's reflectance)
        if (kMode == kAdjoint && pass == 1 && id == kPlane && S.grad_tex != nullptr && active_next) {
          const V3 g{(dL.x * Lrem.x) / fmaxf(an.x, 1e-8f), (dL.y * Lrem.y) / fmaxf(an.y, 1e-8f),
                     (dL.z * Lrem.z) / fmaxf(an.z, 1e-8f)};
          tex_scatter(S, tl, g);
          ++cnt.grad_events;
        }
        if (kMode == kTape && id == kPlane && active_next) {
          ev = true;
          ev_p = p;
          ev_l = Ln;  // radiance gathered before the vertex's reflectance acts
          ++cnt.grad_events;
        }
        if (kMode == kForward && pass == 1 && id == kPlane && S.grad_tex != nullptr && active_next) {
          const V3 tt = tex_tangent(S, tl);
          dL = V3{dL.x + Lrem.x * (tt.x / fmaxf(an.x, 1e-8f)), dL.y + Lrem.y * (tt.y / fmaxf(an.y, 1e-8f)),
                  dL.z + Lrem.z * (tt.z / fmaxf(an.z, 1e-8f))};
          ++cnt.grad_events;
        }
        // ----- emitter sampling (plugins/twostatepath.py:294-312)
        const float e0 = next1d(rng), e1 = next1d(rng);
        if (active_next && cos_i > 0.0f) {
          const V3 lp{S.light_c.x + fmaf(2.0f, e0, -1.0f) * S.light_hx, S.light_c.y,
                      S.light_c.z + fmaf(2.0f, e1, -1.0f) * S.light_hz};
          const V3 v{lp.x - p.x, lp.y - p.y, lp.z - p.z};
          const float dist2 = dot3(v, v);
          const float dist = sqrtf(dist2);
          const float inv_dist = 1.0f / dist;
          const V3 wl{v.x * inv_dist, v.y * inv_dist, v.z * inv_dist};
          const float cos_l = wl.y;  // light normal is -y
          const float cos_o = dot3(n, wl);
          if (cos_l > 0.0f && cos_o > 0.0f) {
            const float pdf_l = dist2 / (cos_l * S.light_area);
            const V3 org = offset_origin(p, n, wl);
            ++cnt.shadow_rays;
            if (!occluded(S, org, wl, dist)) {
              const float pdf_b = kInvPi * cos_o;
              const float mis = mis_power(pdf_l, pdf_b);
              const V3 ew{S.light_le.x / pdf_l, S.light_le.y / pdf_l, S.light_le.z / pdf_l};
              const V3 vn{(an.x * kInvPi) * cos_o, (an.y * kInvPi) * cos_o, (an.z * kInvPi) * cos_o};
              const V3 cn{((bn.x * mis) * vn.x) * ew.x, ((bn.y * mis) * vn.y) * ew.y,
                          ((bn.z * mis) * vn.z) * ew.z};
              Ln = V3{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
              if (kMode == kTwoState) {
                const V3 vo{(ao.x * kInvPi) * cos_o, (ao.y * kInvPi) * cos_o, (ao.z * kInvPi) * cos_o};
                Lo = V3{Lo.x + ((bo.x * mis) * vo.x) * ew.x, Lo.y + ((bo.y * mis) * vo.y) * ew.y,
                        Lo.z + ((bo.z * mis) * vo.z) * ew.z};
              }
              if (kMode == kAdjoint || kMode == kForward) Lrem = V3{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
            }
          }
        }
        // ----- BSDF sampling of `new` (plugins/twostatepath.py:316-333)
        pcg_skip1(rng);  // 1D component (diffuse sampling ignores it)
        const float s0 = next1d(rng), s1 = next1d(rng);
        bool alive = active_next && cos_i > 0.0f;
        if (alive) {
          // cosine-weighted hemisphere around n; cos_theta_o = lz exactly
          const float r = sqrtf(s0);
          float sn, cs;
          sincos_2pi(s1, sn, cs);
          const float lz = sqrtf(fmaxf(0.0f, 1.0f - s0));
          V3 ts, tt;
          onb(n, ts, tt);
          const float lx = r * cs, ly = r * sn;
          const V3 wo{fmaf(lz, n.x, fmaf(ly, tt.x, lx * ts.x)), fmaf(lz, n.y, fmaf(ly, tt.y, lx * ts.y)),
                      fmaf(lz, n.z, fmaf(ly, tt.z, lx * ts.z))};
          const float pdf = kInvPi * lz;
          if (pdf > 0.0f) {
            if (kMode == kTwoState) {
              const V3 vold{(ao.x * kInvPi) * lz, (ao.y * kInvPi) * lz, (ao.z * kInvPi) * lz};
              bo = V3{bo.x * (vold.x / pdf), bo.y * (vold.y / pdf), bo.z * (vold.z / pdf)};
            }
            bn = V3{bn.x * an.x, bn.y * an.y, bn.z * an.z};  // diffuse sample weight = reflectance
            prev_pdf = pdf;
            prev_delta = false;
            o = offset_origin(p, n, wo);
            d = wo;
          } else {
            alive = false;
          }
        }
        if (!alive) {
          bn = V3{0, 0, 0};
          bo = V3{0, 0, 0};
        }
        // ----- Russian roulette (plugins/twostatepath.py:343-355)
        const float bmax = fmaxf(fmaxf(bn.x, bn.y), bn.z);
        alive = alive && bmax != 0.0f;
        const float rr_prob = fminf(bmax, 0.95f);
        const float ur = next1d(rng);
        if (depth >= S.rr_depth) {
          const float inv = 1.0f / rr_prob;
          bn = V3{bn.x * inv, bn.y * inv, bn.z * inv};
          bo = V3{bo.x * inv, bo.y * inv, bo.z * inv};
          alive = alive && ur < rr_prob;
        }
        depth += 1;
        finished = !alive;
      }
    }

    if (kMode == kTape) {
      const float4 a = make_float4(ev_p.x, ev_p.z, __uint_as_float((uint32_t)path), 0.0f);
      const float4 b = make_float4(ev_l.x, ev_l.y, ev_l.z, 0.0f);
      if (!tape_append_n<2>(Q, tc, ev && !lost, a, b)) lost = true;
    }

    if (finished) {
      if (kMode == kTape) {
        Q.path_ltot[path] = make_float4(Ln.x, Ln.y, Ln.z, lost ? 1.0f : 0.0f);
        if (lost) Q.lost_list[atomicAdd(Q.lost_count, 1ull)] = (uint32_t)path;
      }
      if ((kMode == kAdjoint || kMode == kForward) && pass == 0) {
        Ltot = Ln;
        pass = 1;
        phase = kSStart;
      } else {
        if (kMode == kForward && (dL.x != 0.0f || dL.y != 0.0f || dL.z != 0.0f)) {
          const float fs = (float)S.spp;
          float* o = S.out_img + (int64_t)pix * 3;
          atomicAdd(o + 0, dL.x / fs);
          atomicAdd(o + 1, dL.y / fs);
          atomicAdd(o + 2, dL.z / fs);
        }
        if (kMode == kTwoState || kMode == kSingle) {
          float4* out = Q.path_out + path * (kMode == kTwoState ? 2 : 1);
          out[0] = make_float4(Ln.x, Ln.y, Ln.z, 0.0f);
          if (kMode == kTwoState) out[1] = make_float4(Lo.x, Lo.y, Lo.z, 0.0f);
        }
        ++cnt.paths;
        phase = kSIdle;
      }
    }
  }
  if (kMode == kTape) tape_close(Q, tc);  // the unused slots of the warp's last chunk
}

}  // namespace rcv
