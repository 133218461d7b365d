// Two-state volumetric path tracer, single-state tracer and seed-replay
// adjoint for a heterogeneous medium in the unit cube behind a null boundary,
// lit by a constant white environment (radiance 1).
//
// Restates the per-path algorithm of the reference:
//   plugins/twostatevolpath.py:141-385  sample_twostates (main loop)
//   plugins/twostatevolpath.py:387-479  sample_emitter_twostates (NEE with
//                                       two-state ratio tracking)
//   plugins/twostatemedium.py:15-107    sample_interaction_twostates
// and, for the adjoint, path replay backpropagation (Vicini et al. 2021) of
// the single-state estimator that a two-state integrator renders when its
// medium delegates every query to `new` (plugins/twostatemedium.py:125-151).
//
// Random-number order per path (one PCG32 stream per path):
//   film 2D, channel 1D, [camera iteration: RR 1D; on a cube hit the null
//   BSDF sample 1D + 2D], then per medium iteration: RR 1D, free flight 1D,
//   on a valid collision real/null 1D; on a real scattering event below
//   max_depth: phase 1D + 2D, NEE direction 2D, one 1D per ratio-tracking
//   step.  An escaping path draws the null BSDF sample (1D + 2D) and the RR
//   1D of the outside iteration before the environment is added.
//
// Execution shape: one thread owns `chunk` consecutive samples of a pixel and
// regenerates a new path as soon as one finishes; the main path and its NEE
// shadow walk share one loop body ("one free-flight step per iteration") so
// that warps stay converged on the density lookups, which dominate the cost.
#pragma once
#include "rcv_device.cuh"

namespace rcv {

// Packed lookup cell: 8 corners of the old and the new density, 64 bytes.
//   [0] old v000 v100 v010 v110   [1] old v001 v101 v011 v111
//   [2] new v000 ...              [3] new v001 ...
struct VolJob {
  // film / camera
  int32_t width, height, spp, chunk;  // chunk = samples per thread
  V3 cam_o, cam_f, cam_r, cam_u;
  // integrator
  int32_t max_depth, rr_depth, hide_emitters;
  uint32_t seed;
  // medium
  int32_t dx, dy, dz;
  float scale;
  const float4* __restrict__ cells;   // (dz+1)(dy+1)(dx+1) * 4
  const float4* __restrict__ albedo;  // dz*dy*dx * 2 (old, new) or null
  float albedo_const[3];
  const uint32_t* maxbits;  // [0] max old density, [1] max new density (bits)
  // outputs
  float* out_old;  // two-state: H; single: unused
  float* out_new;  // two-state: F; single: image
  // adjoint
  const float* grad_img;
  float4* grad_cells;   // (dz+1)(dy+1)(dx+1) * 2
  float4* grad_albedo;  // dz*dy*dx (rgb + pad) or null
  unsigned long long* counters;
  int64_t thread_begin;  // first global thread of this job (batched launches)
  int64_t thread_count;  // width*height*(spp/chunk)
};

enum TraceMode { kTwoState = 0, kSingle = 1, kAdjoint = 2 };

struct Counts {
  uint32_t paths, lookups, nee_lookups, scatters;
  uint32_t grad_events, albedo_events;  // adjoint: density / albedo scatters
};

__device__ __forceinline__ float bits_to_float(uint32_t b) { return __uint_as_float(b); }

__device__ __forceinline__ void camera_ray(const VolJob& J, int px, int py, float u0, float u1,
                                           V3& o, V3& d) {
  const float fx = (float)px + u0;
  const float fy = (float)py + u1;
  const float nx = fx / (float)J.width;
  const float ny = fy / (float)J.height;
  const float a = 2.0f * nx - 1.0f;
  const float b = 1.0f - 2.0f * ny;
  V3 r;
  r.x = (J.cam_f.x + a * J.cam_r.x) + b * J.cam_u.x;
  r.y = (J.cam_f.y + a * J.cam_r.y) + b * J.cam_u.y;
  r.z = (J.cam_f.z + a * J.cam_r.z) + b * J.cam_u.z;
  const float len = sqrtf((r.x * r.x + r.y * r.y) + r.z * r.z);
  d = V3{r.x / len, r.y / len, r.z / len};
  o = J.cam_o;
}

struct Lookup {
  Axis ax, ay, az;
  int64_t cell;
};

__device__ __forceinline__ Lookup locate(const VolJob& J, const V3& x) {
  Lookup l;
  l.ax = axis_coord(x.x, J.dx);
  l.ay = axis_coord(x.y, J.dy);
  l.az = axis_coord(x.z, J.dz);
  l.cell = ((int64_t)l.az.cell * (J.dy + 1) + l.ay.cell) * (J.dx + 1) + l.ax.cell;
  return l;
}

__device__ __forceinline__ void density2(const VolJob& J, const Lookup& l, float& rho_old,
                                         float& rho_new) {
  const float4* c = J.cells + l.cell * 4;
  const float4 o0 = __ldg(c + 0), o1 = __ldg(c + 1), n0 = __ldg(c + 2), n1 = __ldg(c + 3);
  rho_old = trilerp(o0, o1, l.ax.f, l.ay.f, l.az.f);
  rho_new = trilerp(n0, n1, l.ax.f, l.ay.f, l.az.f);
}

__device__ __forceinline__ float density_new(const VolJob& J, const Lookup& l) {
  const float4* c = J.cells + l.cell * 4;
  const float4 n0 = __ldg(c + 2), n1 = __ldg(c + 3);
  return trilerp(n0, n1, l.ax.f, l.ay.f, l.az.f);
}

__device__ __forceinline__ int clampi(int v, int hi) { return v < 0 ? 0 : (v > hi ? hi : v); }

// Trilinear RGB albedo of one state (state 0 = old, 1 = new).
__device__ __forceinline__ V3 albedo_at(const VolJob& J, const Lookup& l, int state) {
  if (J.albedo == nullptr) return V3{J.albedo_const[0], J.albedo_const[1], J.albedo_const[2]};
  const int x0 = clampi(l.ax.cell - 1, J.dx - 1), x1 = clampi(l.ax.cell, J.dx - 1);
  const int y0 = clampi(l.ay.cell - 1, J.dy - 1), y1 = clampi(l.ay.cell, J.dy - 1);
  const int z0 = clampi(l.az.cell - 1, J.dz - 1), z1 = clampi(l.az.cell, J.dz - 1);
  auto at = [&](int x, int y, int z) {
    return __ldg(J.albedo + (((int64_t)z * J.dy + y) * J.dx + x) * 2 + state);
  };
  const float4 a000 = at(x0, y0, z0), a100 = at(x1, y0, z0), a010 = at(x0, y1, z0),
               a110 = at(x1, y1, z0), a001 = at(x0, y0, z1), a101 = at(x1, y0, z1),
               a011 = at(x0, y1, z1), a111 = at(x1, y1, z1);
  const float fx = l.ax.f, fy = l.ay.f, fz = l.az.f;
  V3 r;
  {
    const float c00 = lerpf(a000.x, a100.x, fx), c10 = lerpf(a010.x, a110.x, fx);
    const float c01 = lerpf(a001.x, a101.x, fx), c11 = lerpf(a011.x, a111.x, fx);
    r.x = lerpf(lerpf(c00, c10, fy), lerpf(c01, c11, fy), fz);
  }
  {
    const float c00 = lerpf(a000.y, a100.y, fx), c10 = lerpf(a010.y, a110.y, fx);
    const float c01 = lerpf(a001.y, a101.y, fx), c11 = lerpf(a011.y, a111.y, fx);
    r.y = lerpf(lerpf(c00, c10, fy), lerpf(c01, c11, fy), fz);
  }
  {
    const float c00 = lerpf(a000.z, a100.z, fx), c10 = lerpf(a010.z, a110.z, fx);
    const float c01 = lerpf(a001.z, a101.z, fx), c11 = lerpf(a011.z, a111.z, fx);
    r.z = lerpf(lerpf(c00, c10, fy), lerpf(c01, c11, fy), fz);
  }
  return r;
}

// Scatters g * (trilinear weight of each corner) into the cell gradient.
__device__ __forceinline__ void scatter_density(const VolJob& J, const Lookup& l, float g) {
  const float fx = l.ax.f, fy = l.ay.f, fz = l.az.f;
  const float gx0 = 1.0f - fx, gy0 = 1.0f - fy, gz0 = 1.0f - fz;
  const float a = g * gz0, b = g * fz;
  const float a0 = a * gy0, a1 = a * fy, b0 = b * gy0, b1 = b * fy;
  float4* dst = J.grad_cells + l.cell * 2;
  atomicAdd(dst + 0, make_float4(a0 * gx0, a0 * fx, a1 * gx0, a1 * fx));
  atomicAdd(dst + 1, make_float4(b0 * gx0, b0 * fx, b1 * gx0, b1 * fx));
}

__device__ __forceinline__ void scatter_albedo(const VolJob& J, const Lookup& l, const V3& g) {
  const int x0 = clampi(l.ax.cell - 1, J.dx - 1), x1 = clampi(l.ax.cell, J.dx - 1);
  const int y0 = clampi(l.ay.cell - 1, J.dy - 1), y1 = clampi(l.ay.cell, J.dy - 1);
  const int z0 = clampi(l.az.cell - 1, J.dz - 1), z1 = clampi(l.az.cell, J.dz - 1);
  const float fx = l.ax.f, fy = l.ay.f, fz = l.az.f;
  const float wx[2] = {1.0f - fx, fx}, wy[2] = {1.0f - fy, fy}, wz[2] = {1.0f - fz, fz};
  const int xs[2] = {x0, x1}, ys[2] = {y0, y1}, zs[2] = {z0, z1};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int i = k & 1, j = (k >> 1) & 1, m = k >> 2;
    const float w = (wz[m] * wy[j]) * wx[i];
    float4* dst = J.grad_albedo + ((int64_t)zs[m] * J.dy + ys[j]) * J.dx + xs[i];
    atomicAdd(dst, make_float4(g.x * w, g.y * w, g.z * w, 0.0f));
  }
}

// Russian roulette at the top of an iteration (plugins/twostatevolpath.py:182-188).
// Returns false when the path terminates.
template <int kMode>
__device__ __forceinline__ bool roulette(const VolJob& J, Pcg32& rng, int depth, V3& bn, V3& bo) {
  bool alive = (bn.x != 0.0f || bn.y != 0.0f || bn.z != 0.0f);
  if (kMode == kTwoState) alive = alive || (bo.x != 0.0f || bo.y != 0.0f || bo.z != 0.0f);
  if (!alive) return false;
  float m = fmaxf(fmaxf(bn.x, bn.y), bn.z);
  if (kMode == kTwoState) m = fmaxf(fmaxf(fmaxf(bn.x, bo.x), fmaxf(bn.y, bo.y)), fmaxf(bn.z, bo.z));
  const float q = fminf(m, 0.99f);
  const float u = next1d(rng);
  if (depth > J.rr_depth) {
    if (!(u < q)) return false;
    const float inv = 1.0f / q;
    bn = V3{bn.x * inv, bn.y * inv, bn.z * inv};
    if (kMode == kTwoState) bo = V3{bo.x * inv, bo.y * inv, bo.z * inv};
  }
  return true;
}

enum PathPhase { kStart = 0, kMain = 1, kNee = 2, kNeeAdj = 3 };

// Traces samples [s0, s1) of pixel `pix`; adds each path's radiance to
// acc_old / acc_new (in sample order).  In adjoint mode, scatters gradients
// instead and leaves the accumulators untouched.
template <int kMode>
__device__ void trace_samples(const VolJob& J, int pix, int s0, int s1, V3& acc_old, V3& acc_new,
                              Counts& cnt) {
  const float mu_old = J.scale * bits_to_float(__ldg(J.maxbits + 0));
  const float mu_new = J.scale * bits_to_float(__ldg(J.maxbits + 1));
  const float mu = (kMode == kTwoState) ? fmaxf(mu_old, mu_new) : mu_new;
  const int px = pix % J.width, py = pix / J.width;
  const float mis = 0.5f;  // power heuristic between two equal 1/(4 pi) pdfs
  const float emit_weight = 1.0f / kInvFourPi;

  V3 dL{0.0f, 0.0f, 0.0f};
  if (kMode == kAdjoint) {
    const float* g = J.grad_img + (int64_t)pix * 3;
    const float inv = (float)J.spp;
    dL = V3{g[0] / inv, g[1] / inv, g[2] / inv};
  }

  Pcg32 rng, rng_nee;
  int s = s0;
  int phase = kStart;
  int pass = 0;  // adjoint: 0 = radiance pass, 1 = replay pass
  // main path state
  V3 p, d, inv_d;
  float t_rem = 0.0f;
  V3 bo{1, 1, 1}, bn{1, 1, 1}, Lo{0, 0, 0}, Ln{0, 0, 0};
  V3 Lrem{0, 0, 0}, Ltot{0, 0, 0};
  int depth = 0;
  // NEE state
  V3 q, w;
  float tr_rem = 0.0f, tro = 1.0f, trn = 1.0f;
  V3 wo_next;
  float s_nee = 0.0f;

  while (s < s1) {
    if (phase == kStart) {
      seed_lane(rng, J.seed, (uint32_t)((int64_t)pix * J.spp + s));
      const float u0 = next1d(rng), u1 = next1d(rng);
      V3 o;
      camera_ray(J, px, py, u0, u1, o, d);
      (void)next1d(rng);  // colour channel for free-flight sampling (grey extinction)
      bo = V3{1, 1, 1};
      bn = V3{1, 1, 1};
      Lo = V3{0, 0, 0};
      Ln = V3{0, 0, 0};
      depth = 0;
      if (kMode == kAdjoint) Lrem = Ltot;
      bool done = !roulette<kMode>(J, rng, depth, bn, bo);
      float tn = 0.0f, tf = -1.0f;
      if (!done) {
        inv_d = recip(d);
        slab(o, inv_d, tn, tf);
        if (!(tn <= tf && tf > 0.0f)) {
          // camera ray misses the cube: environment seen directly
          if (!J.hide_emitters) {
            Ln = V3{Ln.x + bn.x, Ln.y + bn.y, Ln.z + bn.z};
            if (kMode == kTwoState) Lo = V3{Lo.x + bo.x, Lo.y + bo.y, Lo.z + bo.z};
          }
          done = true;
        }
      }
      if (done) {
        goto path_done;
      }
      // null BSDF of the cube boundary: the sample is drawn and discarded
      (void)next1d(rng);
      (void)next1d(rng);
      (void)next1d(rng);
      p = advance(o, fmaxf(tn, 0.0f), d);
      {
        float a, b;
        slab(p, inv_d, a, b);
        t_rem = b;
      }
      phase = kMain;
    }

    {
      // ------------------------------------------------ one free-flight step
      V3 org, dir;
      float tmax;
      Pcg32* r = &rng;
      if (phase == kMain) {
        if (!roulette<kMode>(J, rng, depth, bn, bo)) goto path_done;
        org = p;
        dir = d;
        tmax = t_rem;
      } else {
        org = q;
        dir = w;
        tmax = tr_rem;
        if (phase == kNeeAdj) r = &rng_nee;
      }
      const float t = free_flight(next1d(*r), mu);
      const bool valid = t <= tmax;
      Lookup lk;
      float rho_o = 0.0f, rho_n = 0.0f;
      V3 x;
      if (valid) {
        x = advance(org, t, dir);
        lk = locate(J, x);
        if (kMode == kTwoState)
          density2(J, lk, rho_o, rho_n);
        else
          rho_n = density_new(J, lk);
        if (phase == kMain) {
          ++cnt.lookups;
        } else {
          ++cnt.nee_lookups;
        }
      }
      const float st_o = J.scale * rho_o, st_n = J.scale * rho_n;

      if (phase == kMain) {
        if (valid) {
          const float ur = next1d(rng);
          float prob;
          if (kMode == kTwoState)
            prob = (st_n / mu + st_o / mu) * 0.5f;
          else
            prob = st_n / mu;
          if (ur >= prob) {
            // null collision (plugins/twostatevolpath.py:227-231, 256-257)
            if (kMode == kTwoState) {
              const float sn_o = mu - st_o, sn_n = mu - st_n;
              const float den = sn_n + sn_o;
              const float wn = (2.0f * sn_n) / den, wo = (2.0f * sn_o) / den;
              bn = V3{bn.x * wn, bn.y * wn, bn.z * wn};
              bo = V3{bo.x * wo, bo.y * wo, bo.z * wo};
            } else if (kMode == kAdjoint && pass == 1) {
              const float sn = mu - st_n;
              const float sd = (dL.x * Lrem.x + dL.y * Lrem.y) + dL.z * Lrem.z;
              scatter_density(J, lk, -(J.scale * sd) / sn);
              ++cnt.grad_events;
            }
            p = x;
            t_rem = t_rem - t;
          } else {
            // real scattering event (plugins/twostatevolpath.py:249-281)
            depth += 1;
            if (depth >= J.max_depth) goto path_done;
            ++cnt.scatters;
            const V3 an = albedo_at(J, lk, 1);
            const V3 ss_n{st_n * an.x, st_n * an.y, st_n * an.z};
            if (kMode == kTwoState) {
              const V3 ao = albedo_at(J, lk, 0);
              const V3 ss_o{st_o * ao.x, st_o * ao.y, st_o * ao.z};
              const float den = st_n + st_o;
              bn = V3{bn.x * ((2.0f * ss_n.x) / den), bn.y * ((2.0f * ss_n.y) / den),
                      bn.z * ((2.0f * ss_n.z) / den)};
              bo = V3{bo.x * ((2.0f * ss_o.x) / den), bo.y * ((2.0f * ss_o.y) / den),
                      bo.z * ((2.0f * ss_o.z) / den)};
            } else {
              bn = V3{bn.x * (ss_n.x / st_n), bn.y * (ss_n.y / st_n), bn.z * (ss_n.z / st_n)};
              if (kMode == kAdjoint && pass == 1) {
                const float sd = (dL.x * Lrem.x + dL.y * Lrem.y) + dL.z * Lrem.z;
                scatter_density(J, lk, (J.scale * sd) / st_n);
                ++cnt.grad_events;
                if (J.grad_albedo != nullptr) {
                  ++cnt.albedo_events;
                  const V3 ga{(dL.x * Lrem.x) / fmaxf(an.x, 1e-8f),
                              (dL.y * Lrem.y) / fmaxf(an.y, 1e-8f),
                              (dL.z * Lrem.z) / fmaxf(an.z, 1e-8f)};
                  scatter_albedo(J, lk, ga);
                }
              }
            }
            // isotropic phase sample (1D unused + 2D)
            (void)next1d(rng);
            const float pu0 = next1d(rng), pu1 = next1d(rng);
            wo_next = uniform_sphere(pu0, pu1);
            // NEE towards the environment, then ratio tracking
            const float nu0 = next1d(rng), nu1 = next1d(rng);
            w = uniform_sphere(nu0, nu1);
            q = x;
            p = x;
            {
              float a, b;
              slab(q, recip(w), a, b);
              tr_rem = b;
            }
            tro = 1.0f;
            trn = 1.0f;
            if (kMode == kAdjoint && pass == 1) rng_nee = rng;
            phase = kNee;
          }
        } else {
          // leaves the cube: null BSDF sample, outside iteration RR, environment
          (void)next1d(rng);
          (void)next1d(rng);
          (void)next1d(rng);
          if (!roulette<kMode>(J, rng, depth, bn, bo)) goto path_done;
          if (!(J.hide_emitters && depth == 0)) {
            const float k = depth == 0 ? 1.0f : mis;
            const V3 cn{bn.x * k, bn.y * k, bn.z * k};
            Ln = V3{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
            if (kMode == kTwoState) Lo = V3{Lo.x + bo.x * k, Lo.y + bo.y * k, Lo.z + bo.z * k};
            if (kMode == kAdjoint) Lrem = V3{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
          }
          goto path_done;
        }
      } else if (phase == kNee) {
        bool finished = !valid;
        if (valid) {
          // ratio tracking (plugins/twostatevolpath.py:443-452)
          trn = trn * ((mu - st_n) / mu);
          if (kMode == kTwoState) tro = tro * ((mu - st_o) / mu);
          q = x;
          tr_rem = tr_rem - t;
          finished = (kMode == kTwoState) ? (trn == 0.0f && tro == 0.0f) : (trn == 0.0f);
        }
        if (finished) {
          const float ev = emit_weight;
          const float en = ev * trn;
          const V3 cn{((bn.x * kInvFourPi) * mis) * en, ((bn.y * kInvFourPi) * mis) * en,
                      ((bn.z * kInvFourPi) * mis) * en};
          Ln = V3{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
          if (kMode == kTwoState) {
            const float eo = ev * tro;
            Lo = V3{Lo.x + ((bo.x * kInvFourPi) * mis) * eo, Lo.y + ((bo.y * kInvFourPi) * mis) * eo,
                    Lo.z + ((bo.z * kInvFourPi) * mis) * eo};
          }
          if (kMode == kAdjoint && pass == 1) {
            // replay the shadow walk to back-propagate through its transmittance
            s_nee = (dL.x * cn.x + dL.y * cn.y) + dL.z * cn.z;
            Lrem = V3{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
            q = p;
            {
              float a, b;
              slab(q, recip(w), a, b);
              tr_rem = b;
            }
            trn = 1.0f;
            phase = kNeeAdj;
          } else {
            d = wo_next;
            inv_d = recip(d);
            {
              float a, b;
              slab(p, inv_d, a, b);
              t_rem = b;
            }
            phase = kMain;
          }
        }
      } else {  // kNeeAdj: second walk with the saved stream
        bool finished = !valid;
        if (valid) {
          const float sn = mu - st_n;
          if (sn > 0.0f) {
            scatter_density(J, lk, -(J.scale * s_nee) / sn);
            ++cnt.grad_events;
          }
          trn = trn * (sn / mu);
          q = x;
          tr_rem = tr_rem - t;
          finished = trn == 0.0f;
        }
        if (finished) {
          d = wo_next;
          inv_d = recip(d);
          {
            float a, b;
            slab(p, inv_d, a, b);
            t_rem = b;
          }
          phase = kMain;
        }
      }
      continue;
    }

  path_done:
    if (kMode == kAdjoint && pass == 0) {
      // radiance pass finished: replay the same path with gradients
      Ltot = Ln;
      pass = 1;
      phase = kStart;
      continue;
    }
    if (kMode != kAdjoint) {
      acc_new = V3{acc_new.x + Ln.x, acc_new.y + Ln.y, acc_new.z + Ln.z};
      if (kMode == kTwoState) acc_old = V3{acc_old.x + Lo.x, acc_old.y + Lo.y, acc_old.z + Lo.z};
    }
    ++cnt.paths;
    pass = 0;
    phase = kStart;
    ++s;
  }
}

}  // namespace rcv
