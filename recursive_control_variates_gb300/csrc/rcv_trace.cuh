// Persistent tracer loop with deferred expensive events.
//
// Every warp pulls batches of path indices from one global counter and hands
// them to idle lanes.  A lane is always in one of these phases:
//   kStart    path (or adjoint replay pass) waiting to be initialised
//   kMain     walking the main path: one free-flight step per iteration
//   kScatter  real scattering event waiting to be processed (albedo lookups,
//             phase and NEE direction sampling, adjoint scatter)
//   kNee      walking the NEE shadow ray (ratio tracking)
//   kNeeAdj   adjoint only: replaying the shadow walk to scatter gradients
// Path starts and scattering events cost 100-200 instructions while a
// free-flight step costs a few dozen; executing them as soon as one lane
// needs them would leave the other 31 lanes waiting in almost every
// iteration.  Lanes that reach one park in kStart / kScatter and the warp runs
// that branch only when at least `defer` lanes wait (or when no lane can walk),
// so the expensive branches run with many lanes and the free-flight step
// stays converged.  The per-path random-number order is unchanged, so results
// do not depend on the schedule.
#pragma once
#include "rcv_volume.cuh"

namespace rcv {

enum PathPhase { kIdle = 0, kStart = 1, kMain = 2, kScatter = 3, kNee = 4, kNeeAdj = 5 };

// Job of a global path index: binary search in the launch's job table.
__device__ __forceinline__ const VolJob& job_of(const VolJob& single, const Queue& Q, int64_t path) {
  if (Q.jobs == nullptr) return single;
  int lo = 0, hi = Q.njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (Q.jobs[mid].path_begin <= path)
      lo = mid;
    else
      hi = mid - 1;
  }
  return Q.jobs[lo];
}

template <int kMode>
__device__ void trace_persistent(const VolJob& single, const Queue& Q, Counts& cnt) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  const float mis = 0.5f;  // power heuristic between two equal 1/(4 pi) pdfs
  const float emit_weight = 1.0f / kInvFourPi;
  const unsigned defer = (unsigned)Q.defer;

  int64_t batch_next = 0, batch_end = 0;
  bool queue_empty = false;
  int64_t path = 0;
  const VolJob* Jp = &single;
  int phase = kIdle;
  int pass = 0;  // adjoint: 0 = radiance pass, 1 = replay pass
  float mu = 0.0f, inv_mu = 0.0f, half_inv_mu = 0.0f;
  int pix = 0;
  uint32_t sid = 0;  // sample index within the job: pixel * spp + sample
  V3 dL{0.0f, 0.0f, 0.0f};

  Pcg32 rng, rng_nee;
  // main path state
  V3 p, d;
  float t_rem = 0.0f;
  V3 bo{1, 1, 1}, bn{1, 1, 1}, Lo{0, 0, 0}, Ln{0, 0, 0};
  V3 Lrem{0, 0, 0}, Ltot{0, 0, 0};
  int depth = 0;
  float sc_n = 0.0f, sc_o = 0.0f;  // sigma_t of both states at a pending scattering event
  // NEE state
  V3 q, w;
  float tr_rem = 0.0f, tro = 1.0f, trn = 1.0f;
  V3 wo_next;
  float s_nee = 0.0f;
  // adjoint: NEE transmittances of the radiance pass, reused by the replay
  // pass (same random numbers, so the same values); the replay then walks
  // each shadow ray once, on the main stream, instead of twice
  constexpr int kTrStore = 16;
  float tr_store[kMode == kAdjoint ? kTrStore : 1];
  int n_store = 0, i_event = 0;
  bool nee_saved_rng = false;  // kNeeAdj draws from rng_nee (after a full walk)

  while (true) {
    // ------------------------------------------- hand new paths to idle lanes
    unsigned need = __ballot_sync(0xffffffffu, phase == kIdle);
    while (need != 0u && !queue_empty) {
      if (batch_next == batch_end) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(Q.counter, (unsigned long long)Q.batch);
        b = __shfl_sync(0xffffffffu, b, 0);
        if ((int64_t)b >= Q.total) {
          queue_empty = true;
          break;
        }
        batch_next = (int64_t)b;
        batch_end = min((int64_t)b + Q.batch, Q.total);
      }
      const unsigned avail = (unsigned)(batch_end - batch_next);
      const unsigned take = min((unsigned)__popc(need), avail);
      const unsigned rank = (unsigned)__popc(need & lt_mask);
      if (((need >> lane) & 1u) && rank < take) {
        path = batch_next + rank;
        phase = kStart;
        pass = 0;
      }
      batch_next += take;
      need = __ballot_sync(0xffffffffu, phase == kIdle);
    }
    const unsigned m_start = __ballot_sync(0xffffffffu, phase == kStart);
    const unsigned m_scat = __ballot_sync(0xffffffffu, phase == kScatter);
    const unsigned m_walk = __ballot_sync(0xffffffffu, phase >= kMain && phase != kScatter);
    if (queue_empty && (m_start | m_scat | m_walk) == 0u) break;
    // Once the queue is empty no new lanes arrive to fill a deferred branch;
    // waiting would only make the warp's last paths take turns.
    const unsigned need_lanes = queue_empty ? 1u : defer;
    const bool run_start =
        (unsigned)__popc(m_start) >= need_lanes || (m_walk == 0u && m_scat == 0u && m_start != 0u);
    const bool run_scat = (unsigned)__popc(m_scat) >= need_lanes || (m_walk == 0u && m_scat != 0u);

    bool finished = false;  // the lane's current path (or pass) ends this iteration

    // ------------------------------------------------------------ path start
    if (run_start && phase == kStart) {
      if (kMode == kAdjoint) {
        if (pass == 0) n_store = 0;
        i_event = 0;
      }
      if (pass == 0) {
        Jp = &job_of(single, Q, path);
        const VolJob& Jn = *Jp;
        const float mu_old = Jn.scale * bits_to_float(__ldg(Jn.maxbits + 0));
        const float mu_new = Jn.scale * bits_to_float(__ldg(Jn.maxbits + 1));
        mu = (kMode == kTwoState) ? fmaxf(mu_old, mu_new) : mu_new;
        inv_mu = 1.0f / mu;
        half_inv_mu = 0.5f * inv_mu;
        // k-th pixel of the job's hand-out order, sample s of that pixel
        const int64_t local = path - Jn.path_begin;
        const uint32_t k = (uint32_t)(local / Jn.spp);
        const uint32_t smp = (uint32_t)(local - (int64_t)k * Jn.spp);
        pix = Jn.pixel_order != nullptr ? (int)__ldg(Jn.pixel_order + k) : (int)k;
        sid = (uint32_t)pix * (uint32_t)Jn.spp + smp;
        if (kMode == kAdjoint) {
          const float* g = Jn.grad_img + (int64_t)pix * 3;
          const float fs = (float)Jn.spp;
          dL = V3{g[0] / fs, g[1] / fs, g[2] / fs};
        }
      }
      const VolJob& J = *Jp;
      seed_lane(rng, J.seed, sid);
      const float u0 = next1d(rng), u1 = next1d(rng);
      V3 o;
      camera_ray(J, pix % J.width, pix / J.width, u0, u1, o, d);
      (void)next1d(rng);  // colour channel for free-flight sampling (grey extinction)
      bo = V3{1, 1, 1};
      bn = V3{1, 1, 1};
      Lo = V3{0, 0, 0};
      Ln = V3{0, 0, 0};
      depth = 0;
      if (kMode == kAdjoint) Lrem = Ltot;
      if (!roulette<kMode>(J, rng, depth, bn, bo)) {
        finished = true;
      } else {
        const V3 inv_d = recip(d);
        float tn, tf;
        slab(o, inv_d, tn, tf);
        if (!(tn <= tf && tf > 0.0f)) {
          // camera ray misses the cube: environment seen directly
          if (!J.hide_emitters) {
            Ln = V3{Ln.x + bn.x, Ln.y + bn.y, Ln.z + bn.z};
            if (kMode == kTwoState) Lo = V3{Lo.x + bo.x, Lo.y + bo.y, Lo.z + bo.z};
          }
          finished = true;
        } else {
          // null BSDF of the cube boundary: its 1D + 2D sample is drawn and discarded
          pcg_skip3(rng);
          p = advance(o, fmaxf(tn, 0.0f), d);
          float a;
          slab(p, inv_d, a, t_rem);
          phase = kMain;
        }
      }
    }

    // ------------------------------------------------- real scattering event
    if (run_scat && phase == kScatter) {
      const VolJob& J = *Jp;
      const Lookup lk = locate(J, p);
      const float st_n = sc_n, st_o = sc_o;
      const V3 an = albedo_at(J, lk, 1);
      const V3 ss_n{st_n * an.x, st_n * an.y, st_n * an.z};
      if (kMode == kTwoState) {
        // plugins/twostatevolpath.py:259-260
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
            const V3 ga{(dL.x * Lrem.x) / fmaxf(an.x, 1e-8f), (dL.y * Lrem.y) / fmaxf(an.y, 1e-8f),
                        (dL.z * Lrem.z) / fmaxf(an.z, 1e-8f)};
            scatter_albedo(J, lk, ga);
          }
        }
      }
      // isotropic phase sample (1D unused + 2D), plugins/twostatevolpath.py:275
      pcg_skip1(rng);
      const float pu0 = next1d(rng), pu1 = next1d(rng);
      wo_next = uniform_sphere(pu0, pu1);
      // NEE towards the environment, then ratio tracking
      const float nu0 = next1d(rng), nu1 = next1d(rng);
      w = uniform_sphere(nu0, nu1);
      q = p;
      {
        float a;
        slab(q, recip(w), a, tr_rem);
      }
      tro = 1.0f;
      trn = 1.0f;
      phase = kNee;
      if (kMode == kAdjoint && pass == 1) {
        if (i_event < n_store) {
          // transmittance known from the radiance pass: add the NEE
          // contribution now and walk the shadow ray once to scatter its
          // gradient, drawing from the main stream as the full walk would
          const float en = emit_weight * tr_store[i_event];
          const V3 cn{((bn.x * kInvFourPi) * mis) * en, ((bn.y * kInvFourPi) * mis) * en,
                      ((bn.z * kInvFourPi) * mis) * en};
          s_nee = (dL.x * cn.x + dL.y * cn.y) + dL.z * cn.z;
          Lrem = V3{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
          nee_saved_rng = false;
          phase = kNeeAdj;
        } else {
          rng_nee = rng;
          nee_saved_rng = true;
        }
        ++i_event;
      }
    }

    // --------------------------------------------------- free-flight step
    if (phase == kMain || phase == kNee || phase == kNeeAdj) {
      const VolJob& J = *Jp;
      bool alive = true;
      V3 org, dir;
      float tmax;
      Pcg32* r = &rng;
      if (phase == kMain) {
        alive = roulette<kMode>(J, rng, depth, bn, bo);
        org = p;
        dir = d;
        tmax = t_rem;
      } else {
        org = q;
        dir = w;
        tmax = tr_rem;
        if (kMode == kAdjoint && phase == kNeeAdj && nee_saved_rng) r = &rng_nee;
      }
      if (!alive) {
        finished = true;
      } else {
        const float t = free_flight(next1d(*r), mu, inv_mu);
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
          if (phase == kMain)
            ++cnt.lookups;
          else
            ++cnt.nee_lookups;
        }
        const float st_o = J.scale * rho_o, st_n = J.scale * rho_n;

        if (phase == kMain) {
          if (valid) {
            const float ur = next1d(rng);
            // real-collision probability: mean of both states' sigma_t / mu
            // (plugins/twostatevolpath.py:222-225); equal states give exactly
            // the single-state sigma_t / mu
            float prob;
            if (kMode == kTwoState)
              prob = (st_n + st_o) * half_inv_mu;
            else
              prob = st_n * inv_mu;
            if (ur >= prob) {
              // null collision (plugins/twostatevolpath.py:227-231, 256-257);
              // the two weights sum to 2, equal states give exactly 1
              if (kMode == kTwoState) {
                const float sn_o = mu - st_o, sn_n = mu - st_n;
                const float den = sn_n + sn_o;
                const float wn = (2.0f * sn_n) / den, wo = 2.0f - wn;
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
              // real scattering event (plugins/twostatevolpath.py:249-253)
              depth += 1;
              if (depth >= J.max_depth) {
                finished = true;
              } else {
                ++cnt.scatters;
                p = x;
                sc_n = st_n;
                sc_o = st_o;
                phase = kScatter;
              }
            }
          } else {
            // leaves the cube: null BSDF sample, outside iteration RR, environment
            pcg_skip3(rng);
            if (roulette<kMode>(J, rng, depth, bn, bo) && !(J.hide_emitters && depth == 0)) {
              const float k = depth == 0 ? 1.0f : mis;
              const V3 cn{bn.x * k, bn.y * k, bn.z * k};
              Ln = V3{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
              if (kMode == kTwoState) Lo = V3{Lo.x + bo.x * k, Lo.y + bo.y * k, Lo.z + bo.z * k};
              if (kMode == kAdjoint) Lrem = V3{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
            }
            finished = true;
          }
        } else if (phase == kNee) {
          bool done = !valid;
          if (valid) {
            // ratio tracking (plugins/twostatevolpath.py:443-452)
            trn = trn * ((mu - st_n) * inv_mu);
            if (kMode == kTwoState) tro = tro * ((mu - st_o) * inv_mu);
            q = x;
            tr_rem = tr_rem - t;
            done = (kMode == kTwoState) ? (trn == 0.0f && tro == 0.0f) : (trn == 0.0f);
          }
          if (done) {
            const float en = emit_weight * trn;
            const V3 cn{((bn.x * kInvFourPi) * mis) * en, ((bn.y * kInvFourPi) * mis) * en,
                        ((bn.z * kInvFourPi) * mis) * en};
            Ln = V3{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
            if (kMode == kTwoState) {
              const float eo = emit_weight * tro;
              Lo = V3{Lo.x + ((bo.x * kInvFourPi) * mis) * eo, Lo.y + ((bo.y * kInvFourPi) * mis) * eo,
                      Lo.z + ((bo.z * kInvFourPi) * mis) * eo};
            }
            if (kMode == kAdjoint && pass == 1) {
              // replay the shadow walk to back-propagate through its transmittance
              s_nee = (dL.x * cn.x + dL.y * cn.y) + dL.z * cn.z;
              Lrem = V3{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
              q = p;
              float a;
              slab(q, recip(w), a, tr_rem);
              trn = 1.0f;
              phase = kNeeAdj;
            } else {
              if (kMode == kAdjoint && n_store < kTrStore) tr_store[n_store++] = trn;
              d = wo_next;
              float a;
              slab(p, recip(d), a, t_rem);
              phase = kMain;
            }
          }
        } else {  // kNeeAdj: second walk with the saved stream
          bool done = !valid;
          if (valid) {
            const float sn = mu - st_n;
            if (sn > 0.0f) {
              scatter_density(J, lk, -(J.scale * s_nee) / sn);
              ++cnt.grad_events;
            }
            trn = trn * (sn * inv_mu);
            q = x;
            tr_rem = tr_rem - t;
            done = trn == 0.0f;
          }
          if (done) {
            d = wo_next;
            float a;
            slab(p, recip(d), a, t_rem);
            phase = kMain;
          }
        }
      }
    }

    // -------------------------------------------------------------- path end
    if (finished) {
      if (kMode == kAdjoint && pass == 0) {
        // radiance pass finished: replay the same path with gradients
        Ltot = Ln;
        pass = 1;
        phase = kStart;
      } else {
        if (kMode != kAdjoint) {
          float4* o = Q.path_out + (Jp->path_begin + sid) * (kMode == kTwoState ? 2 : 1);
          o[0] = make_float4(Ln.x, Ln.y, Ln.z, 0.0f);
          if (kMode == kTwoState) o[1] = make_float4(Lo.x, Lo.y, Lo.z, 0.0f);
        }
        ++cnt.paths;
        phase = kIdle;
      }
    }
  }
}

}  // namespace rcv
