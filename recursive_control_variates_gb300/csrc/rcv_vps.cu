// volpathsimple (plugins/volpathsimple.py): the reference's simplified
// volumetric path tracer and its differential-ratio-tracking adjoint, the
// `adjoint_integrator` of every grid experiment (experiments.py:131,245,364).
//
// Primal (VolpathSimpleIntegrator.sample, :53-327), per loop iteration:
// Russian roulette (1D); a real interaction by delta tracking
// (sample_real_interaction, :349-395: per collision a free-flight 1D and,
// inside the segment, a real/null 1D); NEE towards the environment (2D + one
// 1D per ratio-tracking step, :398-491); the phase sample (1D + 2D).  A path
// that leaves the cube sees the environment with the MIS weight of its last
// scattering event (:296-321).  After reaching the medium, one 1D seeds the
// adjoint's second stream (:103-113).
//
// Adjoint: a primal pass gives L; a replay with L_rem = L - (NEE so far)
// back-propagates
//   - the scattering term at each real interaction, MIS weight s^2/(1+s^2),
//     s = sigma_t (:160-186);
//   - the transmittance of each last segment by 4 uniform samples (:597-620);
//   - each NEE shadow ray by replaying its ratio tracking (:412-422, :481-505);
//   - differential ratio tracking: for every segment (escaping or not) a
//     reservoir keeps one, weighted by the throughput (:743-778); at the end a
//     distance is resampled on it in proportion to the transmittance and a
//     recursive path estimates the in-scattered radiance, MIS 1/(1+s^2)
//     (:508-594, :623-668).  Without subsampling this runs at every segment.
// The extra random numbers come from a second stream seeded with
// sample_tea_32(bits of lane 0's seeding draw, 1) (:108-113).
// sample_interaction_drt belongs to the Mitsuba fork the reference depends
// on; it is restated as a distance from the majorant's exponential truncated
// to the segment, weight = ratio-tracking transmittance / pdf.
//
// One thread per path, sequential: this integrator is the alternative
// adjoint, and its recursive DRT paths do not fit the persistent queue's
// phase machine.  The arithmetic follows the oracle's float sequence.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "rcv_common.h"
#include "rcv_pack.cuh"
#include "rcv_volume.cuh"

namespace rcv {

struct VpsParams {
  int32_t use_nee, use_drt, use_drt_subsampling, use_drt_mis;
  uint32_t alt_seed;   // seed of the adjoint's second stream
  int32_t pad;
  float4* path_out;    // primal: per-path radiance
};

struct VpsSeg {
  V3 o, d;
  float tmax;
};

// kEnv: the job has an environment map (else the constant white environment).
template <bool kEnv>
struct Vps {
  const VolJob& J;
  const VpsParams& P;
  float mu, inv_mu;  // global majorant of `new` (scale * max density) and 1/mu

  __device__ float flight(Pcg32& r, const V3& o, const V3& d, float tmax, float& m) const {
    const float u = next1d(r);
    m = mu;
    if (J.sg[0] > 0) {
      const float tau = -log_unit(1.0f - u);
      return supergrid_flight(J, J.sg_new, o, d, tmax, tau, m);
    }
    return free_flight(u, mu, inv_mu);
  }

  __device__ float sigma_t(const Lookup& l) const { return J.scale * density_new(J, l); }

  __device__ float real_interaction(Pcg32& r, const VpsSeg& seg) const {
    V3 p = seg.o;
    float rem = seg.tmax, t_acc = 0.0f;
    for (;;) {
      float m;
      const float t = flight(r, p, seg.d, rem, m);
      if (!(t <= rem)) return kInf;
      const V3 x = advance(p, t, seg.d);
      const float st = sigma_t(locate(J, x));
      const float ratio = m != 0.0f ? st / m : 0.0f;
      const float u = next1d(r);
      t_acc = t_acc + t;
      if (u < ratio) return t_acc;
      p = x;
      rem = rem - t;
    }
  }

  // Ratio tracking from o along w to tmax; with `adj`, scatters adj . dlog T.
  __device__ float transmittance(Pcg32& r, const V3& o, const V3& w, float tmax, const V3* adj) const {
    V3 q = o;
    float rem = tmax, tr = 1.0f;
    for (;;) {
      float m;
      const float t = flight(r, q, w, rem, m);
      if (!(t <= rem)) break;
      const V3 x = advance(q, t, w);
      const Lookup l = locate(J, x);
      const float sn = m - sigma_t(l);
      const float contrib = m != 0.0f ? sn / m : sn;
      if (adj != nullptr && contrib > 0.0f) {
        const float wn = (adj->x + adj->y) + adj->z;
        scatter_density(J, l, -(J.scale * wn) / sn);
      }
      tr = tr * contrib;
      q = x;
      rem = rem - t;
      if (tr == 0.0f) break;
    }
    return tr;
  }

  __device__ float exit_distance(const V3& o, const V3& d) const {
    float tn, tf;
    slab(o, recip(d), tn, tf);
    return tf;
  }

  // NEE towards the environment (sample_emitter_for_nee, :393-417): the
  // constant one sampled uniformly (MIS 1/2 against the phase function), a
  // map by importance with the power heuristic.
  __device__ V3 nee(Pcg32& r, const V3& x, const V3& thr, const V3* dL) const {
    Pcg32 replay = r;
    const float u0 = next1d(r), u1 = next1d(r);
    V3 w, e{0.0f, 0.0f, 0.0f};
    if (kEnv) {
      V3 Le;
      float pdf;
      w = to_box(J, env_sample(J.env, u0, u1, Le, pdf));
      float k = 0.0f;
      if (pdf > 0.0f && pdf < kInf) k = (kInvFourPi * env_mis(pdf, kInvFourPi)) / pdf;
      e = V3{Le.x * k, Le.y * k, Le.z * k};
    } else {
      w = to_box(J, uniform_sphere(u0, u1));
    }
    const float tf = exit_distance(x, w);
    const float tr = transmittance(r, x, w, tf, nullptr);
    V3 c;
    if (kEnv) {
      c = V3{(thr.x * e.x) * tr, (thr.y * e.y) * tr, (thr.z * e.z) * tr};
    } else {
      const float mis = 0.5f;
      const float en = (1.0f / kInvFourPi) * tr;
      c = V3{((thr.x * kInvFourPi) * mis) * en, ((thr.y * kInvFourPi) * mis) * en,
             ((thr.z * kInvFourPi) * mis) * en};
    }
    if (dL != nullptr) {
      const V3 adj{dL->x * c.x, dL->y * c.y, dL->z * c.z};
      pcg_skip1(replay);
      pcg_skip1(replay);
      transmittance(replay, x, w, tf, &adj);
    }
    return c;
  }

  __device__ V3 primal_from(Pcg32& r, VpsSeg seg, int depth, bool has_scattered, bool active) const {
    V3 L{0, 0, 0}, thr{1, 1, 1};
    bool escaped = false;
    while (active) {
      const float q = fminf(fmaxf(fmaxf(thr.x, thr.y), thr.z), 0.99f);
      const bool rr = depth > J.rr_depth;
      const bool alive = thr.x != 0.0f || thr.y != 0.0f || thr.z != 0.0f;
      const float u = next1d(r);
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
      const V3 x = advance(seg.o, t, seg.d);
      const Lookup lx = locate(J, x);
      const V3 a = albedo_at(J, albedo_lookup(J, lx, x), 1);
      has_scattered = true;
      thr = V3{thr.x * a.x, thr.y * a.y, thr.z * a.z};
      depth += 1;
      if (depth >= J.max_depth) break;
      if (P.use_nee) {
        const V3 c = nee(r, x, thr, nullptr);
        L = V3{L.x + c.x, L.y + c.y, L.z + c.z};
      }
      pcg_skip1(r);
      const float pu0 = next1d(r), pu1 = next1d(r);
      seg.o = x;
      seg.d = to_box(J, uniform_sphere(pu0, pu1));
      const float tf = exit_distance(seg.o, seg.d);
      if (!(tf > 0.0f)) break;  // accidental escape (:279-283)
      seg.tmax = tf;
    }
    if (escaped && !(depth <= 0 && J.hide_emitters)) {
      if (kEnv) {
        // map hit: power heuristic against NEE after a scattering event (:280-298)
        float pdf;
        const V3 Le = env_along(seg.d, pdf);
        const float k = (P.use_nee && has_scattered) ? env_mis(kInvFourPi, pdf) : 1.0f;
        L = V3{L.x + (thr.x * Le.x) * k, L.y + (thr.y * Le.y) * k, L.z + (thr.z * Le.z) * k};
      } else {
        const float k = (P.use_nee && has_scattered) ? 0.5f : 1.0f;
        L = V3{L.x + thr.x * k, L.y + thr.y * k, L.z + thr.z * k};
      }
    }
    return L;
  }

  // Radiance of the environment map along a box direction and the pdf of
  // sampling it (the direction made a unit world direction first).
  __device__ V3 env_along(const V3& d, float& pdf) const {
    V3 wd{d.x * J.box.x, d.y * J.box.y, d.z * J.box.z};
    const float inv_len = 1.0f / sqrtf(fmaf(wd.z, wd.z, fmaf(wd.y, wd.y, wd.x * wd.x)));
    wd = V3{wd.x * inv_len, wd.y * inv_len, wd.z * inv_len};
    float u, v, st;
    env_uv(wd, u, v, st);
    pdf = env_pdf(J.env, u, v, st);
    return env_eval_uv(J.env, u, v);
  }

  // Camera ray, colour-channel draw, medium entry (reach_medium, :329-346);
  // `d` is the camera ray (for the environment when it misses the medium).
  __device__ bool camera(Pcg32& r, int pix, VpsSeg& seg, V3& d) const {
    const float u0 = next1d(r), u1 = next1d(r);
    V3 o;
    camera_ray(J, pix % J.width, pix / J.width, u0, u1, o, d);
    pcg_skip1(r);
    const V3 inv_d = recip(d);
    float tn, tf;
    slab(o, inv_d, tn, tf);
    if (!(tn <= tf && tf > 0.0f)) return false;
    seg.o = advance(o, fmaxf(tn, 0.0f), d);
    seg.d = d;
    float a;
    slab(seg.o, inv_d, a, seg.tmax);
    return true;
  }

  __device__ V3 render_path(uint32_t sid, int pix) const {
    Pcg32 r;
    seed_lane(r, J.seed, sid);
    VpsSeg seg;
    V3 d;
    if (!camera(r, pix, seg, d)) {
      if (J.hide_emitters) return V3{0.0f, 0.0f, 0.0f};
      if (kEnv) {
        float pdf;
        return env_along(d, pdf);
      }
      return V3{1.0f, 1.0f, 1.0f};
    }
    pcg_skip1(r);  // seeds the adjoint's second stream
    return primal_from(r, seg, 0, false, true);
  }

  __device__ void drt(Pcg32& alt, const VpsSeg& seg, int depth, const V3& adj) const {
    if (!(mu > 0.0f)) return;
    const float e = exp_nonpos(-(mu * seg.tmax));
    const float u = next1d(alt);
    const float tp = -log_unit(1.0f - u * (1.0f - e)) / mu;
    const float pdf = (mu * exp_nonpos(-(mu * tp))) / (1.0f - e);
    const float tr = transmittance(alt, seg.o, seg.d, tp, nullptr);
    const float wdrt = tr / pdf;
    const V3 x = advance(seg.o, tp, seg.d);
    const Lookup l = locate(J, x);
    const AlbedoLookup al = albedo_lookup(J, l, x);
    const float st = sigma_t(l);
    const V3 a = albedo_at(J, al, 1);
    V3 Li{0, 0, 0};
    if (P.use_nee) Li = nee(alt, x, V3{1, 1, 1}, nullptr);
    pcg_skip1(alt);
    const float pu0 = next1d(alt), pu1 = next1d(alt);
    VpsSeg next{x, to_box(J, uniform_sphere(pu0, pu1)), 0.0f};
    const float tf = exit_distance(next.o, next.d);
    const bool ok = tf > 0.0f;
    next.tmax = tf;
    const int next_depth = depth + 1;
    const bool active = ok && next_depth < J.max_depth;
    if (active) pcg_skip1(alt);  // the recursive call's seeding draw (:103)
    const V3 Lr = primal_from(alt, next, next_depth, true, active);
    Li = V3{Li.x + Lr.x, Li.y + Lr.y, Li.z + Lr.z};
    const float mis = P.use_drt_mis ? 1.0f / (1.0f + st * st) : 1.0f;
    const float k0 = mis * wdrt;
    const V3 k{(k0 * adj.x) * Li.x, (k0 * adj.y) * Li.y, (k0 * adj.z) * Li.z};
    scatter_density(J, l, J.scale * ((k.x * a.x + k.y * a.y) + k.z * a.z));
    if (J.grad_albedo != nullptr) scatter_albedo(J, al, V3{k.x * st, k.y * st, k.z * st});
  }

  __device__ void backward_path(uint32_t sid, int pix, const V3& dL) const {
    const V3 Ltot = render_path(sid, pix);
    Pcg32 r, alt;
    seed_lane(r, J.seed, sid);
    seed_lane(alt, P.alt_seed, sid);
    VpsSeg seg;
    V3 d;
    if (!camera(r, pix, seg, d)) return;
    pcg_skip1(r);
    V3 res = Ltot, thr{1, 1, 1};
    int depth = 0;
    V3 wsum{0, 0, 0}, cur{0, 0, 0};
    bool have = false;
    VpsSeg keep{};
    int keep_depth = 0;
    for (;;) {
      const float q = fminf(fmaxf(fmaxf(thr.x, thr.y), thr.z), 0.99f);
      const bool rr = depth > J.rr_depth;
      const bool alive = thr.x != 0.0f || thr.y != 0.0f || thr.z != 0.0f;
      const float u = next1d(r);
      if (!alive || (rr && !(u < q))) break;
      if (rr) {
        const float iq = 1.0f / q;
        thr = V3{thr.x * iq, thr.y * iq, thr.z * iq};
      }
      const float t = real_interaction(r, seg);
      const bool escape = !(t < kInf);
      if (P.use_drt) {
        if (P.use_drt_subsampling) {
          wsum = V3{wsum.x + thr.x, wsum.y + thr.y, wsum.z + thr.z};
          const float pick = next1d(alt);
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
        const V3 x = advance(seg.o, t, seg.d);
        const Lookup l = locate(J, x);
        const AlbedoLookup al = albedo_lookup(J, l, x);
        const float st = sigma_t(l);
        const V3 a = albedo_at(J, al, 1);
        if (!P.use_drt || P.use_drt_mis) {
          const float mis = P.use_drt ? (st * st) / (1.0f + st * st) : 1.0f;
          const float inv_pdf = 1.0f / st;
          const V3 k{((mis * dL.x) * (res.x / fmaxf(1e-8f, a.x))) * inv_pdf,
                     ((mis * dL.y) * (res.y / fmaxf(1e-8f, a.y))) * inv_pdf,
                     ((mis * dL.z) * (res.z / fmaxf(1e-8f, a.z))) * inv_pdf};
          scatter_density(J, l, J.scale * ((k.x * a.x + k.y * a.y) + k.z * a.z));
          if (J.grad_albedo != nullptr) scatter_albedo(J, al, V3{k.x * st, k.y * st, k.z * st});
        }
      }
      {
        const float interval = escape ? seg.tmax : t;
        const float w = (dL.x * res.x + dL.y * res.y) + dL.z * res.z;
        const float coef = -(w * (interval * 0.25f));
        for (int j = 0; j < 4; ++j) {
          const float tj = next1d(alt) * interval;
          scatter_density(J, locate(J, advance(seg.o, tj, seg.d)), J.scale * coef);
        }
      }
      if (escape) break;
      const V3 x = advance(seg.o, t, seg.d);
      const Lookup lx = locate(J, x);
      const V3 a = albedo_at(J, albedo_lookup(J, lx, x), 1);
      thr = V3{thr.x * a.x, thr.y * a.y, thr.z * a.z};
      depth += 1;
      if (depth >= J.max_depth) break;
      if (P.use_nee) {
        const V3 c = nee(r, x, thr, &dL);
        res = V3{res.x - c.x, res.y - c.y, res.z - c.z};
      }
      pcg_skip1(r);
      const float pu0 = next1d(r), pu1 = next1d(r);
      seg.o = x;
      seg.d = to_box(J, uniform_sphere(pu0, pu1));
      const float tf = exit_distance(seg.o, seg.d);
      if (!(tf > 0.0f)) break;
      seg.tmax = tf;
    }
    if (P.use_drt && P.use_drt_subsampling && have) {
      const float dmean = ((cur.x + cur.y) + cur.z) / 3.0f;
      if (dmean != 0.0f) {
        const float wmean = ((wsum.x + wsum.y) + wsum.z) / 3.0f;
        const V3 sw{(wmean * cur.x) / dmean, (wmean * cur.y) / dmean, (wmean * cur.z) / dmean};
        drt(alt, keep, keep_depth, V3{sw.x * dL.x, sw.y * dL.y, sw.z * dL.z});
      }
    }
  }
};

template <bool kAdj, bool kEnv>
__global__ void __launch_bounds__(128) vps_kernel(const __grid_constant__ VolJob J,
                                                  const __grid_constant__ VpsParams P) {
  const float mu = J.scale * bits_to_float(__ldg(J.maxbits + 1));
  const Vps<kEnv> v{J, P, mu, 1.0f / mu};
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t path = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; path < J.path_count; path += stride) {
    const int pix = (int)(path / J.spp);
    const uint32_t sid = (uint32_t)path;  // pixel * spp + sample
    if (kAdj) {
      const float* g = J.grad_img + (int64_t)pix * 3;
      const float fs = (float)J.spp;
      v.backward_path(sid, pix, V3{g[0] / fs, g[1] / fs, g[2] / fs});
    } else {
      const V3 L = v.render_path(sid, pix);
      P.path_out[path] = make_float4(L.x, L.y, L.z, 0.0f);
    }
  }
}

// sample_tea_32(bits of lane 0's fourth draw, 1)[0] (:108-113).
static uint32_t vps_alt_seed(uint32_t seed) {
  Pcg32 r;
  seed_lane(r, seed, 0u);
  next1d(r);
  next1d(r);
  next1d(r);
  const float u = next1d(r);
  uint32_t bits;
  std::memcpy(&bits, &u, 4);
  uint32_t a, b;
  tea(bits, 1u, 4, a, b);
  return a;
}

static int vps_setup(const rcv_medium* m, const rcv_sensor* s, const rcv_volpath_options* o,
                     const rcv_volpathsimple_flags* f, uint32_t seed, int spp, VolJob* J, VpsParams* P) {
  int rc = make_volume_job(m, s, o, seed, spp, J);
  if (rc) return rc;
  std::memset(P, 0, sizeof(*P));
  const rcv_volpathsimple_flags def{1, 1, 1, 1};
  const rcv_volpathsimple_flags& F = f ? *f : def;
  P->use_nee = F.use_nee != 0;
  P->use_drt = F.use_drt != 0;
  P->use_drt_subsampling = F.use_drt_subsampling != 0;
  P->use_drt_mis = F.use_drt_mis != 0;
  P->alt_seed = vps_alt_seed(seed);
  return RCV_OK;
}

// Grid-stride launch: at most 16 blocks of 128 threads per SM.
static unsigned vps_grid(int64_t paths) {
  static std::once_flag once;
  static int sms = 1;
  std::call_once(once, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
  });
  int64_t blocks = (paths + 127) / 128;
  if (blocks > int64_t(sms) * 16) blocks = int64_t(sms) * 16;
  return (unsigned)(blocks < 1 ? 1 : blocks);
}

}  // namespace rcv

using namespace rcv;

extern "C" uint64_t rcv_volpathsimple_workspace_bytes(int32_t width, int32_t height, int32_t spp) {
  if (width <= 0 || height <= 0 || spp <= 0) return 0;
  return align256(uint64_t(width) * height * spp * 16u);
}

extern "C" int rcv_render_volpathsimple(const rcv_medium* m, const rcv_sensor* s, const rcv_volpath_options* o,
                                        const rcv_volpathsimple_flags* f, uint32_t seed, int32_t spp, float* img,
                                        void* workspace, void* stream) {
  RCV_REQUIRE(img != nullptr && workspace != nullptr, "image / workspace are NULL");
  RCV_REQUIRE((reinterpret_cast<uintptr_t>(workspace) & 255u) == 0, "workspace must be 256-byte aligned");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  VolJob J;
  VpsParams P;
  int rc = vps_setup(m, s, o, f, seed, spp, &J, &P);
  if (rc) return rc;
  P.path_out = static_cast<float4*>(workspace);
  if (J.env.valid)
    vps_kernel<false, true><<<vps_grid(J.path_count), 128, 0, st>>>(J, P);
  else
    vps_kernel<false, false><<<vps_grid(J.path_count), 128, 0, st>>>(J, P);
  rc = launched("volpathsimple launch");
  if (rc) return rc;
  return launch_reduce(false, P.path_out, 0, int64_t(J.width) * J.height, J.spp, img, nullptr, st);
}

extern "C" int rcv_render_backward_volpathsimple(const rcv_medium* m, const rcv_sensor* s,
                                                 const rcv_volpath_options* o, const rcv_volpathsimple_flags* f,
                                                 uint32_t seed, int32_t spp, const float* grad_img,
                                                 float* grad_density, float* grad_albedo, void* stream) {
  RCV_REQUIRE(grad_img != nullptr && grad_density != nullptr, "gradient buffers are NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  VolJob J;
  VpsParams P;
  int rc = vps_setup(m, s, o, f, seed, spp, &J, &P);
  if (rc) return rc;
  const bool want_albedo = grad_albedo != nullptr && m->albedo_old != nullptr;
  rc = reset_gradients(m, want_albedo, st);
  if (rc) return rc;
  if (!want_albedo) J.grad_albedo = nullptr;
  J.grad_img = grad_img;
  if (J.env.valid)
    vps_kernel<true, true><<<vps_grid(J.path_count), 128, 0, st>>>(J, P);
  else
    vps_kernel<true, false><<<vps_grid(J.path_count), 128, 0, st>>>(J, P);
  rc = launched("volpathsimple adjoint launch");
  if (rc) return rc;
  return launch_fold(m, grad_density, want_albedo ? grad_albedo : nullptr, st);
}
