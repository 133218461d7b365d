// Gradient of the adjoint from the event tape of the kTape radiance pass.
//
// Path replay backpropagation (Vicini et al. 2021) scatters, at every event of
// a path, dL . L_rem times a factor of the event into the grid gradient, with
// L_rem = L - (radiance gathered before the event).  The replay tasks of
// kReplay retrace every segment to find the events again.  The kTape radiance
// pass instead records each event as it happens (its position and a
// reference), and this file turns the tape into the gradient in two flat
// launches, the same arithmetic as the replay event by event
// (plugins/twostatevolpath.py:141-479 for the events; the adjoint
// semantics of Mitsuba's prb_volpath):
//   tape_weights_kernel  per event record and per path, dL . L_rem of every
//                        kind of event that refers to it, once dL is known;
//   tape_scatter_kernel  per tape slot: the event's extinction term that
//                        the radiance pass kept beside it (and at
//                        scattering events the albedo from the medium),
//                        the event's factor, and the gradient scatter:
//                          null collision   -scale * (dL . L_rem) / sigma_n
//                          scattering event  scale * (dL . L_rem) / sigma_t,
//                                            albedo: dL * L_rem / albedo
//                          shadow-walk step -scale * (dL . c_nee) / sigma_n
//                                            (where sigma_n > 0)
// with sigma_n = majorant - sigma_t (the collision's majorant: global or
// the supergrid cell's) and sigma_t of the new state, both as the radiance
// pass computed them.
// Events of a path that lost an event or a record are skipped; kReplay
// replays that path whole.  Batched launches find each event's job through
// its path (binary search in the job table, once per record and path).
#include "rcv_common.h"
#include "rcv_volume.cuh"

namespace rcv {

// Job of a global path index: the single job, or a binary search in the
// launch's job table (batched launches).
__device__ __forceinline__ int tape_job(const VolJob* jobs, int njobs, uint32_t path) {
  if (jobs == nullptr) return 0;
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].path_begin <= (int64_t)path)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Pixel of a path of the job (the hand-out order maps the k-th pixel slot).
__device__ __forceinline__ int tape_pixel(const VolJob& J, uint32_t path) {
  const uint32_t k = (path - (uint32_t)J.path_begin) / (uint32_t)J.spp;
  return J.pixel_order != nullptr ? (int)__ldg(J.pixel_order + k) : (int)k;
}

__device__ __forceinline__ V3 tape_dL(const VolJob& J, int pix) {
  const float* g = J.grad_img + (int64_t)pix * 3;
  const float fs = (float)J.spp;
  return V3{g[0] / fs, g[1] / fs, g[2] / fs};
}

// Record k (2 float4: [path, radiance gathered before the event's NEE
// contribution] [NEE contribution]) -> weights [dL . L_rem after the NEE
// contribution (the next segment), dL . c_nee (the shadow walk), dL . L_rem
// (the event), job] [dL * L_rem per channel (the event's albedo)].  Path p ->
// [dL . L (its camera segment), job].  Job -1: the path is replayed instead
// and its events are skipped.
__global__ void tape_weights_kernel(const __grid_constant__ VolJob single, const VolJob* __restrict__ jobs,
                                    int njobs, const float4* __restrict__ rec,
                                    const unsigned long long* __restrict__ rec_count, int64_t rec_cap,
                                    float4* __restrict__ w, const float4* __restrict__ ltot,
                                    float2* __restrict__ cam_w, int64_t paths) {
  const int64_t nrec = min((int64_t)*rec_count, rec_cap);
  const int64_t n = max(nrec, paths);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    if (i < nrec) {
      const float4 r0 = rec[2 * i], r1 = rec[2 * i + 1];
      const uint32_t path = __float_as_uint(r0.x);
      const float4 lt = ltot[path];
      if (lt.w != 0.0f) {
        w[2 * i] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
      } else {
        const int j = tape_job(jobs, njobs, path);
        const VolJob& J = jobs != nullptr ? jobs[j] : single;
        const V3 g = tape_dL(J, tape_pixel(J, path));
        const V3 lr{lt.x - r0.y, lt.y - r0.z, lt.z - r0.w};
        const V3 ls{lr.x - r1.x, lr.y - r1.y, lr.z - r1.z};
        const float s_event = (g.x * lr.x + g.y * lr.y) + g.z * lr.z;
        const float s_next = (g.x * ls.x + g.y * ls.y) + g.z * ls.z;
        const float s_nee = (g.x * r1.x + g.y * r1.y) + g.z * r1.z;
        w[2 * i] = make_float4(s_next, s_nee, s_event, __int_as_float(j));
        w[2 * i + 1] = make_float4(g.x * lr.x, g.y * lr.y, g.z * lr.z, 0.0f);
      }
    }
    if (i < paths) {
      const float4 lt = ltot[i];
      float2 c = make_float2(0.0f, __int_as_float(-1));
      if (lt.w == 0.0f) {
        const int j = tape_job(jobs, njobs, (uint32_t)i);
        const VolJob& J = jobs != nullptr ? jobs[j] : single;
        const V3 g = tape_dL(J, tape_pixel(J, (uint32_t)i));
        c = make_float2((g.x * lt.x + g.y * lt.y) + g.z * lt.z, __int_as_float(j));
      }
      cam_w[i] = c;
    }
  }
}

template <bool kCount>
__global__ void __launch_bounds__(256) tape_scatter_kernel(const __grid_constant__ VolJob single,
                                                           const VolJob* __restrict__ jobs,
                                                           const float4* __restrict__ tape,
                                                           const unsigned long long* __restrict__ tape_count,
                                                           int64_t tape_cap, const float4* __restrict__ w,
                                                           const float2* __restrict__ cam_w,
                                                           const float* __restrict__ tape_f,
                                                           unsigned long long* counters) {
  const int64_t n = min((int64_t)*tape_count, tape_cap);
  uint32_t ge = 0, ae = 0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float4 ev = __ldcs(tape + i);
    const uint32_t ref = __float_as_uint(ev.w);
    if (ref == kTapeEmpty) continue;
    const uint32_t kind = ref >> 30, idx = ref & kTapeIndexMask;
    float s;
    int j;
    if (kind == kEvCamera) {
      const float2 c = __ldg(cam_w + idx);
      s = c.x;
      j = __float_as_int(c.y);
    } else {
      const float4 wr = __ldg(w + 2 * (int64_t)idx);
      s = kind == kEvSegment ? wr.x : (kind == kEvShadow ? wr.y : wr.z);
      j = __float_as_int(wr.w);
    }
    if (j < 0) continue;
    const VolJob& J = jobs != nullptr ? jobs[j] : single;
    const V3 x{ev.x, ev.y, ev.z};
    const Lookup lk = locate(J, x);
    const float f = __ldcs(tape_f + i);  // sigma_t (scattering event) or sigma_n
    if (kind == kEvScatter) {
      scatter_density(J, lk, (J.scale * s) / f);
      if (kCount) ++ge;
      if (J.grad_albedo != nullptr) {
        const AlbedoLookup alk = albedo_lookup(J, lk, x);
        const V3 an = albedo_at(J, alk, 1);
        const float4 ga = __ldg(w + 2 * (int64_t)idx + 1);
        scatter_albedo(J, alk,
                       V3{ga.x / fmaxf(an.x, 1e-8f), ga.y / fmaxf(an.y, 1e-8f), ga.z / fmaxf(an.z, 1e-8f)});
        if (kCount) ++ae;
      }
    } else {
      const float sn = f;
      if (kind != kEvShadow || sn > 0.0f) {
        scatter_density(J, lk, -(J.scale * s) / sn);
        if (kCount) ++ge;
      }
    }
  }
  if (kCount && counters != nullptr) {
    ge = __reduce_add_sync(0xffffffffu, ge);
    ae = __reduce_add_sync(0xffffffffu, ae);
    if ((threadIdx.x & 31) == 0) {
      if (ge) atomicAdd(counters + RCV_COUNTER_GRAD_EVENTS, (unsigned long long)ge);
      if (ae) atomicAdd(counters + RCV_COUNTER_ALBEDO_EVENTS, (unsigned long long)ae);
    }
  }
}

int launch_tape_gradient(const VolJob& single, const VolJob* jobs, int njobs, const AdjBuffers& A, float4* weights,
                         float2* cam_w, int64_t paths, uint64_t* counters, int sms, cudaStream_t st) {
  const int block = 256;
  tape_weights_kernel<<<grid_for(A.ckpt_cap > paths ? A.ckpt_cap : paths, block), block, 0, st>>>(
      single, jobs, njobs, A.ckpt, A.ckpt_count, A.ckpt_cap, weights, A.path_ltot, cam_w, paths);
  int rc = launched("tape_weights launch");
  if (rc) return rc;
  const unsigned grid = (unsigned)(sms > 0 ? sms : 1) * 8u;
  unsigned long long* c = reinterpret_cast<unsigned long long*>(counters);
  if (counters != nullptr)
    tape_scatter_kernel<true><<<grid, block, 0, st>>>(single, jobs, A.tape, A.tape_count, A.tape_cap, weights,
                                                       cam_w, A.tape_f, c);
  else
    tape_scatter_kernel<false><<<grid, block, 0, st>>>(single, jobs, A.tape, A.tape_count, A.tape_cap, weights,
                                                        cam_w, A.tape_f, c);
  return launched("tape_scatter launch");
}

}  // namespace rcv
