// Persistent tracer loop with deferred expensive events.
//
// Every warp pulls batches of path indices from one global counter and hands
// them to idle lanes.  A lane is always in one of these phases:
//   kStart    path (or adjoint replay pass) waiting to be initialised
//   kMain     walking the main path: one free-flight step per iteration
//   kScatter  real scattering event waiting to be processed (albedo lookups,
//             phase and NEE direction sampling, adjoint scatter)
//   kNee      walking the NEE shadow ray (ratio tracking)
//   kNeeAdj   adjoint replay only: walking the shadow ray again to scatter
//             its gradients
// Path starts and scattering events cost 100-200 instructions while a
// free-flight step costs a few dozen; executing them as soon as one lane
// needs them would leave the other 31 lanes waiting in almost every
// iteration.  Lanes that reach one park in kStart / kScatter and the warp runs
// that branch only when at least `defer` lanes wait (or when no lane can walk),
// so the expensive branches run with many lanes and the free-flight step
// stays converged.  The per-path random-number order is unchanged, so results
// do not depend on the schedule.
//
// Adjoint (path replay backpropagation, Vicini et al. 2021) in two launches.
// The gradient of an event is dL . L_rem times a factor of the event, where
// L_rem = L - (radiance gathered before the event) is only known once the
// path has ended.
//   kAdjoint  radiance pass: traces the path on `new`, stores its total
//             radiance L and, at every real scattering event, a 64-byte
//             checkpoint (random-number state, position, depth, throughput,
//             radiance so far, NEE contribution).
//   kReplay   a queue of replay tasks: the segment of every path from the
//             camera to its first scattering event, then one task per
//             checkpoint (that scattering event, its NEE shadow ray and the
//             segment to the next event).  Each task replays its segment with
//             the same random numbers and scatters the gradients; a task
//             stops at the next scattering event, which has its own task.
// A path whose checkpoints did not fit is replayed whole by its camera task.
//   kForward  the same replay tasks for forward-mode derivatives: at each
//             event where kReplay scatters dL . L_rem times a factor into the
//             grid gradient, it adds L_rem times the factor applied to the
//             tangent field to the task's image derivative, which goes to its
//             pixel at the end of the task.
// Replaying segments instead of whole paths keeps every task short, so the
// launch does not end on a few paths that scatter dozens of times.
//   kTape     the radiance pass without checkpoints: it records every
//             gradient event of the path (main-walk null collisions, real
//             scattering events, shadow-walk steps) on a tape, as its
//             position and a reference to the path or to the record of its
//             scattering event (radiance gathered before it, NEE
//             contribution).  The gradient is then one flat pass over the
//             tape (rcv_tape.cu), which recomputes each event's factor from
//             the medium; paths whose events did not fit are replayed whole
//             by kReplay over the lost list.
#pragma once
#include "rcv_volume.cuh"

namespace rcv {

enum PathPhase { kIdle = 0, kStart = 1, kMain = 2, kScatter = 3, kNee = 4, kNeeAdj = 5 };

// Replay task kinds.
enum TaskKind { kTaskSegment = 0, kTaskWhole = 1, kTaskCheckpoint = 2 };

// Checkpoint record (4 float4): [path, depth, rng.state lo, hi] [p, bn.x]
// [bn.y, bn.z, Lacc.x, Lacc.y] [Lacc.z, cn]; Lacc = radiance gathered before
// the event's NEE contribution cn.
__device__ __forceinline__ void write_checkpoint(float4* rec, uint32_t path, int depth, uint64_t state,
                                                 const V3& p, const V3& bn, const V3& lacc, const V3& cn) {
  rec[0] = make_float4(__uint_as_float(path), __int_as_float(depth), __uint_as_float((uint32_t)state),
                       __uint_as_float((uint32_t)(state >> 32)));
  rec[1] = make_float4(p.x, p.y, p.z, bn.x);
  rec[2] = make_float4(bn.y, bn.z, lacc.x, lacc.y);
  rec[3] = make_float4(lacc.z, cn.x, cn.y, cn.z);
}

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

// Warps per tracer block (the cooperative walk keeps 3 x 32 floats per warp in
// shared memory).
constexpr int kTraceWarps = 4;
constexpr int kTraceBlock = 32 * kTraceWarps;

// Cooperative walk of a warp's last paths.
//
// Once the path queue is empty a warp runs until its longest path ends, and
// that path's free-flight steps form one chain of dependent lookups: at full
// size the last paths of a launch (up to 64 scattering events, each with a
// shadow walk) keep a few warps busy for 40 % of the launch time.  A run of
// null collisions of the main walk, or of ratio-tracking steps of the shadow
// walk, needs no result of one step to place the next except the position,
// and the random numbers of step k are at a known offset in the path's stream
// (3 draws per main step below the roulette depth: roulette, distance,
// real/null; 1 per shadow step).  So a group of G lanes evaluates the next G
// steps of one walking path at once: lane k jumps the stream to step k, takes
// its distance, and looks the densities up at its tentative point, assuming
// all earlier steps of the group were null (main) or did not end the shadow
// walk.  The first step that is something else (a real collision, leaving the
// segment, a zero throughput or transmittance) ends the run; the owner lane
// takes the steps before it, and the regular step code then executes that
// step itself.  Positions, remaining distances, null-collision weights and
// transmittances are accumulated in step order with the operations of the
// regular step, so a path gives the same bits whether it walks alone or with
// helpers.  `m` holds the walking lanes (at most 8: G = 32 / 16 / 8 / 4 for
// 1 / 2 / 3-4 / 5-8 paths); `org`, `dir`, `tmax` are the walk's ray and
// remaining distance, `c1`, `c2` its throughputs (main: bn, bo) or
// transmittances (shadow: trn, tro in .x); `s_t`, `s_w1`, `s_w2` are the
// warp's 32-float shared arrays for the steps' distances and weights.
// Returns the number of steps the calling lane's path took (0 for lanes that
// own no walking path).  kTape: every step taken is a gradient event, which
// the lane that evaluated it appends to the tape with the owner's reference
// `ref`; `lost` is set on an owner whose events did not fit.
template <int kMode>
__device__ __forceinline__ int coop_walk(unsigned m, bool main_walk, const VolJob* Jp, Pcg32& rng, float mu,
                                         float inv_mu, float half_inv_mu, V3& org, const V3& dir, float& tmax,
                                         V3& c1, V3& c2, float* s_t, float* s_w1, float* s_w2, const Queue& Q,
                                         TapeCursor& tc, uint32_t ref, bool& lost) {
  constexpr unsigned kFull = 0xffffffffu;
  const unsigned lane = threadIdx.x & 31u;
  const int n = __popc(m);
  const int G = n == 1 ? 32 : (n == 2 ? 16 : (n <= 4 ? 8 : 4));
  const int grp = (int)lane / G;
  const int k = (int)lane & (G - 1);
  const int base = grp * G;
  const bool busy = grp < n;
  // owner of this lane's group: the grp-th walking lane (lanes of idle groups
  // read their own registers and touch no memory)
  unsigned mm = m;
  for (int i = 0; i < grp && mm != 0u; ++i) mm &= mm - 1u;
  const int owner = mm != 0u ? __ffs(mm) - 1 : (int)lane;

  const bool g_main = __shfl_sync(kFull, (int)main_walk, owner) != 0;
  const VolJob* J = (const VolJob*)__shfl_sync(kFull, (unsigned long long)Jp, owner);
  Pcg32 r;
  r.state = __shfl_sync(kFull, (unsigned long long)rng.state, owner);
  r.inc = __shfl_sync(kFull, (unsigned long long)rng.inc, owner);
  const float g_mu = __shfl_sync(kFull, mu, owner);
  const float g_inv = __shfl_sync(kFull, inv_mu, owner);
  const float g_hinv = __shfl_sync(kFull, half_inv_mu, owner);
  const V3 dv{__shfl_sync(kFull, dir.x, owner), __shfl_sync(kFull, dir.y, owner), __shfl_sync(kFull, dir.z, owner)};
  float px = __shfl_sync(kFull, org.x, owner), py = __shfl_sync(kFull, org.y, owner);
  float pz = __shfl_sync(kFull, org.z, owner), tr = __shfl_sync(kFull, tmax, owner);

  // this lane's step: its draws, distance and real/null variable
  r.state = pcg_jump(r.state, r.inc, (g_main ? 3u : 1u) * (uint32_t)k);
  if (g_main) pcg_skip1(r);  // roulette draw, unused below the roulette depth
  const float t = free_flight(next1d(r), g_mu, g_inv);
  const float ur = g_main ? next1d(r) : 0.0f;
  s_t[lane] = t;
  __syncwarp();
  // position and remaining distance before this lane's step, in step order
#pragma unroll 4
  for (int j = 0; j < k; ++j) {
    const float tj = s_t[base + j];
    px = fmaf(tj, dv.x, px);
    py = fmaf(tj, dv.y, py);
    pz = fmaf(tj, dv.z, pz);
    tr = tr - tj;
  }
  const bool valid = busy && t <= tr;
  const V3 x{fmaf(t, dv.x, px), fmaf(t, dv.y, py), fmaf(t, dv.z, pz)};
  float st_o = 0.0f, st_n = 0.0f;
  if (valid) {
    const Lookup lk = locate(*J, x);
    float rho_o = 0.0f, rho_n;
    if (kMode == kTwoState)
      density2(*J, lk, rho_o, rho_n);
    else
      rho_n = density_new(*J, lk);
    st_o = J->scale * rho_o;
    st_n = J->scale * rho_n;
  }
  bool term;
  float w1 = 0.0f, w2 = 0.0f;  // main: null-collision weights (two-state); shadow: transmittance factors
  if (g_main) {
    const float prob = kMode == kTwoState ? (st_n + st_o) * g_hinv : st_n * g_inv;
    term = !(valid && ur >= prob);
    if (kMode == kTwoState) {
      const float sn_o = g_mu - st_o, sn_n = g_mu - st_n;
      w1 = (2.0f * sn_n) / (sn_n + sn_o);
      w2 = 2.0f - w1;
    }
  } else {
    term = !valid;
    w1 = (g_mu - st_n) * g_inv;
    if (kMode == kTwoState) w2 = (g_mu - st_o) * g_inv;
  }
  s_w1[lane] = w1;
  s_w2[lane] = w2;
  const unsigned tb_all = __ballot_sync(kFull, term);
  __syncwarp();

  // the owner takes the steps before the first one that is not a null step
  // (main) or that ends the shadow walk, with its throughputs (main) or
  // transmittances (shadow) multiplied in step order
  const bool own = (m >> lane) & 1u;
  int f = 0, src = (int)lane;
  const int ob = __popc(m & ((1u << lane) - 1u)) * G;
  const unsigned gmask = G == 32 ? kFull : ((1u << G) - 1u);
  if (own) {
    const unsigned tb = (tb_all >> ob) & gmask;
    const int f0 = tb != 0u ? __ffs(tb) - 1 : G;
    f = f0;
    for (int j = 0; j < f0; ++j) {
      const float x1 = s_w1[ob + j], x2 = s_w2[ob + j];
      if (main_walk) {
        // the regular step begins with the roulette's throughput test
        bool alive = c1.x != 0.0f || c1.y != 0.0f || c1.z != 0.0f;
        if (kMode == kTwoState) alive = alive || (c2.x != 0.0f || c2.y != 0.0f || c2.z != 0.0f);
        if (!alive) {
          f = j;
          break;
        }
        if (kMode == kTwoState) {
          c1 = V3{c1.x * x1, c1.y * x1, c1.z * x1};
          c2 = V3{c2.x * x2, c2.y * x2, c2.z * x2};
        }
      } else {
        const float n1 = c1.x * x1, n2 = c2.x * x2;
        const bool done = kMode == kTwoState ? (n1 == 0.0f && n2 == 0.0f) : n1 == 0.0f;
        if (done) {
          f = j;  // the regular step takes this step and ends the walk
          break;
        }
        c1.x = n1;
        if (kMode == kTwoState) c2.x = n2;
      }
    }
    if (f > 0) src = ob + f - 1;
  }
  // state after f steps: position, remaining distance and stream after step
  // f - 1 of the group's lane that took it
  const V3 xs{__shfl_sync(kFull, x.x, src), __shfl_sync(kFull, x.y, src), __shfl_sync(kFull, x.z, src)};
  const float ts = __shfl_sync(kFull, tr - t, src);
  const unsigned long long ss = __shfl_sync(kFull, (unsigned long long)r.state, src);
  if (kMode == kTape) {
    // the group's steps before the first that ends the run are events
    const int fg = __shfl_sync(kFull, f, owner);
    const uint32_t rg = __shfl_sync(kFull, ref, owner);
    // sigma_n of each step (the cooperative walk runs on the global majorant)
    const bool ok = tape_append(Q, tc, busy && k < fg, x, rg, g_mu - st_n);
    const unsigned bad = __ballot_sync(kFull, !ok);
    if (own && ((bad >> ob) & gmask) != 0u) lost = true;
  }
  if (f == 0) return 0;
  org = xs;
  tmax = ts;
  rng.state = ss;
  return f;
}

// dLoss/dL of one path of pixel `pix` (the pixel value is the mean of its
// samples), as the replay uses it.
__device__ __forceinline__ V3 pixel_dL(const VolJob& J, int pix) {
  const float* g = J.grad_img + (int64_t)pix * 3;
  const float fs = (float)J.spp;
  return V3{g[0] / fs, g[1] / fs, g[2] / fs};
}

// Environment map seen along the box direction d (made a unit world
// direction first): radiance, and the pdf of sampling that direction for NEE.
__device__ __forceinline__ V3 env_radiance_dir(const VolJob& J, const V3& d, float& pdf) {
  V3 wd{d.x * J.box.x, d.y * J.box.y, d.z * J.box.z};
  const float inv_len = 1.0f / sqrtf(fmaf(wd.z, wd.z, fmaf(wd.y, wd.y, wd.x * wd.x)));
  wd = V3{wd.x * inv_len, wd.y * inv_len, wd.z * inv_len};
  float u, v, st;
  env_uv(wd, u, v, st);
  pdf = env_pdf(J.env, u, v, st);
  return env_eval_uv(J.env, u, v);
}

// kSG: the launch may contain media with a majorant supergrid.  kCount: the
// launch accumulates the RCV_COUNTER_* event counts (off, the counters cost
// no registers).
// kEnv: the launch's job has an environment map (else the constant white
// environment; the two are separate kernels so that the constant one carries
// none of the map's code).
template <int kMode, bool kSG, bool kCount, bool kEnv>
__device__ void trace_persistent(const VolJob& single, const Queue& Q, Counts& cnt) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  const float mis = 0.5f;  // power heuristic between two equal 1/(4 pi) pdfs
  const float emit_weight = 1.0f / kInvFourPi;
  const unsigned defer = (unsigned)Q.defer;
  // replay tasks, scattering the image gradient (kReplay) or gathering a
  // tangent field (kForward)
  constexpr bool kRep = kMode == kReplay || kMode == kForward;
  // radiance passes of the adjoint (checkpoints or tape)
  constexpr bool kRad = kMode == kAdjoint || kMode == kTape;
  constexpr bool kCoop = kMode == kTwoState || kMode == kSingle || kRad;
  __shared__ float s_coop[kCoop ? kTraceWarps * 96 : 1];  // cooperative walk: distances, weights
  // environment map: each lane's NEE weight e = Le / pdf * phase * MIS of its
  // pending shadow ray, kept here from the scattering event to the end of the
  // walk instead of in registers
  __shared__ float s_env[kEnv ? kTraceWarps * 32 * 3 : 1];
  float* env_e = s_env + (kEnv ? threadIdx.x * 3 : 0);
  // replay: camera tasks [0, paths) (after a tape pass: the paths on the lost
  // list), then the checkpoints that were written
  const int64_t total = !kRep ? Q.total
                              : (Q.lost_list != nullptr ? (int64_t)*Q.lost_count
                                                        : Q.total + min((int64_t)*Q.ckpt_count, Q.ckpt_cap));

  int64_t batch_next = 0, batch_end = 0;
  bool queue_empty = false;
  int64_t path = 0;
  const VolJob* Jp = &single;
  int phase = kIdle;
  float mu = 0.0f, inv_mu = 0.0f;  // half of inv_mu is recomputed where needed (one register less)
  int pix = 0;
  uint32_t sid = 0;  // sample index within the job: pixel * spp + sample
  V3 dL{0.0f, 0.0f, 0.0f};  // kForward: the task's image derivative
  // kReplay: dL . L_rem with dL = dLoss/dL of the pixel; it changes only with
  // L_rem, and dL itself is recomputed from the image gradient at the events
  // that need it per channel (fewer registers live through the walk)
  float s_main = 0.0f;

  Pcg32 rng;
  // whole-path replay: state of the stream of the second shadow walk (its
  // increment is rng.inc)
  uint64_t nee_state = 0;
  // main path state
  V3 p, d;
  float t_rem = 0.0f;
  V3 bo{1, 1, 1}, bn{1, 1, 1}, Lo{0, 0, 0}, Ln{0, 0, 0};
  int depth = 0;
  float sc_n = 0.0f, sc_o = 0.0f;  // sigma_t of both states at a pending scattering event
  // NEE state
  V3 q, w;
  float tr_rem = 0.0f, tro = 1.0f, trn = 1.0f;
  V3 wo_next;
  // adjoint radiance pass: random-number state at the pending scattering event
  uint64_t ck_state = 0;
  bool ck_lost = false;  // a checkpoint (kTape: an event or event record) of this path did not fit
  // kTape: reference of the path's next events (kind << 30 | path or event
  // record), and the warp's tape chunk
  uint32_t tref = 0;
  TapeCursor tc{0u, 0u};
  // replay
  // replay: radiance the path gathers after its current point,
  // L_rem = L - (radiance gathered so far), kept instead of L and the sum so far
  V3 Lrem{0, 0, 0}, cn_task{0, 0, 0};
  uint32_t ck_slot = 0;  // replay checkpoint task: its record (the NEE contribution is re-read there)
  float s_nee = 0.0f;
  int task = kTaskSegment;
  bool own_event = false;  // checkpoint task: its scattering event is still to be processed
  // loop iterations: a path's length is n_iter - iter0 when it ends
  uint32_t n_iter = 0, iter0 = 0;

  while (true) {
    ++n_iter;
    // ------------------------------------------- hand new paths to idle lanes
    unsigned need = __ballot_sync(0xffffffffu, phase == kIdle);
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
        path = batch_next + rank;
        phase = kStart;
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

    bool finished = false;  // the lane's current path (or task) ends this iteration
    // kTape: this iteration's events, appended where the warp has
    // reconverged: a walk step (1: null collision at p, 2: shadow-walk step
    // at q) with its reference and sigma_n, and the scattering event at p
    // processed in this iteration with its sigma_t
    int ev_kind = 0;
    uint32_t ev_ref = 0;
    float ev_f = 0.0f, ev_sf = 0.0f;
    bool ev_scat = false;

    // ------------------------------------------------------------ path start
    if (run_start && phase == kStart) {
      iter0 = n_iter;
      // replay: a checkpoint task resumes at its scattering event
      const bool resume = kRep && Q.lost_list == nullptr && path >= Q.total;
      float4 r0, r1, r2, r3;
      if (resume) {
        ck_slot = (uint32_t)(path - Q.total);
        const float4* rec = Q.ckpt + (path - Q.total) * 4;
        r0 = rec[0];
        r1 = rec[1];
        r2 = rec[2];
        r3 = rec[3];
        path = (int64_t)__float_as_uint(r0.x);
      } else if (kRep && Q.lost_list != nullptr) {
        path = (int64_t)Q.lost_list[path];  // a path the tape could not hold
      }
      Jp = &job_of(single, Q, path);
      const VolJob& J = *Jp;
      const float mu_old = J.scale * bits_to_float(__ldg(J.maxbits + 0));
      const float mu_new = J.scale * bits_to_float(__ldg(J.maxbits + 1));
      mu = (kMode == kTwoState) ? fmaxf(mu_old, mu_new) : mu_new;
      inv_mu = 1.0f / mu;
      // k-th pixel of the job's hand-out order, sample s of that pixel
      // 32-bit index arithmetic: a job has fewer than 2^32 paths
      const uint32_t local = (uint32_t)(path - J.path_begin);
      const uint32_t uspp = (uint32_t)J.spp;
      const uint32_t k = local / uspp;
      const uint32_t smp = local - k * uspp;
      pix = J.pixel_order != nullptr ? (int)__ldg(J.pixel_order + k) : (int)k;
      sid = (uint32_t)pix * (uint32_t)J.spp + smp;
      seed_lane(rng, J.seed, sid);
      bo = V3{1, 1, 1};
      bn = V3{1, 1, 1};
      Lo = V3{0, 0, 0};
      Ln = V3{0, 0, 0};
      depth = 0;
      if (kRad) ck_lost = false;
      if (kMode == kTape) tref = (kEvCamera << 30) | (uint32_t)path;
      if (kRep) {
        if (kMode == kForward) dL = V3{0.0f, 0.0f, 0.0f};
        const float4 lt = Q.path_ltot[path];
        Lrem = V3{lt.x, lt.y, lt.z};
        task = resume ? kTaskCheckpoint : (lt.w != 0.0f ? kTaskWhole : kTaskSegment);
      }
      if (resume) {
        if (task != kTaskCheckpoint || Q.path_ltot[path].w != 0.0f) {
          finished = true;  // the path is replayed whole by its camera task
        } else {
          depth = __float_as_int(r0.y);
          rng.state = (uint64_t)__float_as_uint(r0.z) | ((uint64_t)__float_as_uint(r0.w) << 32);
          p = V3{r1.x, r1.y, r1.z};
          bn = V3{r1.w, r2.x, r2.y};
          Ln = V3{r2.z, r2.w, r3.x};
          Lrem = V3{Lrem.x - Ln.x, Lrem.y - Ln.y, Lrem.z - Ln.z};
          if (kMode == kForward) cn_task = V3{r3.y, r3.z, r3.w};
          sc_n = J.scale * density_new(J, locate(J, p));
          own_event = true;
          phase = kScatter;
        }
      } else {
        const float u0 = next1d(rng), u1 = next1d(rng);
        V3 o;
        const uint32_t py = (uint32_t)pix / (uint32_t)J.width;
        camera_ray(J, (int)((uint32_t)pix - py * (uint32_t)J.width), (int)py, u0, u1, o, d);
        (void)next1d(rng);  // colour channel for free-flight sampling (grey extinction)
        if (!roulette<kMode>(J, rng, depth, bn, bo)) {
          finished = true;
        } else {
          const V3 inv_d = recip(d);
          float tn, tf;
          slab(o, inv_d, tn, tf);
          if (!(tn <= tf && tf > 0.0f)) {
            // camera ray misses the cube: environment seen directly
            if (!J.hide_emitters) {
              if (kEnv) {
                float pdf;
                const V3 Le = env_radiance_dir(J, d, pdf);
                Ln = V3{Ln.x + bn.x * Le.x, Ln.y + bn.y * Le.y, Ln.z + bn.z * Le.z};
                if (kMode == kTwoState) Lo = V3{Lo.x + bo.x * Le.x, Lo.y + bo.y * Le.y, Lo.z + bo.z * Le.z};
              } else {
                Ln = V3{Ln.x + bn.x, Ln.y + bn.y, Ln.z + bn.z};
                if (kMode == kTwoState) Lo = V3{Lo.x + bo.x, Lo.y + bo.y, Lo.z + bo.z};
              }
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
    }

    if (kMode == kReplay && run_start && iter0 == n_iter) {
      const V3 g = pixel_dL(*Jp, pix);  // the task started in this iteration
      s_main = (g.x * Lrem.x + g.y * Lrem.y) + g.z * Lrem.z;
    }

    // ------------------------------------------------- real scattering event
    if (run_scat && phase == kScatter) {
      const VolJob& J = *Jp;
      if (kRep && task == kTaskSegment) {
        finished = true;  // the event has its own checkpoint task
      } else if (kRep && task == kTaskCheckpoint && !own_event) {
        finished = true;
      } else {
        const Lookup lk = locate(J, p);
        const AlbedoLookup alk = albedo_lookup(J, lk, p);
        const float st_n = sc_n, st_o = sc_o;
        const V3 an = albedo_at(J, alk, 1);
        const V3 ss_n{st_n * an.x, st_n * an.y, st_n * an.z};
        if (kMode == kTwoState) {
          // plugins/twostatevolpath.py:259-260
          const V3 ao = albedo_at(J, alk, 0);
          const V3 ss_o{st_o * ao.x, st_o * ao.y, st_o * ao.z};
          // one division: 2 / (st_n + st_o) equals 1 / st_n exactly for equal
          // states, so those keep the single-state weights bit for bit
          const float k2 = 2.0f / (st_n + st_o);
          bn = V3{bn.x * (ss_n.x * k2), bn.y * (ss_n.y * k2), bn.z * (ss_n.z * k2)};
          bo = V3{bo.x * (ss_o.x * k2), bo.y * (ss_o.y * k2), bo.z * (ss_o.z * k2)};
        } else {
          if (kMode == kReplay) {
            // d log(sigma_s) / d density and d log(albedo) / d albedo at the event
            const V3 Lr = Lrem;
            const V3 g = pixel_dL(J, pix);
            const float sd = s_main;  // (g . Lr)
            scatter_density(J, lk, (J.scale * sd) / st_n);
            if (kCount) ++cnt.grad_events;
            if (J.grad_albedo != nullptr) {
              if (kCount) ++cnt.albedo_events;
              const V3 ga{(g.x * Lr.x) / fmaxf(an.x, 1e-8f), (g.y * Lr.y) / fmaxf(an.y, 1e-8f),
                          (g.z * Lr.z) / fmaxf(an.z, 1e-8f)};
              scatter_albedo(J, alk, ga);
            }
          } else if (kMode == kForward) {
            // the same terms applied to the tangent field: L_rem times
            // d log(sigma_s) along the tangent, per channel
            const V3 Lr = Lrem;
            const float f = (J.scale * tangent_density(J, lk)) / st_n;
            dL = V3{dL.x + Lr.x * f, dL.y + Lr.y * f, dL.z + Lr.z * f};
            if (kCount) ++cnt.grad_events;
            if (J.grad_albedo != nullptr) {
              if (kCount) ++cnt.albedo_events;
              const V3 ta = tangent_albedo(J, alk);
              dL = V3{dL.x + Lr.x * (ta.x / fmaxf(an.x, 1e-8f)), dL.y + Lr.y * (ta.y / fmaxf(an.y, 1e-8f)),
                      dL.z + Lr.z * (ta.z / fmaxf(an.z, 1e-8f))};
            }
          }
          // a checkpoint already holds the throughput after the event
          if (!(kRep && task == kTaskCheckpoint)) {
            const float k1 = 1.0f / st_n;
            bn = V3{bn.x * (ss_n.x * k1), bn.y * (ss_n.y * k1), bn.z * (ss_n.z * k1)};
          }
        }
        if (kMode == kAdjoint) ck_state = rng.state;
        if (kMode == kTape && !ck_lost) {
          // the event's record, written when its shadow walk ends; the walk's
          // steps refer to it (a path without one is replayed instead)
          const unsigned long long k = atomicAdd(Q.ckpt_count, 1ull);
          if ((int64_t)k < Q.ckpt_cap) {
            tref = (kEvShadow << 30) | (uint32_t)k;
            ev_scat = true;  // the event itself
            ev_sf = st_n;
          } else {
            ck_lost = true;
            tref = (kEvCamera << 30) | (uint32_t)path;
          }
        }
        // isotropic phase sample (1D unused + 2D), plugins/twostatevolpath.py:275
        pcg_skip1(rng);
        const float pu0 = next1d(rng), pu1 = next1d(rng);
        wo_next = to_box(J, uniform_sphere(pu0, pu1));
        {
          // exit distance of the next segment, needed when the NEE walk
          // ends; computed here, where many lanes run together
          float a;
          slab(p, recip(wo_next), a, t_rem);
        }
        // NEE towards the environment, then ratio tracking
        const float nu0 = next1d(rng), nu1 = next1d(rng);
        if (kEnv) {
          // NEE towards the environment map (plugins/twostatevolpath.py:315-344):
          // importance-sampled direction, power-heuristic weight against the
          // phase function's pdf
          V3 Le;
          float pdf;
          w = to_box(J, env_sample(J.env, nu0, nu1, Le, pdf));
          float k = 0.0f;
          if (pdf > 0.0f && pdf < kInf) k = (kInvFourPi * env_mis(pdf, kInvFourPi)) / pdf;
          env_e[0] = Le.x * k;
          env_e[1] = Le.y * k;
          env_e[2] = Le.z * k;
        } else {
          w = to_box(J, uniform_sphere(nu0, nu1));
        }
        q = p;
        {
          float a;
          slab(q, recip(w), a, tr_rem);
        }
        tro = 1.0f;
        trn = 1.0f;
        phase = kNee;
        if (kRep) {
          if (task == kTaskCheckpoint) {
            // NEE contribution known from the radiance pass: one shadow walk
            // on the main stream scatters its gradient (gathers the tangent)
            V3 cn = cn_task;
            if (kMode == kReplay) {
              const float4 r3 = Q.ckpt[(int64_t)ck_slot * 4 + 3];
              cn = V3{r3.y, r3.z, r3.w};
            }
            Lrem = V3{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
            if (kMode == kReplay) {
              const V3 g = pixel_dL(J, pix);
              s_nee = (g.x * cn.x + g.y * cn.y) + g.z * cn.z;
              s_main = (g.x * Lrem.x + g.y * Lrem.y) + g.z * Lrem.z;
            }
            own_event = false;
            phase = kNeeAdj;
          } else {
            nee_state = rng.state;  // whole-path replay: walk for the transmittance, then again
          }
        }
      }
    }

    // ------------------------- cooperative walk of the last paths (see above)
    if (kCoop && queue_empty) {
      bool elig = false;
      if (!finished) {
        if (phase == kNee) {
          elig = true;
        } else if (phase == kMain) {
          bool alive = bn.x != 0.0f || bn.y != 0.0f || bn.z != 0.0f;
          if (kMode == kTwoState) alive = alive || (bo.x != 0.0f || bo.y != 0.0f || bo.z != 0.0f);
          elig = alive && depth <= Jp->rr_depth;
        }
        if (kSG && elig && Jp->sg[0] > 0) elig = false;
      }
      const unsigned m_coop = __ballot_sync(0xffffffffu, elig);
      const int n_coop = __popc(m_coop);
      if (n_coop >= 1 && n_coop <= 8) {
        const bool mw = phase == kMain;
        V3 org = mw ? p : q;
        const V3 dir = mw ? d : w;
        float tmax = mw ? t_rem : tr_rem;
        V3 c1 = mw ? bn : V3{trn, 0.0f, 0.0f};
        V3 c2 = mw ? bo : V3{tro, 0.0f, 0.0f};
        float* s = s_coop + (threadIdx.x >> 5) * 96;
        const int f = coop_walk<kMode>(m_coop, mw, Jp, rng, mu, inv_mu, 0.5f * inv_mu, org, dir, tmax, c1, c2, s,
                                       s + 32, s + 64, Q, tc, tref, ck_lost);
        if (f > 0) {
          if (mw) {
            p = org;
            t_rem = tmax;
            bn = c1;
            if (kMode == kTwoState) bo = c2;
            if (kCount) cnt.lookups += (unsigned)f;
          } else {
            q = org;
            tr_rem = tmax;
            trn = c1.x;
            if (kMode == kTwoState) tro = c2.x;
            if (kCount) cnt.nee_lookups += (unsigned)f;
          }
          iter0 -= (uint32_t)f;  // the path's cost counts its steps
        }
      }
    }

    // --------------------------------------------------- free-flight step
    if (phase == kMain || phase == kNee || phase == kNeeAdj) {
      const VolJob& J = *Jp;
      bool alive = true;
      V3 org, dir;
      float tmax;
      // whole-path replay: the second shadow walk draws from the saved stream
      // (chosen by value, not through a pointer, which would put both
      // streams in local memory)
      bool nee_stream = false;
      if (phase == kMain) {
        alive = roulette<kMode>(J, rng, depth, bn, bo);
        org = p;
        dir = d;
        tmax = t_rem;
      } else {
        org = q;
        dir = w;
        tmax = tr_rem;
        nee_stream = kRep && phase == kNeeAdj && task == kTaskWhole;
      }
      if (!alive) {
        finished = true;
      } else {
        // majorant of this collision: global, or the supergrid cell it lies in
        float mu_c = mu, inv_c = inv_mu, hinv_c = 0.5f * inv_mu;
        float t;
        if (kSG && J.sg[0] > 0) {
          const float tau = -log_unit(1.0f - (nee_stream ? next1d_state(nee_state, rng.inc) : next1d(rng)));
          t = supergrid_flight(J, kMode == kTwoState ? J.sg_two : J.sg_new, org, dir, tmax, tau, mu_c);
          inv_c = 1.0f / mu_c;
          hinv_c = 0.5f * inv_c;
        } else {
          t = free_flight(nee_stream ? next1d_state(nee_state, rng.inc) : next1d(rng), mu, inv_mu);
        }
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
          if (kCount) {
            if (phase == kMain)
              ++cnt.lookups;
            else
              ++cnt.nee_lookups;
          }
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
              prob = (st_n + st_o) * hinv_c;
            else
              prob = st_n * inv_c;
            if (ur >= prob) {
              // null collision (plugins/twostatevolpath.py:227-231, 256-257);
              // the two weights sum to 2, equal states give exactly 1
              if (kMode == kTwoState) {
                const float sn_o = mu_c - st_o, sn_n = mu_c - st_n;
                const float den = sn_n + sn_o;
                const float wn = (2.0f * sn_n) / den, wo = 2.0f - wn;
                bn = V3{bn.x * wn, bn.y * wn, bn.z * wn};
                bo = V3{bo.x * wo, bo.y * wo, bo.z * wo};
              } else if (kMode == kReplay) {
                const float sn = mu_c - st_n;
                scatter_density(J, lk, -(J.scale * s_main) / sn);
                if (kCount) ++cnt.grad_events;
              } else if (kMode == kForward) {
                const float sn = mu_c - st_n;
                const V3 Lr = Lrem;
                const float f = -(J.scale * tangent_density(J, lk)) / sn;
                dL = V3{dL.x + Lr.x * f, dL.y + Lr.y * f, dL.z + Lr.z * f};
                if (kCount) ++cnt.grad_events;
              }
              p = x;
              t_rem = t_rem - t;
              if (kMode == kTape) {
                ev_kind = 1;
                ev_ref = tref;
                ev_f = mu_c - st_n;
              }
            } else {
              // real scattering event (plugins/twostatevolpath.py:249-253)
              depth += 1;
              if (depth >= J.max_depth) {
                finished = true;
              } else {
                if (kCount) ++cnt.scatters;
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
              if (kEnv) {
                // environment map hit after a phase sample: power heuristic
                // against NEE (plugins/twostatevolpath.py:288-308)
                float pdf;
                const V3 Le = env_radiance_dir(J, d, pdf);
                const float k = depth == 0 ? 1.0f : env_mis(kInvFourPi, pdf);
                Ln = V3{Ln.x + (bn.x * Le.x) * k, Ln.y + (bn.y * Le.y) * k, Ln.z + (bn.z * Le.z) * k};
                if (kMode == kTwoState)
                  Lo = V3{Lo.x + (bo.x * Le.x) * k, Lo.y + (bo.y * Le.y) * k, Lo.z + (bo.z * Le.z) * k};
              } else {
                const float k = depth == 0 ? 1.0f : mis;
                Ln = V3{Ln.x + bn.x * k, Ln.y + bn.y * k, Ln.z + bn.z * k};
                if (kMode == kTwoState) Lo = V3{Lo.x + bo.x * k, Lo.y + bo.y * k, Lo.z + bo.z * k};
              }
            }
            finished = true;
          }
        } else if (phase == kNee) {
          bool done = !valid;
          if (valid) {
            // ratio tracking (plugins/twostatevolpath.py:443-452)
            trn = trn * ((mu_c - st_n) * inv_c);
            if (kMode == kTwoState) tro = tro * ((mu_c - st_o) * inv_c);
            q = x;
            tr_rem = tr_rem - t;
            if (kMode == kTape) {
              ev_kind = 2;
              ev_ref = tref;
              ev_f = mu_c - st_n;
            }
            done = (kMode == kTwoState) ? (trn == 0.0f && tro == 0.0f) : (trn == 0.0f);
          }
          if (done) {
            V3 cn;
            if (kEnv) {
              cn = V3{(bn.x * env_e[0]) * trn, (bn.y * env_e[1]) * trn, (bn.z * env_e[2]) * trn};
            } else {
              const float en = emit_weight * trn;
              cn = V3{((bn.x * kInvFourPi) * mis) * en, ((bn.y * kInvFourPi) * mis) * en,
                      ((bn.z * kInvFourPi) * mis) * en};
            }
            if (kMode == kAdjoint && !ck_lost) {
              const unsigned long long slot = atomicAdd(Q.ckpt_count, 1ull);
              if ((int64_t)slot < Q.ckpt_cap)
                write_checkpoint(Q.ckpt + slot * 4, (uint32_t)path, depth, ck_state, p, bn, Ln, cn);
              else
                ck_lost = true;
            }
            if (kMode == kTape && (tref >> 30) == kEvShadow) {
              // the scattering event's record: its path, the radiance gathered
              // before its NEE contribution, and that contribution; the event
              // itself goes on the tape, and the next segment's null
              // collisions refer to the record too
              const uint32_t k = tref & kTapeIndexMask;
              float4* rec = Q.ckpt + (int64_t)k * 2;
              __stcs(rec, make_float4(__uint_as_float((uint32_t)path), Ln.x, Ln.y, Ln.z));
              __stcs(rec + 1, make_float4(cn.x, cn.y, cn.z, 0.0f));
              tref = (kEvSegment << 30) | k;
            }
            Ln = V3{Ln.x + cn.x, Ln.y + cn.y, Ln.z + cn.z};
            if (kRep) Lrem = V3{Lrem.x - cn.x, Lrem.y - cn.y, Lrem.z - cn.z};
            if (kMode == kTwoState) {
              if (kEnv) {
                Lo = V3{Lo.x + (bo.x * env_e[0]) * tro, Lo.y + (bo.y * env_e[1]) * tro,
                        Lo.z + (bo.z * env_e[2]) * tro};
              } else {
                const float eo = emit_weight * tro;
                Lo = V3{Lo.x + ((bo.x * kInvFourPi) * mis) * eo, Lo.y + ((bo.y * kInvFourPi) * mis) * eo,
                        Lo.z + ((bo.z * kInvFourPi) * mis) * eo};
              }
            }
            if (kRep) {
              // whole-path replay: walk the shadow ray again (saved stream) to
              // back-propagate through its transmittance
              if (kMode == kReplay) {
                const V3 g = pixel_dL(*Jp, pix);
                s_nee = (g.x * cn.x + g.y * cn.y) + g.z * cn.z;
                s_main = (g.x * Lrem.x + g.y * Lrem.y) + g.z * Lrem.z;
              } else {
                cn_task = cn;
              }
              q = p;
              float a;
              slab(q, recip(w), a, tr_rem);
              trn = 1.0f;
              phase = kNeeAdj;
            } else {
              d = wo_next;  // t_rem was set at the scattering event
              phase = kMain;
            }
          }
        } else {  // kNeeAdj: the shadow walk with gradients
          bool done = !valid;
          if (valid) {
            const float sn = mu_c - st_n;
            if (sn > 0.0f) {
              if (kMode == kForward) {
                const float f = -(J.scale * tangent_density(J, lk)) / sn;
                dL = V3{dL.x + cn_task.x * f, dL.y + cn_task.y * f, dL.z + cn_task.z * f};
              } else {
                scatter_density(J, lk, -(J.scale * s_nee) / sn);
              }
              if (kCount) ++cnt.grad_events;
            }
            trn = trn * (sn * inv_c);
            q = x;
            tr_rem = tr_rem - t;
            done = trn == 0.0f;
          }
          if (done) {
            d = wo_next;  // t_rem was set at the scattering event
            phase = kMain;
          }
        }
      }
    }

    if (kMode == kTape) {
      if (!tape_append(Q, tc, ev_kind != 0 && !ck_lost, ev_kind == 2 ? q : p, ev_ref, ev_f)) ck_lost = true;
      if (!tape_append(Q, tc, ev_scat && !ck_lost, p, (kEvScatter << 30) | (tref & kTapeIndexMask), ev_sf))
        ck_lost = true;
    }

    // -------------------------------------------------------------- path end
    if (finished) {
      if (kMode == kTwoState || kMode == kSingle) {
        float4* o = Q.path_out + (Jp->path_begin + sid) * (kMode == kTwoState ? 2 : 1);
        __stcs(o, make_float4(Ln.x, Ln.y, Ln.z, 0.0f));
        if (kMode == kTwoState) __stcs(o + 1, make_float4(Lo.x, Lo.y, Lo.z, 0.0f));
      }
      if (kRad) __stcs(Q.path_ltot + path, make_float4(Ln.x, Ln.y, Ln.z, ck_lost ? 1.0f : 0.0f));
      if (kMode == kTape && ck_lost) Q.lost_list[atomicAdd(Q.lost_count, 1ull)] = (uint32_t)path;
      if (kMode == kForward && (dL.x != 0.0f || dL.y != 0.0f || dL.z != 0.0f)) {
        // the task's share of its pixel's derivative (the pixel value is the
        // mean of its samples)
        const float fs = (float)Jp->spp;
        float* o = Jp->out_img + (int64_t)pix * 3;
        atomicAdd(o + 0, dL.x / fs);
        atomicAdd(o + 1, dL.y / fs);
        atomicAdd(o + 2, dL.z / fs);
      }
      if (kCount && !kRep) ++cnt.paths;
      if (Jp->pixel_cost != nullptr) red_add_u32(Jp->pixel_cost + pix, n_iter - iter0);
      phase = kIdle;
    }
  }
  if (kMode == kTape) tape_close(Q, tc);  // the unused slots of the warp's last chunk
}

}  // namespace rcv
