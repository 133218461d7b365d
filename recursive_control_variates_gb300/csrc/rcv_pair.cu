// The two independent tracers of an optimisation step in one persistent
// launch: the two-state primal render (the control-variate images H and F,
// plugins/twostatevolpath.py:91-138) and the adjoint's radiance pass with
// its event tape, which needs only the parameters and the gradient seed.
//
// Each tracer alone ends on its longest paths (depth up to max_depth, each
// scattering event followed by a shadow walk) while most of the GPU idles;
// run one after the other, the second starts its own longest paths only as
// the first one's blocks retire.  Here every warp runs both tracers in turn,
// the warps of half of the SM pairs starting with the two-state paths and
// the others with the radiance-pass paths, so that the longest paths of both
// (handed out first by the cost order) start together and the bulk of
// either tracer fills the GPU around them.  Each tracer keeps its own queue, pixel order, random
// streams and outputs: the results are those of the two separate launches.
#include <cuda_runtime.h>

#include <mutex>

#include "rcv_common.h"
#include "rcv_trace.cuh"

namespace rcv {

template <bool kSG, bool kEnv>
__global__ void __launch_bounds__(kTraceBlock, 5)
    trace_pair_kernel(const __grid_constant__ VolJob JA, const __grid_constant__ Queue QA,
                      const __grid_constant__ VolJob JB, const __grid_constant__ Queue QB) {
  Counts cnt{0, 0, 0, 0, 0, 0};
  // The tracer a warp runs first goes by its SM pair (TPC): every warp of a
  // TPC starts on the same tracer.  Measured on GB300 (512^2, 16 + 16 spp,
  // depth 64): with the choice by warp or by SM, so that the two SMs of a
  // TPC ran both tracers' code at once, the paired launch took 4.2 ms; by
  // TPC (or by die) 2.4 ms, against 1.56 + 1.42 ms for the two launches
  // alone -- as if the two SMs of a TPC shared an instruction cache that
  // holds the hot code of one tracer but not of two.
  unsigned smid;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
  const bool primal_first = ((smid >> 1) & 1u) == 0u;
  // each tracer returns once its queue is empty and the warp's paths ended
  // (written out rather than as a loop over the two: the loop form keeps
  // state of both bodies live and spills ~200 B a thread)
  if (primal_first) trace_persistent<kTwoState, kSG, false, kEnv>(JA, QA, cnt);
  trace_persistent<kTape, kSG, false, kEnv>(JB, QB, cnt);
  if (!primal_first) trace_persistent<kTwoState, kSG, false, kEnv>(JA, QA, cnt);
}

using PairKernel = void (*)(VolJob, Queue, VolJob, Queue);
static const PairKernel kPairKernels[4] = {trace_pair_kernel<false, false>, trace_pair_kernel<true, false>,
                                           trace_pair_kernel<false, true>, trace_pair_kernel<true, true>};

static int pair_blocks_per_sm(int variant) {
  static std::once_flag once;
  static int blocks[4];
  std::call_once(once, [] {
    for (int v = 0; v < 4; ++v) {
      blocks[v] = 1;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[v], kPairKernels[v], kTraceBlock, 0);
      if (blocks[v] < 1) blocks[v] = 1;
    }
  });
  return blocks[variant];
}

void warm_pair_config() { (void)pair_blocks_per_sm(0); }

int launch_pair(const VolJob& JA, const Queue& QA, const VolJob& JB, const Queue& QB, const rcv_volpath_options* o,
                cudaStream_t st, bool supergrid) {
  RCV_REQUIRE(QA.counters == nullptr && QB.counters == nullptr, "the paired launch does not count events");
  RCV_REQUIRE(QA.path_out != nullptr && QB.tape != nullptr, "the paired launch needs the primal's path "
                                                            "radiance and the adjoint's tape");
  RCV_REQUIRE((QA.jobs == nullptr) == (QB.jobs == nullptr), "the paired launch takes two single jobs or two "
                                                            "job tables");
  const bool single = QA.jobs == nullptr;
  const bool sg = supergrid || (single && (JA.sg[0] > 0 || JB.sg[0] > 0));
  // an environment map belongs to a single job (job tables take the constant environment)
  const bool env = single && JA.env.valid != 0;
  RCV_REQUIRE(!single || (JB.env.valid != 0) == env, "the paired jobs must share their environment");
  const int variant = (sg ? 1 : 0) + (env ? 2 : 0);
  int per_sm = pair_blocks_per_sm(variant);
  if (o != nullptr && o->blocks_per_sm > 0 && o->blocks_per_sm < per_sm) per_sm = o->blocks_per_sm;
  const int64_t warps_needed = (QA.total + QA.batch - 1) / QA.batch + (QB.total + QB.batch - 1) / QB.batch;
  int64_t blocks = (warps_needed + kTraceWarps - 1) / kTraceWarps;
  const int64_t cap = int64_t(tracer_sm_count()) * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  kPairKernels[variant]<<<(unsigned)blocks, kTraceBlock, 0, st>>>(JA, QA, JB, QB);
  return launched("paired trace kernel launch");
}

}  // namespace rcv
