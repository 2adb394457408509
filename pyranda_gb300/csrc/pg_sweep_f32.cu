// FP32 instantiation of the directional sweeps (the fast path: single-precision
// arithmetic on FP64 inputs and outputs).
#include "pg_sweep.cuh"

namespace pg {

int launch_sweep_f32(const OpRef& op, const KParams& P, int dir, int epi, void* st) {
  return dispatch_kind<float>(op, P, dir, epi, st);
}

}  // namespace pg
