// FP32 instantiation of the 9-point directional sweeps (d8 with the exact
// fixed-point RHS, the compact and the Gaussian filters), in its own
// translation unit so that it compiles beside pg_sweep_f32.cu.
#include "pg_sweep.cuh"

namespace pg {

int launch_sweep_f32_r4(const OpRef& op, const KParams& P, int dir, int epi, void* st) {
  return dispatch_kind_r4<float>(op, P, dir, epi, st);
}

}  // namespace pg
