// FP64 instantiation of the directional sweeps and the sweep launcher.
#include "pg_sweep.cuh"

namespace pg {

int launch_sweep_f32(const DevOp& op, const KParams& P, int dir, int epi, void* st);

int launch_sweep(const DevOp& op, int precision, const SweepLaunch& s, void* stream) {
  KParams P;
  P.in = s.in;
  P.out = s.out;
  P.scratch = s.scratch;
  P.rhs = op.rhs;
  P.lu = op.lu;
  P.n = op.n;
  P.nx = s.nx;
  P.ny = s.ny;
  P.nz = s.nz;
  P.epi_scale = s.epi_scale;
  for (int k = 0; k < 9; k++) P.ri[k] = op.rhs_in[k];
  if (s.dir == 0) P.nlines = (int64_t)s.ny * s.nz;
  else if (s.dir == 1) P.nlines = (int64_t)s.nx * s.nz;
  else P.nlines = (int64_t)s.nx * s.ny;
  if (P.nlines <= 0) return PG_OK;
  if ((int64_t)s.nx * s.ny * s.nz >= ((int64_t)1 << 31)) {
    set_error("field of %lld points: the sweeps address fields of fewer than 2^31 points",
              (long long)s.nx * s.ny * s.nz);
    return PG_EBADSHAPE;
  }
  if (precision == PG_FP32) return launch_sweep_f32(op, P, s.dir, s.epi, stream);
  return dispatch_kind<double>(op, P, s.dir, s.epi, stream);
}

}  // namespace pg
