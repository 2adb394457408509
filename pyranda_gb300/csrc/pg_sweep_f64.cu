// FP64 instantiation of the directional sweeps and the sweep launcher.
#include "pg_sweep.cuh"

namespace pg {

int launch_sweep_f32(const OpRef& op, const KParams& P, int dir, int epi, void* st);

int launch_sweep(int precision, const SweepLaunch& s, void* stream) {
  const OpRef& op = *s.op;
  KParams P;
  P.in = s.in;
  P.out = s.out;
  P.scratch = s.scratch;
  P.ops = op.dev;
  P.nops = op.nops;
  P.nlines = op.nlines;
  P.scale_pow = s.scale_pow;
  P.emax = s.emax;
  if (P.nlines <= 0) return PG_OK;
  if (precision == PG_FP32 && op.kind == OPK_D8 && op.exact && !op.null_op) {
    if (!s.emax || !s.moff) {
      set_error("sweep: the exact d8 RHS needs the exponent workspace");
      return PG_EINVAL;
    }
    if (!s.emax_ready) {
      const int rc = launch_max_exponent(s.in, s.moff, op.nops, s.emax, stream);
      if (rc) return rc;
    }
  }
  if (precision == PG_FP32) return launch_sweep_f32(op, P, s.dir, s.epi, stream);
  return dispatch_kind<double>(op, P, s.dir, s.epi, stream);
}

}  // namespace pg
