// FP64 instantiation of the directional sweeps and the sweep launcher.
#include "pg_sweep.cuh"

namespace pg {

int launch_sweep_f32(const DevOp& op, const KParams& P, int dir, int epi, int lb, int64_t nb, void* st);

int launch_sweep(const DevOp& op, int precision, const SweepLaunch& s, void* stream) {
  KParams P;
  P.in = s.in;
  P.out = s.out;
  P.rhs = op.rhs;
  P.lu = op.lu;
  P.n = op.n;
  P.nx = s.nx;
  P.ny = s.ny;
  P.nz = s.nz;
  P.epi_scale = s.epi_scale;
  for (int k = 0; k < 9; k++) P.ri[k] = op.rhs_in[k];
  const size_t esz = precision == PG_FP32 ? 4 : 8;
  // lines per CTA: 32 while the tile fits twice per SM, else 16, else 8
  int lb = 32;
  while (lb > 8 && (size_t)op.n * (lb + 1) * esz > 110 * 1024) lb /= 2;
  if ((size_t)op.n * (lb + 1) * esz > 220 * 1024) {
    set_error("line length %d too long for one tile", op.n);
    return PG_EBADSHAPE;
  }
  int64_t nblocks;
  if (s.dir == 0) {
    nblocks = ((int64_t)s.ny * s.nz + lb - 1) / lb;
    P.tiles_i = 1;
  } else {
    P.tiles_i = (s.nx + lb - 1) / lb;
    nblocks = (int64_t)P.tiles_i * (s.dir == 1 ? s.nz : s.ny);
  }
  if (nblocks <= 0) return PG_OK;
  if (precision == PG_FP32) return launch_sweep_f32(op, P, s.dir, s.epi, lb, nblocks, stream);
  return dispatch_kind<double>(op, P, s.dir, s.epi, lb, nblocks, stream);
}

}  // namespace pg
