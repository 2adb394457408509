// FP32 instantiation of the directional sweeps (the fast path: single-precision
// arithmetic on FP64 inputs and outputs).
#include "pg_sweep.cuh"

namespace pg {

int launch_sweep_f32(const OpRef& op, const KParams& P, int dir, int epi, void* st) {
  return dispatch_kind<float>(op, P, dir, epi, st);
}

namespace {

// One thread per point: the d8 RHS of its row along DIR, exactly as the
// banded FP32 sweep forms it (64-bit fixed point at the member's exponent;
// edge rows with their integer weights, interior rows with iw), rounded once
// to FP32.
template <bool PER, int DIR>
__global__ void __launch_bounds__(256) d8_rhs_kernel(const MemberOp* __restrict__ ops, int nops,
                                                     const double* __restrict__ in, const int* __restrict__ emax,
                                                     int64_t npts, double* __restrict__ rhs) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npts;
       p += (int64_t)gridDim.x * blockDim.x) {
    int m = 0;
    if (nops > 1) {  // the member owning point p: last entry with off <= p
      int lo = 0, hi = nops - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ops[mid].off <= p) lo = mid;
        else hi = mid - 1;
      }
      m = lo;
    }
    const MemberOp& op = ops[m];
    const int64_t q = p - op.off;
    const int nx = op.nx, ny = op.ny, n = op.n;
    int i, st;
    if (DIR == 0) {
      i = (int)(q % nx);
      st = 1;
    } else if (DIR == 1) {
      i = (int)((q / nx) % ny);
      st = nx;
    } else {
      i = (int)(q / ((int64_t)nx * ny));
      st = nx * ny;
    }
    const int E = __ldg(emax + m);
    const Line<long long> ln{in + p - (int64_t)i * st, st, n, E};
    long long s;
    if (i < 4 || i >= n - 4) {
      s = edge_rhs<long long, 4, PER, int>(ln, i, op.rhs_i);
    } else {
      const long long mc = ln.v(i);
      s = 0;
#pragma unroll
      for (int l = 0; l < 9; l++)
        if (l != 4) s += (long long)op.iw[l] * (ln.v(i + l - 4) - mc);
    }
    rhs[p] = f2d_bits(fixed_to_float(s, E, op.wscale));
  }
}

template <bool PER>
int launch_d8_rhs_dir(const OpRef& op, const double* in, double* rhs, int dir, const int* emax, int64_t npts,
                      void* stream) {
  const int64_t b = (npts + 255) / 256;
  const unsigned blocks = (unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
  cudaStream_t s = (cudaStream_t)stream;
  if (dir == 0) d8_rhs_kernel<PER, 0><<<blocks, 256, 0, s>>>(op.dev, op.nops, in, emax, npts, rhs);
  else if (dir == 1) d8_rhs_kernel<PER, 1><<<blocks, 256, 0, s>>>(op.dev, op.nops, in, emax, npts, rhs);
  else d8_rhs_kernel<PER, 2><<<blocks, 256, 0, s>>>(op.dev, op.nops, in, emax, npts, rhs);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("d8 rhs: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

}  // namespace

int launch_d8_rhs(const OpRef& op, const double* in, double* rhs, int dir, const int* emax, int64_t npts,
                  void* stream) {
  if (op.kind != OPK_D8 || !op.exact || op.null_op) {
    set_error("d8 rhs: the operator has no exact fixed-point RHS");
    return PG_EINVAL;
  }
  return op.periodic ? launch_d8_rhs_dir<true>(op, in, rhs, dir, emax, npts, stream)
                     : launch_d8_rhs_dir<false>(op, in, rhs, dir, emax, npts, stream);
}

}  // namespace pg
