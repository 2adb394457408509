// FP32 instantiation of the directional sweeps (the fast path: single-precision
// arithmetic on FP64 inputs and outputs).
#include "pg_sweep.cuh"

namespace pg {

int launch_sweep_f32_r4(const OpRef& op, const KParams& P, int dir, int epi, void* st);  // pg_sweep_f32_r4.cu

int launch_sweep_f32(const OpRef& op, const KParams& P, int dir, int epi, void* st) {
  if (op.kind == OPK_D1 || op.kind == OPK_D2 || op.kind == OPK_D4) return dispatch_kind_r3<float>(op, P, dir, epi, st);
  return launch_sweep_f32_r4(op, P, dir, epi, st);
}

namespace {

// The d8 RHS of every row along DIR, exactly as the banded FP32 sweep forms
// it (64-bit fixed point at the member's exponent; edge rows with their
// integer weights, interior rows as iw[0] x the 8th difference), rounded once
// to FP32.  One thread owns a run of kRun rows of one line (blockIdx.y = run):
// each value is loaded and converted once, and the interior rows come from a
// cascade of differences primed with the 8 values before the first of them.
constexpr int kRun = 16;

template <bool PER, int DIR>
__global__ void __launch_bounds__(128) d8_rhs_kernel(const MemberOp* __restrict__ ops, int nops, long long nlines,
                                                     const double* __restrict__ in, const int* __restrict__ emax,
                                                     double* __restrict__ rhs) {
  const int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nlines) return;
  int m = 0;
  if (nops > 1) {  // the member owning line L: last entry with line0 <= L
    int lo = 0, hi = nops - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (ops[mid].line0 <= L) lo = mid;
      else hi = mid - 1;
    }
    m = lo;
  }
  const MemberOp& op = ops[m];
  const int n = op.n;
  const int i0 = blockIdx.y * kRun;
  if (i0 >= n) return;
  const int64_t Lm = L - op.line0;
  const int nx = op.nx, ny = op.ny;
  int64_t base;
  int st;
  if (DIR == 0) {
    base = Lm * nx;
    st = 1;
  } else if (DIR == 1) {
    base = (Lm / nx) * (int64_t)nx * ny + (Lm % nx);
    st = nx;
  } else {
    base = (Lm / nx) * (int64_t)nx + (Lm % nx);
    st = nx * ny;
  }
  base += op.off;
  const int E = __ldg(emax + m);
  const Line<long long> ln{in + base, st, n, E};
  double* __restrict__ out = rhs + base;
  const float wi = op.wscale * (float)op.iw[0];
  Cascade cas{};
  bool primed = false;
  const int i1 = min(i0 + kRun, n);
  for (int i = i0; i < i1; i++) {
    float r;
    if (i < 4 || i >= n - 4) {
      r = fixed_to_float(edge_rhs<long long, 4, PER, int>(ln, i, op.rhs_i, op.bcl, op.bch), E, op.wscale);
    } else {
      if (!primed) {
#pragma unroll
        for (int k = 0; k < 8; k++) cas.push(ln.v(i - 4 + k));
        primed = true;
      }
      r = fixed_to_float(cas.push(ln.v(i + 4)), E, wi);
    }
    out[(int64_t)i * st] = f2d_bits(r);
  }
}

template <bool PER>
int launch_d8_rhs_dir(const OpRef& op, const double* in, double* rhs, int dir, const int* emax, int nmax,
                      void* stream) {
  const dim3 grid((unsigned)((op.nlines + 127) / 128), (unsigned)((nmax + kRun - 1) / kRun));
  cudaStream_t s = (cudaStream_t)stream;
  if (dir == 0) d8_rhs_kernel<PER, 0><<<grid, 128, 0, s>>>(op.dev, op.nops, op.nlines, in, emax, rhs);
  else if (dir == 1) d8_rhs_kernel<PER, 1><<<grid, 128, 0, s>>>(op.dev, op.nops, op.nlines, in, emax, rhs);
  else d8_rhs_kernel<PER, 2><<<grid, 128, 0, s>>>(op.dev, op.nops, op.nlines, in, emax, rhs);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("d8 rhs: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

}  // namespace

int launch_d8_rhs(const OpRef& op, const double* in, double* rhs, int dir, const int* emax, int nmax,
                  void* stream) {
  if (op.kind != OPK_D8 || !op.exact || op.null_op || nmax < 1 || op.nlines < 1) {
    set_error("d8 rhs: the operator has no exact fixed-point RHS");
    return PG_EINVAL;
  }
  return op.periodic ? launch_d8_rhs_dir<true>(op, in, rhs, dir, emax, nmax, stream)
                     : launch_d8_rhs_dir<false>(op, in, rhs, dir, emax, nmax, stream);
}

}  // namespace pg
