// Pointwise and reduction kernels: the fused LSRK(5,4) stage update, the
// Courant / diffusion time-step limits, global reductions and the mesh fill.
// These are HBM-bound; they use grid-stride loops over 2 doubles per thread
// (16-byte accesses) sized to a multiple of the SM count.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>

#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxVar = 16;

int grid_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  const int64_t cap = 152 * 8;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

int check(const char* what) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

__global__ void fill_kernel(double* __restrict__ o, double v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    o[i] = v;
}

__global__ void copy_kernel(double* __restrict__ o, const double* __restrict__ a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    o[i] = a[i];
}

struct RkArgs {
  double* U[kMaxVar];
  double* PHI[kMaxVar];
  const double* F[kMaxVar];
};

// pyranda.py:800-804:  tmp1 = A*PHI ; PHI = dt*F + tmp1 ; tmp2 = B*PHI ; U = U + tmp2
// DT_FIELD: one dt per point (an ensemble advances each member with its own dt)
template <bool DT_FIELD>
__global__ void rk_stage_kernel(const RkArgs a, int nvar, const double* __restrict__ dtp, double A, double B,
                                int64_t n) {
  const double dt0 = DT_FIELD ? 0.0 : *dtp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double dt = DT_FIELD ? dtp[i] : dt0;
    for (int v = 0; v < nvar; v++) {
      // rounding spelled out (one product, then two fused multiply-adds): the fused EOM
      // kernels that apply a stage themselves repeat exactly these operations
      const double phi = __fma_rn(dt, a.F[v][i], __dmul_rn(A, a.PHI[v][i]));
      a.PHI[v][i] = phi;
      a.U[v][i] = __fma_rn(B, phi, a.U[v][i]);
    }
  }
}

// Block reduction helper: op 0 = sum, 1 = max, 2 = min.
template <int OP>
__device__ __forceinline__ double combine(double a, double b) {
  if (OP == 0) return a + b;
  if (OP == 1) return fmax(a, b);
  return fmin(a, b);
}

template <int OP>
__device__ __forceinline__ double identity() {
  if (OP == 0) return 0.0;
  if (OP == 1) return -INFINITY;  // max of an all -inf input is -inf, as in numpy
  return INFINITY;
}

template <int OP>
__device__ double block_reduce(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v = combine<OP>(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : identity<OP>();
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v = combine<OP>(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// NaN propagation: fmax/fmin drop NaNs, so a NaN anywhere would be hidden; a
// separate flag keeps numpy's behaviour (max/min of data holding NaN is NaN).
template <int OP>
__global__ void reduce_partial(const double* __restrict__ in, int64_t n, double* __restrict__ partial) {
  double acc = identity<OP>();
  bool nan = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = in[i];
    nan |= (x != x);
    acc = combine<OP>(acc, x);
  }
  acc = block_reduce<OP>(acc);
  const int anynan = __syncthreads_or(nan);
  if (threadIdx.x == 0) partial[blockIdx.x] = anynan ? NAN : acc;
}

template <int OP>
__global__ void reduce_final(const double* __restrict__ partial, int np, double* __restrict__ out) {
  double acc = identity<OP>();
  bool nan = false;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const double x = partial[i];
    nan |= (x != x);
    acc = combine<OP>(acc, x);
  }
  acc = block_reduce<OP>(acc);
  const int anynan = __syncthreads_or(nan);
  if (threadIdx.x == 0) *out = anynan ? NAN : acc;
}

// courant: vrate = |u|/d1 + |v|/d2 + |w|/d3 ; crate = |c|/GridLen ; max(vrate+crate).
// The spacings are uniform, so each division is a multiplication by the
// reciprocal computed once on the host (FP64 division costs ~10 FP64-pipe
// instructions on GB300; the product differs from the quotient by <= 1 ulp).
__global__ void courant_partial(const double* __restrict__ u, const double* __restrict__ v,
                                const double* __restrict__ w, const double* __restrict__ c, double vconst,
                                double wconst, double r1, double r2, double r3, double rgl, int64_t n,
                                double* __restrict__ partial) {
  double acc = -INFINITY;
  bool nan = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double vv = v ? v[i] : vconst;
    const double ww = w ? w[i] : wconst;
    const double vrate = fabs(u[i]) * r1 + fabs(vv) * r2 + fabs(ww) * r3;
    const double x = vrate + fabs(c[i]) * rgl;
    nan |= (x != x);
    acc = fmax(acc, x);
  }
  acc = block_reduce<1>(acc);
  const int anynan = __syncthreads_or(nan);
  if (threadIdx.x == 0) partial[blockIdx.x] = anynan ? NAN : acc;
}

__global__ void invert_scalar(double* p) { *p = 1.0 / *p; }

// The diffusion limit min(rho GridLen^2 / max(1e-12, bulk)) in two passes.
// FP64 division runs on GB300's slow FP64 pipe (~10 instructions each), so
// pass 1 estimates every quotient in FP32 (integer FP64->FP32 conversion,
// correctly rounded FP32 divide; relative error < 4e-7) and pass 2 evaluates
// the FP64 quotient only where the estimate is within 1e-5 of the smallest
// estimate: the true minimiser is always among those, so the result is the
// exact FP64 minimum.  Points whose values are not finite or beyond 2^60 in
// magnitude are always evaluated exactly.  As in the one-pass form, NaN in
// rho makes the result NaN and a NaN bulk is floored by fmax.
struct DiffEst {
  float e;
  bool exact;
  bool nan;
};

__device__ __forceinline__ float d2f_int(double d) {  // FP64 -> FP32 by integer operations
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned mag = hi & 0x7fffffffu;
  unsigned f = ((mag - (896u << 20)) << 3) | (lo >> 29);
  f += (lo >> 28) & 1u;
  f = (mag < (897u << 20)) ? 0u : f;
  return __uint_as_float(f | (hi & 0x80000000u));
}

__device__ __forceinline__ DiffEst diff_estimate(double rho, double bulk, float gl2) {
  const unsigned rh = (unsigned)__double2hiint(rho), rl = (unsigned)__double2loint(rho);
  const unsigned bh = (unsigned)__double2hiint(bulk);
  const unsigned re = (rh >> 20) & 0x7ffu, be = (bh >> 20) & 0x7ffu;
  DiffEst d;
  d.nan = (re == 0x7ffu) && (((rh & 0xfffffu) | rl) != 0u);
  d.exact = (re >= 1023u + 60u) || (be >= 1023u + 60u);
  d.e = (d2f_int(rho) * gl2) / fmaxf(1.0e-12f, d2f_int(bulk));
  return d;
}

// partial[b]: block b's smallest estimate; partial[gridDim.x + b]: 1 if block b holds a point
// that pass 2 must evaluate exactly whatever its estimate
__global__ void diff_estimate_partial(const double* __restrict__ bulk, const double* __restrict__ rho, float gl2,
                                      int64_t n, double* __restrict__ partial) {
  float acc = FLT_MAX;
  bool nan = false, exact = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const DiffEst d = diff_estimate(rho[i], bulk[i], gl2);
    nan |= d.nan;
    exact |= d.exact;
    if (!d.exact) acc = fminf(acc, d.e);
  }
  double v = block_reduce<2>((double)acc);
  const int anynan = __syncthreads_or(nan);
  const int anyexact = __syncthreads_or(exact);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = anynan ? NAN : v;
    partial[gridDim.x + blockIdx.x] = anyexact ? 1.0 : 0.0;
  }
}

__global__ void diff_exact_partial(const double* __restrict__ bulk, const double* __restrict__ rho, double gl,
                                   float gl2, int64_t n, const double* __restrict__ est_min,
                                   double* __restrict__ partial) {
  const double m = *est_min;
  const float lim = (float)(m + fabs(m) * 1.0e-5 + 1.0e-38);
  // a block whose points (the same grid-stride set as in pass 1) all estimate above the limit
  // holds no candidate: it skips its loads
  const double bmin = partial[blockIdx.x];
  const bool bexact = partial[gridDim.x + blockIdx.x] != 0.0;
  __syncthreads();  // every thread has read the pass-1 values before thread 0 overwrites them
  if (m == m && !bexact && !(bmin <= (double)lim)) {
    if (threadIdx.x == 0) partial[blockIdx.x] = INFINITY;
    return;
  }
  double acc = INFINITY;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double r = rho[i], b = bulk[i];
    const DiffEst d = diff_estimate(r, b, gl2);
    if (d.exact || d.e <= lim) acc = fmin(acc, r * gl * gl / fmax(1.0e-12, b));
  }
  acc = block_reduce<2>(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = (m != m) ? NAN : acc;
}

__global__ void finite_kernel(const double* __restrict__ in, int64_t n, int* flag) {
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(in[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(flag, 1);
}

// mesh.f90:169-211 (Cartesian): cell-centred coordinates from the face origin
__global__ void mesh_kernel(int which, double* __restrict__ out, int nx, int ny, int nz, double x1, double y1,
                            double z1, double dx, double dy, double dz, double cval) {
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(p % nx);
    const int j = (int)((p / nx) % ny);
    const int k = (int)(p / ((int64_t)nx * ny));
    double v;
    // mesh.f90:181-183: x1 + REAL(2*i-1)*half*dx, evaluated without contraction
    if (which == 0) v = __dadd_rn(x1, __dmul_rn(__dmul_rn((double)(2 * (i + 1) - 1), 0.5), dx));
    else if (which == 1) v = __dadd_rn(y1, __dmul_rn(__dmul_rn((double)(2 * (j + 1) - 1), 0.5), dy));
    else if (which == 2) v = __dadd_rn(z1, __dmul_rn(__dmul_rn((double)(2 * (k + 1) - 1), 0.5), dz));
    else v = cval;
    out[p] = v;
  }
}

// ---------------------------------------------------------------------------
// Ensemble (segmented) reductions: block b works on member b / kSegBlocks.
// ---------------------------------------------------------------------------
enum { SEG_SUM = 0, SEG_MAX = 1, SEG_MIN = 2, SEG_COURANT = 3, SEG_DIFF = 4 };

template <int KIND>
__global__ void seg_partial(const double* __restrict__ a, const double* __restrict__ b,
                            const double* __restrict__ w, const double* __restrict__ c, double vconst,
                            double wconst, const double* __restrict__ mconst, const long long* __restrict__ moff,
                            double* __restrict__ partial) {
  constexpr int OP = (KIND == SEG_SUM) ? 0 : ((KIND == SEG_MAX || KIND == SEG_COURANT) ? 1 : 2);
  const int m = blockIdx.x / kSegBlocks, sub = blockIdx.x % kSegBlocks;
  const long long lo = moff[m], hi = moff[m + 1];
  double r1 = 0, r2 = 0, r3 = 0, rgl = 0, gl = 0;
  if (KIND == SEG_COURANT) {
    r1 = mconst[m * 5 + 0];
    r2 = mconst[m * 5 + 1];
    r3 = mconst[m * 5 + 2];
    rgl = mconst[m * 5 + 3];
  }
  if (KIND == SEG_DIFF) gl = mconst[m * 5 + 4];
  double acc = identity<OP>();
  bool nan = false;
  for (long long i = lo + (long long)sub * blockDim.x + threadIdx.x; i < hi; i += (long long)kSegBlocks * blockDim.x) {
    double x;
    if (KIND == SEG_COURANT) {
      const double vv = b ? b[i] : vconst;
      const double ww = w ? w[i] : wconst;
      x = fabs(a[i]) * r1 + fabs(vv) * r2 + fabs(ww) * r3 + fabs(c[i]) * rgl;
    } else if (KIND == SEG_DIFF) {
      x = b[i] * gl * gl / fmax(1.0e-12, a[i]);
    } else {
      x = a[i];
    }
    nan |= (x != x);
    acc = combine<OP>(acc, x);
  }
  acc = block_reduce<OP>(acc);
  const int anynan = __syncthreads_or(nan);
  if (threadIdx.x == 0) partial[blockIdx.x] = anynan ? NAN : acc;
}

template <int OP>
__global__ void seg_final(const double* __restrict__ partial, int invert, double* __restrict__ member) {
  const int m = blockIdx.x;
  double acc = identity<OP>();
  bool nan = false;
  for (int i = threadIdx.x; i < kSegBlocks; i += blockDim.x) {
    const double x = partial[m * kSegBlocks + i];
    nan |= (x != x);
    acc = combine<OP>(acc, x);
  }
  acc = block_reduce<OP>(acc);
  const int anynan = __syncthreads_or(nan);
  if (threadIdx.x == 0) member[m] = anynan ? NAN : (invert ? 1.0 / acc : acc);
}

__global__ void seg_broadcast(const double* __restrict__ member, const long long* __restrict__ moff, int nmem,
                              int64_t n, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nmem - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (moff[mid] <= i) lo = mid;
      else hi = mid - 1;
    }
    out[i] = member[lo];
  }
}

template <int KIND>
int seg_run(const double* a, const double* b, const double* w, const double* c, double vconst, double wconst,
            const double* mconst, const long long* moff, int nmem, int64_t npts, double* partial,
            double* out_field, double* out_member, void* stream) {
  constexpr int OP = (KIND == SEG_SUM) ? 0 : ((KIND == SEG_MAX || KIND == SEG_COURANT) ? 1 : 2);
  cudaStream_t s = (cudaStream_t)stream;
  double* member = out_member ? out_member : partial + (size_t)nmem * kSegBlocks;
  seg_partial<KIND><<<nmem * kSegBlocks, kThreads, 0, s>>>(a, b, w, c, vconst, wconst, mconst, moff, partial);
  seg_final<OP><<<nmem, kThreads, 0, s>>>(partial, KIND == SEG_COURANT ? 1 : 0, member);
  count_launch(2);
  if (out_field) {
    seg_broadcast<<<grid_for(npts), kThreads, 0, s>>>(member, moff, nmem, npts, out_field);
    count_launch();
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("segmented reduction: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

}  // namespace

int launch_fill(double* out, double value, int64_t n, void* stream) {
  if (n <= 0) return PG_OK;
  fill_kernel<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(out, value, n);
  return check("fill");
}

int launch_copy(double* out, const double* in, int64_t n, void* stream) {
  if (n <= 0 || out == in) return PG_OK;
  copy_kernel<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(out, in, n);
  return check("copy");
}

int launch_rk_stage(int nvar, double* const* U, double* const* PHI, const double* const* F, const double* dt,
                    double A, double B, int64_t n, int dt_is_field, void* stream) {
  RkArgs a;
  for (int v0 = 0; v0 < nvar; v0 += kMaxVar) {
    const int m = nvar - v0 < kMaxVar ? nvar - v0 : kMaxVar;
    for (int v = 0; v < m; v++) {
      a.U[v] = U[v0 + v];
      a.PHI[v] = PHI[v0 + v];
      a.F[v] = F[v0 + v];
    }
    if (dt_is_field) rk_stage_kernel<true><<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(a, m, dt, A, B, n);
    else rk_stage_kernel<false><<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(a, m, dt, A, B, n);
    int rc = check("rk_stage");
    if (rc) return rc;
  }
  return PG_OK;
}

int launch_reduce(int op, const double* in, int64_t n, double* partial, double* out, void* stream) {
  const int g = grid_for(n) < kReduceBlocks ? grid_for(n) : kReduceBlocks;
  cudaStream_t s = (cudaStream_t)stream;
  if (op == 0) {
    reduce_partial<0><<<g, kThreads, 0, s>>>(in, n, partial);
    reduce_final<0><<<1, kThreads, 0, s>>>(partial, g, out);
  } else if (op == 1) {
    reduce_partial<1><<<g, kThreads, 0, s>>>(in, n, partial);
    reduce_final<1><<<1, kThreads, 0, s>>>(partial, g, out);
  } else {
    reduce_partial<2><<<g, kThreads, 0, s>>>(in, n, partial);
    reduce_final<2><<<1, kThreads, 0, s>>>(partial, g, out);
  }
  count_launch();
  return check("reduce");
}

int launch_courant(const double* u, const double* v, const double* w, const double* c, double vconst,
                   double wconst, const double d[3], double gridlen, int64_t n, double* partial, double* out,
                   void* stream) {
  const int g = grid_for(n) < kReduceBlocks ? grid_for(n) : kReduceBlocks;
  cudaStream_t s = (cudaStream_t)stream;
  courant_partial<<<g, kThreads, 0, s>>>(u, v, w, c, vconst, wconst, 1.0 / d[0], 1.0 / d[1], 1.0 / d[2],
                                         1.0 / gridlen, n, partial);
  reduce_final<1><<<1, kThreads, 0, s>>>(partial, g, out);
  invert_scalar<<<1, 1, 0, s>>>(out);
  count_launch(2);
  return check("courant");
}

int launch_diff(const double* bulk, const double* rho, double gl, int64_t n, double* partial, double* out,
                void* stream) {
  const int g = grid_for(n) < kReduceBlocks ? grid_for(n) : kReduceBlocks;
  cudaStream_t s = (cudaStream_t)stream;
  // pass 1: FP32 estimates -> *out holds their minimum (or NaN)
  diff_estimate_partial<<<g, kThreads, 0, s>>>(bulk, rho, (float)(gl * gl), n, partial);
  reduce_final<2><<<1, kThreads, 0, s>>>(partial, g, out);
  // pass 2: the exact FP64 quotient where the estimate is within 1e-5 of that minimum
  diff_exact_partial<<<g, kThreads, 0, s>>>(bulk, rho, gl, (float)(gl * gl), n, out, partial);
  reduce_final<2><<<1, kThreads, 0, s>>>(partial, g, out);
  count_launch(4);
  return check("diff");
}

// The fixed-point scale of the exact d8 RHS: per member the largest biased
// exponent field of its values (bits 52..62; infinities and NaN give 2047).
__global__ void max_exponent_kernel(const double* __restrict__ in, const long long* __restrict__ moff,
                                    int* __restrict__ emax) {
  const int m = blockIdx.y;
  const long long a = moff[m], b = moff[m + 1];
  unsigned e = 0;
  for (long long i = a + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < b;
       i += (long long)gridDim.x * blockDim.x)
    e = max(e, ((unsigned)__double2hiint(in[i]) >> 20) & 0x7ffu);
  e = __reduce_max_sync(0xffffffffu, e);
  if ((threadIdx.x & 31) == 0 && e) atomicMax(emax + m, (int)e);
}

int launch_max_exponent(const double* in, const long long* moff, int nmem, int* emax, void* stream) {
  if (nmem <= 0) return PG_OK;
  cudaError_t e = cudaMemsetAsync(emax, 0, sizeof(int) * (size_t)nmem, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    set_error("max_exponent: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  const int bx = std::max(1, std::min(152 * 8, (152 * 8 + nmem - 1) / nmem * 2));
  max_exponent_kernel<<<dim3((unsigned)bx, (unsigned)nmem), kThreads, 0, (cudaStream_t)stream>>>(in, moff, emax);
  return check("max_exponent");
}

int launch_check_finite(const double* in, int64_t n, int* flag, void* stream) {
  if (n <= 0) return PG_OK;
  finite_kernel<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(in, n, flag);
  return check("check_finite");
}

// Cylindrical-coordinate pointwise forms (x = radius r, mesh.f90:172-175:
// r = x1 + (2 i - 1) dx / 2, evaluated without contraction as the mesh is).
// CellVol = d1 2 pi r d3 for one point along y, else d1 (r dy) d3 (mesh.f90:213-225).
__device__ __forceinline__ double cyl_radius(int64_t p, int nx, double x1, double dx) {
  const int i = (int)(p % nx);
  return __dadd_rn(x1, __dmul_rn(__dmul_rn((double)(2 * (i + 1) - 1), 0.5), dx));
}

// out may alias a or c (in-place forms), so no pointer is __restrict__; operands
// an op does not use may be null and are never read.
__global__ void cyl_kernel(int op, int64_t n, int nx, int ny, double x1, double dx, double dy, double dz,
                           const double* a, const double* b, const double* c, const double* e, const double* f,
                           double* out) {
  const double pi = 3.141592653589793;  // acos(-1) in FP64
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const double r = cyl_radius(p, nx, x1, dx);
    double v;
    switch (op) {
      case CYL_MUL_R: v = __dmul_rn(r, a[p]); break;                    // xgrid*f
      case CYL_MUL_R2: v = __dmul_rn(__dmul_rn(r, r), a[p]); break;     // xgrid**2*f
      case CYL_DIV_R: v = a[p] / r; break;                              // f/xgrid
      case CYL_DIVV: v = __dadd_rn(__dadd_rn(a[p], b[p]) / r, c[p]); break;  // (fA+fB)/xgrid + fC
      case CYL_DIVT_X:  // (fA+fB-fyy)/xgrid + fC
        v = __dadd_rn(__dsub_rn(__dadd_rn(a[p], b[p]), e[p]) / r, c[p]);
        break;
      case CYL_DIVT_Y:  // fA/xgrid**2 + (fB+fyx-fxy)/xgrid + fC
        v = __dadd_rn(__dadd_rn(a[p] / __dmul_rn(r, r), __dsub_rn(__dadd_rn(b[p], e[p]), f[p]) / r), c[p]);
        break;
      case CYL_D2: v = __dmul_rn(r, dy); break;
      case CYL_GRIDLEN: v = (ny == 1) ? fmin(dx, dz) : fmin(fmin(dx, __dmul_rn(r, dy)), dz); break;
      default: {  // CYL_CELLVOL_MUL / CYL_CELLVOL_DIV / CYL_CELLVOL: only the first two read a
        const double cv = (ny == 1) ? __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(dx, 2.0), pi), r), dz)
                                    : __dmul_rn(__dmul_rn(dx, __dmul_rn(r, dy)), dz);
        if (op == CYL_CELLVOL_MUL) v = __dmul_rn(a[p], cv);
        else if (op == CYL_CELLVOL_DIV) v = a[p] / cv;
        else v = cv;
      }
    }
    out[p] = v;
  }
}

int launch_cyl(int op, int64_t n, int nx, int ny, double x1, double dx, double dy, double dz, const double* a,
               const double* b, const double* c, const double* e, const double* f, double* out, void* stream) {
  // operands each form reads: a for 0-7, b and c for the divergences, e for the divT rows, f for DIVT_Y
  const bool ok = out && op >= CYL_MUL_R && op <= CYL_GRIDLEN && (op > CYL_CELLVOL_DIV || a) &&
                  (op < CYL_DIVV || op > CYL_DIVT_Y || (b && c)) && (op < CYL_DIVT_X || op > CYL_DIVT_Y || e) &&
                  (op != CYL_DIVT_Y || f);
  if (!ok) {
    set_error("cylindrical form %d: missing operand", op);
    return PG_EINVAL;
  }
  cyl_kernel<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(op, n, nx, ny, x1, dx, dy, dz, a, b, c, e, f, out);
  return check("cylindrical form");
}

int launch_mesh(int which, double* out, int nx, int ny, int nz, const double x1f[3], const double d[3],
                const double dm[3], void* stream) {
  double cval = 0.0;
  if (which >= 3 && which <= 5) cval = dm[which - 3];
  if (which == 6) cval = fmin(fmin(dm[0], dm[1]), dm[2]);
  if (which == 7) cval = d[0] * d[1] * d[2];
  const int64_t n = (int64_t)nx * ny * nz;
  mesh_kernel<<<grid_for(n), kThreads, 0, (cudaStream_t)stream>>>(which, out, nx, ny, nz, x1f[0], x1f[1], x1f[2],
                                                                  d[0], d[1], d[2], cval);
  return check("mesh");
}

}  // namespace pg

namespace pg {

int launch_seg_reduce(int op, const double* in, const long long* moff, int nmem, int64_t npts, double* partial,
                      double* out_field, double* out_member, void* stream) {
  if (op == 0) return seg_run<SEG_SUM>(in, nullptr, nullptr, nullptr, 0, 0, nullptr, moff, nmem, npts, partial,
                                        out_field, out_member, stream);
  if (op == 1) return seg_run<SEG_MAX>(in, nullptr, nullptr, nullptr, 0, 0, nullptr, moff, nmem, npts, partial,
                                        out_field, out_member, stream);
  return seg_run<SEG_MIN>(in, nullptr, nullptr, nullptr, 0, 0, nullptr, moff, nmem, npts, partial, out_field,
                          out_member, stream);
}

int launch_seg_courant(const double* u, const double* v, const double* w, const double* c, double vconst,
                       double wconst, const double* mconst, const long long* moff, int nmem, int64_t npts,
                       double* partial, double* out_field, void* stream) {
  return seg_run<SEG_COURANT>(u, v, w, c, vconst, wconst, mconst, moff, nmem, npts, partial, out_field, nullptr,
                              stream);
}

int launch_seg_diff(const double* bulk, const double* rho, const double* mconst, const long long* moff, int nmem,
                    int64_t npts, double* partial, double* out_field, void* stream) {
  return seg_run<SEG_DIFF>(bulk, rho, nullptr, nullptr, 0, 0, mconst, moff, nmem, npts, partial, out_field,
                           nullptr, stream);
}

}  // namespace pg
