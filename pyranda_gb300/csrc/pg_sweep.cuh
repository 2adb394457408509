// Directional compact-operator sweeps for sm_103a (templates; instantiated in
// pg_sweep_f64.cu and pg_sweep_f32.cu).
//
// One thread owns one grid line and streams it once forward and once
// backward:
//   forward:  RHS stencil through a register window (compact_d1.f90:113-193,
//             compact_r4.f90:106-193) fused with the forward substitution of
//             the line solve (the reference's bpentLUS3x / ppentLUS3x,
//             pentadiagonal.f90:629-684, solve the same systems from its own
//             factorisation; the tables here are the Crout / Schur-complement
//             ones of pg_setup.cpp); the forward values go to a scratch array
//             laid out [position][line], so every access to it is coalesced
//             whatever the sweep direction;
//   backward: back substitution, fused with the epilogue (filter add-back
//             compact_r4.f90:209-234, ring max operators.f90:636-639,
//             divergence accumulation) and the store.
// Nothing is staged in shared memory, so occupancy is bounded only by the
// number of lines and by registers.  y/z sweeps read and write coalesced (the
// 32 lines of a warp are 32 x-neighbours); x sweeps read each line's 32-byte
// sectors through L1.  The forward window lives in a 16-slot register ring
// that doubles as the prefetch queue; the backward loop prefetches 8 rows
// ahead.  Offsets along a line are 32-bit (fields hold fewer than 2^31
// points).  The d1 metric 1/dx is folded into the RHS weights on the host.
//
// On GB300 FP64 issues at ~1/58 of the FP32 rate (measured 1.2 TFLOP/s): the
// FP64 sweeps are bound by FP64 instruction count, the FP32 sweeps (fast path)
// by HBM.  The FP32 path converts FP64<->FP32 with integer bit operations,
// because GB300 runs F2F conversions on the FP64 pipe.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <type_traits>

#include "pg_internal.h"

namespace pg {

struct KParams {
  const double* __restrict__ in;
  double* __restrict__ out;
  void* __restrict__ scratch;  // forward-elimination values (T); member m's lines at [off_m + position*lines_m + line]
  const MemberOp* ops;         // one entry per grid of the launch
  int nops;
  long long nlines;            // lines over all grids
  int scale_pow;               // ring epilogues: scale = dm^scale_pow
  const int* emax;             // exact d8 RHS: per grid the largest exponent of `in`
};

constexpr int kSweepThreads = 128;

namespace {

template <typename T>
__device__ __forceinline__ T ldc(const T* p) { return __ldg(p); }

// FP64 -> FP32 by integer operations (GB300 runs F2F on its FP64 pipe): the
// exponent is re-biased in the high word and the mantissa rounded to nearest
// (ties away from zero).  Values below the FP32 normal range flush to signed
// zero; the fast path only sees finite field values inside the FP32 range
// (infinities and NaNs of the FP64 fields are caught by pg_check_finite).
__device__ __forceinline__ float d2f_bits(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned mag = hi & 0x7fffffffu;
  unsigned f = ((mag - (896u << 20)) << 3) | (lo >> 29);
  f += (lo >> 28) & 1u;
  f = (mag < (897u << 20)) ? 0u : f;
  return __uint_as_float(f | (hi & 0x80000000u));
}

// FP32 -> FP64 by integer operations: exact for normal numbers, zero stays
// zero (FP32 subnormals flush to zero).
__device__ __forceinline__ double f2d_bits(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned mag = u & 0x7fffffffu;
  unsigned hi = ((mag >> 3) + (896u << 20)) | (u & 0x80000000u);
  unsigned lo = u << 29;
  if (mag < 0x00800000u) { hi = u & 0x80000000u; lo = 0u; }
  return __hiloint2double((int)hi, (int)lo);
}

// FP64 -> FP32 value + FP32 residual, without the FP64 pipe: hi is d2f_bits(d)
// and r = d - hi is read from the 29 mantissa bits hi dropped (minus 2^29 when
// hi rounded up), scaled by the exponent.  hi + r carries ~48 bits of d;
// residuals of |d| < 2^-76 flush to zero.
__device__ __forceinline__ float2 split_f64(double d) {
  const unsigned dh = (unsigned)__double2hiint(d), dl = (unsigned)__double2loint(d);
  const int e = (int)((dh >> 20) & 0x7ffu);
  const int low = (int)((dl & 0x1FFFFFFFu) - (((dl >> 28) & 1u) << 29));
  float r = (float)low * __uint_as_float((unsigned)max(e - 948, 0) << 23);
  r = (e >= 948) ? r : 0.0f;
  r = (dh >> 31) ? -r : r;
  return make_float2(d2f_bits(d), r);
}

// Exact d8 RHS of the FP32 sweeps.  The 8th difference of a smooth field
// cancels about 40 of its 53 bits, more than FP32 holds.  The d8 weights are
// integers times one scale (c10d8: 60 x binomial coefficients), so every
// value of the grid becomes a 64-bit fixed-point number at the grid's largest
// binary exponent E (53 significant bits for the largest values, round half
// up), the weighted sums of the RHS are exact in 64-bit integers (at most
// 2^62 in magnitude: 254 units of weight times 2^54), and the only rounding
// is the conversion of the exact sum to FP32 before the solve.
// (branch-free, so that a prefetched load is not waited for before its use)
__device__ __forceinline__ long long to_fixed(double d, int E) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const int ex = (int)((b >> 52) & 0x7ffULL);
  const int sh = E - ex;
  const int shc = min(max(sh, 0), 62);
  const long long mant = (long long)((b & 0xfffffffffffffULL) | (1ULL << 52));
  long long m = (mant + ((1LL << shc) >> 1)) >> shc;
  m = (ex == 0 || sh >= 54) ? 0LL : m;
  return (b >> 63) ? -m : m;
}

// s x 2^(E - 1075) x w in FP32: the significand rounded to nearest even,
// below the FP32 normal range flushed to zero; NaN when E marks an infinity
// or NaN in the grid.
__device__ __forceinline__ float fixed_to_float(long long s, int E, float w) {
  if (E >= 2047) return __uint_as_float(0x7fc00000u);
  const int k = E - 1075;  // the value is s x 2^k
  if (k >= -126 && k <= 64) {
    // the hardware conversion rounds |s| to 24 bits to nearest, ties to even, as the integer
    // path below; the power of two is exact while the product stays normal (|s| < 2^63)
    float f = __ll2float_rn(s) * __uint_as_float((unsigned)(k + 127) << 23);
    if (fabsf(f) < 1.17549435e-38f) f = 0.0f;  // below the FP32 normal range: zero, as below
    f *= w;
    return f;
  }
  if (s == 0) return 0.0f;
  const unsigned long long a = (unsigned long long)(s < 0 ? -s : s);
  int top = 63 - __clzll((long long)a);
  unsigned long long sig;
  if (top <= 23) {
    sig = a << (23 - top);
  } else {
    const int sh = top - 23;
    sig = a >> sh;
    const unsigned long long rem = a & ((1ULL << sh) - 1ULL), half = 1ULL << (sh - 1);
    sig += (rem > half || (rem == half && (sig & 1ULL))) ? 1ULL : 0ULL;
    if (sig >> 24) {
      sig >>= 1;
      top++;
    }
  }
  const int be = top + E - 948;  // biased FP32 exponent of a x 2^(E - 1075)
  float f;
  if (be <= 0) f = 0.0f;
  else if (be >= 255) f = __uint_as_float(0x7f800000u);
  else f = __uint_as_float(((unsigned)be << 23) | ((unsigned)sig & 0x7fffffu));
  f *= w;
  return s < 0 ? -f : f;
}

// Running differences of a stream: after push(x_p), c[q] holds the q-th
// backward difference at p (q = 0..7) and push returns the 8th.  |x| <= 2^53
// keeps every difference within 2^61.
struct Cascade {
  long long c[8];
  __device__ __forceinline__ long long push(long long x) {
    long long t = x;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const long long u = t - c[q];
      c[q] = t;
      t = u;
    }
    return t;
  }
};

template <typename T>
__device__ __forceinline__ T from_f64(double v) { return (T)v; }
template <>
__device__ __forceinline__ float from_f64<float>(double v) { return d2f_bits(v); }
template <typename T>
__device__ __forceinline__ double to_f64(T v) { return (double)v; }

// a grid value as the RHS arithmetic's type (E: the fixed-point exponent)
template <typename TR>
__device__ __forceinline__ TR load_as(double v, int) { return from_f64<TR>(v); }
template <>
__device__ __forceinline__ long long load_as<long long>(double v, int E) { return to_fixed(v, E); }

// an RHS value as the solve's type
__device__ __forceinline__ float solve_value(float x, int, float) { return x; }
__device__ __forceinline__ double solve_value(double x, int, float) { return x; }
__device__ __forceinline__ float solve_value(long long x, int E, float w) { return fixed_to_float(x, E, w); }

// type of the RHS weight tables read by each RHS arithmetic
template <typename TR> struct WeightOf { using type = TR; };
template <> struct WeightOf<long long> { using type = int; };
template <>
__device__ __forceinline__ double to_f64<float>(float v) { return f2d_bits(v); }

template <int EPI>
__device__ __forceinline__ double epilogue(double r, double v_in, double o, double scale, bool addback) {
  const double val = addback ? r + v_in : r;
  if (EPI == EPI_STORE) return val;
  if (EPI == EPI_ADD) return o + val;
  if (EPI == EPI_RING_SET) return fabs(val) * scale;
  return fmax(o, fabs(val) * scale);
}

constexpr int kRing = 16;  // ring-buffer slots of the forward window (window + prefetch)
constexpr int kPFB = 8;    // prefetch distance of the backward loop

template <typename T> struct V4;
template <> struct V4<float> {
  float a, b, c, d;
  static __device__ __forceinline__ V4 ld(const float* p) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    return V4{v.x, v.y, v.z, v.w};
  }
};
template <> struct V4<double> {
  double a, b, c, d;
  static __device__ __forceinline__ V4 ld(const double* p) {
    const double2 u = __ldg(reinterpret_cast<const double2*>(p));
    const double2 w = __ldg(reinterpret_cast<const double2*>(p) + 1);
    return V4{u.x, u.y, w.x, w.y};
  }
};

// Access to one line of the input field (32-bit offsets from the line base).
template <typename T>
struct Line {
  const double* __restrict__ in;  // first point of the line
  int stride, n;
  int e;                          // fixed-point exponent (T = long long)
  __device__ __forceinline__ T v(int p) const { return load_as<T>(in[p * stride], e); }
  __device__ __forceinline__ T w(int p) const {  // periodic wrap
    const int q = p < 0 ? p + n : (p >= n ? p - n : p);
    return v(q);
  }
};

// RHS of one edge row (rows 0..3 and n-4..n-1) straight from the line, with
// the reference's periodic-halo formulas or, at a non-periodic end, the
// formulas of its boundary code (bcl lower end, bch upper end): the
// difference form anchored at the end point for one-sided (0), symmetric (+1)
// and extended (2) rows, plain sums for antisymmetric (-1) rows
// (compact_d1.f90:119-193, compact_r3.f90:88-157, compact_r4.f90:106-193).
template <typename T, int KIND, bool PER, typename W, typename LN>
__device__ __forceinline__ T edge_rhs(const LN& ln, int i, const W* __restrict__ R, int bcl = 0, int bch = 0) {
  const int n = ln.n;
  const W* r = R + i * 9;
  const bool lower = i < n / 2;
  const bool anti = !PER && (lower ? bcl : bch) == -1;
  if (KIND == 1) {
    if (PER)  // compact_d1.f90:141-147, :185-191 (the halo is the wrapped line)
      return ldc(r + 4) * (ln.w(i + 1) - ln.w(i - 1)) + ldc(r + 5) * (ln.w(i + 2) - ln.w(i - 2)) +
             ldc(r + 6) * (ln.w(i + 3) - ln.w(i - 3));
    if (i == 3 || i == n - 4)  // interior formula with the boundary rows' weights
      return ldc(r + 4) * (ln.v(i + 1) - ln.v(i - 1)) + ldc(r + 5) * (ln.v(i + 2) - ln.v(i - 2)) +
             ldc(r + 6) * (ln.v(i + 3) - ln.v(i - 3));
    if (anti) {  // compact_d1.f90:121-128, :163-170: sum of weights times values on the line
      T s = T(0);
      for (int l = 0; l < 7; l++) {
        const int p = i + l - 3;
        if (p >= 0 && p < n) s += ldc(r + l) * ln.v(p);
      }
      return s;
    }
    if (i == 0 || i == 1) {  // compact_d1.f90:131-134
      const T v0 = ln.v(0);
      T s = T(0);
      for (int l = (i == 0 ? 4 : 3); l <= 6; l++) s += ldc(r + l) * (ln.v(l - 3 + i) - v0);
      return s;
    }
    if (i == 2)  // compact_d1.f90:135
      return ldc(r + 4) * (ln.v(3) - ln.v(1)) + ldc(r + 5) * (ln.v(4) - ln.v(0)) + ldc(r + 6) * (ln.v(5) - ln.v(0));
    const T vn = ln.v(n - 1);
    if (i == n - 3)  // compact_d1.f90:178
      return ldc(r + 0) * (ln.v(n - 6) - vn) + ldc(r + 1) * (ln.v(n - 5) - vn) +
             ldc(r + 2) * (ln.v(n - 4) - ln.v(n - 2));
    T s = T(0);  // rows n-2, n-1 (compact_d1.f90:179-180)
    const int top = (i == n - 2) ? 3 : 2;
    for (int l = 0; l <= top; l++) s += ldc(r + l) * (ln.v(i - 3 + l) - vn);
    return s;
  }
  if (KIND == 3) {  // 7-point difference form about the row's own point (compact_r3.f90:124-136, :146-157)
    const T vc = ln.v(i);
    T s = T(0);
    if (PER) {
      for (int l = 0; l < 7; l++) s += ldc(r + l) * (ln.w(i + l - 3) - vc);
    } else {  // points beyond a non-periodic end count as zero; antisymmetric rows add (sum of weights) v_i
      T sumr = T(0);
      for (int l = 0; l < 7; l++) {
        const int p = i + l - 3;
        s += ldc(r + l) * ((p >= 0 && p < n) ? ln.v(p) - vc : -vc);
        sumr += ldc(r + l);
      }
      if (anti) s += sumr * vc;
    }
    return s;
  }
  if (PER) {  // two partial sums (compact_r4.f90:131-138, :180-189)
    const T vc = ln.v(i);
    T s1 = T(0), s2 = T(0);
    if (i < 4) {
      for (int l = 0; l <= 3 - i; l++) s1 += ldc(r + l) * (ln.v(i + l - 4 + n) - vc);
      for (int l = 4 - i; l <= 8; l++) s2 += ldc(r + l) * (ln.v(i + l - 4) - vc);
    } else {
      const int q = n - 1 - i;
      for (int l = 0; l <= 4 + q; l++) s1 += ldc(r + l) * (ln.v(i + l - 4) - vc);
      for (int l = 5 + q; l <= 8; l++) s2 += ldc(r + l) * (ln.v(i + l - 4 - n) - vc);
    }
    return s1 + s2;
  }
  T s = T(0);
  if (anti) {  // compact_r4.f90:108-117, :157-166: sum of weights times values on the line
    for (int l = 0; l < 9; l++) {
      const int p = i + l - 4;
      if (p >= 0 && p < n) s += ldc(r + l) * ln.v(p);
    }
    return s;
  }
  // one-sided / symmetric / extended closures (compact_r4.f90:120-125, :166-171)
  if (i < 4) {
    const T v0 = ln.v(0);
    for (int l = 5 - i; l <= 8; l++) s += ldc(r + l) * (ln.v(l + i - 4) - v0);
  } else {
    const T vn = ln.v(n - 1);
    const int q = n - 1 - i;
    for (int l = 0; l <= 3 + q; l++) s += ldc(r + l) * (ln.v(i + l - 4) - vn);
  }
  return s;
}

// Interior RHS from the ring: the window of row i starts at slot k.
template <typename T, int KIND>
__device__ __forceinline__ T ring_rhs(const T* ring, int k, const T* ai) {
  if (KIND == 1) {
    return ai[4] * (ring[(k + 4) % kRing] - ring[(k + 2) % kRing]) +
           ai[5] * (ring[(k + 5) % kRing] - ring[(k + 1) % kRing]) +
           ai[6] * (ring[(k + 6) % kRing] - ring[(k + 0) % kRing]);
  }
  if (KIND == 3) {
    const T vc3 = ring[(k + 3) % kRing];
    T s3 = T(0);
#pragma unroll
    for (int l = 0; l < 7; l++)
      if (l != 3) s3 += (ring[(k + l) % kRing] - vc3) * ai[l];
    return s3;
  }
  const T vc = ring[(k + 4) % kRing];
  T s = T(0);
  s += (ring[(k + 0) % kRing] - vc) * ai[0];
  s += (ring[(k + 1) % kRing] - vc) * ai[1];
  s += (ring[(k + 2) % kRing] - vc) * ai[2];
  s += (ring[(k + 3) % kRing] - vc) * ai[3];
  s += (ring[(k + 5) % kRing] - vc) * ai[5];
  s += (ring[(k + 6) % kRing] - vc) * ai[6];
  s += (ring[(k + 7) % kRing] - vc) * ai[7];
  s += (ring[(k + 8) % kRing] - vc) * ai[8];
  return s;
}

// KIND: 1 = d1 evaluator, 3 = r3 evaluator (d2, d4), 4 = r4 evaluator.  DIR: 0 = x, 1 = y, 2 = z.
// TR: the RHS arithmetic (T, or long long for the exact d8 RHS of FP32 sweeps).
template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, int DIR, int EPI, typename TR = T>
__global__ void __launch_bounds__(kSweepThreads) sweep_kernel(const KParams P) {
  constexpr bool kExact = std::is_same<TR, long long>::value;
  const int64_t L = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= P.nlines) return;
  // the grid (ensemble member) owning this line: last entry with line0 <= L
  int m = 0;
  if (P.nops > 1) {
    int lo = 0, hi = P.nops - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (P.ops[mid].line0 <= L) lo = mid;
      else hi = mid - 1;
    }
    m = lo;
  }
  const MemberOp& op = P.ops[m];
  const int64_t Lm = L - op.line0;
  const int n = op.n;
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
  const double* __restrict__ pin = P.in + base;
  double* __restrict__ pout = P.out + base;
  const int E = kExact ? __ldg(P.emax + m) : 0;
  const float wsc = kExact ? op.wscale : 1.0f;
  const Line<TR> ln{pin, st, n, E};
  using W = typename WeightOf<TR>::type;
  const W* __restrict__ R = reinterpret_cast<const W*>(kExact ? (const void*)op.rhs_i : op.rhs);
  const T* __restrict__ C = reinterpret_cast<const T*>(op.lu);  // 12 per row
  T* __restrict__ ps = reinterpret_cast<T*>(P.scratch) + op.off + Lm;  // row i at ps[i * nl]
  const int nl = (int)op.lines;
  constexpr bool kReadOut = (EPI == EPI_ADD || EPI == EPI_RING_MAX);
  const double sc = (P.scale_pow == 2) ? op.dm * op.dm : (P.scale_pow == 1 ? op.dm : 1.0);
  constexpr int H = (KIND == 4) ? 4 : 3;  // stencil half width

  // edge rows first: they may need wrapped values of the far end of the line
  T e[8];
#pragma unroll
  for (int q = 0; q < 8; q++)
    e[q] = solve_value(edge_rhs<TR, KIND, PER, W>(ln, q < 4 ? q : n - 8 + q, R, op.bcl, op.bch), E, wsc);

  auto put = [&](int p, T x, double vin, double o) {
    pout[p * st] = epilogue<EPI>(to_f64<T>(x), vin, o, sc, ADDBACK);
  };
  auto put_load = [&](int p, T x) {
    const double vin = ADDBACK ? pin[p * st] : 0.0;
    const double o = kReadOut ? pout[p * st] : 0.0;
    put(p, x, vin, o);
  };

  // ---------------------------------------------------------------- forward
  // Solve tables (12 per row, pg_setup.cpp solve_tables): forward
  // z_i = rho r_i - alpha z_{i-1} - beta z_{i-2}; on periodic lines also the
  // border sums t0 += G_0i z_i, t1 += G_1i z_i over rows 0..n-3.  Rows whose
  // multipliers reach before the line start hold zeros, so every row takes the
  // same formula.
  T rm1 = T(0), rm2 = T(0), t1 = T(0), t2 = T(0), rN1 = T(0), rN = T(0);
  auto fwd_row = [&](int i, T rhs) {
    const V4<T> f = V4<T>::ld(C + i * 12);  // rho alpha beta G_0i
    T z = f.a * rhs;
    z -= f.c * rm2;
    z -= f.b * rm1;
    if (PER) {
      t1 += f.d * z;
      t2 += ldc(C + i * 12 + 8) * z;
    }
    return z;
  };
  // edge rows (0..3 and n-4..n-1)
  auto fwd_edge = [&](int i, T rhs) {
    if (!IMPL) {
      put_load(i, rhs);
      return;
    }
    if (PER && i >= n - 2) {  // the two border unknowns are solved after the sweep
      if (i == n - 2) rN1 = rhs;
      else rN = rhs;
      return;
    }
    const T z = fwd_row(i, rhs);
    if (i < n - 2) ps[i * nl] = z;
    rm2 = rm1;
    rm1 = z;
  };
  // interior rows (4 <= i <= n-5)
  auto fwd_in = [&](int i, T rhs) {
    if (!IMPL) {
      put_load(i, rhs);
      return;
    }
    const T z = fwd_row(i, rhs);
    ps[i * nl] = z;
    rm2 = rm1;
    rm1 = z;
  };

  // implicit: the first rows' forward elimination; explicit operators store them after the window
  // below is filled, so that an in-place call (in == out) still reads the original rows 0..3
  if (IMPL) {
#pragma unroll
    for (int q = 0; q < 4; q++) fwd_edge(q, e[q]);
  }

  // interior rows 4 .. n-5: ring[s] holds v[i0 - H + s] at the start of a block
  // of kRing rows; the slot of the oldest value is refilled kRing positions ahead
  {
    TR ai[9];
#pragma unroll
    for (int k = 0; k < 9; k++) ai[k] = kExact ? (TR)op.iw[k] : (TR)op.ri[k];
    // the exact RHS keeps the raw FP64 values in the ring and converts a value when it is used
    using RT = typename std::conditional<kExact, double, TR>::type;
    auto ld = [&](int p) -> RT {
      if constexpr (kExact) return pin[p * st];
      else return ln.v(p);
    };
    RT ring[kRing];
#pragma unroll
    for (int s2 = 0; s2 < kRing; s2++) {
      const int p = 4 - H + s2;
      ring[s2] = (p < n) ? ld(p) : RT(0);
    }
    if (!IMPL) {
#pragma unroll
      for (int q = 0; q < 4; q++) fwd_edge(q, e[q]);
    }
    // exact d8: the interior weights are iw[0] x (1, -8, 28, -56, 70, -56, 28, -8, 1), so the
    // RHS of row i is iw[0] times the 8th backward difference at i + 4, kept by a cascade of
    // first differences (8 integer subtractions per point); primed with points 0..7
    Cascade cas{};
    if constexpr (kExact) {
#pragma unroll
      for (int s2 = 0; s2 < 8; s2++) cas.push(to_fixed(ring[s2], E));
    }
    const float wi = kExact ? wsc * (float)op.iw[0] : 0.0f;
    auto rhs_at = [&](int k) -> T {
      if constexpr (kExact) return fixed_to_float(cas.push(to_fixed(ring[(k + 8) % kRing], E)), E, wi);
      else return solve_value(ring_rhs<TR, KIND>(ring, k, ai), E, wsc);
    };
    int i0 = 4;
    for (; i0 + kRing <= n - 4; i0 += kRing) {  // whole blocks: no guards
#pragma unroll
      for (int k = 0; k < kRing; k++) {
        const int i = i0 + k;
        const T rhs = rhs_at(k);
        const int p = i - H + kRing;
        ring[k] = (p < n) ? ld(p) : RT(0);
        fwd_in(i, rhs);
      }
    }
#pragma unroll
    for (int k = 0; k < kRing; k++) {  // last partial block
      const int i = i0 + k;
      if (i <= n - 5) {
        const T rhs = rhs_at(k);
        const int p = i - H + kRing;
        ring[k] = (p < n) ? ld(p) : RT(0);
        fwd_in(i, rhs);
      }
    }
  }

#pragma unroll
  for (int q = 4; q < 8; q++) fwd_edge(n - 8 + q, e[q]);
  if (!IMPL) return;

  // --------------------------------------------------------------- backward
  // x_i = z_i - u1 x_{i+1} - u2 x_{i+2} (- F_i0 x_{n-2} - F_i1 x_{n-1} on periodic lines)
  T x1, x2, xa = T(0), xb = T(0);
  if (PER) {  // border unknowns x_B = S^-1 (r_B - t); S^-1 sits in row n-2
    const V4<T> si = V4<T>::ld(C + (n - 2) * 12);
    const T b0 = rN1 - t1, b1 = rN - t2;
    xa = si.a * b0 + si.b * b1;
    xb = si.c * b0 + si.d * b1;
    put_load(n - 1, xb);
    put_load(n - 2, xa);
    x1 = T(0);  // the interior block's band ends at row n-3; F carries the coupling to x_B
    x2 = T(0);
  } else {  // the last two forward values are still in registers
    x2 = rm1;
    x1 = rm2 - ldc(C + (n - 2) * 12 + 4) * x2;
    put_load(n - 1, x2);
    put_load(n - 2, x1);
  }
  T pr[kPFB];
  double pv[kPFB], po[kPFB];
#pragma unroll
  for (int k = 0; k < kPFB; k++) {
    const int p = n - 3 - k;
    pr[k] = (p >= 0) ? ps[p * nl] : T(0);
    pv[k] = (ADDBACK && p >= 0) ? pin[p * st] : 0.0;
    po[k] = (kReadOut && p >= 0) ? pout[p * st] : 0.0;
  }
  for (int i = n - 3; i >= 0; i -= kPFB) {
#pragma unroll
    for (int k = 0; k < kPFB; k++) {
      const int ii = i - k;
      if (ii >= 0) {
        const T z = pr[k];
        const double vin = pv[k], o = po[k];
        const int p = ii - kPFB;
        pr[k] = (p >= 0) ? ps[p * nl] : T(0);
        if (ADDBACK) pv[k] = (p >= 0) ? pin[p * st] : 0.0;
        if (kReadOut) po[k] = (p >= 0) ? pout[p * st] : 0.0;
        const V4<T> g = V4<T>::ld(C + ii * 12 + 4);  // u1 u2 F_i0 F_i1
        T x = z;
        if (PER) {
          x -= g.d * xb;
          x -= g.c * xa;
        }
        x -= g.b * x2;
        x -= g.a * x1;  // short chain through x1: one fused multiply-add
        x2 = x1;
        x1 = x;
        put(ii, x, vin, o);
      }
    }
  }
}

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, int DIR, int EPI, typename TR = T>
int launch_t(const KParams& P, void* stream) {
  const int64_t nb = (P.nlines + kSweepThreads - 1) / kSweepThreads;
  sweep_kernel<T, KIND, PER, IMPL, ADDBACK, DIR, EPI, TR>
      <<<(unsigned)nb, kSweepThreads, 0, (cudaStream_t)stream>>>(P);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("sweep launch: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, unsigned EPIS, typename TR, int DIR>
int dispatch_epi(const KParams& P, int epi, void* st) {
  if constexpr ((EPIS >> EPI_STORE) & 1u)
    if (epi == EPI_STORE) return launch_t<T, KIND, PER, IMPL, ADDBACK, DIR, EPI_STORE, TR>(P, st);
  if constexpr ((EPIS >> EPI_ADD) & 1u)
    if (epi == EPI_ADD) return launch_t<T, KIND, PER, IMPL, ADDBACK, DIR, EPI_ADD, TR>(P, st);
  if constexpr ((EPIS >> EPI_RING_SET) & 1u)
    if (epi == EPI_RING_SET) return launch_t<T, KIND, PER, IMPL, ADDBACK, DIR, EPI_RING_SET, TR>(P, st);
  if constexpr ((EPIS >> EPI_RING_MAX) & 1u)
    if (epi == EPI_RING_MAX) return launch_t<T, KIND, PER, IMPL, ADDBACK, DIR, EPI_RING_MAX, TR>(P, st);
  set_error("sweep: epilogue %d is not built for this operator", epi);
  return PG_EINVAL;
}

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, unsigned EPIS, typename TR = T>
int dispatch_dir_epi(const KParams& P, int dir, int epi, void* st) {
  if (dir == 0) return dispatch_epi<T, KIND, PER, IMPL, ADDBACK, EPIS, TR, 0>(P, epi, st);
  if (dir == 1) return dispatch_epi<T, KIND, PER, IMPL, ADDBACK, EPIS, TR, 1>(P, epi, st);
  return dispatch_epi<T, KIND, PER, IMPL, ADDBACK, EPIS, TR, 2>(P, epi, st);
}

// The 3- and 7-point operators (d1, d2, d4) and the 9-point ones (d8, the
// filters), in separate functions so that a translation unit can instantiate
// one family.
template <typename T>
int dispatch_kind_r3(const OpRef& op, const KParams& P, int dir, int epi, void* st) {
  switch (op.kind) {
    case OPK_D1:
      return op.periodic ? dispatch_dir_epi<T, 1, true, true, false, kEpiStoreAdd>(P, dir, epi, st)
                         : dispatch_dir_epi<T, 1, false, true, false, kEpiStoreAdd>(P, dir, epi, st);
    case OPK_D2:
      return op.periodic ? dispatch_dir_epi<T, 3, true, true, false, kEpiStoreAdd>(P, dir, epi, st)
                         : dispatch_dir_epi<T, 3, false, true, false, kEpiStoreAdd>(P, dir, epi, st);
    case OPK_D4:
      return op.periodic ? dispatch_dir_epi<T, 3, true, false, false, kEpiStore>(P, dir, epi, st)
                         : dispatch_dir_epi<T, 3, false, false, false, kEpiStore>(P, dir, epi, st);
    default:
      set_error("sweep: operator %d is not a 3- or 7-point operator", op.kind);
      return PG_EINVAL;
  }
}

template <typename T>
int dispatch_kind_r4(const OpRef& op, const KParams& P, int dir, int epi, void* st) {
  switch (op.kind) {
    case OPK_D8: {
      // FP32 sweeps take the exact fixed-point RHS where the weights allow it
      using TRX = typename std::conditional<std::is_same<T, float>::value, long long, T>::type;
      if (std::is_same<T, float>::value && op.exact)
        return op.periodic ? dispatch_dir_epi<T, 4, true, true, false, kEpiRing, TRX>(P, dir, epi, st)
                           : dispatch_dir_epi<T, 4, false, true, false, kEpiRing, TRX>(P, dir, epi, st);
      return op.periodic ? dispatch_dir_epi<T, 4, true, true, false, kEpiRing>(P, dir, epi, st)
                         : dispatch_dir_epi<T, 4, false, true, false, kEpiRing>(P, dir, epi, st);
    }
    case OPK_SF:
      return op.periodic ? dispatch_dir_epi<T, 4, true, true, true, kEpiStore>(P, dir, epi, st)
                         : dispatch_dir_epi<T, 4, false, true, true, kEpiStore>(P, dir, epi, st);
    case OPK_GF:
      return op.periodic ? dispatch_dir_epi<T, 4, true, false, true, kEpiStore>(P, dir, epi, st)
                         : dispatch_dir_epi<T, 4, false, false, true, kEpiStore>(P, dir, epi, st);
    default:
      set_error("sweep: operator %d is not a 9-point operator", op.kind);
      return PG_EINVAL;
  }
}

template <typename T>
int dispatch_kind(const OpRef& op, const KParams& P, int dir, int epi, void* st) {
  return (op.kind == OPK_D1 || op.kind == OPK_D2 || op.kind == OPK_D4) ? dispatch_kind_r3<T>(op, P, dir, epi, st)
                                                                       : dispatch_kind_r4<T>(op, P, dir, epi, st);
}

}  // namespace

}  // namespace pg
