// Directional compact-operator sweeps for sm_103a.
//
// One CTA owns a tile of LB lines (LB = blockDim.x, one thread per line) and
// the whole length n of those lines.  The tile is staged in shared memory with
// coalesced loads (x lines: each line is contiguous; y/z lines: the LB lines
// are LB consecutive x positions), then every thread evaluates its own line
// in place in shared memory:
//   1. RHS stencil      compact_d1.f90:113-193 (d1) / compact_r4.f90:106-193 (r4)
//   2. banded solve     pentadiagonal.f90:629-651 (bpentLUS3x)
//      or cyclic solve  pentadiagonal.f90:654-684 (ppentLUS3x)
//   3. fused epilogue   filter add-back (compact_r4.f90:209-234), ring max
//                       (operators.f90:636-639), divergence accumulation
// and the tile is written back coalesced.  The d1 metric 1/dx is folded into
// the RHS weights on the host.
//
// On GB300 FP64 issues at ~1/58 of the FP32 rate (measured 1.2 TFLOP/s), so
// these sweeps are bound by FP64 instruction count, not by HBM; the kernel is
// written to keep the FP64 work per point minimal (FMA-contracted forms) and
// leaves loads, address arithmetic and the tile transpose to the other pipes.
#include <cuda_runtime.h>

#pragma once
#include <cstdio>

#include "pg_internal.h"

namespace pg {

struct KParams {
  const double* __restrict__ in;
  double* __restrict__ out;
  const void* rhs;  // n x 9 per-row RHS weights (T)
  const void* lu;   // n x 9 per-row solve coefficients (T)
  int n, nx, ny, nz;
  int tiles_i;      // y/z sweeps: number of LB-wide tiles along x
  double epi_scale;
  double ri[9];     // interior RHS weights
};

namespace {



template <typename T>
__device__ __forceinline__ T ldc(const T* p) { return __ldg(p); }

// ---------------------------------------------------------------------------
// RHS of one line, in place on a shared-memory column c[p*lds].
// Edge rows (4 per side) are evaluated first from the untouched column and
// kept in registers; the interior rows then stream through a register window.
// ---------------------------------------------------------------------------
template <typename T, bool PER>
__device__ __forceinline__ void rhs_d1(T* c, int lds, int n, const T* __restrict__ R,
                                       const T a5, const T a6, const T a7) {
  auto V = [&](int p) -> T { return c[p * lds]; };
  auto W = [&](int p) -> T { return c[((p % n + n) % n) * lds]; };
  T e[8];
  if (PER) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int i = q < 4 ? q : n - 8 + q;
      const T* r = R + i * 9;
      e[q] = ldc(r + 4) * (W(i + 1) - W(i - 1)) + ldc(r + 5) * (W(i + 2) - W(i - 2)) +
             ldc(r + 6) * (W(i + 3) - W(i - 3));
    }
  } else {
    // one-sided closures, boundary code 0 (compact_d1.f90:131-139, :175-183)
    const T* r0 = R;
    const T* r1 = R + 9;
    const T* r2 = R + 18;
    const T* r3 = R + 27;
    const T v0 = V(0), v1 = V(1), v2 = V(2), v3 = V(3), v4 = V(4), v5 = V(5), v6 = V(6);
    T s = T(0);
    s += ldc(r0 + 4) * (v1 - v0);
    s += ldc(r0 + 5) * (v2 - v0);
    s += ldc(r0 + 6) * (v3 - v0);
    e[0] = s;
    s = T(0);
    s += ldc(r1 + 3) * (v1 - v0);
    s += ldc(r1 + 4) * (v2 - v0);
    s += ldc(r1 + 5) * (v3 - v0);
    s += ldc(r1 + 6) * (v4 - v0);
    e[1] = s;
    e[2] = ldc(r2 + 4) * (v3 - v1) + ldc(r2 + 5) * (v4 - v0) + ldc(r2 + 6) * (v5 - v0);
    e[3] = ldc(r3 + 4) * (v4 - v2) + ldc(r3 + 5) * (v5 - v1) + ldc(r3 + 6) * (v6 - v0);
    const int m = n - 1;
    const T u0 = V(m), u1 = V(m - 1), u2 = V(m - 2), u3 = V(m - 3), u4 = V(m - 4), u5 = V(m - 5),
            u6 = V(m - 6);
    const T* q4 = R + (m - 3) * 9;
    const T* q5 = R + (m - 2) * 9;
    const T* q6 = R + (m - 1) * 9;
    const T* q7 = R + m * 9;
    e[4] = ldc(q4 + 4) * (u2 - u4) + ldc(q4 + 5) * (u1 - u5) + ldc(q4 + 6) * (u0 - u6);
    e[5] = ldc(q5 + 0) * (u5 - u0) + ldc(q5 + 1) * (u4 - u0) + ldc(q5 + 2) * (u3 - u1);
    s = T(0);
    s += ldc(q6 + 0) * (u4 - u0);
    s += ldc(q6 + 1) * (u3 - u0);
    s += ldc(q6 + 2) * (u2 - u0);
    s += ldc(q6 + 3) * (u1 - u0);
    e[6] = s;
    s = T(0);
    s += ldc(q7 + 0) * (u3 - u0);
    s += ldc(q7 + 1) * (u2 - u0);
    s += ldc(q7 + 2) * (u1 - u0);
    e[7] = s;
  }
  // interior rows 4 .. n-5 through a 7-point register window
  T w0 = V(1), w1 = V(2), w2 = V(3), w3 = V(4), w4 = V(5), w5 = V(6), w6 = V(7);
  for (int i = 4; i <= n - 5; i++) {
    const T r = a5 * (w4 - w2) + a6 * (w5 - w1) + a7 * (w6 - w0);
    const T nxt = (i + 4 < n) ? V(i + 4) : T(0);
    c[i * lds] = r;
    w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = w5; w5 = w6; w6 = nxt;
  }
#pragma unroll
  for (int q = 0; q < 8; q++) c[(q < 4 ? q : n - 8 + q) * lds] = e[q];
}

template <typename T, bool PER>
__device__ __forceinline__ void rhs_r4(T* c, int lds, int n, const T* __restrict__ R, const T* ai) {
  auto V = [&](int p) -> T { return c[p * lds]; };
  T e[8];
  if (PER) {
    // periodic halo rows: two partial sums as compact_r4.f90:131-138, :180-189
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const T* r = R + i * 9;
      const T vc = V(i);
      T s1 = T(0), s2 = T(0);
      for (int l = 0; l <= 3 - i; l++) s1 += ldc(r + l) * (V(i + l - 4 + n) - vc);
      for (int l = 4 - i; l <= 8; l++) s2 += ldc(r + l) * (V(i + l - 4) - vc);
      e[i] = s1 + s2;
    }
#pragma unroll
    for (int q = 3; q >= 0; q--) {
      const int i = n - 1 - q;
      const T* r = R + i * 9;
      const T vc = V(i);
      T s1 = T(0), s2 = T(0);
      for (int l = 0; l <= 4 + q; l++) s1 += ldc(r + l) * (V(i + l - 4) - vc);
      for (int l = 5 + q; l <= 8; l++) s2 += ldc(r + l) * (V(i + l - 4 - n) - vc);
      e[7 - q] = s1 + s2;
    }
  } else {
    // one-sided closures (compact_r4.f90:120-125, :166-171)
    const T v0 = V(0), vn = V(n - 1);
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const T* r = R + i * 9;
      T s = T(0);
      for (int l = 5 - i; l <= 8; l++) s += ldc(r + l) * (V(l + i - 4) - v0);
      e[i] = s;
    }
#pragma unroll
    for (int q = 3; q >= 0; q--) {
      const int i = n - 1 - q;
      const T* r = R + i * 9;
      T s = T(0);
      for (int l = 0; l <= 3 + q; l++) s += ldc(r + l) * (V(i + l - 4) - vn);
      e[7 - q] = s;
    }
  }
  // interior rows 4 .. n-5: sum_l (v[i+l-4] - v[i]) * a_l   (compact_r4.f90:144-156)
  T w[9];
#pragma unroll
  for (int k = 0; k < 9; k++) w[k] = (k < n) ? V(k) : T(0);  // n == 8 has no interior row
  for (int i = 4; i <= n - 5; i++) {
    const T vc = w[4];
    T s = T(0);
    s += (w[0] - vc) * ai[0];
    s += (w[1] - vc) * ai[1];
    s += (w[2] - vc) * ai[2];
    s += (w[3] - vc) * ai[3];
    s += (w[5] - vc) * ai[5];
    s += (w[6] - vc) * ai[6];
    s += (w[7] - vc) * ai[7];
    s += (w[8] - vc) * ai[8];
    const T nxt = (i + 5 < n) ? V(i + 5) : T(0);
    c[i * lds] = s;
#pragma unroll
    for (int k = 0; k < 8; k++) w[k] = w[k + 1];
    w[8] = nxt;
  }
#pragma unroll
  for (int q = 0; q < 8; q++) c[(q < 4 ? q : n - 8 + q) * lds] = e[q];
}

// bpentLUS3x on one column (pentadiagonal.f90:629-651), pull form of the
// forward elimination: r_k -= r_{k-2} c1_k ; r_k -= r_{k-1} c2_k.
template <typename T>
__device__ __forceinline__ void solve_banded(T* c, int lds, int n, const T* __restrict__ L) {
  T rm2 = c[0];
  T rm1 = c[lds] - rm2 * ldc(L + 9 + 1);
  c[lds] = rm1;
  for (int i = 2; i < n; i++) {
    const T* l = L + i * 9;
    const T r = (c[i * lds] - rm2 * ldc(l + 0)) - rm1 * ldc(l + 1);
    c[i * lds] = r;
    rm2 = rm1;
    rm1 = r;
  }
  T x2 = rm1 * ldc(L + (n - 1) * 9 + 2);
  c[(n - 1) * lds] = x2;
  T x1 = (rm2 - ldc(L + (n - 2) * 9 + 3) * x2) * ldc(L + (n - 2) * 9 + 2);
  c[(n - 2) * lds] = x1;
  for (int i = n - 3; i >= 0; i--) {
    const T* l = L + i * 9;
    const T x = (c[i * lds] - ldc(l + 3) * x1 - ldc(l + 4) * x2) * ldc(l + 2);
    c[i * lds] = x;
    x2 = x1;
    x1 = x;
  }
}

// ppentLUS3x on one column (pentadiagonal.f90:654-684): bordered LU of the
// cyclic pentadiagonal system.
template <typename T>
__device__ __forceinline__ void solve_cyclic(T* c, int lds, int n, const T* __restrict__ L) {
  T rm2 = c[0];
  T rm1 = c[lds] - ldc(L + 9 + 1) * rm2;
  c[lds] = rm1;
  T t1 = ldc(L + 5) * rm2 + ldc(L + 9 + 5) * rm1;
  T t2 = ldc(L + 6) * rm2 + ldc(L + 9 + 6) * rm1;
  for (int i = 2; i <= n - 3; i++) {
    const T* l = L + i * 9;
    const T r = c[i * lds] - ldc(l + 1) * rm1 - ldc(l + 0) * rm2;
    c[i * lds] = r;
    t1 += ldc(l + 5) * r;
    t2 += ldc(l + 6) * r;
    rm2 = rm1;
    rm1 = r;
  }
  const T* la = L + (n - 2) * 9;
  const T* lb = L + (n - 1) * 9;
  const T rN1 = c[(n - 2) * lds] - t1;
  const T xN = (c[(n - 1) * lds] - t2 - ldc(la + 6) * rN1) * ldc(lb + 2);
  const T xN1 = (rN1 - ldc(la + 8) * xN) * ldc(la + 2);
  c[(n - 1) * lds] = xN;
  c[(n - 2) * lds] = xN1;
  T x1 = xN1, x2 = xN;
  for (int i = n - 3; i >= 0; i--) {
    const T* l = L + i * 9;
    const T x = (c[i * lds] - ldc(l + 3) * x1 - ldc(l + 4) * x2 - ldc(l + 7) * xN1 - ldc(l + 8) * xN) *
                ldc(l + 2);
    c[i * lds] = x;
    x2 = x1;
    x1 = x;
  }
}

template <int EPI>
__device__ __forceinline__ double epilogue(double r, double v_in, double* o, double scale, bool addback) {
  const double val = addback ? r + v_in : r;
  if (EPI == EPI_STORE) return val;
  if (EPI == EPI_ADD) return *o + val;
  if (EPI == EPI_RING_SET) return fabs(val) * scale;
  return fmax(*o, fabs(val) * scale);
}

// KIND: 1 = d1 evaluator, 4 = r4 evaluator.  DIR: 0 = x, 1 = y, 2 = z.
template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, int DIR, int EPI>
__global__ void __launch_bounds__(32) sweep_kernel(const KParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  const int lb = blockDim.x;
  const int lds = lb + 1;
  const int t = threadIdx.x;
  const int n = P.n, nx = P.nx, ny = P.ny;

  // tile decode
  int64_t base_t;   // base offset of this thread's line
  int64_t stride;   // element stride along the line
  bool valid;
  int64_t line0 = 0;
  int nlines = 0;
  if (DIR == 0) {
    const int64_t total = (int64_t)ny * P.nz;
    line0 = (int64_t)blockIdx.x * lb;
    nlines = (int)(total - line0 < (int64_t)lb ? total - line0 : (int64_t)lb);
    valid = t < nlines;
    base_t = (line0 + t) * nx;
    stride = 1;
  } else {
    const int b = blockIdx.x;
    const int ti = b % P.tiles_i;
    const int outer = b / P.tiles_i;
    const int i = ti * lb + t;
    valid = i < nx;
    if (DIR == 1) {
      base_t = (int64_t)outer * nx * ny + i;
      stride = nx;
    } else {
      base_t = (int64_t)outer * nx + i;
      stride = (int64_t)nx * ny;
    }
  }

  // stage the tile
  if (DIR == 0) {
    for (int l = 0; l < nlines; l++) {
      const double* src = P.in + (line0 + l) * nx;
      for (int p = t; p < n; p += lb) s[p * lds + l] = (T)src[p];
    }
  } else if (valid) {
    const double* src = P.in + base_t;
    int p = 0;
    for (; p + 4 <= n; p += 4) {
      const double a0 = src[(int64_t)p * stride], a1 = src[(int64_t)(p + 1) * stride];
      const double a2 = src[(int64_t)(p + 2) * stride], a3 = src[(int64_t)(p + 3) * stride];
      s[p * lds + t] = (T)a0;
      s[(p + 1) * lds + t] = (T)a1;
      s[(p + 2) * lds + t] = (T)a2;
      s[(p + 3) * lds + t] = (T)a3;
    }
    for (; p < n; p++) s[p * lds + t] = (T)src[(int64_t)p * stride];
  }
  __syncthreads();

  if (valid) {
    T* c = s + t;
    const T* R = reinterpret_cast<const T*>(P.rhs);
    const T* L = reinterpret_cast<const T*>(P.lu);
    if (KIND == 1) {
      rhs_d1<T, PER>(c, lds, n, R, (T)P.ri[4], (T)P.ri[5], (T)P.ri[6]);
    } else {
      T ai[9];
#pragma unroll
      for (int k = 0; k < 9; k++) ai[k] = (T)P.ri[k];
      rhs_r4<T, PER>(c, lds, n, R, ai);
    }
    if (IMPL) {
      if (PER) solve_cyclic<T>(c, lds, n, L);
      else solve_banded<T>(c, lds, n, L);
    }
  }
  __syncthreads();

  // write back with the fused epilogue
  const double sc = P.epi_scale;
  if (DIR == 0) {
    for (int l = 0; l < nlines; l++) {
      const int64_t off = (line0 + l) * nx;
      for (int p = t; p < n; p += lb) {
        const double r = (double)s[p * lds + l];
        const double vin = ADDBACK ? P.in[off + p] : 0.0;
        P.out[off + p] = epilogue<EPI>(r, vin, P.out + off + p, sc, ADDBACK);
      }
    }
  } else if (valid) {
    for (int p = 0; p < n; p++) {
      const int64_t off = base_t + (int64_t)p * stride;
      const double r = (double)s[p * lds + t];
      const double vin = ADDBACK ? P.in[off] : 0.0;
      P.out[off] = epilogue<EPI>(r, vin, P.out + off, sc, ADDBACK);
    }
  }
}

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, int DIR, int EPI>
int launch_t(const KParams& P, int lb, int64_t nblocks, void* stream) {
  auto kern = sweep_kernel<T, KIND, PER, IMPL, ADDBACK, DIR, EPI>;
  const size_t smem = (size_t)P.n * (lb + 1) * sizeof(T);
  static bool attr_set = false;
  static size_t attr_val = 0;
  if (!attr_set || attr_val < smem) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error("cudaFuncSetAttribute(smem=%zu): %s", smem, cudaGetErrorString(e));
      return PG_ECUDA;
    }
    attr_set = true;
    attr_val = smem;
  }
  kern<<<(unsigned)nblocks, lb, smem, (cudaStream_t)stream>>>(P);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("sweep launch: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK>
int dispatch_dir_epi(const KParams& P, int dir, int epi, int lb, int64_t nb, void* st) {
#define PG_EPI_CASES(D)                                                                   \
  switch (epi) {                                                                          \
    case EPI_STORE: return launch_t<T, KIND, PER, IMPL, ADDBACK, D, EPI_STORE>(P, lb, nb, st);       \
    case EPI_ADD: return launch_t<T, KIND, PER, IMPL, ADDBACK, D, EPI_ADD>(P, lb, nb, st);           \
    case EPI_RING_SET: return launch_t<T, KIND, PER, IMPL, ADDBACK, D, EPI_RING_SET>(P, lb, nb, st); \
    default: return launch_t<T, KIND, PER, IMPL, ADDBACK, D, EPI_RING_MAX>(P, lb, nb, st);           \
  }
  if (dir == 0) { PG_EPI_CASES(0) }
  if (dir == 1) { PG_EPI_CASES(1) }
  PG_EPI_CASES(2)
#undef PG_EPI_CASES
}

template <typename T>
int dispatch_kind(const DevOp& op, const KParams& P, int dir, int epi, int lb, int64_t nb, void* st) {
  switch (op.kind) {
    case OPK_D1:
      return op.periodic ? dispatch_dir_epi<T, 1, true, true, false>(P, dir, epi, lb, nb, st)
                         : dispatch_dir_epi<T, 1, false, true, false>(P, dir, epi, lb, nb, st);
    case OPK_D8:
      return op.periodic ? dispatch_dir_epi<T, 4, true, true, false>(P, dir, epi, lb, nb, st)
                         : dispatch_dir_epi<T, 4, false, true, false>(P, dir, epi, lb, nb, st);
    case OPK_SF:
      return op.periodic ? dispatch_dir_epi<T, 4, true, true, true>(P, dir, epi, lb, nb, st)
                         : dispatch_dir_epi<T, 4, false, true, true>(P, dir, epi, lb, nb, st);
    default:
      return op.periodic ? dispatch_dir_epi<T, 4, true, false, true>(P, dir, epi, lb, nb, st)
                         : dispatch_dir_epi<T, 4, false, false, true>(P, dir, epi, lb, nb, st);
  }
}

}  // namespace

}  // namespace pg
