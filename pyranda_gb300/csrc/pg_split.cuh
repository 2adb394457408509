// Shared parts of the split-line sweeps: launch parameters, the tile
// accessors and RHS windows, shared-memory layout helpers, and the
// register-resident kernel (seg_kernel, instantiated by pg_seg_r3.cu and
// pg_seg_r4.cu).  pg_split.cu holds the tile form and the dispatch.
#pragma once
#include "pg_sweep.cuh"

namespace pg {

struct SParams {  // one split-sweep launch
  const double* in;  // may equal out: a CTA reads all of its lines before it writes any
  double* out;
  const MemberOp* ops;
  const SplitOp* sops;
  const SplitTile* tiles;
  int scale_pow;
  const int* emax;
};

// Launch the register-resident form for one operator (epi: pg_epilogue).
// pg_seg_r3.cu: d1, d2, d4 (KIND 1 and 3); pg_seg_r4.cu: d8, the filters (KIND 4).
int seg_launch_r3(const OpRef& op, const SParams& P, const SplitSet& ss, int dir, int epi, void* stream);
int seg_launch_r4(const OpRef& op, const SParams& P, const SplitSet& ss, int dir, int epi, void* stream);


namespace {

constexpr int kSplitThreads = 256;
constexpr int kBatch = 8;  // global loads a thread has in flight in the load and store phases


// One line of the tile in shared memory (raw FP64 values), read as the RHS
// arithmetic's type -- the accessors edge_rhs uses.
template <typename TR>
struct SLine {
  const double* v0;
  int n, e;
  __device__ __forceinline__ TR v(int p) const { return load_as<TR>(v0[p], e); }
  __device__ __forceinline__ TR w(int p) const {
    const int q = p < 0 ? p + n : (p >= n ? p - n : p);
    return v(q);
  }
};

// The RHS of an interior row from its window of 2H+1 values (win[H] = the
// row's own point), in the difference form of the reference
// (compact_d1.f90:152-160, compact_r3.f90, compact_r4.f90:144-156).
// Values are FP64 (T = double) or FP32 hi + lo pairs (T = float): every
// difference v_k - v_c is (hi_k - hi_c) + (lo_k - lo_c), exact to FP32
// rounding of the difference itself, so a large mean or a slowly varying
// field costs no accuracy before the weights are applied.
template <int KIND>
__device__ __forceinline__ double window_rhs(const double* v, const double* ai) {
  if (KIND == 1) return ai[4] * (v[4] - v[2]) + ai[5] * (v[5] - v[1]) + ai[6] * (v[6] - v[0]);
  constexpr int H = (KIND == 4) ? 4 : 3;
  double s = 0.0;
#pragma unroll
  for (int l = 0; l < 2 * H + 1; l++)
    if (l != H) s += (v[l] - v[H]) * ai[l];
  return s;
}
template <int KIND>
__device__ __forceinline__ float window_rhs(const float2* v, const float* ai) {
  auto d = [&](int k, int c) { return (v[k].x - v[c].x) + (v[k].y - v[c].y); };
  if (KIND == 1) return ai[4] * d(4, 2) + ai[5] * d(5, 1) + ai[6] * d(6, 0);
  if (KIND == 4) {
    // the 9-point operators (d8, both filters) have symmetric interior weights
    // (checked when the tables are built): the hi differences pair up about the
    // centre, and the residuals, small against the differences, enter as
    // sum_k a_k (lo_{+k} + lo_{-k}) - 2 (sum_k a_k) lo_c
    float s = 0.0f, sl = 0.0f, a2 = 0.0f;
#pragma unroll
    for (int k = 1; k <= 4; k++) {
      s += ai[4 + k] * ((v[4 + k].x - v[4].x) + (v[4 - k].x - v[4].x));
      sl += ai[4 + k] * (v[4 + k].y + v[4 - k].y);
      a2 += ai[4 + k];
    }
    return s + (sl - 2.0f * a2 * v[4].y);
  }
  constexpr int H = (KIND == 4) ? 4 : 3;
  float s = 0.0f;
#pragma unroll
  for (int l = 0; l < 2 * H + 1; l++)
    if (l != H) s += d(l, H) * ai[l];
  return s;
}

// A thread's result of row i in the 8-byte slot of its input value: FP64 as
// is, FP32 as the first half of an 8-byte access (a 4-byte access at an
// 8-byte stride would meet 2-way bank conflicts across the lanes' rows).
__device__ __forceinline__ void slot_st(double* p, double v) { *p = v; }
__device__ __forceinline__ void slot_st(double* p, float v) {
  asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"((unsigned)__cvta_generic_to_shared(p)), "f"(v), "f"(0.0f)
               : "memory");
}
template <typename T>
__device__ __forceinline__ T slot_ld(const double* p);
template <>
__device__ __forceinline__ double slot_ld<double>(const double* p) { return *p; }
template <>
__device__ __forceinline__ float slot_ld<float>(const double* p) {
  float a;
  [[maybe_unused]] float b;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(a), "=f"(b) : "r"((unsigned)__cvta_generic_to_shared(p))
               : "memory");
  return a;
}

__host__ __device__ constexpr size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }
__host__ __device__ inline int row_stride(int n) { return (n & 1) ? n : n + 1; }  // odd: conflict-free columns

// Shared memory of one tile: line bases, the tile of raw FP64 values (each
// slot later holds the thread's own results in place), the segment tips.
template <typename T>
__host__ __device__ inline size_t split_smem(int n, int S, int nl) {
  const int ld = row_stride(n);
  return al16((size_t)nl * 8) + al16((size_t)nl * ld * sizeof(double)) + (size_t)nl * (4 * S + 1) * sizeof(T);
}

// ---------------------------------------------------------------------------
// Register-resident form of the FP32 split sweep, for grids whose lines are a
// multiple of kSplitSeg points long (every segment exactly 32 rows).  The
// thread's 32 rows are unrolled: their RHS, forward and backward substitution
// and reduced-system correction run in registers, and shared memory holds only
// the segment tips (plus, along x, the staged tile).  Along y and z a warp's
// lanes are 32 neighbouring lines at one position, so each thread reads its
// rows (and 3-4 halo rows on each side) and writes its results straight from
// and to global memory, every warp access one contiguous run.  Along x the
// tile is staged through shared memory as in split_kernel.  The arithmetic is
// split_kernel's (FP32 hi + lo pair differences, the exact fixed-point d8 RHS,
// FP32 solves), so the two forms agree to FP32 rounding.

// One line in global memory, read as the RHS arithmetic's type (edge rows).
template <typename TR>
struct GLine {
  const double* p;
  long long st;
  int n, e;
  __device__ __forceinline__ TR v(int q) const { return load_as<TR>(__ldg(p + q * st), e); }
  __device__ __forceinline__ TR w(int q) const { return v(q < 0 ? q + n : (q >= n ? q - n : q)); }
};

// Tips of line l, segment j at tips[l * (4S + 4) + 4j]: 16-byte rows whose stride keeps the
// lanes of a quarter warp (neighbouring lines) on distinct banks.
__host__ __device__ inline size_t seg_tips_bytes(int S, int nl) { return al16((size_t)nl * (4 * S + 4) * 4); }

template <int KIND, bool PER, bool IMPL, bool ADDBACK, int DIR, int EPI, bool EXACT>
__global__ void __launch_bounds__(kSplitThreads, EXACT ? 4 : 3) seg_kernel(const SParams P) {
  constexpr int H = (KIND == 4) ? 4 : 3;
  constexpr int L = kSplitSeg;
  constexpr bool kStage = (DIR == 0);  // x through a staged tile (direct per-thread runs of a line thrash L1)
  extern __shared__ __align__(16) unsigned char s_buf[];
  const SplitTile tile = P.tiles[blockIdx.x];
  const MemberOp& op = P.ops[tile.op];
  const SplitOp so = P.sops[tile.op];
  const int n = op.n, S = so.S, nl = tile.nlines;
  const int tid = threadIdx.x, tld = 4 * S + 4;
  const int nx = op.nx, ny = op.ny;
  const long long st = (DIR == 0) ? 1 : (DIR == 1 ? (long long)nx : (long long)nx * ny);
  const int ld = row_stride(n);
  float* tips = reinterpret_cast<float*>(s_buf);
  long long* sbase = reinterpret_cast<long long*>(s_buf + seg_tips_bytes(S, nl));
  double* sv = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(sbase) + al16((size_t)nl * 8));
  auto line_base = [&](int li) -> long long {
    const long long Lm = tile.line0 + li;
    long long b;
    if (DIR == 0) b = Lm * nx;
    else if (DIR == 1) b = (Lm / nx) * (long long)nx * ny + (Lm % nx);
    else b = Lm;
    return b + op.off;
  };
  const int NE = n * nl;
  const int qs = kSplitThreads / n, qr = kSplitThreads % n;  // x: element tid of the tile is (tid / n, tid % n)
  if (kStage) {  // stage the tile: a warp reads a contiguous run of one line
    for (int li = tid; li < nl; li += blockDim.x) sbase[li] = line_base(li);
    __syncthreads();
    int es = tid / n, ef = tid % n;
    for (int e0 = tid; e0 < NE; e0 += kSplitThreads * kBatch) {
      double v[kBatch];
      int so_[kBatch], fo_[kBatch];
#pragma unroll
      for (int k = 0; k < kBatch; k++) {
        so_[k] = es;
        fo_[k] = ef;
        v[k] = (e0 + k * kSplitThreads < NE) ? __ldg(P.in + sbase[es] + ef) : 0.0;
        ef += qr;
        es += qs;
        if (ef >= n) {
          ef -= n;
          es++;
        }
      }
#pragma unroll
      for (int k = 0; k < kBatch; k++)
        if (e0 + k * kSplitThreads < NE) sv[so_[k] * ld + fo_[k]] = v[k];
    }
    __syncthreads();
  }

  const int l = tid % nl, j = tid / nl;
  const bool active = j < S;
  const int p0 = j * L;
  const long long gb = kStage ? 0 : line_base(l);
  const double* gl = P.in + gb;
  const double* vl = sv + l * ld;
  // the raw value at position p0 + k of the thread's line, k in [-H, L + H): rows outside the
  // segment wrap (periodic) or clamp to the line (their rows are the one-sided edge rows)
  auto raw = [&](int k) -> double {
    int p = p0 + k;
    if (k < 0 || k >= L) {
      if (PER) p = p < 0 ? p + n : (p >= n ? p - n : p);
      else p = min(max(p, 0), n - 1);
    }
    return kStage ? vl[p] : __ldg(gl + p * st);
  };
  const int E = EXACT ? __ldg(P.emax + tile.op) : 0;
  const float wsc = EXACT ? op.wscale : 1.0f;
  float z[L];
  if (active) {
    // one-sided / boundary-code edge rows of the first and last segment (FP64 or exact arithmetic)
    const bool elo = !PER && j == 0, ehi = !PER && j == S - 1;
    float re[8];
#pragma unroll
    for (int q = 0; q < 8; q++) re[q] = 0.0f;
    if (elo || ehi) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int i = q < 4 ? q : n - 8 + q;
        if (q < 4 ? !elo : !ehi) continue;
        if (EXACT) {
          if (kStage)
            re[q] = fixed_to_float(edge_rhs<long long, KIND, false, int>(SLine<long long>{vl, n, E}, i, op.rhs_i,
                                                                         op.bcl, op.bch), E, wsc);
          else
            re[q] = fixed_to_float(edge_rhs<long long, KIND, false, int>(GLine<long long>{gl, st, n, E}, i, op.rhs_i,
                                                                         op.bcl, op.bch), E, wsc);
        } else {
          const float* R = reinterpret_cast<const float*>(op.rhs);  // the FP32 operator's weights
          if (kStage)
            re[q] = (float)edge_rhs<double, KIND, false, float>(SLine<double>{vl, n, 0}, i, R, op.bcl, op.bch);
          else
            re[q] = (float)edge_rhs<double, KIND, false, float>(GLine<double>{gl, st, n, 0}, i, R, op.bcl, op.bch);
        }
      }
    }
    const float* __restrict__ C = reinterpret_cast<const float*>(so.row) + (size_t)p0 * 12;
    float z1 = 0.0f, z2 = 0.0f;
    auto put = [&](int k, float r) {
      if (k < 4 && elo) r = re[k];
      if (k >= L - 4 && ehi) r = re[k - L + 8];
      if (IMPL) {  // forward substitution of the segment block (Crout: z = rho r - alpha z1 - beta z2)
        const V4<float> f = V4<float>::ld(C + k * 12);
        float zz = f.a * r;
        zz -= f.c * z2;
        zz -= f.b * z1;
        z2 = z1;
        z1 = zz;
        r = zz;
      }
      z[k] = r;
    };
    if constexpr (EXACT) {
      Cascade cas{};
#pragma unroll
      for (int k = 0; k < 8; k++) cas.push(to_fixed(raw(k - 4), E));
      const float wi = wsc * (float)op.iw[0];
#pragma unroll
      for (int k = 0; k < L; k++) put(k, fixed_to_float(cas.push(to_fixed(raw(k + 4), E)), E, wi));
    } else {
      float ai[9];
#pragma unroll
      for (int k = 0; k < 9; k++) ai[k] = (float)op.ri[k];
      float2 win[2 * H + 1];
#pragma unroll
      for (int k = 0; k < 2 * H; k++) win[k] = split_f64(raw(k - H));
#pragma unroll
      for (int k = 0; k < L; k++) {
        win[2 * H] = split_f64(raw(k + H));
        put(k, window_rhs<KIND>(win, ai));
#pragma unroll
        for (int m = 0; m < 2 * H; m++) win[m] = win[m + 1];
      }
    }
    if (IMPL) {  // backward substitution with the unit upper factor, then the tips
      float y1 = 0.0f, y2 = 0.0f;
#pragma unroll
      for (int k = L - 1; k >= 0; k--) {
        const V4<float> g = V4<float>::ld(C + k * 12 + 4);  // u1 u2 . .
        float y = z[k];
        y -= g.b * y2;
        y -= g.a * y1;
        z[k] = y;
        y2 = y1;
        y1 = y;
      }
      *reinterpret_cast<float4*>(tips + l * tld + 4 * j) = make_float4(z[0], z[1], z[L - 2], z[L - 1]);
    }
  }
  __syncthreads();  // the tips are published, and every read of this tile's input is done

  if (IMPL && active) {  // the neighbouring tips from the reduced system, then the correction
    const float* __restrict__ Gj = reinterpret_cast<const float*>(so.G) + (size_t)j * 16 * S;
    const int g0 = __ldg(so.win + 2 * j), gc = __ldg(so.win + 2 * j + 1);
    const float* tl = tips + l * tld;
    float q0 = 0.0f, q1 = 0.0f, q2 = 0.0f, q3 = 0.0f;
    const int T4 = 4 * S;
    auto dot4 = [](float q, const float4 g, const float4 t) {  // the order of split_kernel's sums
      q += g.x * t.x;
      q += g.y * t.y;
      q += g.z * t.z;
      q += g.w * t.w;
      return q;
    };
    for (int k = 0; k < gc; k++) {
      int js = g0 + k;
      js = js >= S ? js - S : js;
      const float4 t = *reinterpret_cast<const float4*>(tl + 4 * js);
      q0 = dot4(q0, __ldg(reinterpret_cast<const float4*>(Gj + 4 * js)), t);
      q1 = dot4(q1, __ldg(reinterpret_cast<const float4*>(Gj + T4 + 4 * js)), t);
      q2 = dot4(q2, __ldg(reinterpret_cast<const float4*>(Gj + 2 * T4 + 4 * js)), t);
      q3 = dot4(q3, __ldg(reinterpret_cast<const float4*>(Gj + 3 * T4 + 4 * js)), t);
    }
    const float* __restrict__ C = reinterpret_cast<const float*>(so.row) + (size_t)p0 * 12;
#pragma unroll
    for (int k = 0; k < L; k++) {
      const V4<float> sp = V4<float>::ld(C + k * 12 + 8);  // W_0 W_1 V_0 V_1
      float x = z[k];
      x -= sp.a * q0;
      x -= sp.b * q1;
      x -= sp.c * q2;
      x -= sp.d * q3;
      z[k] = x;
    }
  }

  constexpr bool kReadOut = (EPI == EPI_ADD || EPI == EPI_RING_MAX);
  const double sc = (P.scale_pow == 2) ? op.dm * op.dm : (P.scale_pow == 1 ? op.dm : 1.0);
  if (!kStage) {  // straight to global memory, 8 rows at a time (their epilogue inputs read first)
    if (active) {
      double* go = P.out + gb;
      const double* gi = P.in + gb;
#pragma unroll
      for (int k0 = 0; k0 < L; k0 += kBatch) {
        double vin[kBatch], o[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; k++) {
          const long long off = (long long)(p0 + k0 + k) * st;
          vin[k] = ADDBACK ? gi[off] : 0.0;
          o[k] = kReadOut ? go[off] : 0.0;
        }
#pragma unroll
        for (int k = 0; k < kBatch; k++)
          go[(long long)(p0 + k0 + k) * st] = epilogue<EPI>(to_f64<float>(z[k0 + k]), vin[k], o[k], sc, ADDBACK);
      }
    }
    return;
  }
  // x: results into the tile's slots, then the coalesced store of split_kernel
  double* wl = sv + l * ld;
  if (active) {
#pragma unroll
    for (int k = 0; k < L; k++) slot_st(wl + p0 + k, z[k]);
  }
  __syncthreads();
  int es = tid / n, ef = tid % n;
  for (int e0 = tid; e0 < NE; e0 += kSplitThreads * kBatch) {
    long long g[kBatch];
    double vin[kBatch], o[kBatch];
    float r[kBatch];
#pragma unroll
    for (int k = 0; k < kBatch; k++) {
      const bool ok = e0 + k * kSplitThreads < NE;
      g[k] = ok ? sbase[es] + ef : -1;
      r[k] = ok ? slot_ld<float>(sv + es * ld + ef) : 0.0f;
      vin[k] = (ADDBACK && ok) ? P.in[g[k]] : 0.0;
      o[k] = (kReadOut && ok) ? P.out[g[k]] : 0.0;
      ef += qr;
      es += qs;
      if (ef >= n) {
        ef -= n;
        es++;
      }
    }
#pragma unroll
    for (int k = 0; k < kBatch; k++)
      if (g[k] >= 0) P.out[g[k]] = epilogue<EPI>(to_f64<float>(r[k]), vin[k], o[k], sc, ADDBACK);
  }
}


}  // namespace
}  // namespace pg
