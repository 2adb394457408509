// Split-line compact sweeps: every line is cut into segments of kSplitSeg
// points and each segment is solved by its own thread; the segments are
// joined by the reduced system of their tip unknowns.
//
// The reference splits a line the same way across MPI ranks when a
// direction is decomposed (local banded solve with coupling columns,
// compact_basetype.f90:171-197; a 4x4 block tridiagonal solve of the
// gathered boundary values, pentadiagonal.f90:160-626; the local correction,
// compact_d1.f90:242-337).  Here the "ranks" are the threads of one CTA, the
// reduced system is the same for every line of a grid, so its inverse is
// formed once on the host (pg_setup.cpp build_split) and applied as small dot
// products, and everything between the one read and the one write of a line
// stays on chip:
//   1. the CTA loads a tile of whole lines, coalesced for every direction
//      (x: a warp reads a run of one line; y, z: a warp reads one position of
//      32 neighbouring lines), converted once, into shared memory;
//   2. thread (line l, segment j) forms the RHS of its rows from shared memory
//      (edge rows with the reference's one-sided / periodic formulas), then
//      the local forward and backward substitution of its segment block, and
//      publishes the four tip values;
//   3. after a barrier each thread takes the tips it needs from the reduced
//      solve (its window of neighbouring segments) and corrects its rows:
//      x = y - W xbot_{j-1} - V xtop_{j+1};
//   4. the CTA stores the tile coalesced, with the fused epilogue (filter
//      add-back in FP64, accumulate, ring max).
// No scratch field is written or read back, the serial chain of a thread is
// one segment (not one line) long, and a line may be longer than the dense
// path's 1024 points (up to 256 segments).  The tile keeps the raw FP64
// values.  T = float is the fast path's arithmetic: RHS differences from FP32
// hi + lo pairs of the FP64 values, d8 with the exact 64-bit fixed-point RHS,
// FP32 solves; T = double follows the reference arithmetic.
#include "pg_sweep.cuh"

namespace pg {
namespace {

constexpr int kSplitThreads = 256;
constexpr int kBatch = 8;  // global loads a thread has in flight in the load and store phases

struct SParams {
  const double* in;  // may equal out: a CTA reads all of its lines before it writes any
  double* out;
  const MemberOp* ops;
  const SplitOp* sops;
  const SplitTile* tiles;
  int scale_pow;
  const int* emax;
};

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
  float a, b;
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

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, int DIR, int EPI, typename TR>
__global__ void __launch_bounds__(kSplitThreads, 3) split_kernel(const SParams P) {
  constexpr bool kExact = std::is_same<TR, long long>::value;
  constexpr bool kPair = std::is_same<T, float>::value && !kExact;  // FP32 differences from hi + lo pairs
  constexpr int H = (KIND == 4) ? 4 : 3;
  using W = typename WeightOf<TR>::type;
  extern __shared__ __align__(16) unsigned char s_buf[];
  const SplitTile tile = P.tiles[blockIdx.x];
  const MemberOp& op = P.ops[tile.op];
  const SplitOp so = P.sops[tile.op];
  const int n = op.n, S = so.S, nl = tile.nlines;
  const int ld = row_stride(n), tld = 4 * S + 1;
  long long* sbase = reinterpret_cast<long long*>(s_buf);
  double* sv = reinterpret_cast<double*>(s_buf + al16((size_t)nl * 8));
  T* tips = reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(sv) + al16((size_t)nl * ld * sizeof(double)));
  const int tid = threadIdx.x;
  const int nx = op.nx, ny = op.ny;
  const long long st = (DIR == 0) ? 1 : (DIR == 1 ? (long long)nx : (long long)nx * ny);
  for (int l = tid; l < nl; l += blockDim.x) {
    const long long Lm = tile.line0 + l;
    long long b;
    if (DIR == 0) b = Lm * nx;
    else if (DIR == 1) b = (Lm / nx) * (long long)nx * ny + (Lm % nx);
    else b = Lm;
    sbase[l] = b + op.off;
  }
  __syncthreads();

  // 1. load the tile (every input value of these lines is read before any output is written).
  // Element e of the tile is (slow, fast) = (e / fe, e % fe) with the fast index the one that is
  // contiguous in memory (x: the position along the line; y, z: the line), so consecutive threads
  // read consecutive addresses; each thread issues kBatch loads before it stores any of them.
  const int fe = (DIR == 0) ? n : nl;
  const int NE = n * nl;  // elements of the tile
  const int qs = kSplitThreads / fe, qr = kSplitThreads % fe;
  {
    int es = tid / fe, ef = tid % fe;  // (slow, fast) of element tid
    for (int e0 = tid; e0 < NE; e0 += kSplitThreads * kBatch) {
      double v[kBatch];
      int so_[kBatch], fo_[kBatch];
#pragma unroll
      for (int k = 0; k < kBatch; k++) {
        so_[k] = es;
        fo_[k] = ef;
        const int li = (DIR == 0) ? es : ef, pi = (DIR == 0) ? ef : es;
        v[k] = (e0 + k * kSplitThreads < NE) ? __ldg(P.in + sbase[li] + (long long)pi * st) : 0.0;
        ef += qr;
        es += qs;
        if (ef >= fe) {
          ef -= fe;
          es++;
        }
      }
#pragma unroll
      for (int k = 0; k < kBatch; k++)
        if (e0 + k * kSplitThreads < NE) {
          const int li = (DIR == 0) ? so_[k] : fo_[k], pi = (DIR == 0) ? fo_[k] : so_[k];
          sv[li * ld + pi] = v[k];
        }
    }
  }
  __syncthreads();

  // 2. thread (line l, segment j): RHS and local solve of rows [a, b).  It first copies what it
  // reads outside its own rows (the 4 values on each side) and forms the one-sided edge rows, whose
  // stencils reach 8 points in; after a barrier every thread owns its rows and writes its results
  // in place of its own input values (slot i of the line holds z_i, then y_i, then x_i, as T).
  const int l = tid % nl, j = tid / nl;
  const bool active = j < S;
  const T* __restrict__ C = reinterpret_cast<const T*>(so.row);  // 12 per position
  const int E = kExact ? __ldg(P.emax + tile.op) : 0;
  const float wsc = kExact ? op.wscale : 1.0f;
  int a = 0, b = 0;
  double* vl = sv + l * ld;  // slot i: the input value, later this thread's result of row i
  double hl[4] = {0.0, 0.0, 0.0, 0.0}, hr[4] = {0.0, 0.0, 0.0, 0.0};
  T re[8];
#pragma unroll
  for (int q = 0; q < 8; q++) re[q] = T(0);
  if (active) {
    a = __ldg(so.start + j);
    b = __ldg(so.start + j + 1);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      int p = a - 4 + k;
      p = p < 0 ? p + n : p;
      hl[k] = (PER || a - 4 + k >= 0) ? vl[p] : 0.0;
      p = b + k;
      p = p >= n ? p - n : p;
      hr[k] = (PER || b + k < n) ? vl[p] : 0.0;
    }
    if (!PER) {  // the one-sided rows 0..3 and n-4..n-1 (reference formulas, compact_d1.f90:131-180,
                 // compact_r4.f90:120-125,166-171), only in the first and last segment
      if (kExact) {
        const SLine<long long> ln{vl, n, E};
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int i = q < 4 ? q : n - 8 + q;
          if (i >= a && i < b) re[q] = (T)fixed_to_float(edge_rhs<long long, KIND, false, int>(ln, i, op.rhs_i, op.bcl, op.bch), E, wsc);
        }
      } else {  // FP64 arithmetic on the raw values (8 rows of a line)
        const SLine<double> ln{vl, n, 0};
        const W* R = reinterpret_cast<const W*>(op.rhs);
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int i = q < 4 ? q : n - 8 + q;
          if (i >= a && i < b) re[q] = (T)edge_rhs<double, KIND, false, W>(ln, i, R, op.bcl, op.bch);
        }
      }
    }
  }
  __syncthreads();
  if (active) {
    T z1 = T(0), z2 = T(0);
    auto put = [&](int i, T r) {
      if (IMPL) {  // forward substitution of the segment block (Crout: z = rho r - alpha z1 - beta z2)
        const V4<T> f = V4<T>::ld(C + i * 12);
        T z = f.a * r;
        z -= f.c * z2;
        z -= f.b * z1;
        z2 = z1;
        z1 = z;
        r = z;
      }
      slot_st(vl + i, r);
    };
    // rows in order: the lower one-sided rows, the interior rows [ia, ib), the upper one-sided rows
    const int ia = PER ? a : max(a, 4), ib = PER ? b : min(b, n - 4);
    const int iv = max(ia, min(ib, b - H));  // interior rows below iv read ahead inside the segment
    // the value at ia - H + k (k < 2H): the left halo when the window starts at the segment's first row.
    // The window is primed before the lower one-sided rows store their results over slots 0..3.
    auto first = [&](int k) -> double { return (ia == a && k < H) ? hl[k + 4 - H] : vl[ia - H + k]; };
    auto lower_edge_rows = [&]() {
      if (!PER) {
#pragma unroll
        for (int q = 0; q < 4; q++)
          if (q >= a && q < b) put(q, re[q]);
      }
    };
    if (ia >= ib) lower_edge_rows();
    if (ia < ib) {
      if constexpr (kExact) {
        // iw[0] x the 8th difference, exact in 64-bit integers, kept by a cascade of differences
        Cascade cas{};
#pragma unroll
        for (int k = 0; k < 8; k++) cas.push(to_fixed(first(k), E));
        lower_edge_rows();
        const float wi = wsc * (float)op.iw[0];
        int i = ia;
        for (; i < iv; i++) put(i, fixed_to_float(cas.push(to_fixed(vl[i + 4], E)), E, wi));
#pragma unroll
        for (int t = 0; t < 4; t++)
          if (i + t < ib) put(i + t, fixed_to_float(cas.push(to_fixed(hr[t], E)), E, wi));
      } else if constexpr (kPair) {
        float ai[9];
#pragma unroll
        for (int k = 0; k < 9; k++) ai[k] = (float)op.ri[k];
        float2 win[2 * H + 1];
#pragma unroll
        for (int k = 0; k < 2 * H; k++) win[k] = split_f64(first(k));
        lower_edge_rows();
        auto row = [&](int i, double next) {
          win[2 * H] = split_f64(next);
          put(i, window_rhs<KIND>(win, ai));
#pragma unroll
          for (int k = 0; k < 2 * H; k++) win[k] = win[k + 1];
        };
        int i = ia;
        for (; i < iv; i++) row(i, vl[i + H]);
#pragma unroll
        for (int t = 0; t < H; t++)
          if (i + t < ib) row(i + t, hr[t]);
      } else {
        double ai[9];
#pragma unroll
        for (int k = 0; k < 9; k++) ai[k] = op.ri[k];
        double win[2 * H + 1];
#pragma unroll
        for (int k = 0; k < 2 * H; k++) win[k] = first(k);
        lower_edge_rows();
        auto row = [&](int i, double next) {
          win[2 * H] = next;
          put(i, (T)window_rhs<KIND>(win, ai));
#pragma unroll
          for (int k = 0; k < 2 * H; k++) win[k] = win[k + 1];
        };
        int i = ia;
        for (; i < iv; i++) row(i, vl[i + H]);
#pragma unroll
        for (int t = 0; t < H; t++)
          if (i + t < ib) row(i + t, hr[t]);
      }
    }
    if (!PER) {
#pragma unroll
      for (int q = 4; q < 8; q++) {
        const int i = n - 8 + q;
        if (i >= a && i < b && i >= ib) put(i, re[q]);
      }
    }
    if (IMPL) {  // backward substitution with the unit upper factor
      T y1 = T(0), y2 = T(0);
      for (int i = b - 1; i >= a; i--) {
        const V4<T> g = V4<T>::ld(C + i * 12 + 4);  // u1 u2 . .
        T y = slot_ld<T>(vl + i);
        y -= g.b * y2;
        y -= g.a * y1;
        slot_st(vl + i, y);
        y2 = y1;
        y1 = y;
      }
      T* tp = tips + l * tld + 4 * j;
      tp[0] = slot_ld<T>(vl + a);
      tp[1] = slot_ld<T>(vl + a + 1);
      tp[2] = slot_ld<T>(vl + b - 2);
      tp[3] = slot_ld<T>(vl + b - 1);
    }
  }
  __syncthreads();

  // 3. the neighbouring tips from the reduced system, then the correction
  if (IMPL && active) {
    const T* __restrict__ Gj = reinterpret_cast<const T*>(so.G) + (size_t)j * 16 * S;
    const int g0 = __ldg(so.win + 2 * j), gc = __ldg(so.win + 2 * j + 1);
    const T* tl = tips + l * tld;
    T q0 = T(0), q1 = T(0), q2 = T(0), q3 = T(0);
    const int T4 = 4 * S;
    for (int k = 0; k < gc; k++) {
      int js = g0 + k;
      js = js >= S ? js - S : js;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const int idx = 4 * js + c;
        const T t = tl[idx];
        q0 += ldc(Gj + idx) * t;
        q1 += ldc(Gj + T4 + idx) * t;
        q2 += ldc(Gj + 2 * T4 + idx) * t;
        q3 += ldc(Gj + 3 * T4 + idx) * t;
      }
    }
    for (int i = a; i < b; i++) {
      const V4<T> sp = V4<T>::ld(C + i * 12 + 8);  // W_0 W_1 V_0 V_1
      T x = slot_ld<T>(vl + i);
      x -= sp.a * q0;
      x -= sp.b * q1;
      x -= sp.c * q2;
      x -= sp.d * q3;
      slot_st(vl + i, x);
    }
  }
  __syncthreads();

  // 4. store with the fused epilogue, in the order of the load (inputs of the epilogue batched)
  constexpr bool kReadOut = (EPI == EPI_ADD || EPI == EPI_RING_MAX);
  const double sc = (P.scale_pow == 2) ? op.dm * op.dm : (P.scale_pow == 1 ? op.dm : 1.0);
  {
    int es = tid / fe, ef = tid % fe;
    for (int e0 = tid; e0 < NE; e0 += kSplitThreads * kBatch) {
      long long g[kBatch];
      double vin[kBatch], o[kBatch];
      T r[kBatch];
#pragma unroll
      for (int k = 0; k < kBatch; k++) {
        const int li = (DIR == 0) ? es : ef, pi = (DIR == 0) ? ef : es;
        const bool ok = e0 + k * kSplitThreads < NE;
        g[k] = ok ? sbase[li] + (long long)pi * st : -1;
        r[k] = ok ? slot_ld<T>(sv + li * ld + pi) : T(0);
        vin[k] = (ADDBACK && ok) ? P.in[g[k]] : 0.0;
        o[k] = (kReadOut && ok) ? P.out[g[k]] : 0.0;
        ef += qr;
        es += qs;
        if (ef >= fe) {
          ef -= fe;
          es++;
        }
      }
#pragma unroll
      for (int k = 0; k < kBatch; k++)
        if (g[k] >= 0) P.out[g[k]] = epilogue<EPI>(to_f64<T>(r[k]), vin[k], o[k], sc, ADDBACK);
    }
  }
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

template <int KIND, bool PER, bool IMPL, bool ADDBACK, int DIR, int EPI, bool EXACT>
int launch_seg(const SParams& P, const SplitSet& ss, void* stream) {
  const size_t smem = DIR == 0 ? ss.smem_seg_x : ss.smem_seg_yz;
  auto k = seg_kernel<KIND, PER, IMPL, ADDBACK, DIR, EPI, EXACT>;
  static size_t attr = 0;
  if (smem > attr) {
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error("split sweep: %s (%zu bytes of shared memory)", cudaGetErrorString(e), smem);
      return PG_ECUDA;
    }
    attr = smem;
  }
  k<<<ss.ntiles, kSplitThreads, smem, (cudaStream_t)stream>>>(P);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("split sweep launch: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

template <int KIND, bool PER, bool IMPL, bool ADDBACK, bool EXACT = false>
int seg_dir_epi(const SParams& P, const SplitSet& ss, int dir, int epi, void* st) {
#define PG_SEG_EPI(D)                                                                               \
  switch (epi) {                                                                                    \
    case EPI_STORE: return launch_seg<KIND, PER, IMPL, ADDBACK, D, EPI_STORE, EXACT>(P, ss, st);       \
    case EPI_ADD: return launch_seg<KIND, PER, IMPL, ADDBACK, D, EPI_ADD, EXACT>(P, ss, st);           \
    case EPI_RING_SET: return launch_seg<KIND, PER, IMPL, ADDBACK, D, EPI_RING_SET, EXACT>(P, ss, st); \
    default: return launch_seg<KIND, PER, IMPL, ADDBACK, D, EPI_RING_MAX, EXACT>(P, ss, st);           \
  }
  if (dir == 0) { PG_SEG_EPI(0) }
  if (dir == 1) { PG_SEG_EPI(1) }
  PG_SEG_EPI(2)
#undef PG_SEG_EPI
}

int seg_kind(const OpRef& op, const SParams& P, const SplitSet& ss, int dir, int epi, void* st) {
  switch (op.kind) {
    case OPK_D1:
      return op.periodic ? seg_dir_epi<1, true, true, false>(P, ss, dir, epi, st)
                         : seg_dir_epi<1, false, true, false>(P, ss, dir, epi, st);
    case OPK_D8:
      if (op.exact)
        return op.periodic ? seg_dir_epi<4, true, true, false, true>(P, ss, dir, epi, st)
                           : seg_dir_epi<4, false, true, false, true>(P, ss, dir, epi, st);
      return op.periodic ? seg_dir_epi<4, true, true, false>(P, ss, dir, epi, st)
                         : seg_dir_epi<4, false, true, false>(P, ss, dir, epi, st);
    case OPK_SF:
      return op.periodic ? seg_dir_epi<4, true, true, true>(P, ss, dir, epi, st)
                         : seg_dir_epi<4, false, true, true>(P, ss, dir, epi, st);
    case OPK_D2:
      return op.periodic ? seg_dir_epi<3, true, true, false>(P, ss, dir, epi, st)
                         : seg_dir_epi<3, false, true, false>(P, ss, dir, epi, st);
    case OPK_D4:
      return op.periodic ? seg_dir_epi<3, true, false, false>(P, ss, dir, epi, st)
                         : seg_dir_epi<3, false, false, false>(P, ss, dir, epi, st);
    default:
      return op.periodic ? seg_dir_epi<4, true, false, true>(P, ss, dir, epi, st)
                         : seg_dir_epi<4, false, false, true>(P, ss, dir, epi, st);
  }
}

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, int DIR, int EPI, typename TR>
int launch_s(const SParams& P, const SplitSet& ss, void* stream) {
  const size_t smem = sizeof(T) == 8 ? ss.smem64 : ss.smem32;
  auto k = split_kernel<T, KIND, PER, IMPL, ADDBACK, DIR, EPI, TR>;
  static size_t attr = 0;
  if (smem > attr) {
    const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) {
      set_error("split sweep: %s (%zu bytes of shared memory)", cudaGetErrorString(e), smem);
      return PG_ECUDA;
    }
    attr = smem;
  }
  k<<<ss.ntiles, kSplitThreads, smem, (cudaStream_t)stream>>>(P);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("split sweep launch: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, typename TR = T>
int split_dir_epi(const SParams& P, const SplitSet& ss, int dir, int epi, void* st) {
#define PG_SPLIT_EPI(D)                                                                             \
  switch (epi) {                                                                                    \
    case EPI_STORE: return launch_s<T, KIND, PER, IMPL, ADDBACK, D, EPI_STORE, TR>(P, ss, st);       \
    case EPI_ADD: return launch_s<T, KIND, PER, IMPL, ADDBACK, D, EPI_ADD, TR>(P, ss, st);           \
    case EPI_RING_SET: return launch_s<T, KIND, PER, IMPL, ADDBACK, D, EPI_RING_SET, TR>(P, ss, st); \
    default: return launch_s<T, KIND, PER, IMPL, ADDBACK, D, EPI_RING_MAX, TR>(P, ss, st);           \
  }
  if (dir == 0) { PG_SPLIT_EPI(0) }
  if (dir == 1) { PG_SPLIT_EPI(1) }
  PG_SPLIT_EPI(2)
#undef PG_SPLIT_EPI
}

template <typename T>
int split_kind(const OpRef& op, const SParams& P, const SplitSet& ss, int dir, int epi, void* st) {
  switch (op.kind) {
    case OPK_D1:
      return op.periodic ? split_dir_epi<T, 1, true, true, false>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 1, false, true, false>(P, ss, dir, epi, st);
    case OPK_D8: {
      using TRX = typename std::conditional<std::is_same<T, float>::value, long long, T>::type;
      if (std::is_same<T, float>::value && op.exact)
        return op.periodic ? split_dir_epi<T, 4, true, true, false, TRX>(P, ss, dir, epi, st)
                           : split_dir_epi<T, 4, false, true, false, TRX>(P, ss, dir, epi, st);
      return op.periodic ? split_dir_epi<T, 4, true, true, false>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 4, false, true, false>(P, ss, dir, epi, st);
    }
    case OPK_SF:
      return op.periodic ? split_dir_epi<T, 4, true, true, true>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 4, false, true, true>(P, ss, dir, epi, st);
    case OPK_D2:
      return op.periodic ? split_dir_epi<T, 3, true, true, false>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 3, false, true, false>(P, ss, dir, epi, st);
    case OPK_D4:
      return op.periodic ? split_dir_epi<T, 3, true, false, false>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 3, false, false, false>(P, ss, dir, epi, st);
    default:
      return op.periodic ? split_dir_epi<T, 4, true, false, true>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 4, false, false, true>(P, ss, dir, epi, st);
  }
}

}  // namespace

size_t split_smem_bytes(int precision, bool, int n, int S, int nl) {
  return precision == PG_FP64 ? split_smem<double>(n, S, nl) : split_smem<float>(n, S, nl);
}

// Shared memory of the register-resident form: the tips, plus (x) the line bases and the tile.
size_t seg_smem(int dir, int n, int S, int nl) {
  size_t b = seg_tips_bytes(S, nl);
  if (dir == 0) b += al16((size_t)nl * 8) + (size_t)nl * row_stride(n) * sizeof(double);
  return b;
}

int launch_split(int precision, const OpRef& op, const SplitSet& ss, const double* in, double* out, int dir, int epi,
                 int scale_pow, const int* emax, void* stream) {
  if (!ss.ok || ss.ntiles == 0) return PG_OK;
  SParams P{in, out, op.dev, ss.sops, ss.tiles, scale_pow, emax};
  // the register-resident form wherever every segment is 32 rows long
  if (precision == PG_FP32 && ss.seg32)
    return seg_kind(op, P, ss, dir, epi, stream);
  if (precision == PG_FP32) return split_kind<float>(op, P, ss, dir, epi, stream);
  return split_kind<double>(op, P, ss, dir, epi, stream);
}

}  // namespace pg
