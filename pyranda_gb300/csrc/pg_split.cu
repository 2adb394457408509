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
#include "pg_split.cuh"

namespace pg {
namespace {

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

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, unsigned EPIS, typename TR, int DIR>
int split_epi(const SParams& P, const SplitSet& ss, int epi, void* st) {
  if constexpr ((EPIS >> EPI_STORE) & 1u)
    if (epi == EPI_STORE) return launch_s<T, KIND, PER, IMPL, ADDBACK, DIR, EPI_STORE, TR>(P, ss, st);
  if constexpr ((EPIS >> EPI_ADD) & 1u)
    if (epi == EPI_ADD) return launch_s<T, KIND, PER, IMPL, ADDBACK, DIR, EPI_ADD, TR>(P, ss, st);
  if constexpr ((EPIS >> EPI_RING_SET) & 1u)
    if (epi == EPI_RING_SET) return launch_s<T, KIND, PER, IMPL, ADDBACK, DIR, EPI_RING_SET, TR>(P, ss, st);
  if constexpr ((EPIS >> EPI_RING_MAX) & 1u)
    if (epi == EPI_RING_MAX) return launch_s<T, KIND, PER, IMPL, ADDBACK, DIR, EPI_RING_MAX, TR>(P, ss, st);
  set_error("split sweep: epilogue %d is not built for this operator", epi);
  return PG_EINVAL;
}

template <typename T, int KIND, bool PER, bool IMPL, bool ADDBACK, unsigned EPIS, typename TR = T>
int split_dir_epi(const SParams& P, const SplitSet& ss, int dir, int epi, void* st) {
  if (dir == 0) return split_epi<T, KIND, PER, IMPL, ADDBACK, EPIS, TR, 0>(P, ss, epi, st);
  if (dir == 1) return split_epi<T, KIND, PER, IMPL, ADDBACK, EPIS, TR, 1>(P, ss, epi, st);
  return split_epi<T, KIND, PER, IMPL, ADDBACK, EPIS, TR, 2>(P, ss, epi, st);
}

template <typename T>
int split_kind(const OpRef& op, const SParams& P, const SplitSet& ss, int dir, int epi, void* st) {
  switch (op.kind) {
    case OPK_D1:
      return op.periodic ? split_dir_epi<T, 1, true, true, false, kEpiStoreAdd>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 1, false, true, false, kEpiStoreAdd>(P, ss, dir, epi, st);
    case OPK_D8: {
      using TRX = typename std::conditional<std::is_same<T, float>::value, long long, T>::type;
      if (std::is_same<T, float>::value && op.exact)
        return op.periodic ? split_dir_epi<T, 4, true, true, false, kEpiRing, TRX>(P, ss, dir, epi, st)
                           : split_dir_epi<T, 4, false, true, false, kEpiRing, TRX>(P, ss, dir, epi, st);
      return op.periodic ? split_dir_epi<T, 4, true, true, false, kEpiRing>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 4, false, true, false, kEpiRing>(P, ss, dir, epi, st);
    }
    case OPK_SF:
      return op.periodic ? split_dir_epi<T, 4, true, true, true, kEpiStore>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 4, false, true, true, kEpiStore>(P, ss, dir, epi, st);
    case OPK_D2:
      return op.periodic ? split_dir_epi<T, 3, true, true, false, kEpiStoreAdd>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 3, false, true, false, kEpiStoreAdd>(P, ss, dir, epi, st);
    case OPK_D4:
      return op.periodic ? split_dir_epi<T, 3, true, false, false, kEpiStore>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 3, false, false, false, kEpiStore>(P, ss, dir, epi, st);
    default:
      return op.periodic ? split_dir_epi<T, 4, true, false, true, kEpiStore>(P, ss, dir, epi, st)
                         : split_dir_epi<T, 4, false, false, true, kEpiStore>(P, ss, dir, epi, st);
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
    return (op.kind == OPK_D1 || op.kind == OPK_D2 || op.kind == OPK_D4) ? seg_launch_r3(op, P, ss, dir, epi, stream)
                                                                           : seg_launch_r4(op, P, ss, dir, epi, stream);
  if (precision == PG_FP32) return split_kind<float>(op, P, ss, dir, epi, stream);
  return split_kind<double>(op, P, ss, dir, epi, stream);
}

}  // namespace pg
