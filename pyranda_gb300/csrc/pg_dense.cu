// Dense compact operators on the tensor cores (tcgen05, split TF32).
//
// For a line of n <= 1024 points every compact operator of this library is a
// fixed linear map out = D v with D = A^-1 B (the reference builds the same
// matrix as `sm` in compact_basetype.f90:199-205).  Applying D to all lines
// of a field is a GEMM:
//   x lines (contiguous):     OUT[lines, pos] = V[lines, k] . D^T[k, pos]
//   y / z lines (strided):    OUT[pos, lines] = D[pos, k]   . V^T[k, lines]
// Both run here as tcgen05.mma kind::tf32 with FP32 accumulators in tensor
// memory.  TF32 keeps 11 significant bits, so D and v are each split into
// hi + lo TF32 parts and the product is hi.hi + hi.lo + lo.hi (three MMAs per
// K step; the dropped lo.lo term is ~2^-22 relative).  D is split once on the
// host into hi/lo planes already in the shared-memory layout the MMA reads
// (K-major, 128-byte swizzle) and copied per K chunk with cp.async.bulk; the
// FP64 field is converted and split while it is staged.  The epilogue goes
// through shared memory so that global stores are coalesced, and applies the
// same fused epilogues as the banded sweeps (store / accumulate / ring, with
// the filters' FP64 add-back of v).
//
// One CTA computes one output tile of 128 lines x up to 256 positions: for x
// lines one accumulator (M = lines, N = positions), for y and z lines up to
// two (M = 128 positions each, N = lines), over the full K = n in chunks of
// 32, double buffered.  Every wait is bounded; on a time-out the kernel records
// PG_ETIMEOUT in the status word, stops issuing work and still frees its
// tensor memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "pg_internal.h"
#include "pg_sweep.cuh"
#include "pg_tc.cuh"

namespace pg {
namespace {

constexpr int kDenseThreads = 512;  // 16 warps: latency hiding for the staging and the epilogue
constexpr int kKC = 32;               // K elements per chunk: one 128-byte row of TF32
constexpr int kStageBytes = 98304;    // V hi/lo + D hi/lo of one chunk
constexpr int kStages = 2;
constexpr int kSmemBytes = kStages * kStageBytes + 1024;  // + alignment slack
constexpr int kTmemCols = 256;

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, M = 128, N = n (multiple of 16, <= 256).
__device__ __forceinline__ uint32_t idesc_tf32(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, int acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

// TF32 of an FP32 value: round the low 13 mantissa bits to nearest (ties away).
__device__ __forceinline__ uint32_t tf32_bits(float x) {
  return (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u;
}

// One staging item: v_{kb-1} and v_kb .. v_kb+7 of one line (v at p[k * st]),
// the two adjacent 16-byte chunks of 4 differences a thread stages per K chunk.
struct Item {
  double v[9];
};

__device__ __forceinline__ void load_item(const double* __restrict__ p, bool ok, int kb, int n, int periodic,
                                          int64_t st, Item& it) {
  const int km1 = (kb > 0) ? kb - 1 : (periodic ? n - 1 : -1);
  it.v[0] = (ok && km1 >= 0 && km1 < n) ? __ldg(p + km1 * st) : 0.0;
#pragma unroll
  for (int j = 0; j < 8; j++) it.v[j + 1] = (ok && kb + j < n) ? __ldg(p + (kb + j) * st) : 0.0;
}

// The eight differences w_k = v_k - v_{k-1}, k = kb .. kb+7, as TF32 hi / lo.
// w_0 is the wrap difference v_0 - v_{n-1} on periodic lines and 0
// otherwise; k >= n gives 0.  Each v is split into FP32 value + residual
// first, so a difference keeps ~48 bits of v before its own rounding to FP32.
// direct: the values v_k themselves (their FP32 value + residual).
__device__ __forceinline__ void difference_item(const Item& it, bool ok, int kb, int n, int periodic, int direct,
                                                uint32_t* h, uint32_t* l) {
  float2 prev = split_f64(it.v[0]);
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const int k = kb + j;
    float f = 0.0f;
    if (ok && k < n) {
      const float2 v = split_f64(it.v[j + 1]);
      if (direct) f = v.x + v.y;
      else if (k > 0 || periodic) f = (v.x - prev.x) + (v.y - prev.y);
      prev = v;
    }
    h[j] = tf32_bits(f);
    l[j] = tf32_bits(f - __uint_as_float(h[j]));
  }
}

__device__ __forceinline__ int64_t line_base(const DenseOp& op, int dir, int64_t l) {
  if (dir == 0) return op.off + l * op.nx;
  if (dir == 1) return op.off + (l / op.nx) * (int64_t)op.nx * op.ny + (l % op.nx);
  return op.off + l;
}

struct DParams {
  const double* in;
  double* out;
  const DenseOp* ops;
  const DenseTile* tiles;
  int* status;
  int scale_pow;
};

// ORIENT 0: lines are the MMA's M (x direction); 1: lines are its N (y, z).
template <int ORIENT, int DIR, int EPI, bool ADDBACK>
__global__ void __launch_bounds__(kDenseThreads, 1) dense_kernel(const DParams P) {
  extern __shared__ uint8_t dsm_raw[];
  __shared__ __align__(8) uint64_t full_bar[kStages];
  __shared__ __align__(8) uint64_t mma_bar[kStages];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_bad;
  __shared__ long long s_base[128];  // per line: offset of its first point
  uint8_t* smem = dsm_raw + ((1024u - (smem_u32(dsm_raw) & 1023u)) & 1023u);

  const DenseTile tile = P.tiles[blockIdx.x];
  const DenseOp op = P.ops[tile.op];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n = op.n;
  const int st = (DIR == 0) ? 1 : (DIR == 1 ? op.nx : op.nx * op.ny);

  // Tile geometry: V rows are the tile's 128 lines, D rows its output
  // positions [drow0, drow0 + 256).  x: one accumulator, N = positions.
  // y, z: NP accumulators (one per 128 positions, M = 128 each), N = lines,
  // so the lines are staged once for all 256 positions.
  int drow0, drows, vrows, N, NP;
  drow0 = tile.part * 256;
  if (ORIENT == 0) {
    drows = min(256, ((n + 15) & ~15) - drow0);
    vrows = 128;
    N = drows;
    NP = 1;
  } else {
    NP = min(2, (n - drow0 + 127) / 128);
    drows = NP * 128;
    vrows = (tile.nlines + 15) & ~15;
    N = vrows;
  }
  constexpr uint32_t vbytes = 16384u;  // one V plane of a stage: 128 rows
  constexpr uint32_t dbytes = 32768u;  // one D plane of a stage: 256 rows
  const uint32_t dcopy = (uint32_t)drows * 128u;  // bytes of the D rows this tile reads

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&mma_bar[s], 1);
    }
    s_bad = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < 128) s_base[tid] = (tid < tile.nlines) ? line_base(op, DIR, tile.line0 + tid) : 0;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = idesc_tf32(N);
  const int kchunks = op.kchunks;
  bool bad = false;
  int issued = -1, committed = -1;  // thread 0: last chunk whose D copy / MMAs were issued
  // this thread's staging item: 16-byte chunks 2 qp and 2 qp + 1 of row item_r in every K chunk
  // (128 rows x 4 chunk pairs = 512 threads; y, z: consecutive threads take consecutive lines)
  static_assert(kDenseThreads == 512, "one chunk pair of one row per thread");
  const int item_r = (ORIENT == 0) ? (tid >> 2) : (tid & 127);
  const int item_q = 2 * ((ORIENT == 0) ? (tid & 3) : (tid >> 7));
  const int64_t vst = (ORIENT == 0) ? 1 : st;
  const double* const item_p = P.in + s_base[item_r];
  const bool item_ok = item_r < tile.nlines;
  Item cur, nxt;
  load_item(item_p, item_ok, item_q * 4, n, op.periodic, vst, cur);

  for (int c = 0; c < kchunks && !bad; c++) {
    const int s = c & 1;
    uint8_t* st_base = smem + s * kStageBytes;
    uint8_t* v_hi = st_base;
    uint8_t* v_lo = st_base + vbytes;
    uint8_t* d_hi = st_base + 2 * vbytes;
    uint8_t* d_lo = d_hi + dbytes;
    // the next chunk's loads go out first, so they are in flight across this chunk's work
    if (c + 1 < kchunks) load_item(item_p, item_ok, (c + 1) * kKC + item_q * 4, n, op.periodic, vst, nxt);
    // the MMAs that last read this stage (chunk c - 2) must be complete
    if (c >= 2 && !mbar_wait(&mma_bar[s], ((c >> 1) + 1) & 1)) bad = true;
    if (__syncthreads_or(bad)) break;
    if (tid == 0) {
      const uint32_t* plane = op.dsw + (size_t)c * 2 * op.rows * 32;
      mbar_expect_tx(&full_bar[s], 2 * dcopy);
      bulk_copy(d_hi, plane + (size_t)drow0 * 32, dcopy, &full_bar[s]);
      bulk_copy(d_lo, plane + (size_t)op.rows * 32 + (size_t)drow0 * 32, dcopy, &full_bar[s]);
      issued = c;
    }
    // stage V: 16-byte chunks of 4 consecutive k (differences, split into TF32 hi / lo)
    const int k0 = c * kKC;
    {
      const int r = item_r, q = item_q;
      uint32_t h[8], l[8];
      difference_item(cur, item_ok, k0 + q * 4, n, op.periodic, op.direct, h, l);
      if (ORIENT == 0 || r < vrows) {
        *reinterpret_cast<uint4*>(v_hi + swz(r, q)) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4*>(v_lo + swz(r, q)) = make_uint4(l[0], l[1], l[2], l[3]);
        *reinterpret_cast<uint4*>(v_hi + swz(r, q + 1)) = make_uint4(h[4], h[5], h[6], h[7]);
        *reinterpret_cast<uint4*>(v_lo + swz(r, q + 1)) = make_uint4(l[4], l[5], l[6], l[7]);
      }
    }
    cur = nxt;
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      if (!mbar_wait(&full_bar[s], (c >> 1) & 1)) {
        s_bad = 1;
      } else {
        tc_fence_after();
        for (int pp = 0; pp < NP; pp++) {
          // y, z: accumulator pp (TMEM columns 128 pp ..) takes D rows 128 pp ..
          const uint32_t dofs = (ORIENT == 0) ? 0u : (uint32_t)pp * 16384u;
          const uint32_t a_hi = smem_u32(ORIENT == 0 ? v_hi : d_hi) + dofs;
          const uint32_t a_lo = smem_u32(ORIENT == 0 ? v_lo : d_lo) + dofs;
          const uint32_t b_hi = smem_u32(ORIENT == 0 ? d_hi : v_hi), b_lo = smem_u32(ORIENT == 0 ? d_lo : v_lo);
          const uint32_t acc = tmem + (uint32_t)(pp * 128);
#pragma unroll
          for (int kk = 0; kk < kKC / 8; kk++) {
            const uint32_t o = kk * 32;  // 8 TF32 = 32 bytes along K
            mma_tf32(acc, sdesc(a_hi + o), sdesc(b_lo + o), idesc, (c > 0 || kk > 0) ? 1 : 0);
            mma_tf32(acc, sdesc(a_lo + o), sdesc(b_hi + o), idesc, 1);
            mma_tf32(acc, sdesc(a_hi + o), sdesc(b_hi + o), idesc, 1);
          }
        }
        mma_commit(&mma_bar[s]);
        committed = c;
      }
    }
    __syncthreads();
    bad = s_bad != 0;
  }
  // all MMAs complete (the last commit covers every earlier one)
  if (!bad) {
    const int cl = kchunks - 1;
    if (!mbar_wait(&mma_bar[cl & 1], (cl >> 1) & 1)) bad = true;
  }
  tc_fence_after();
  if (__syncthreads_or(bad)) {
    if (tid == 0) {
      atomicExch(P.status, (int)PG_ETIMEOUT);
      // let this CTA's own copies and MMAs in flight finish (bounded) before
      // its shared and tensor memory go away
      if (issued > committed) mbar_wait(&full_bar[issued & 1], (issued >> 1) & 1);
      if (committed >= 0) mbar_wait(&mma_bar[committed & 1], (committed >> 1) & 1);
      tc_fence_after();
    }
    __syncthreads();
  } else {
    // tensor memory -> shared tile T[row][col] (row = TMEM lane), padded rows
    float* T = reinterpret_cast<float*>(smem);
    const int ncol = (ORIENT == 0) ? N : NP * 128;  // TMEM columns in use (y, z: accumulator pp at 128 pp)
    const int ld = ncol + 1;
    // warp w reads TMEM lanes 32 (w % 4) ..; the warp groups w / 4 take turns over 8-column blocks
    const int q = warp & 3, h = warp >> 2;
    const int row = q * 32 + lane;
    for (int col = 8 * h; col < ncol; col += 8 * (kDenseThreads / 128)) {
      float r[8];
      tmem_ld8(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)col, r);
#pragma unroll
      for (int i = 0; i < 8; i++) T[row * ld + col + i] = r[i];
    }
    __syncthreads();
    const double sc = (P.scale_pow == 2) ? op.dm * op.dm : (P.scale_pow == 1 ? op.dm : 1.0);
    constexpr bool kReadOut = (EPI == EPI_ADD || EPI == EPI_RING_MAX);
    // warps take rows, lanes consecutive columns: coalesced stores, no index division
    constexpr int kWarps = kDenseThreads / 32;
    if (ORIENT == 0) {
      const int nl = tile.nlines, npos = min(N, n - drow0);
      for (int r = warp; r < nl; r += kWarps) {
        const int64_t b = s_base[r] + drow0;
        for (int col = lane; col < npos; col += 32) {
          const int64_t a = b + col;
          const double vin = ADDBACK ? P.in[a] : 0.0;
          const double o = kReadOut ? P.out[a] : 0.0;
          P.out[a] = epilogue<EPI>(f2d_bits(T[r * ld + col]), vin, o, sc, ADDBACK);
        }
      }
    } else {
      // position drow0 + 128 pp + r of line col is T[r][128 pp + col]
      const int nl = tile.nlines, npos = min(NP * 128, n - drow0);
      for (int pr = warp; pr < npos; pr += kWarps) {
        const int pp = pr >> 7, r = pr & 127;
        const int64_t b = (int64_t)(drow0 + pr) * st;
        const float* trow = T + r * ld + pp * 128;
        for (int col = lane; col < nl; col += 32) {
          const int64_t a = s_base[col] + b;
          const double vin = ADDBACK ? P.in[a] : 0.0;
          const double o = kReadOut ? P.out[a] : 0.0;
          P.out[a] = epilogue<EPI>(f2d_bits(trow[col]), vin, o, sc, ADDBACK);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// The bounded-wait path on its own: one CTA waits on an mbarrier that
// nothing ever arrives at, gives up after limit_ns and records PG_ETIMEOUT
// in the status word -- what the dense kernel does when a copy or an MMA
// never completes.  No copies are in flight and no tensor memory is held.
__global__ void wait_selftest_kernel(int* status, unsigned long long limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const bool ok = mbar_wait(&bar, 0, limit_ns);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(status, (int)PG_ETIMEOUT);
}

template <int ORIENT, int DIR, int EPI, bool ADDBACK>
int launch_one(const DParams& p, int ntiles, cudaStream_t st) {
  static bool attr = false;
  auto k = dense_kernel<ORIENT, DIR, EPI, ADDBACK>;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) {
      set_error("dense sweep: %s", cudaGetErrorString(e));
      return PG_ECUDA;
    }
    attr = true;
  }
  k<<<ntiles, kDenseThreads, kSmemBytes, st>>>(p);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("dense sweep: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

template <int ORIENT, int DIR>
int launch_epi(const DParams& p, int ntiles, int epi, bool addback, cudaStream_t st) {
  if (addback) {
    if (epi != EPI_STORE) {
      set_error("dense sweep: add-back operators only store");
      return PG_EINVAL;
    }
    return launch_one<ORIENT, DIR, EPI_STORE, true>(p, ntiles, st);
  }
  switch (epi) {
    case EPI_STORE: return launch_one<ORIENT, DIR, EPI_STORE, false>(p, ntiles, st);
    case EPI_ADD: return launch_one<ORIENT, DIR, EPI_ADD, false>(p, ntiles, st);
    case EPI_RING_SET: return launch_one<ORIENT, DIR, EPI_RING_SET, false>(p, ntiles, st);
    default: return launch_one<ORIENT, DIR, EPI_RING_MAX, false>(p, ntiles, st);
  }
}

}  // namespace

int launch_wait_selftest(int* status, unsigned limit_ms, void* stream) {
  wait_selftest_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(status, (unsigned long long)limit_ms * 1000000ull);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("wait self-test: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

int launch_dense(const DenseSet& ds, const double* in, double* out, int dir, int epi, int scale_pow, int* status,
                 void* stream) {
  if (ds.ntiles == 0) return PG_OK;
  DParams p{in, out, ds.ops, ds.tiles, status, scale_pow};
  cudaStream_t st = (cudaStream_t)stream;
  if (dir == 0) return launch_epi<0, 0>(p, ds.ntiles, epi, ds.addback, st);
  if (dir == 1) return launch_epi<1, 1>(p, ds.ntiles, epi, ds.addback, st);
  return launch_epi<1, 2>(p, ds.ntiles, epi, ds.addback, st);
}

// ---------------------------------------------------------------------------
// Host side: D from the banded operator, split into the swizzled TF32 planes.
// ---------------------------------------------------------------------------
namespace {

uint32_t host_tf32(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return (u + 0x1000u) & 0xFFFFE000u;
}

float host_f(uint32_t u) {
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}

}  // namespace

// D (row-major n x n, FP64) -> [kchunk][hi, lo][rows][32] TF32 words, rows
// padded to a multiple of 128 with zeros, each 8-row group 128B-swizzled.
void split_dense(const std::vector<double>& D, int n, std::vector<uint32_t>& out, int& rows, int& kchunks) {
  rows = (n + 127) / 128 * 128;
  kchunks = (n + kKC - 1) / kKC;
  out.assign((size_t)kchunks * 2 * rows * kKC, 0u);
  for (int c = 0; c < kchunks; c++)
    for (int r = 0; r < n; r++)
      for (int k = 0; k < kKC; k++) {
        const int col = c * kKC + k;
        if (col >= n) continue;
        const double v = D[(size_t)r * n + col];
        const uint32_t hb = host_tf32((float)v);
        const uint32_t lb = host_tf32((float)(v - (double)host_f(hb)));
        const int q = (k >> 2) ^ (r & 7);
        const size_t w = (size_t)r * kKC + q * 4 + (k & 3);
        out[((size_t)c * 2 + 0) * rows * kKC + w] = hb;
        out[((size_t)c * 2 + 1) * rows * kKC + w] = lb;
      }
}

}  // namespace pg
