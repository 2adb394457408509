// Learned LAD closure: a small MLP that predicts the artificial bulk viscosity
// beta and conductivity kappa of the LAD method from local features.
//
// Features of a point (kLadIn = 55, padded to kLadK = 64 inputs): the
// 27-point (3 x 3 x 3) stencils of  div(u) * D  and  |grad rho| * D  (|grad rho|
// by second-order central differences, lad_gradmag_kernel) around
// it (periodic directions wrap, one-sided directions clamp, a direction of one
// point repeats the point), then D itself, where D is the largest mesh
// spacing (the spacing across the shocks of the training problems, so that
// features and targets keep their scale between grids of other aspect ratios).  Each input is normalised, x = (f - mean) / std, with the
// training set's statistics.
//
// Network: 64 -> 64 -> 64 -> 64 -> 2, ReLU on the hidden layers, BF16 weights
// and BF16 activations between layers, FP32 accumulation.  The two outputs
// are normalised targets
//   y0 = beta / (rho D)             (a velocity scale)
//   y1 = kappa dt / (rho cv D^2)    (dimensionless)
// so that   beta = max(0, y0 s0 + m0) rho D,   kappa = max(0, y1 s1 + m1) rho cv D^2 / dt.
//
// Inference (lad_infer_tc_kernel) fuses the feature gather with the network on
// the 5th-generation tensor cores (tcgen05.mma kind::f16, BF16 operands in
// shared memory, FP32 accumulators in tensor memory) and raises a device flag
// when any raw output leaves [ylo, yhi] (the training range with a margin):
// the plain LAD closure is then the fallback.
// Training (lad_train_tc_kernel) runs the forward with the same BF16 rounding
// points and the backward on the tensor cores (mma.sync BF16 -> FP32, the
// FP32 gradients as BF16 hi + lo), MSE loss, FP32 gradient accumulation, and
// an Adam step in lad_adam_kernel.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "pg_internal.h"
#include "pg_sweep.cuh"  // d2f_bits: FP64 -> FP32 without the FP64 pipe
#include "pg_tc.cuh"     // tcgen05 helpers

namespace pg {
namespace {

constexpr int kIn = PG_LAD_IN;        // 55 features
constexpr int kK = PG_LAD_K;          // 64 padded inputs
constexpr int kH = PG_LAD_HIDDEN;     // 64
constexpr int kOut = PG_LAD_OUT;      // 2
constexpr int kTrainRows = 64;        // rows of a training CTA

__device__ __forceinline__ int wrapc(int i, int n, int per) {
  if (n == 1) return 0;
  if (per) return (i < 0) ? i + n : (i >= n ? i - n : i);
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// raw (unnormalised) feature f of point (i, j, k)
__device__ __forceinline__ float feature(const double* __restrict__ div, const double* __restrict__ gmag,
                                         const LadGrid& g, int i, int j, int k, int f) {
  if (f >= kIn) return 0.0f;
  if (f == kIn - 1) return (float)g.delta;  // raw features are f32(v) * f32(D), in FP32
  const int s = f % 27;
  const int di = s % 3 - 1, dj = (s / 3) % 3 - 1, dk = s / 9 - 1;
  const int64_t p = (int64_t)wrapc(i + di, g.n[0], g.per[0]) +
                    (int64_t)g.n[0] * (wrapc(j + dj, g.n[1], g.per[1]) + (int64_t)g.n[1] * wrapc(k + dk, g.n[2], g.per[2]));
  const double v = (f < 27) ? div[p] : gmag[p];
  return d2f_bits(v) * (float)g.delta;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One input column of the network: where its value sits in the staged
// neighbourhood (relative to the point) and its normalisation.
struct alignas(16) ColInfo {
  int off;
  float xm, xs;  // mean and 1/std
  int pad;
};

// parameter offsets (PG_LAD_NPARAM layout)
constexpr int kW1 = 0, kW2 = kH * kK, kW3 = kW2 + kH * kH, kW4 = kW3 + kH * kH, kB1 = kW4 + kOut * kH,
              kB2 = kB1 + kH, kB3 = kB2 + kH, kB4 = kB3 + kH;
static_assert(kB1 == PG_LAD_NWEIGHT && kB4 + kOut == PG_LAD_NPARAM, "parameter layout");

// Inference tile: 128 consecutive x-points of one (j, k) row.  The 3 x 3 rows
// around it (130 points each: one halo point per side) of div*D and
// |grad rho|*D are staged once in shared memory (rows 0..17), beside a row of
// D (18) and a row of zeros (19) for the constant and padding columns; every
// point's 64 features are read from there.
constexpr int kTileX = 128;
constexpr int kHaloX = kTileX + 2;
constexpr int kNbRows = 2 * 9 + 2;

// ----------------------------------------------------------- inference, tcgen05
// The same tile and features, with the network on the 5th-generation tensor
// cores.  One CTA of 128 threads owns a 128-point row tile (M = 128, one
// thread per point) and loops over tiles (persistent grid, one wave).  Per
// tile: each thread writes its 64 normalised BF16 features as row r of the A
// tile in shared memory (K-major, 128-byte swizzle); one thread issues the
// four K = 16 steps of tcgen05.mma kind::f16 (BF16 x BF16 -> FP32 in tensor
// memory, N = 64) against W1 and commits them to an mbarrier; every thread
// then reads its row of the accumulator (tcgen05.ld), adds the bias, applies
// ReLU and writes the row back, packed to BF16, as the next layer's A tile;
// the same for W2 and W3.  The 64 -> 2 output layer runs as one more MMA with
// W4 padded to N = 16 rows (the bias added after).  The weights are staged
// once per CTA in the same swizzled layout (the B operands: N rows of K = 64).
// Every wait is bounded: on a time-out the CTA records PG_ETIMEOUT in the
// status word, waits (bounded) for its own MMAs and still frees its tensor
// memory.
constexpr int kTcThreads = 128;
constexpr int kTcTmemCols = 64;
constexpr int kTcMaxResident = 8;  // 8 x 64 TMEM columns = the SM's 512
constexpr int kTcOutRows = 16;     // the output layer's N (kOut rows + zero rows)

struct TcSmem {                    // placed at a 1024-byte boundary
  uint8_t a[128 * 128];            // A: 128 rows x 64 BF16
  uint8_t w[3][kH * 128];          // B of the hidden layers: 64 rows (outputs) x 64 BF16 (inputs)
  uint8_t w4[kTcOutRows * 128];    // B of the output layer: rows >= kOut are zero
  float nb[kNbRows * kHaloX];      // the neighbourhood of the tile (rows 0..17 staged, 18: D, 19: zeros)
  float b[3][kH];
  float b4[kOut];
  ColInfo col[kK];
  uint64_t bar;
  uint32_t tmem_slot;
};

__global__ void __launch_bounds__(kTcThreads, 4) lad_infer_tc_kernel(const LadInferArgs A) {
  extern __shared__ __align__(16) unsigned char lad_tc_raw[];
  const uint32_t raw = smem_u32(lad_tc_raw);
  TcSmem& S = *reinterpret_cast<TcSmem*>(lad_tc_raw + (((raw + 1023u) & ~1023u) - raw));
  const pg_lad_model& M = A.model;
  const __nv_bfloat16* W = reinterpret_cast<const __nv_bfloat16*>(M.wbf16);
  const float* P = M.params;
  const int tid = threadIdx.x, warp = tid >> 5;
  const LadGrid& G = A.grid;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_slot)),
                 "r"(kTcTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&S.bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // weights: row n of a layer, 16-byte chunk q = inputs 8q .. 8q + 7 (BF16, already rounded)
  for (int i = tid; i < 3 * kH * 8; i += blockDim.x) {
    const int l = i / (kH * 8), n = (i / 8) % kH, q = i % 8;
    const int base = (l == 0 ? kW1 : (l == 1 ? kW2 : kW3)) + n * kK + 8 * q;
    *reinterpret_cast<uint4*>(S.w[l] + swz(n, q)) = *reinterpret_cast<const uint4*>(W + base);
  }
  for (int i = tid; i < kTcOutRows * 8; i += blockDim.x) {
    const int n = i / 8, q = i % 8;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (n < kOut) v = *reinterpret_cast<const uint4*>(W + kW4 + n * kH + 8 * q);
    *reinterpret_cast<uint4*>(S.w4 + swz(n, q)) = v;
  }
  for (int i = tid; i < kH; i += blockDim.x) {
    S.b[0][i] = P[kB1 + i];
    S.b[1][i] = P[kB2 + i];
    S.b[2][i] = P[kB3 + i];
  }
  if (tid < kOut) S.b4[tid] = P[kB4 + tid];
  for (int c = tid; c < kK; c += blockDim.x) {
    ColInfo ci;
    if (c < 2 * 27) {
      const int f = c / 27, s2 = c - f * 27;
      ci.off = (f * 9 + s2 / 3) * kHaloX + s2 % 3;
    } else {
      ci.off = (c == kIn - 1 ? 18 : 19) * kHaloX;
    }
    ci.xm = M.xmean[c];
    ci.xs = M.xinvstd[c];
    ci.pad = 0;
    S.col[c] = ci;
  }
  for (int xx = tid; xx < kHaloX; xx += blockDim.x) {
    S.nb[18 * kHaloX + xx] = (float)G.delta;
    S.nb[19 * kHaloX + xx] = 0.0f;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem_slot;
  const uint32_t a_addr = smem_u32(S.a);
  const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 lanes (= rows)

  const int nx = G.n[0], ny = G.n[1], nz = G.n[2];
  const int nxb = (nx + kTileX - 1) / kTileX;
  const long long ntiles = (long long)nxb * ny * nz;
  const float dl = (float)G.delta;
  const float fb = d2f_bits(G.delta), fk = d2f_bits(A.cv * G.delta * G.delta / A.dt[0]);
  bool out_of_range = false, bad = false;
  uint32_t phase = 0;
  const int r = tid;  // this thread's row: point x0 + r of the tile; also halo column r of the staging
  // the 36 halo elements beyond column 127 (columns 128 and 129 of the 18 rows): threads 0..35
  const int xr = (tid < 36) ? (tid >> 1) : -1, xc = kTileX + (tid & 1);

  // one layer: the A tile against B (n rows) into the accumulator; false on a time-out
  auto layer = [&](const uint8_t* B, int n) -> bool {
    fence_proxy_async();  // this thread's A row is visible to the tensor core
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t b_addr = smem_u32(B), idesc = idesc_bf16(n);
#pragma unroll
      for (int kk = 0; kk < kK / 16; kk++)
        tc_mma_bf16(tmem, sdesc(a_addr + kk * 32), sdesc(b_addr + kk * 32), idesc, kk > 0 ? 1 : 0);
      mma_commit(&S.bar);
    }
    const bool ok = mbar_wait(&S.bar, phase & 1);
    phase++;
    tc_fence_after();
    return ok;
  };
  // this thread's accumulator row + bias, ReLU, packed to BF16 as row r of the next A tile
  auto hidden = [&](int l) {
#pragma unroll
    for (int c0 = 0; c0 < kH; c0 += 32) {
      uint32_t u[32];
      tmem_ld16(tlane + (uint32_t)c0, u);
      tmem_ld16(tlane + (uint32_t)(c0 + 16), u + 16);
      tmem_wait_ld();
      uint32_t pk[16];
#pragma unroll
      for (int i = 0; i < 16; i++)
        pk[i] = pack_bf16(fmaxf(__uint_as_float(u[2 * i]) + S.b[l][c0 + 2 * i], 0.0f),
                          fmaxf(__uint_as_float(u[2 * i + 1]) + S.b[l][c0 + 2 * i + 1], 0.0f));
#pragma unroll
      for (int q = 0; q < 4; q++)
        *reinterpret_cast<uint4*>(S.a + swz(r, c0 / 8 + q)) =
            make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
    }
  };

  for (long long tile = blockIdx.x; tile < ntiles && !bad; tile += gridDim.x) {
    const int xb = (int)(tile % nxb);
    const long long row = tile / nxb;
    const int j = (int)(row % ny), k = (int)(row / ny);
    const int x0 = xb * kTileX;
    const int x = x0 + r;
    const int64_t prow = (int64_t)nx * (j + (int64_t)ny * k);
    const double rho_d = (x < nx) ? __ldg(A.rho + prow + x) : 1.0;
    {  // the neighbourhood, rows (f, dj, dk) x halo columns x0 - 1 .. x0 + 128: loads first, then stores
      const int xa = wrapc(x0 - 1 + r, nx, G.per[0]);
      const int xe = wrapc(x0 - 1 + xc, nx, G.per[0]);
      double v[18], ve = 0.0;
#pragma unroll
      for (int rr = 0; rr < 9; rr++) {
        const int jj = wrapc(j + rr % 3 - 1, ny, G.per[1]), kk = wrapc(k + rr / 3 - 1, nz, G.per[2]);
        const int64_t ro = (int64_t)nx * (jj + (int64_t)ny * kk);
        v[rr] = __ldg(A.div + ro + xa);
        v[9 + rr] = __ldg(A.gmag + ro + xa);
        if (xr == rr) ve = __ldg(A.div + ro + xe);
        if (xr == 9 + rr) ve = __ldg(A.gmag + ro + xe);
      }
      __syncthreads();  // the previous tile's neighbourhood is no longer read
#pragma unroll
      for (int q = 0; q < 18; q++) S.nb[q * kHaloX + r] = d2f_bits(v[q]) * dl;
      if (xr >= 0) S.nb[xr * kHaloX + xc] = d2f_bits(ve) * dl;
    }
    __syncthreads();
    {  // the features of point x0 + r, normalised and packed to BF16
#pragma unroll
      for (int q = 0; q < 8; q++) {
        uint32_t pk[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
          const ColInfo c0 = S.col[8 * q + 2 * h], c1 = S.col[8 * q + 2 * h + 1];
          pk[h] = pack_bf16((S.nb[c0.off + r] - c0.xm) * c0.xs, (S.nb[c1.off + r] - c1.xm) * c1.xs);
        }
        *reinterpret_cast<uint4*>(S.a + swz(r, q)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    if (!layer(S.w[0], kH)) bad = true;
    if (__syncthreads_or(bad)) break;
    hidden(0);
    if (!layer(S.w[1], kH)) bad = true;
    if (__syncthreads_or(bad)) break;
    hidden(1);
    if (!layer(S.w[2], kH)) bad = true;
    if (__syncthreads_or(bad)) break;
    hidden(2);
    if (!layer(S.w4, kTcOutRows)) bad = true;
    if (__syncthreads_or(bad)) break;
    uint32_t u[8];
    tmem_ld8_nowait(tlane, u);
    tmem_wait_ld();
    if (x < nx) {
      const float y0 = __uint_as_float(u[0]) + S.b4[0], y1 = __uint_as_float(u[1]) + S.b4[1];
      out_of_range |= !(y0 >= M.ylo[0] && y0 <= M.yhi[0] && y1 >= M.ylo[1] && y1 <= M.yhi[1]);
      const float rho = d2f_bits(rho_d);
      A.beta[prow + x] = f2d_bits(fmaxf(0.0f, fmaf(y0, M.ys[0], M.ym[0])) * rho * fb);
      A.kappa[prow + x] = f2d_bits(fmaxf(0.0f, fmaf(y1, M.ys[1], M.ym[1])) * rho * fk);
    }
    tc_fence_before();  // this tile's accumulator reads are done before the next tile's MMAs
  }
  if (bad && tid == 0) {
    atomicExch(A.status, (int)PG_ETIMEOUT);
    mbar_wait(&S.bar, (phase - 1) & 1);  // the MMAs still in flight (bounded)
  }
  if (__syncthreads_or(out_of_range) && tid == 0) atomicExch(A.flag, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols) : "memory");
  }
}

// |grad rho| by central differences, FP32 arithmetic: one thread per point,
// 32-bit indices (fields hold fewer than 2^31 points).
__global__ void lad_gradmag_kernel(const double* __restrict__ rho, const LadGrid G, double* __restrict__ out) {
  const unsigned nx = (unsigned)G.n[0], ny = (unsigned)G.n[1], nz = (unsigned)G.n[2];
  const unsigned np = nx * ny * nz;
  const unsigned st[3] = {1u, nx, nx * ny};
  for (unsigned p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    const unsigned r = p / nx;
    const unsigned idx[3] = {p - r * nx, r % ny, r / ny};
    float g2 = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const unsigned n = (unsigned)G.n[d], i = idx[d];
      if (n == 1) continue;
      unsigned lo, hi;
      float sc = G.rd[d];
      if (G.per[d]) {
        lo = (i == 0) ? n - 1 : i - 1;
        hi = (i == n - 1) ? 0 : i + 1;
        sc *= 0.5f;
      } else {
        lo = (i == 0) ? 0 : i - 1;
        hi = (i == n - 1) ? n - 1 : i + 1;
        if (i != 0 && i != n - 1) sc *= 0.5f;
      }
      const float a = d2f_bits(rho[p + (hi - i) * st[d]]), b = d2f_bits(rho[p - (i - lo) * st[d]]);
      const float dd = (a - b) * sc;
      g2 = fmaf(dd, dd, g2);
    }
    out[p] = f2d_bits(sqrtf(g2));
  }
}

// ----------------------------------------------------------------- training
// Feature rows for given points (training-set extraction): X[s][0..63] BF16.
__global__ void lad_features_kernel(const double* __restrict__ div, const double* __restrict__ gmag, LadGrid G,
                                    const int64_t* __restrict__ pts, int64_t ns, float* __restrict__ raw) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ns * kK;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = q / kK;
    const int f = (int)(q % kK);
    const int64_t p = pts[s];
    if (p < 0 || p >= (int64_t)G.n[0] * G.n[1] * G.n[2]) {  // not a point of the grid
      raw[q] = 0.0f;
      continue;
    }
    const int i = (int)(p % G.n[0]);
    const int j = (int)((p / G.n[0]) % G.n[1]);
    const int k = (int)(p / ((int64_t)G.n[0] * G.n[1]));
    raw[q] = feature(div, gmag, G, i, j, k, f);
  }
}

// Normalise raw feature rows into BF16 network inputs.
__global__ void lad_normalize_kernel(const float* __restrict__ raw, int64_t ns, const float* __restrict__ xm,
                                     const float* __restrict__ xs, __nv_bfloat16* __restrict__ X) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ns * kK;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int f = (int)(q % kK);
    X[q] = __float2bfloat16((raw[q] - xm[f]) * xs[f]);
  }
}

// ------------------------------------------------------- training, tensor cores
// The same step on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32
// accumulation).  One CTA = 64 rows of the batch, 4 warps of 16 rows.
//  forward:  per warp, each layer's FP32 accumulator fragments become the
//            next layer's BF16 A fragments in registers (bias, ReLU, BF16
//            rounding as in inference); the output layer pads N to 8;
//  backward: dY_l (the gradient at layer l's pre-activation, FP32) enters the
//            MMAs as BF16 hi + lo (two products), so the gradient keeps ~16
//            bits before its FP32 accumulation;
//            dH_{l-1} = dY_l W_l per warp (A = dY_l from its own fragments,
//            B = W_l^T from shared memory), masked by H_{l-1} > 0;
//            dW_l = dY_l^T H_{l-1} over the CTA's 64 rows (A = dY_l^T and
//            B = H_{l-1}^T from shared memory, each warp 16 output rows);
//            the 2-output layer's gradients and every bias gradient are
//            shuffle/shared-memory sums.  Gradients go to G with one atomic
//            per parameter per CTA.
constexpr int kTcTrainWarps = 4;
constexpr int kLd = kH + 8;  // BF16 row stride of the shared-memory operands (staggers banks)

struct TrainTcSmem {
  __nv_bfloat16 w[3][kH][kLd];    // W_l[o][q]   (forward B: rows o, consecutive q)
  __nv_bfloat16 wt[2][kH][kLd];   // W_l^T[q][o] for l = 2, 3 (backward B)
  __nv_bfloat16 w4[8][kLd];       // output layer, rows >= kOut zero
  __nv_bfloat16 ht[3][kH][kLd];   // X^T, H1^T, H2^T: [feature][row of the CTA]
  float dyt[kH][kTrainRows + 4];  // dY_l^T: [output][row]
  float w4f[kOut][kH];
  float b[3][kH];
  float b4[kOut];
  float red[kTcTrainWarps][kH];   // per-warp bias-gradient partials
  float loss[kTcTrainWarps];
};

__device__ __forceinline__ uint32_t ld_u32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// FP32 -> BF16 hi + BF16 lo (lo = the rounding residual of hi)
__device__ __forceinline__ void split_bf16(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

__global__ void __launch_bounds__(kTcTrainWarps * 32) lad_train_tc_kernel(const LadTrainArgs A) {
  extern __shared__ __align__(16) unsigned char lad_train_raw[];
  TrainTcSmem& S = *reinterpret_cast<TrainTcSmem*>(lad_train_raw);
  const pg_lad_model& M = A.model;
  const __nv_bfloat16* W = reinterpret_cast<const __nv_bfloat16*>(M.wbf16);
  const float* P = M.params;
  const __nv_bfloat16* X = reinterpret_cast<const __nv_bfloat16*>(A.X);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const int nthr = kTcTrainWarps * 32;
  const int64_t row0 = (int64_t)blockIdx.x * kTrainRows;
  const int nr = (int)((A.rows - row0) < kTrainRows ? (A.rows - row0) : kTrainRows);
  const __nv_bfloat16 z = __float2bfloat16(0.0f);
  for (int i = tid; i < kH * kK; i += nthr) {
    const int o = i / kK, q = i % kK;
    S.w[0][o][q] = W[kW1 + i];
    S.w[1][o][q] = W[kW2 + i];
    S.w[2][o][q] = W[kW3 + i];
    S.wt[0][q][o] = W[kW2 + i];
    S.wt[1][q][o] = W[kW3 + i];
  }
  for (int i = tid; i < 8 * kH; i += nthr) S.w4[i / kH][i % kH] = (i / kH < kOut) ? W[kW4 + i] : z;
  for (int i = tid; i < kOut * kH; i += nthr) S.w4f[i / kH][i % kH] = __bfloat162float(W[kW4 + i]);
  for (int i = tid; i < kH; i += nthr) {
    S.b[0][i] = P[kB1 + i];
    S.b[1][i] = P[kB2 + i];
    S.b[2][i] = P[kB3 + i];
  }
  if (tid < kOut) S.b4[tid] = P[kB4 + tid];
  // this warp's rows: r0 + g and r0 + g + 8 of the CTA
  const int r0 = warp * 16, ra = r0 + g, rb = r0 + g + 8;
  const bool va = ra < nr, vb = rb < nr;
  // X as A fragments (rows beyond the batch are zero) and as X^T in shared memory
  uint32_t ax[4][4];
#pragma unroll
  for (int kt = 0; kt < 4; kt++) {
#pragma unroll
    for (int h = 0; h < 4; h++) {
      const int rr = (h & 1) ? rb : ra, cc = kt * 16 + 2 * t + (h >> 1) * 8;
      const bool ok = (h & 1) ? vb : va;
      ax[kt][h] = ok ? ld_u32(X + (row0 + rr) * kK + cc) : 0u;
      const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162*>(&ax[kt][h]);
      S.ht[0][cc][rr] = v.x;
      S.ht[0][cc + 1][rr] = v.y;
    }
  }
  __syncthreads();
  // one forward layer: c = b + A W^T, then ReLU -> BF16 A fragments of the next layer (and H^T)
  auto forward = [&](const uint32_t (*a)[4], int l, uint32_t (*an)[4], int store) {
    float c[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const float b0 = S.b[l][nt * 8 + 2 * t], b1 = S.b[l][nt * 8 + 2 * t + 1];
      c[nt][0] = b0; c[nt][1] = b1; c[nt][2] = b0; c[nt][3] = b1;
#pragma unroll
      for (int kt = 0; kt < 4; kt++)
        mma_bf16(c[nt], a[kt], ld_u32(&S.w[l][nt * 8 + g][kt * 16 + 2 * t]),
                 ld_u32(&S.w[l][nt * 8 + g][kt * 16 + 2 * t + 8]));
    }
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
      an[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
      an[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
      an[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
      an[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
    }
    if (store >= 0) {
#pragma unroll
      for (int kt = 0; kt < 4; kt++)
#pragma unroll
        for (int h = 0; h < 4; h++) {
          const int rr = (h & 1) ? rb : ra, cc = kt * 16 + 2 * t + (h >> 1) * 8;
          const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162*>(&an[kt][h]);
          S.ht[store][cc][rr] = v.x;
          S.ht[store][cc + 1][rr] = v.y;
        }
    }
  };
  uint32_t a1[4][4], a2[4][4], a3[4][4];
  forward(ax, 0, a1, 1);
  forward(a1, 1, a2, 2);
  forward(a2, 2, a3, -1);
  // output layer (N padded to 8): lanes with t = 0 hold outputs 0, 1 of rows ra and rb
  float c4[4] = {S.b4[0], S.b4[1], S.b4[0], S.b4[1]};
  if (t != 0) c4[0] = c4[1] = c4[2] = c4[3] = 0.0f;
#pragma unroll
  for (int kt = 0; kt < 4; kt++)
    mma_bf16(c4, a3[kt], ld_u32(&S.w4[g][kt * 16 + 2 * t]), ld_u32(&S.w4[g][kt * 16 + 2 * t + 8]));
  float dya[2] = {0.f, 0.f}, dyb[2] = {0.f, 0.f}, lsum = 0.f;
  if (t == 0) {
#pragma unroll
    for (int o = 0; o < kOut; o++) {
      if (va) {
        const float e = c4[o] - A.T[(row0 + ra) * kOut + o];
        lsum += e * e;
        dya[o] = 2.0f * e * A.inv_count;
        if (A.Y) A.Y[(row0 + ra) * kOut + o] = c4[o];
      }
      if (vb) {
        const float e = c4[2 + o] - A.T[(row0 + rb) * kOut + o];
        lsum += e * e;
        dyb[o] = 2.0f * e * A.inv_count;
        if (A.Y) A.Y[(row0 + rb) * kOut + o] = c4[2 + o];
      }
    }
  }
#pragma unroll
  for (int o = 0; o < kOut; o++) {  // every lane of row g: the row's dy
    dya[o] = __shfl_sync(0xffffffffu, dya[o], g * 4);
    dyb[o] = __shfl_sync(0xffffffffu, dyb[o], g * 4);
  }
  // dY3 = (dy W4) masked by H3 > 0, in accumulator layout; dW4 = dy^T H3, db4 = sum dy
  float d[8][4];
  float gw4[kOut][8][2];
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const __nv_bfloat162 ha = *reinterpret_cast<const __nv_bfloat162*>(&a3[nt >> 1][(nt & 1) * 2]);
    const __nv_bfloat162 hb = *reinterpret_cast<const __nv_bfloat162*>(&a3[nt >> 1][(nt & 1) * 2 + 1]);
    const float h[4] = {__bfloat162float(ha.x), __bfloat162float(ha.y), __bfloat162float(hb.x), __bfloat162float(hb.y)};
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const int q = nt * 8 + 2 * t + (e & 1);
      const float* dy = (e < 2) ? dya : dyb;
      const float s = dy[0] * S.w4f[0][q] + dy[1] * S.w4f[1][q];
      d[nt][e] = h[e] > 0.0f ? s : 0.0f;
    }
#pragma unroll
    for (int o = 0; o < kOut; o++) {
      gw4[o][nt][0] = dya[o] * h[0] + dyb[o] * h[2];
      gw4[o][nt][1] = dya[o] * h[1] + dyb[o] * h[3];
    }
  }
  // sums over the rows of the warp (lanes with equal t), then over the warps
#pragma unroll
  for (int o = 0; o < kOut; o++)
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
      for (int e = 0; e < 2; e++) {
        float v = gw4[o][nt][e];
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        v += __shfl_xor_sync(0xffffffffu, v, 8);
        v += __shfl_xor_sync(0xffffffffu, v, 16);
        gw4[o][nt][e] = v;
      }
  if (g == 0) {
#pragma unroll
    for (int o = 0; o < kOut; o++)
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        atomicAdd(&A.grad[kW4 + o * kH + nt * 8 + 2 * t], gw4[o][nt][0]);
        atomicAdd(&A.grad[kW4 + o * kH + nt * 8 + 2 * t + 1], gw4[o][nt][1]);
      }
  }
  {
    float sd[kOut];
#pragma unroll
    for (int o = 0; o < kOut; o++) {
      float v = (t == 0) ? dya[o] + dyb[o] : 0.f;
      v += __shfl_xor_sync(0xffffffffu, v, 4);
      v += __shfl_xor_sync(0xffffffffu, v, 8);
      v += __shfl_xor_sync(0xffffffffu, v, 16);
      sd[o] = v;
    }
    if (lane == 0)
      for (int o = 0; o < kOut; o++) atomicAdd(&A.grad[kB4 + o], sd[o]);
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) S.loss[warp] = lsum;

  // hidden layers l = 3, 2, 1 (index 2, 1, 0): d holds dY_l in accumulator layout
  for (int l = 2; l >= 0; l--) {
    // bias gradient: column sums of dY_l over the CTA's rows
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
      for (int e = 0; e < 2; e++) {
        float v = d[nt][e] + d[nt][2 + e];
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        v += __shfl_xor_sync(0xffffffffu, v, 8);
        v += __shfl_xor_sync(0xffffffffu, v, 16);
        if (g == 0) S.red[warp][nt * 8 + 2 * t + e] = v;
      }
    // dY_l^T for the weight gradient
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
      for (int e = 0; e < 4; e++) S.dyt[nt * 8 + 2 * t + (e & 1)][(e < 2) ? ra : rb] = d[nt][e];
    __syncthreads();
    for (int o = tid; o < kH; o += nthr) {
      float v = 0.f;
      for (int w = 0; w < kTcTrainWarps; w++) v += S.red[w][o];
      atomicAdd(&A.grad[(l == 0 ? kB1 : (l == 1 ? kB2 : kB3)) + o], v);
    }
    // dW_l[o][q] = sum_r dY_l[r][o] H_{l-1}[r][q]: this warp's 16 output rows o, all q, K = the 64 rows
    {
      float cw[8][4];
#pragma unroll
      for (int nt = 0; nt < 8; nt++) cw[nt][0] = cw[nt][1] = cw[nt][2] = cw[nt][3] = 0.f;
      const int oa = r0 + g, ob = r0 + g + 8;
#pragma unroll
      for (int kt = 0; kt < 4; kt++) {
        uint32_t ah[4], al[4];
        split_bf16(S.dyt[oa][kt * 16 + 2 * t], S.dyt[oa][kt * 16 + 2 * t + 1], ah[0], al[0]);
        split_bf16(S.dyt[ob][kt * 16 + 2 * t], S.dyt[ob][kt * 16 + 2 * t + 1], ah[1], al[1]);
        split_bf16(S.dyt[oa][kt * 16 + 2 * t + 8], S.dyt[oa][kt * 16 + 2 * t + 9], ah[2], al[2]);
        split_bf16(S.dyt[ob][kt * 16 + 2 * t + 8], S.dyt[ob][kt * 16 + 2 * t + 9], ah[3], al[3]);
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
          const uint32_t b0 = ld_u32(&S.ht[l][nt * 8 + g][kt * 16 + 2 * t]);
          const uint32_t b1 = ld_u32(&S.ht[l][nt * 8 + g][kt * 16 + 2 * t + 8]);
          mma_bf16(cw[nt], ah, b0, b1);
          mma_bf16(cw[nt], al, b0, b1);
        }
      }
      float* gw = A.grad + (l == 0 ? kW1 : (l == 1 ? kW2 : kW3));
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const int q = nt * 8 + 2 * t;
        atomicAdd(&gw[oa * kK + q], cw[nt][0]);
        atomicAdd(&gw[oa * kK + q + 1], cw[nt][1]);
        atomicAdd(&gw[ob * kK + q], cw[nt][2]);
        atomicAdd(&gw[ob * kK + q + 1], cw[nt][3]);
      }
    }
    if (l == 0) break;
    // dY_{l-1} = (dY_l W_l) masked by H_{l-1} > 0 (this warp's rows)
    {
      uint32_t ah[4][4], al[4][4];
#pragma unroll
      for (int kt = 0; kt < 4; kt++) {
        split_bf16(d[2 * kt][0], d[2 * kt][1], ah[kt][0], al[kt][0]);
        split_bf16(d[2 * kt][2], d[2 * kt][3], ah[kt][1], al[kt][1]);
        split_bf16(d[2 * kt + 1][0], d[2 * kt + 1][1], ah[kt][2], al[kt][2]);
        split_bf16(d[2 * kt + 1][2], d[2 * kt + 1][3], ah[kt][3], al[kt][3]);
      }
      const uint32_t (*hb)[4] = (l == 2) ? a2 : a1;
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
          const uint32_t b0 = ld_u32(&S.wt[l - 1][nt * 8 + g][kt * 16 + 2 * t]);
          const uint32_t b1 = ld_u32(&S.wt[l - 1][nt * 8 + g][kt * 16 + 2 * t + 8]);
          mma_bf16(c, ah[kt], b0, b1);
          mma_bf16(c, al[kt], b0, b1);
        }
        const __nv_bfloat162 ha = *reinterpret_cast<const __nv_bfloat162*>(&hb[nt >> 1][(nt & 1) * 2]);
        const __nv_bfloat162 hb2 = *reinterpret_cast<const __nv_bfloat162*>(&hb[nt >> 1][(nt & 1) * 2 + 1]);
        d[nt][0] = __bfloat162float(ha.x) > 0.f ? c[0] : 0.f;
        d[nt][1] = __bfloat162float(ha.y) > 0.f ? c[1] : 0.f;
        d[nt][2] = __bfloat162float(hb2.x) > 0.f ? c[2] : 0.f;
        d[nt][3] = __bfloat162float(hb2.y) > 0.f ? c[3] : 0.f;
      }
    }
    __syncthreads();  // dyt and red are rewritten for the next layer
  }
  __syncthreads();
  if (tid == 0 && A.loss) {
    float lt = 0.f;
    for (int w = 0; w < kTcTrainWarps; w++) lt += S.loss[w];
    atomicAdd(A.loss, lt * A.inv_count);
  }
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters, then the BF16 copies.
__global__ void lad_adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                                const float* __restrict__ g, int n, float lr, float b1, float b2, float eps,
                                float c1, float c2, __nv_bfloat16* __restrict__ pbf, int nbf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    p[i] = pi;
    if (i < nbf) pbf[i] = __float2bfloat16(pi);
  }
}

int lad_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

}  // namespace

int launch_lad_infer(const LadInferArgs& a, void* stream) {
  static int resident = 0;  // CTAs per SM (persistent grid: one wave)
  static int sms = 0;
  const int smem = (int)(sizeof(TcSmem) + 1024);  // + slack for the 1024-byte alignment
  if (resident == 0) {
    cudaError_t e = cudaFuncSetAttribute(lad_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // CTAs per SM from the kernel's own footprint (registers, shared memory + the 1 KB each CTA
    // reserves); the occupancy query reported one CTA per SM for this tensor-memory kernel
    cudaFuncAttributes fa;
    int smem_sm = 0;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, lad_infer_tc_kernel);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e != cudaSuccess) {
      set_error("lad inference: %s", cudaGetErrorString(e));
      return PG_ECUDA;
    }
    const int by_smem = smem_sm / (smem + 1024);
    const int by_regs = 65536 / (kTcThreads * (fa.numRegs > 0 ? fa.numRegs : 255));
    resident = by_smem < by_regs ? by_smem : by_regs;
    // every resident CTA holds kTcTmemCols of the SM's 512 tensor-memory columns
    if (resident > kTcMaxResident) resident = kTcMaxResident;
    if (resident < 1) {
      set_error("lad inference: the kernel does not fit an SM");
      resident = 0;
      return PG_ECUDA;
    }
  }
  const int64_t tiles = (int64_t)((a.grid.n[0] + kTileX - 1) / kTileX) * a.grid.n[1] * a.grid.n[2];
  const int64_t wave = (int64_t)sms * resident;
  const int blocks = (int)(tiles < wave ? tiles : wave);
  lad_infer_tc_kernel<<<blocks, kTcThreads, smem, (cudaStream_t)stream>>>(a);
  count_launch();
  return lad_check("lad inference");
}

int launch_lad_grad_magnitude(const double* rho, const LadGrid& g, double* out, void* stream) {
  const int64_t np = (int64_t)g.n[0] * g.n[1] * g.n[2];
  const int64_t b = (np + 255) / 256;
  lad_gradmag_kernel<<<(unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16), 256, 0, (cudaStream_t)stream>>>(rho, g,
                                                                                                             out);
  count_launch();
  return lad_check("lad grad magnitude");
}

int launch_lad_features(const double* div, const double* gmag, const LadGrid& g, const int64_t* pts, int64_t ns,
                        float* raw, void* stream) {
  const int64_t total = ns * kK;
  const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  lad_features_kernel<<<blocks > 0 ? blocks : 1, 256, 0, (cudaStream_t)stream>>>(div, gmag, g, pts, ns, raw);
  count_launch();
  return lad_check("lad features");
}

int launch_lad_normalize(const float* raw, int64_t ns, const float* xm, const float* xs, void* X, void* stream) {
  const int64_t total = ns * kK;
  const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  lad_normalize_kernel<<<blocks > 0 ? blocks : 1, 256, 0, (cudaStream_t)stream>>>(raw, ns, xm, xs, reinterpret_cast<__nv_bfloat16*>(X));
  count_launch();
  return lad_check("lad normalize");
}

int launch_lad_train(const LadTrainArgs& a, void* stream) {
  static bool attr = false;
  const int smem = (int)sizeof(TrainTcSmem);
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(lad_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) {
      set_error("lad training: %s", cudaGetErrorString(e));
      return PG_ECUDA;
    }
    attr = true;
  }
  if (a.rows <= 0) return PG_OK;
  const int blocks = (int)((a.rows + kTrainRows - 1) / kTrainRows);
  lad_train_tc_kernel<<<blocks, kTcTrainWarps * 32, smem, (cudaStream_t)stream>>>(a);
  count_launch();
  return lad_check("lad training");
}

int launch_lad_adam(float* p, float* m, float* v, const float* g, int n, float lr, float b1, float b2, float eps,
                    int step, void* pbf, int nbf, void* stream) {
  const float c1 = 1.0f / (1.0f - powf(b1, (float)step));
  const float c2 = 1.0f / (1.0f - powf(b2, (float)step));
  lad_adam_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(p, m, v, g, n, lr, b1, b2, eps, c1, c2,
                                                                     reinterpret_cast<__nv_bfloat16*>(pbf), nbf);
  count_launch();
  return lad_check("lad adam");
}

}  // namespace pg
