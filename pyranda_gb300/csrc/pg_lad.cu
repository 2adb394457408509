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
// Inference (lad_infer_kernel) fuses the feature gather with the network on
// the tensor cores (mma.sync m16n8k16 BF16 -> FP32; each layer's accumulator
// fragments are repacked in registers as the next layer's A operand) and
// raises a device flag when any raw output leaves [ylo, yhi] (the training
// range with a margin): the plain LAD closure is then the fallback.
// Training runs the same arithmetic on CUDA cores in lad_train_kernel
// (forward with BF16 rounding at the same points, MSE loss, backward, FP32
// gradient accumulation) and an Adam step in lad_adam_kernel.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "pg_internal.h"
#include "pg_sweep.cuh"  // d2f_bits: FP64 -> FP32 without the FP64 pipe

namespace pg {
namespace {

constexpr int kIn = PG_LAD_IN;        // 55 features
constexpr int kK = PG_LAD_K;          // 64 padded inputs
constexpr int kH = PG_LAD_HIDDEN;     // 64
constexpr int kOut = PG_LAD_OUT;      // 2
constexpr int kInferThreads = 256;    // 8 warps x 16 points = one 128-point row tile
constexpr int kTrainRows = 64;        // rows of a training CTA
constexpr int kTrainThreads = 256;

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

// Shared-memory image of the network for inference: weights as BF16 rows
// [N][K + 8] (the pad staggers banks), biases and normalisation in FP32.
struct InferSmem {
  __nv_bfloat16 w1[kH][kK + 8];
  __nv_bfloat16 w2[kH][kH + 8];
  __nv_bfloat16 w3[kH][kH + 8];
  __nv_bfloat16 w4[8][kH + 8];   // rows >= kOut are zero
  float b1[kH], b2[kH], b3[kH], b4[8];
  ColInfo col[kK];
};

// one hidden layer: A fragments (4 k-tiles) -> ReLU(W A + b) as next A fragments
template <int KT>
__device__ __forceinline__ void layer_relu(const uint32_t (*a)[4], uint32_t (*anext)[4],
                                           const __nv_bfloat16 (*w)[kH + 8], const float* b, int g, int t) {
  float c[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; nt++) {
    const float b0 = b[nt * 8 + 2 * t], b1 = b[nt * 8 + 2 * t + 1];
    c[nt][0] = b0; c[nt][1] = b1; c[nt][2] = b0; c[nt][3] = b1;
#pragma unroll
    for (int kt = 0; kt < KT; kt++) {
      const uint32_t w0 = *reinterpret_cast<const uint32_t*>(&w[nt * 8 + g][kt * 16 + 2 * t]);
      const uint32_t w1 = *reinterpret_cast<const uint32_t*>(&w[nt * 8 + g][kt * 16 + 2 * t + 8]);
      mma_bf16(c[nt], a[kt], w0, w1);
    }
  }
#pragma unroll
  for (int kt = 0; kt < 4; kt++) {
    anext[kt][0] = pack_bf16(fmaxf(c[2 * kt][0], 0.f), fmaxf(c[2 * kt][1], 0.f));
    anext[kt][1] = pack_bf16(fmaxf(c[2 * kt][2], 0.f), fmaxf(c[2 * kt][3], 0.f));
    anext[kt][2] = pack_bf16(fmaxf(c[2 * kt + 1][0], 0.f), fmaxf(c[2 * kt + 1][1], 0.f));
    anext[kt][3] = pack_bf16(fmaxf(c[2 * kt + 1][2], 0.f), fmaxf(c[2 * kt + 1][3], 0.f));
  }
}

// parameter offsets (PG_LAD_NPARAM layout)
constexpr int kW1 = 0, kW2 = kH * kK, kW3 = kW2 + kH * kH, kW4 = kW3 + kH * kH, kB1 = kW4 + kOut * kH,
              kB2 = kB1 + kH, kB3 = kB2 + kH, kB4 = kB3 + kH;
static_assert(kB1 == PG_LAD_NWEIGHT && kB4 + kOut == PG_LAD_NPARAM, "parameter layout");

// One CTA = 128 consecutive x-points of one (j, k) row.  The 3 x 3 rows
// around it (130 points each: one halo point per side) of div*D and
// |grad rho|*D are staged once in shared memory (rows 0..17), after a row of
// D (18) and a row of zeros (19) for the constant and padding columns; every
// warp then builds the features of its 16 points from there and runs the
// network.
constexpr int kTileX = 128;
constexpr int kHaloX = kTileX + 2;
constexpr int kNbRows = 2 * 9 + 2;

__global__ void __launch_bounds__(kInferThreads) lad_infer_kernel(const LadInferArgs A) {
  extern __shared__ __align__(16) unsigned char lad_smem[];
  InferSmem& S = *reinterpret_cast<InferSmem*>(lad_smem);
  float* nbf = reinterpret_cast<float*>(lad_smem + sizeof(InferSmem));
  const pg_lad_model& M = A.model;
  const __nv_bfloat16* W = reinterpret_cast<const __nv_bfloat16*>(M.wbf16);
  const float* P = M.params;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  for (int i = tid; i < kH * kK; i += blockDim.x) S.w1[i / kK][i % kK] = W[kW1 + i];
  for (int i = tid; i < kH * kH; i += blockDim.x) {
    S.w2[i / kH][i % kH] = W[kW2 + i];
    S.w3[i / kH][i % kH] = W[kW3 + i];
  }
  for (int i = tid; i < 8 * kH; i += blockDim.x)
    S.w4[i / kH][i % kH] = (i / kH < kOut) ? W[kW4 + i] : __float2bfloat16(0.0f);
  for (int i = tid; i < kH; i += blockDim.x) {
    S.b1[i] = P[kB1 + i];
    S.b2[i] = P[kB2 + i];
    S.b3[i] = P[kB3 + i];
  }
  if (tid < 8) S.b4[tid] = tid < kOut ? P[kB4 + tid] : 0.0f;
  const LadGrid& G = A.grid;
  for (int c = tid; c < kK; c += blockDim.x) {
    ColInfo ci;
    if (c < 2 * 27) {   // feature f at stencil point s2 = (di+1) + 3 (dj+1) + 9 (dk+1): row (f, dj, dk), x offset di
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
    nbf[18 * kHaloX + xx] = (float)G.delta;
    nbf[19 * kHaloX + xx] = 0.0f;
  }
  const int nx = G.n[0], ny = G.n[1], nz = G.n[2];
  const int nxb = (nx + kTileX - 1) / kTileX;
  const long long ntiles = (long long)nxb * ny * nz;
  const float dl = (float)G.delta;
  // beta = max(0, y0 s0 + m0) rho D,  kappa = max(0, y1 s1 + m1) rho cv D^2 / dt: the factors of the
  // launch once in FP64, the per-point arithmetic in FP32 (GB300's FP64 pipe is 1/58 of FP32)
  const float fb = d2f_bits(G.delta), fk = d2f_bits(A.cv * G.delta * G.delta / A.dt[0]);
  bool out_of_range = false;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int xb = (int)(tile % nxb);
    const long long row = tile / nxb;
    const int j = (int)(row % ny), k = (int)(row / ny);
    const int x0 = xb * kTileX;
    __syncthreads();  // the previous tile's neighbourhood is no longer read
    for (int q = tid; q < 2 * 9 * kHaloX; q += blockDim.x) {
      const int f = q / (9 * kHaloX), rem = q - f * 9 * kHaloX;
      const int rr = rem / kHaloX, xx = rem - rr * kHaloX;
      const int jj = wrapc(j + rr % 3 - 1, ny, G.per[1]), kk = wrapc(k + rr / 3 - 1, nz, G.per[2]);
      const int x = wrapc(x0 - 1 + xx, nx, G.per[0]);
      const int64_t p = (int64_t)x + (int64_t)nx * (jj + (int64_t)ny * kk);
      nbf[q] = d2f_bits(f == 0 ? A.div[p] : A.gmag[p]) * dl;
    }
    __syncthreads();
    const int lx0 = warp * 16;
    if (x0 + lx0 < nx) {
      // A fragments straight from the neighbourhood: column c of row r is feature c of point lx0 + r;
      // a lane holds columns kt*16 + 2t + {0, 1, 8, 9} of rows g and g + 8
      uint32_t a0[4][4], a1[4][4];
      const float* pt = nbf + lx0 + g;
#pragma unroll
      for (int kt = 0; kt < 4; kt++) {
        float v[4][2];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const ColInfo ci = S.col[kt * 16 + 2 * t + (q & 1) + (q >> 1) * 8];
          v[q][0] = (pt[ci.off] - ci.xm) * ci.xs;
          v[q][1] = (pt[ci.off + 8] - ci.xm) * ci.xs;
        }
        a0[kt][0] = pack_bf16(v[0][0], v[1][0]);
        a0[kt][1] = pack_bf16(v[0][1], v[1][1]);
        a0[kt][2] = pack_bf16(v[2][0], v[3][0]);
        a0[kt][3] = pack_bf16(v[2][1], v[3][1]);
      }
      layer_relu<4>(a0, a1, S.w1, S.b1, g, t);
      layer_relu<4>(a1, a0, S.w2, S.b2, g, t);
      layer_relu<4>(a0, a1, S.w3, S.b3, g, t);
      float c[4] = {S.b4[2 * t], S.b4[2 * t + 1], S.b4[2 * t], S.b4[2 * t + 1]};
#pragma unroll
      for (int kt = 0; kt < 4; kt++) {
        const uint32_t w0 = *reinterpret_cast<const uint32_t*>(&S.w4[g][kt * 16 + 2 * t]);
        const uint32_t w1 = *reinterpret_cast<const uint32_t*>(&S.w4[g][kt * 16 + 2 * t + 8]);
        mma_bf16(c, a1[kt], w0, w1);
      }
      // lanes with t == 0 hold outputs 0 and 1 of rows g and g + 8
      if (t == 0) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int x = x0 + lx0 + g + 8 * h;
          if (x < nx) {
            const int64_t p = (int64_t)x + (int64_t)nx * (j + (int64_t)ny * k);
            const float y0 = c[2 * h], y1 = c[2 * h + 1];
            out_of_range |= !(y0 >= M.ylo[0] && y0 <= M.yhi[0] && y1 >= M.ylo[1] && y1 <= M.yhi[1]);
            const float rho = d2f_bits(A.rho[p]);
            // artificial viscosity and conductivity are non-negative (the plain operators are)
            A.beta[p] = f2d_bits(fmaxf(0.0f, fmaf(y0, M.ys[0], M.ym[0])) * rho * fb);
            A.kappa[p] = f2d_bits(fmaxf(0.0f, fmaf(y1, M.ys[1], M.ym[1])) * rho * fk);
          }
        }
      }
    }
  }
  if (__syncthreads_or(out_of_range) && tid == 0) atomicExch(A.flag, 1);
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

struct TrainSmem {
  float w1[kH][kK + 1], w2[kH][kH + 1], w3[kH][kH + 1], w4[kOut][kH + 1];
  float b1[kH], b2[kH], b3[kH], b4[kOut];
  float h1[kTrainRows][kH + 1], h2[kTrainRows][kH + 1], h3[kTrainRows][kH + 1];
  float x[kTrainRows][kK + 1];
  float d[kTrainRows][kH + 1];   // gradient w.r.t. the current layer's pre-activation
  float e[kTrainRows][kH + 1];   // gradient w.r.t. the layer below's output
  float dy[kTrainRows][kOut];
  float loss[kTrainThreads / 32];
};

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16(x)); }

// One CTA: kTrainRows rows of the batch.  Forward in BF16-in / FP32-accumulate
// with BF16 rounding of inputs, weights and hidden activations (the inference
// kernel's arithmetic), loss = mean over rows and outputs of (y - t)^2,
// backward in FP32, gradients added into G (FP32) with atomics.
__global__ void __launch_bounds__(kTrainThreads) lad_train_kernel(const LadTrainArgs A) {
  extern __shared__ __align__(16) unsigned char lad_smem[];
  TrainSmem& S = *reinterpret_cast<TrainSmem*>(lad_smem);
  const pg_lad_model& M = A.model;
  const __nv_bfloat16* W = reinterpret_cast<const __nv_bfloat16*>(M.wbf16);
  const float* P = M.params;
  const __nv_bfloat16* X = reinterpret_cast<const __nv_bfloat16*>(A.X);
  const int tid = threadIdx.x;
  const int64_t row0 = (int64_t)blockIdx.x * kTrainRows;
  const int nr = (int)((A.rows - row0) < kTrainRows ? (A.rows - row0) : kTrainRows);
  for (int i = tid; i < kH * kK; i += kTrainThreads) S.w1[i / kK][i % kK] = __bfloat162float(W[kW1 + i]);
  for (int i = tid; i < kH * kH; i += kTrainThreads) {
    S.w2[i / kH][i % kH] = __bfloat162float(W[kW2 + i]);
    S.w3[i / kH][i % kH] = __bfloat162float(W[kW3 + i]);
  }
  for (int i = tid; i < kOut * kH; i += kTrainThreads) S.w4[i / kH][i % kH] = __bfloat162float(W[kW4 + i]);
  for (int i = tid; i < kH; i += kTrainThreads) {
    S.b1[i] = P[kB1 + i];
    S.b2[i] = P[kB2 + i];
    S.b3[i] = P[kB3 + i];
  }
  if (tid < kOut) S.b4[tid] = P[kB4 + tid];
  for (int i = tid; i < kTrainRows * kK; i += kTrainThreads) {
    const int r = i / kK, f = i % kK;
    S.x[r][f] = (r < nr) ? __bfloat162float(X[(row0 + r) * kK + f]) : 0.0f;
  }
  __syncthreads();
  // forward: h = bf16(relu(W x + b)) for three layers
  auto dense = [&](const float (*w)[kH + 1], const float* b, const float (*in)[kH + 1], float (*out)[kH + 1]) {
    for (int i = tid; i < kTrainRows * kH; i += kTrainThreads) {
      const int r = i / kH, o = i % kH;
      float s = b[o];
      for (int q = 0; q < kH; q++) s += w[o][q] * in[r][q];
      out[r][o] = bf16r(fmaxf(s, 0.0f));
    }
    __syncthreads();
  };
  for (int i = tid; i < kTrainRows * kH; i += kTrainThreads) {
    const int r = i / kH, o = i % kH;
    float s = S.b1[o];
    for (int q = 0; q < kK; q++) s += S.w1[o][q] * S.x[r][q];
    S.h1[r][o] = bf16r(fmaxf(s, 0.0f));
  }
  __syncthreads();
  dense(S.w2, S.b2, S.h1, S.h2);
  dense(S.w3, S.b3, S.h2, S.h3);
  // outputs, loss and dL/dy
  float lsum = 0.0f;
  for (int i = tid; i < kTrainRows * kOut; i += kTrainThreads) {
    const int r = i / kOut, o = i % kOut;
    float s = S.b4[o];
    for (int q = 0; q < kH; q++) s += S.w4[o][q] * S.h3[r][q];
    float g = 0.0f;
    if (r < nr) {
      const float e = s - A.T[(row0 + r) * kOut + o];
      lsum += e * e;
      g = 2.0f * e * A.inv_count;
      if (A.Y) A.Y[(row0 + r) * kOut + o] = s;
    }
    S.dy[r][o] = g;
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((tid & 31) == 0) S.loss[tid >> 5] = lsum;
  __syncthreads();
  if (tid == 0 && A.loss) {
    float l = 0.0f;
    for (int w = 0; w < kTrainThreads / 32; w++) l += S.loss[w];
    atomicAdd(A.loss, l * A.inv_count);
  }
  // layer 4: dW4 = dy^T h3, db4 = sum dy, d(h3) = dy W4 masked by h3 > 0
  for (int i = tid; i < kOut * kH; i += kTrainThreads) {
    const int o = i / kH, q = i % kH;
    float s = 0.0f;
    for (int r = 0; r < kTrainRows; r++) s += S.dy[r][o] * S.h3[r][q];
    atomicAdd(&A.grad[kW4 + i], s);
  }
  if (tid < kOut) {
    float s = 0.0f;
    for (int r = 0; r < kTrainRows; r++) s += S.dy[r][tid];
    atomicAdd(&A.grad[kB4 + tid], s);
  }
  for (int i = tid; i < kTrainRows * kH; i += kTrainThreads) {
    const int r = i / kH, q = i % kH;
    float s = 0.0f;
    for (int o = 0; o < kOut; o++) s += S.dy[r][o] * S.w4[o][q];
    S.d[r][q] = (S.h3[r][q] > 0.0f) ? s : 0.0f;
  }
  __syncthreads();
  // hidden layers 3 and 2: dW = d^T h_below, db = sum d, e = d W masked by h_below > 0
  auto back = [&](const float (*w)[kH + 1], const float (*hb)[kH + 1], float* gw, float* gb) {
    for (int i = tid; i < kH * kH; i += kTrainThreads) {
      const int o = i / kH, q = i % kH;
      float s = 0.0f;
      for (int r = 0; r < kTrainRows; r++) s += S.d[r][o] * hb[r][q];
      atomicAdd(&gw[i], s);
    }
    for (int o = tid; o < kH; o += kTrainThreads) {
      float s = 0.0f;
      for (int r = 0; r < kTrainRows; r++) s += S.d[r][o];
      atomicAdd(&gb[o], s);
    }
    for (int i = tid; i < kTrainRows * kH; i += kTrainThreads) {
      const int r = i / kH, q = i % kH;
      float s = 0.0f;
      for (int o = 0; o < kH; o++) s += S.d[r][o] * w[o][q];
      S.e[r][q] = (hb[r][q] > 0.0f) ? s : 0.0f;
    }
    __syncthreads();
    for (int i = tid; i < kTrainRows * kH; i += kTrainThreads) S.d[i / kH][i % kH] = S.e[i / kH][i % kH];
    __syncthreads();
  };
  back(S.w3, S.h2, A.grad + kW3, A.grad + kB3);
  back(S.w2, S.h1, A.grad + kW2, A.grad + kB2);
  // layer 1: dW1 = d^T x, db1 = sum d
  for (int i = tid; i < kH * kK; i += kTrainThreads) {
    const int o = i / kK, q = i % kK;
    float s = 0.0f;
    for (int r = 0; r < kTrainRows; r++) s += S.d[r][o] * S.x[r][q];
    atomicAdd(&A.grad[kW1 + i], s);
  }
  for (int o = tid; o < kH; o += kTrainThreads) {
    float s = 0.0f;
    for (int r = 0; r < kTrainRows; r++) s += S.d[r][o];
    atomicAdd(&A.grad[kB1 + o], s);
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
  const int smem = (int)(sizeof(InferSmem) + kNbRows * kHaloX * sizeof(float));
  if (resident == 0) {
    cudaError_t e = cudaFuncSetAttribute(lad_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, lad_infer_kernel,
                                                                            kInferThreads, smem);
    if (e != cudaSuccess || resident < 1) {
      set_error("lad inference: %s", e != cudaSuccess ? cudaGetErrorString(e) : "kernel does not fit an SM");
      resident = 0;
      return PG_ECUDA;
    }
  }
  const int64_t tiles = (int64_t)((a.grid.n[0] + kTileX - 1) / kTileX) * a.grid.n[1] * a.grid.n[2];
  const int64_t wave = (int64_t)sms * resident;
  const int blocks = (int)(tiles < wave ? tiles : wave);
  lad_infer_kernel<<<blocks, kInferThreads, smem, (cudaStream_t)stream>>>(a);
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
  const int smem = (int)sizeof(TrainSmem);
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(lad_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) {
      set_error("lad training: %s", cudaGetErrorString(e));
      return PG_ECUDA;
    }
    attr = true;
  }
  if (a.rows <= 0) return PG_OK;
  const int blocks = (int)((a.rows + kTrainRows - 1) / kTrainRows);
  lad_train_kernel<<<blocks, kTrainThreads, smem, (cudaStream_t)stream>>>(a);
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
