// Allocation-free global reduction.
//
// pg_reduce keeps its per-block partial results in a buffer that pg_create
// allocates with cudaMalloc.  Some callers cannot allocate device memory at
// all: code embedded in a host framework whose allocator forbids raw
// cudaMalloc, or code that must not create a pg_handle (and so never owns a
// workspace) because it only needs a sum, max or min of a field it already
// holds.  pg_reduce_noalloc serves them: its scratch is the file-scope device
// array below, which exists in every GPU's memory once the library is loaded
// and stays there until the process exits.
//
// Rules of use (also stated in include/pyranda_gpu.h):
//  - n must not exceed PG_NOALLOC_MAX_VALUES; larger inputs are rejected with
//    PG_EBADSHAPE before anything is launched.
//  - Every call outside a stream capture looks up the array's device address
//    on the current device (cudaGetSymbolAddress), so a device reset between
//    calls is harmless; a call inside a capture reuses the address found by an
//    earlier call, so make one call on each device before capturing.
//  - All calls in the process share the one array.  Two calls whose kernels
//    overlap on the GPU (for example on two streams) race on it; serialise
//    them.  The array keeps the last call's partials; nothing in it has to
//    start at zero because every slot a call reads was written earlier in the
//    same call.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <mutex>

#include "pg_internal.h"

namespace pg {
namespace {

constexpr int kNaThreads = 256;
constexpr int64_t kNaChunk = PG_NOALLOC_CHUNK;           // values reduced by one block
constexpr int kNaMaxBlocks = PG_NOALLOC_MAX_BLOCKS;      // partial slots in the scratch

// The scratch: one partial result per block (32 KiB).
static __device__ __align__(256) double g_noalloc_partials[kNaMaxBlocks];

template <int OP>
__device__ __forceinline__ double na_combine(double a, double b) {
  if (OP == 0) return a + b;
  if (OP == 1) return fmax(a, b);
  return fmin(a, b);
}

template <int OP>
__device__ __forceinline__ double na_identity() {
  if (OP == 0) return 0.0;
  if (OP == 1) return -INFINITY;  // max of an all -inf input is -inf, as in numpy
  return INFINITY;
}

template <int OP>
__device__ double na_block_reduce(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v = na_combine<OP>(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : na_identity<OP>();
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v = na_combine<OP>(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block b reduces the contiguous chunk [b*kNaChunk, min((b+1)*kNaChunk, n)).
// NaN anywhere makes the partial NaN (numpy's max/min/sum behaviour).
template <int OP>
__global__ void na_partial(const double* __restrict__ in, int64_t n, double* __restrict__ partials, int nslots) {
  if ((int)blockIdx.x >= nslots) return;  // never write past the scratch
  const int64_t lo = (int64_t)blockIdx.x * kNaChunk;
  const int64_t hi = lo + kNaChunk < n ? lo + kNaChunk : n;
  double acc = na_identity<OP>();
  bool nan = false;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double x = in[i];
    nan |= (x != x);
    acc = na_combine<OP>(acc, x);
  }
  acc = na_block_reduce<OP>(acc);
  const int anynan = __syncthreads_or(nan);
  if (threadIdx.x == 0) partials[blockIdx.x] = anynan ? NAN : acc;
}

template <int OP>
__global__ void na_final(const double* __restrict__ partials, int np, double* __restrict__ out) {
  double acc = na_identity<OP>();
  bool nan = false;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const double x = partials[i];
    nan |= (x != x);
    acc = na_combine<OP>(acc, x);
  }
  acc = na_block_reduce<OP>(acc);
  const int anynan = __syncthreads_or(nan);
  if (threadIdx.x == 0) *out = anynan ? NAN : acc;
}

// Device address of the scratch on each device.  It is looked up again on
// every call made outside a stream capture, so a device reset between calls
// (which reloads the module, possibly at another address) is picked up; a
// call during a capture uses the address found by an earlier call, because
// the lookup itself may not be issued while a capture is active.
constexpr int kMaxDevices = 64;
double* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

int scratch_for_current_device(cudaStream_t stream, double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error("pg_reduce_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("pg_reduce_noalloc: device %d beyond the %d supported", dev, kMaxDevices);
    return PG_EINVAL;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  const cudaError_t qe = cudaStreamIsCapturing(stream, &cs);
  if (qe != cudaSuccess) (void)cudaGetLastError();  // an implicit capture of the legacy stream: treat as capturing
  const bool capturing = (qe != cudaSuccess) || cs != cudaStreamCaptureStatusNone;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!capturing) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p) {
      set_error("pg_reduce_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      return PG_ECUDA;
    }
    g_scratch_ptr[dev] = static_cast<double*>(p);
  } else if (!g_scratch_ptr[dev]) {
    set_error("pg_reduce_noalloc: first call on device %d made during a stream capture; "
              "call it once before capturing", dev);
    return PG_EINVAL;
  }
  *out = g_scratch_ptr[dev];
  return PG_OK;
}

}  // namespace
}  // namespace pg

extern "C" int pg_reduce_noalloc(int op, const double* in, int64_t n, double* out, void* stream) {
  using namespace pg;
  if (!in || !out || op < 0 || op > 2 || n <= 0) {
    set_error("pg_reduce_noalloc: bad argument (op %d, n %lld)", op, (long long)n);
    return PG_EINVAL;
  }
  if (n > (int64_t)PG_NOALLOC_MAX_VALUES) {
    set_error("pg_reduce_noalloc: n = %lld exceeds the static scratch limit of %lld values",
              (long long)n, (long long)PG_NOALLOC_MAX_VALUES);
    return PG_EBADSHAPE;
  }
  double* partials = nullptr;
  int rc = scratch_for_current_device((cudaStream_t)stream, &partials);
  if (rc != PG_OK) return rc;
  const int nb = (int)((n + kNaChunk - 1) / kNaChunk);  // <= kNaMaxBlocks by the check above
  cudaStream_t s = (cudaStream_t)stream;
  if (op == 0) {
    na_partial<0><<<nb, kNaThreads, 0, s>>>(in, n, partials, kNaMaxBlocks);
    na_final<0><<<1, kNaThreads, 0, s>>>(partials, nb, out);
  } else if (op == 1) {
    na_partial<1><<<nb, kNaThreads, 0, s>>>(in, n, partials, kNaMaxBlocks);
    na_final<1><<<1, kNaThreads, 0, s>>>(partials, nb, out);
  } else {
    na_partial<2><<<nb, kNaThreads, 0, s>>>(in, n, partials, kNaMaxBlocks);
    na_final<2><<<1, kNaThreads, 0, s>>>(partials, nb, out);
  }
  count_launch(2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("pg_reduce_noalloc launch: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}
