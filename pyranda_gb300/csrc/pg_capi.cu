// C ABI of the GB300 compact-operator library (declared in include/pyranda_gpu.h).
//
// A pg_handle replaces one pyranda patch of the parcop module: where parcop
// kept global tables selected by set_patch (pyranda/parcop/objects.f90:22-30,
// :77-89), every call here names its handle explicitly.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "pg_internal.h"

namespace pg {

static thread_local char g_err[512] = "";
static std::atomic<uint64_t> g_launches{0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
}

void count_launch(uint64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

}  // namespace pg

using namespace pg;

struct pg_handle {
  int n[3];
  int periodic[3];
  int precision;
  double d[3];    // patch spacing used by the d1 metric
  double dm[3];   // mesh d1, d2, d3
  double x1f[3];  // lower face coordinates
  DevOp ops[2][OPK_COUNT][3];
  void* tables = nullptr;
  double* work = nullptr;     // one field: temporary of the 3-sweep filters
  double* work2 = nullptr;    // one field: forward-elimination values of a sweep
  double* partial = nullptr;  // reduction partials
  int* status = nullptr;      // device status word (PG_ETIMEOUT from a bounded wait)
  double* host_in = nullptr;  // device buffers of the host-pointer variants
  double* host_out = nullptr;
  cudaStream_t stream = nullptr;
  int64_t npts = 0;
};

namespace {

int cuda_fail(cudaError_t e, const char* what) {
  set_error("%s: %s", what, cudaGetErrorString(e));
  return PG_ECUDA;
}

#define PG_CUDA(call)                                        \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);      \
  } while (0)

bool bad_dir(int d) { return d < 0 || d > 2; }

int sweep(pg_handle* h, int kind, int dir, const double* in, double* out, int epi, double scale, void* st) {
  const DevOp& op = h->ops[h->precision][kind][dir];
  SweepLaunch s{in, out, h->n[0], h->n[1], h->n[2], dir, scale, epi, h->status, h->work2};
  return launch_sweep(op, h->precision, s, st);
}

// null-op semantics of compact_operators.f90: derivatives -> 0, filters -> copy
int null_result(pg_handle* h, int kind, const double* in, double* out, void* st) {
  if (kind == OPK_SF || kind == OPK_GF) return launch_copy(out, in, h->npts, st);
  return launch_fill(out, 0.0, h->npts, st);
}

int apply_one(pg_handle* h, int kind, int dir, const double* in, double* out, void* st) {
  if (h->ops[h->precision][kind][dir].null_op) return null_result(h, kind, in, out, st);
  return sweep(h, kind, dir, in, out, EPI_STORE, 0.0, st);
}

}  // namespace

// ---------------------------------------------------------------------------
// host-pointer variants
// ---------------------------------------------------------------------------
static int host_prepare(pg_handle* h) {
  if (!h->stream) PG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  if (!h->host_in) PG_CUDA(cudaMalloc(&h->host_in, (size_t)h->npts * sizeof(double)));
  if (!h->host_out) PG_CUDA(cudaMalloc(&h->host_out, (size_t)h->npts * sizeof(double)));
  return PG_OK;
}

template <typename F>
static int host_call(pg_handle* h, const double* in, double* out, F&& f) {
  if (!h || !in || !out) return PG_EINVAL;
  int rc = host_prepare(h);
  if (rc) return rc;
  const size_t bytes = (size_t)h->npts * sizeof(double);
  PG_CUDA(cudaMemcpyAsync(h->host_in, in, bytes, cudaMemcpyHostToDevice, h->stream));
  rc = f(h->host_in, h->host_out, (void*)h->stream);
  if (rc) {
    cudaStreamSynchronize(h->stream);
    return rc;
  }
  PG_CUDA(cudaMemcpyAsync(out, h->host_out, bytes, cudaMemcpyDeviceToHost, h->stream));
  PG_CUDA(cudaStreamSynchronize(h->stream));
  return PG_OK;
}


extern "C" {

const char* pg_last_error(void) { return g_err; }

const char* pg_version(void) { return "pyranda_gb300 0.1 (sm_103a)"; }

uint64_t pg_launch_count(void) { return g_launches.load(); }

int pg_create(const pg_grid* g, pg_handle** out) {
  if (!g || !out) {
    set_error("pg_create: NULL argument");
    return PG_EINVAL;
  }
  *out = nullptr;
  if (g->precision != PG_FP64 && g->precision != PG_FP32) {
    set_error("pg_create: bad precision %d", g->precision);
    return PG_EINVAL;
  }
  pg_handle* h = new pg_handle();
  h->precision = g->precision;
  for (int d = 0; d < 3; d++) {
    if (g->n[d] < 1) {
      delete h;
      set_error("pg_create: n[%d] = %d", d, g->n[d]);
      return PG_EBADSHAPE;
    }
    h->n[d] = g->n[d];
    h->periodic[d] = g->periodic[d] ? 1 : 0;
    // parcop.f90:47-56 node extents -> faces; patch.f90:83-85 spacing
    const double dn = (g->xn[d] - g->x1[d]) / (double)std::max(g->n[d] - 1, 1);
    const double f1 = g->x1[d] - dn / 2.0, fn = g->xn[d] + dn / 2.0;
    h->x1f[d] = f1;
    h->d[d] = (fn - f1) / (double)g->n[d];
  }
  // mesh.f90:192-209: a direction of one point takes the larger other spacing
  for (int d = 0; d < 3; d++) {
    if (h->n[d] == 1) {
      const int a = (d + 1) % 3, b = (d + 2) % 3;
      h->dm[d] = std::max(h->d[std::min(a, b)], h->d[std::max(a, b)]);
    } else {
      h->dm[d] = h->d[d];
    }
  }
  h->npts = (int64_t)h->n[0] * h->n[1] * h->n[2];

  // assemble and factor every operator on the host
  OpTables tab[OPK_COUNT][3];
  size_t total = 0;
  for (int k = 0; k < OPK_COUNT; k++)
    for (int d = 0; d < 3; d++) {
      const double scale = (k == OPK_D1) ? h->d[d] : 0.0;
      int rc = build_operator(k, h->n[d], h->periodic[d] != 0, scale, tab[k][d]);
      if (rc != PG_OK) {
        delete h;
        set_error("pg_create: direction %d has %d points; a non-null direction needs at least 8", d, g->n[d]);
        return rc;
      }
      total += (size_t)h->n[d] * (9 + 12) * (sizeof(double) + sizeof(float)) + 64;
    }
  cudaError_t e = cudaMalloc(&h->tables, total);
  if (e != cudaSuccess) {
    delete h;
    set_error("pg_create: cudaMalloc tables: %s", cudaGetErrorString(e));
    return PG_ENOMEM;
  }
  std::vector<unsigned char> host(total);
  size_t off = 0;
  auto put = [&](const std::vector<double>& v, bool f32) -> const void* {
    off = (off + 15) & ~(size_t)15;  // 16-byte aligned rows for vector loads
    const void* dptr = (unsigned char*)h->tables + off;
    if (f32) {
      for (size_t i = 0; i < v.size(); i++) {
        float x = (float)v[i];
        std::memcpy(&host[off + i * 4], &x, 4);
      }
      off += v.size() * 4;
    } else {
      std::memcpy(&host[off], v.data(), v.size() * 8);
      off += v.size() * 8;
    }
    return dptr;
  };
  for (int p = 0; p < 2; p++)
    for (int k = 0; k < OPK_COUNT; k++)
      for (int d = 0; d < 3; d++) {
        const OpTables& t = tab[k][d];
        DevOp& op = h->ops[p][k][d];
        op.kind = k;
        op.n = t.n;
        op.periodic = t.periodic;
        op.implicit = t.implicit;
        op.addback = t.addback;
        op.null_op = t.null_op;
        op.rhs = put(t.rhs, p == PG_FP32);
        // solve coefficients regrouped 12 per row for vector loads:
        // [c1 c2 c6 c7 | c3 c4 c5 c8 | c9 0 0 0]
        std::vector<double> lu12((size_t)t.n * 12, 0.0);
        static const int order[9] = {0, 1, 5, 6, 2, 3, 4, 7, 8};
        for (int i = 0; i < t.n && !t.null_op; i++)
          for (int q = 0; q < 9; q++) lu12[(size_t)i * 12 + q] = t.lu[(size_t)i * 9 + order[q]];
        op.lu = put(lu12, p == PG_FP32);
        const int mid = t.n / 2;
        for (int l = 0; l < 9; l++) op.rhs_in[l] = t.null_op ? 0.0 : t.rhs[(size_t)mid * 9 + l];
      }
  e = cudaMemcpy(h->tables, host.data(), total, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&h->work, (size_t)h->npts * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->work2, (size_t)h->npts * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->partial, (size_t)kReduceBlocks * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(h->status, 0, sizeof(int));
  if (e != cudaSuccess) {
    set_error("pg_create: %s", cudaGetErrorString(e));
    pg_destroy(h);
    return PG_ENOMEM;
  }
  *out = h;
  return PG_OK;
}

int pg_destroy(pg_handle* h) {
  if (!h) return PG_OK;
  if (h->tables) cudaFree(h->tables);
  if (h->work) cudaFree(h->work);
  if (h->work2) cudaFree(h->work2);
  if (h->partial) cudaFree(h->partial);
  if (h->status) cudaFree(h->status);
  if (h->host_in) cudaFree(h->host_in);
  if (h->host_out) cudaFree(h->host_out);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return PG_OK;
}

int pg_device_status(pg_handle* h, int* status) {
  if (!h || !status) return PG_EINVAL;
  int v = 0;
  PG_CUDA(cudaMemcpy(&v, h->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (v != 0) PG_CUDA(cudaMemset(h->status, 0, sizeof(int)));
  *status = v;
  return PG_OK;
}

int pg_set_precision(pg_handle* h, int precision) {
  if (!h || (precision != PG_FP64 && precision != PG_FP32)) return PG_EINVAL;
  h->precision = precision;
  return PG_OK;
}

int pg_get_spacing(const pg_handle* h, double* patch_d, double* mesh_d) {
  if (!h) return PG_EINVAL;
  for (int d = 0; d < 3; d++) {
    if (patch_d) patch_d[d] = h->d[d];
    if (mesh_d) mesh_d[d] = h->dm[d];
  }
  return PG_OK;
}

int pg_d1(pg_handle* h, int dir, const double* in, double* out, void* stream) {
  if (!h || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(h, OPK_D1, dir, in, out, stream);
}

int pg_d8(pg_handle* h, int dir, const double* in, double* out, void* stream) {
  if (!h || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(h, OPK_D8, dir, in, out, stream);
}

int pg_filter(pg_handle* h, int kind, int dir, const double* in, double* out, void* stream) {
  if (!h || !in || !out || (kind != PG_SPECTRAL && kind != PG_GAUSSIAN) || dir < 0 || dir > 3) return PG_EINVAL;
  const int k = kind == PG_SPECTRAL ? OPK_SF : OPK_GF;
  if (dir < 3) return apply_one(h, k, dir, in, out, stream);
  // operators.f90:848-853 / :872-875: x -> y -> z, null directions copy
  int dirs[3], nd = 0;
  for (int d = 0; d < 3; d++)
    if (!h->ops[h->precision][k][d].null_op) dirs[nd++] = d;
  if (nd == 0) return launch_copy(out, in, h->npts, stream);
  // ping-pong so that the last sweep lands in `out`
  const double* src = in;
  for (int q = 0; q < nd; q++) {
    const bool last = (q == nd - 1);
    // with an odd number of remaining sweeps write `out`, else the workspace
    double* dst = ((nd - 1 - q) % 2 == 0) ? out : h->work;
    (void)last;
    int rc = sweep(h, k, dirs[q], src, dst, EPI_STORE, 0.0, stream);
    if (rc) return rc;
    src = dst;
  }
  return PG_OK;
}

int pg_ring(pg_handle* h, const double* in, double* out, void* stream) {
  if (!h || !in || !out) return PG_EINVAL;
  if (in == out) {
    set_error("pg_ring: in and out must differ");
    return PG_EINVAL;
  }
  bool first = true;
  for (int d = 0; d < 3; d++) {
    // ringx: a direction of one point contributes 0 (operators.f90:706-711);
    // d8 on a null direction is also 0 and max(x, 0) = x for x >= 0.
    if (h->n[d] == 1 || h->ops[h->precision][OPK_D8][d].null_op) continue;
    const double s = h->dm[d] * h->dm[d];
    int rc = sweep(h, OPK_D8, d, in, out, first ? EPI_RING_SET : EPI_RING_MAX, s, stream);
    if (rc) return rc;
    first = false;
  }
  if (first) return launch_fill(out, 0.0, h->npts, stream);
  return PG_OK;
}

int pg_ringv(pg_handle* h, const double* vx, const double* vy, const double* vz, double* out, void* stream) {
  if (!h || !vx || !vy || !vz || !out) return PG_EINVAL;
  if (out == vx || out == vy || out == vz) {
    set_error("pg_ringv: out must not alias an input");
    return PG_EINVAL;
  }
  const double* src[3] = {vx, vy, vz};
  bool first = true;
  for (int d = 0; d < 3; d++) {
    if (h->n[d] == 1 || h->ops[h->precision][OPK_D8][d].null_op) continue;
    for (int c = 0; c < 3; c++) {
      int rc = sweep(h, OPK_D8, d, src[c], out, first ? EPI_RING_SET : EPI_RING_MAX, h->dm[d], stream);
      if (rc) return rc;
      first = false;
    }
  }
  if (first) return launch_fill(out, 0.0, h->npts, stream);
  return PG_OK;
}

int pg_grad(pg_handle* h, const double* in, double* gx, double* gy, double* gz, void* stream) {
  if (!h || !in || !gx || !gy || !gz) return PG_EINVAL;
  int rc = apply_one(h, OPK_D1, 0, in, gx, stream);
  if (!rc) rc = apply_one(h, OPK_D1, 1, in, gy, stream);
  if (!rc) rc = apply_one(h, OPK_D1, 2, in, gz, stream);
  return rc;
}

int pg_div(pg_handle* h, const double* fx, const double* fy, const double* fz, double* out, void* stream) {
  if (!h || !fx || !fy || !fz || !out) return PG_EINVAL;
  if (out == fy || out == fz) {
    set_error("pg_div: out must not alias fy or fz");
    return PG_EINVAL;
  }
  const double* f[3] = {fx, fy, fz};
  bool first = true;
  for (int d = 0; d < 3; d++) {
    if (h->ops[h->precision][OPK_D1][d].null_op) continue;  // contributes exactly 0
    int rc = sweep(h, OPK_D1, d, f[d], out, first ? EPI_STORE : EPI_ADD, 0.0, stream);
    if (rc) return rc;
    first = false;
  }
  if (first) return launch_fill(out, 0.0, h->npts, stream);
  return PG_OK;
}

int pg_mesh(pg_handle* h, int which, double* out, void* stream) {
  if (!h || !out || which < 0 || which > 7) return PG_EINVAL;
  return launch_mesh(which, out, h->n[0], h->n[1], h->n[2], h->x1f, h->d, h->dm, stream);
}

int pg_rk_stage(pg_handle* h, int nvar, double* const* U, double* const* PHI, const double* const* F,
                const double* dt, double A, double B, void* stream) {
  if (!h || nvar < 0 || (nvar > 0 && (!U || !PHI || !F || !dt))) return PG_EINVAL;
  if (nvar == 0) return PG_OK;
  return launch_rk_stage(nvar, U, PHI, F, dt, A, B, h->npts, stream);
}

int pg_courant(pg_handle* h, const double* u, const double* v, const double* w, const double* c, double vconst,
               double wconst, double* out, void* stream) {
  if (!h || !u || !c || !out) return PG_EINVAL;
  const double gl = std::min(std::min(h->dm[0], h->dm[1]), h->dm[2]);
  return launch_courant(u, v, w, c, vconst, wconst, h->dm, gl, h->npts, h->partial, out, stream);
}

int pg_diff(pg_handle* h, const double* bulk, const double* rho, double* out, void* stream) {
  if (!h || !bulk || !rho || !out) return PG_EINVAL;
  const double gl = std::min(std::min(h->dm[0], h->dm[1]), h->dm[2]);
  return launch_diff(bulk, rho, gl, h->npts, h->partial, out, stream);
}

int pg_reduce(pg_handle* h, int op, const double* in, int64_t n, double* out, void* stream) {
  if (!h || !in || !out || op < 0 || op > 2 || n <= 0) return PG_EINVAL;
  return launch_reduce(op, in, n, h->partial, out, stream);
}

int pg_check_finite(const double* in, int64_t n, int* flag, void* stream) {
  if (!in || !flag || n < 0) return PG_EINVAL;
  return launch_check_finite(in, n, flag, stream);
}

int pg_d1_host(pg_handle* h, int dir, const double* in, double* out) {
  return host_call(h, in, out, [&](const double* a, double* b, void* s) { return pg_d1(h, dir, a, b, s); });
}

int pg_d8_host(pg_handle* h, int dir, const double* in, double* out) {
  return host_call(h, in, out, [&](const double* a, double* b, void* s) { return pg_d8(h, dir, a, b, s); });
}

int pg_filter_host(pg_handle* h, int kind, int dir, const double* in, double* out) {
  return host_call(h, in, out,
                   [&](const double* a, double* b, void* s) { return pg_filter(h, kind, dir, a, b, s); });
}

int pg_ring_host(pg_handle* h, const double* in, double* out) {
  return host_call(h, in, out, [&](const double* a, double* b, void* s) { return pg_ring(h, a, b, s); });
}

}  // extern "C"
