// C ABI of the GB300 compact-operator library (declared in include/pyranda_gpu.h).
//
// A pg_handle replaces one pyranda patch of the parcop module: where parcop
// kept global tables selected by set_patch (pyranda/parcop/objects.f90:22-30,
// :77-89), every call here names its handle explicitly.  A pg_ensemble holds
// many independent grids of different sizes whose fields are stored back to
// back in one flat buffer; every operator on it is one launch over the lines
// of all members.  A handle is the one-member case of the same machinery.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
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

namespace {

int cuda_fail(cudaError_t e, const char* what) {
  set_error("%s: %s", what, cudaGetErrorString(e));
  return PG_ECUDA;
}

#define PG_CUDA(call)                                   \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// One grid: spacings (parcop.f90:47-56, patch.f90:83-85, mesh.f90:192-209)
// and the host tables of every operator.
struct GridInfo {
  int n[3];
  int periodic[3];
  double d[3];    // patch spacing (the d1 metric)
  double dm[3];   // mesh d1, d2, d3
  double x1f[3];  // lower face coordinates
  int64_t npts;
  int bc[3][2];   // pg_bc per end (non-periodic directions)
  bool symm[3];   // a symmetry plane at either end: the antisymmetric variants differ
  int coordsys;   // pg_coordsys
  double x1[3], xn[3];  // node extents (the default coordinates of a curvilinear grid)
  OpTables tab[OPK_COUNT][3];       // operators for symmetric fields (the default)
  OpTables tab_anti[OPK_COUNT][3];  // variants for antisymmetric fields (compact.f90:80-85, nop = 2)
};

int grid_info(const pg_grid* g, GridInfo& gi, const char* who) {
  for (int d = 0; d < 3; d++) {
    if (g->n[d] < 1) {
      set_error("%s: n[%d] = %d", who, d, g->n[d]);
      return PG_EBADSHAPE;
    }
    gi.n[d] = g->n[d];
    gi.periodic[d] = g->periodic[d] ? 1 : 0;
    gi.x1[d] = g->x1[d];
    gi.xn[d] = g->xn[d];
    for (int e = 0; e < 2; e++) {
      const int b = g->bc[d][e];
      if (b < PG_BC_NONE || b > PG_BC_XTND) {
        set_error("%s: bc[%d][%d] = %d is not a pg_bc", who, d, e, b);
        return PG_EINVAL;
      }
      gi.bc[d][e] = gi.periodic[d] ? PG_BC_NONE : b;
    }
    gi.symm[d] = !gi.periodic[d] && (gi.bc[d][0] == PG_BC_SYMM || gi.bc[d][1] == PG_BC_SYMM);
    const double dn = (g->xn[d] - g->x1[d]) / (double)std::max(g->n[d] - 1, 1);
    const double f1 = g->x1[d] - dn / 2.0, fn = g->xn[d] + dn / 2.0;
    gi.x1f[d] = f1;
    gi.d[d] = (fn - f1) / (double)g->n[d];
  }
  if (g->coordsys < PG_CARTESIAN || g->coordsys > PG_SPHERICAL_RATIO) {
    set_error("%s: coordsys %d is not a pg_coordsys", who, g->coordsys);
    return PG_EINVAL;
  }
  gi.coordsys = g->coordsys;
  for (int d = 0; d < 3; d++) {
    if (gi.n[d] == 1) {
      const int a = (d + 1) % 3, b = (d + 2) % 3;
      gi.dm[d] = std::max(gi.d[std::min(a, b)], gi.d[std::max(a, b)]);
    } else {
      gi.dm[d] = gi.d[d];
    }
  }
  gi.npts = (int64_t)gi.n[0] * gi.n[1] * gi.n[2];
  if (gi.npts >= ((int64_t)1 << 31)) {
    set_error("%s: %lld points; a field must hold fewer than 2^31 points", who, (long long)gi.npts);
    return PG_EBADSHAPE;
  }
  for (int k = 0; k < OPK_COUNT; k++)
    for (int d = 0; d < 3; d++) {
      const double scale = (k == OPK_D1) ? gi.d[d] : ((k == OPK_D2) ? gi.d[d] * gi.d[d] : 0.0);
      int rc = build_operator(k, gi.n[d], gi.periodic[d] != 0, scale, gi.tab[k][d], gi.bc[d][0], gi.bc[d][1], 1);
      if (rc == PG_OK)
        rc = build_operator(k, gi.n[d], gi.periodic[d] != 0, scale, gi.tab_anti[k][d], gi.bc[d][0], gi.bc[d][1], -1);
      if (rc != PG_OK) {
        set_error("%s: direction %d has %d points; a non-null direction needs at least 8", who, d, gi.n[d]);
        return rc;
      }
    }
  return PG_OK;
}

// Device state shared by handles and ensembles.
struct Ctx {
  int precision = PG_FP64;
  int nmem = 0;
  int64_t npts = 0;
  OpRef ops[2][OPK_COUNT][3];
  OpRef anti[2][OPK_COUNT][3];   // the antisymmetric variants (differ where a direction has a symmetry plane)
  bool symm[3] = {false, false, false};
  int coordsys = PG_CARTESIAN;
  double* cyl[3] = {nullptr, nullptr, nullptr};  // non-Cartesian grids: three workspace fields
  double* mf[MF_COUNT] = {};     // spherical and curvilinear grids: the mesh fields (one allocation at mf[0])
  void* blob = nullptr;          // coefficient tables and member-op arrays
  double* work = nullptr;        // one field: x->y->z filter ping-pong
  double* work2 = nullptr;       // one field: forward-elimination scratch of a sweep
  double* partial = nullptr;     // reduction partials (+ per-member results)
  int* status = nullptr;         // device status word
  int* emax = nullptr;           // exact d8 RHS: per member the largest exponent of the sweep input
  int nmax[3] = {0, 0, 0};       // the longest member line along each direction
  long long* moff = nullptr;     // ensembles: member point offsets (nmem + 1)
  double* mconst = nullptr;      // ensembles: per member 1/d1 1/d2 1/d3 1/GridLen GridLen
  double* host_in = nullptr;     // host-pointer variants
  double* host_out = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<MemberOp> mops;    // host copy of the member-op arrays
  // dense split-TF32 operators (PG_DENSE): used for d1 and the two filters
  // where built; d8 (exact fixed-point RHS) and every other case run the
  // FP32 banded sweeps
  bool dense = false;
  bool dense_built = false;
  DenseSet dsets[OPK_COUNT][3];
  bool use_dense[OPK_COUNT][3] = {};  // the sweep plan: dense kernel or FP32 banded
  void* dense_blob = nullptr;
  // split-line sweeps (pg_split.cu): per precision, operator and direction
  bool split_built = false;
  SplitSet splits[2][OPK_COUNT][3];
  bool use_split[2][OPK_COUNT][3] = {};
  void* split_blob = nullptr;
};

void free_ctx(Ctx& c) {
  if (c.blob) cudaFree(c.blob);
  if (c.work) cudaFree(c.work);
  if (c.work2) cudaFree(c.work2);
  if (c.partial) cudaFree(c.partial);
  if (c.status) cudaFree(c.status);
  if (c.emax) cudaFree(c.emax);
  if (c.moff) cudaFree(c.moff);
  if (c.mconst) cudaFree(c.mconst);
  if (c.host_in) cudaFree(c.host_in);
  if (c.host_out) cudaFree(c.host_out);
  if (c.stream) cudaStreamDestroy(c.stream);
  if (c.dense_blob) cudaFree(c.dense_blob);
  if (c.split_blob) cudaFree(c.split_blob);
  for (int q = 0; q < 3; q++)
    if (c.cyl[q]) cudaFree(c.cyl[q]);
  if (c.mf[0]) cudaFree(c.mf[0]);
  c = Ctx();
}

// The d8 RHS weights as integers times one FP32-exact scale, with at most 256
// units of weight per row and an interior row proportional to the 8th
// difference (c10d8: 60 x small integers, stencils.f90:519-526,573-591).
// Then the FP32 sweeps evaluate the RHS exactly in 64-bit fixed point
// (pg_sweep.cuh).
bool integer_weights(const OpTables& t, std::vector<int>& iw, double& w) {
  if (t.kind != OPK_D8 || t.null_op || t.n < 1) return false;
  const size_t mid = (size_t)(t.n / 2);
  w = 0.0;
  for (int l = 0; l < 9 && w == 0.0; l++) w = std::fabs(t.rhs[mid * 9 + l]);
  if (w == 0.0 || (double)(float)w != w) return false;
  iw.assign((size_t)t.n * 9, 0);
  for (int i = 0; i < t.n; i++) {
    int units = 0;
    for (int l = 0; l < 9; l++) {
      const double x = t.rhs[(size_t)i * 9 + l];
      const double q = std::nearbyint(x / w);
      if (q * w != x || std::fabs(q) > 256.0) return false;
      iw[(size_t)i * 9 + l] = (int)q;
      units += std::abs((int)q);
    }
    if (units > 256) return false;
  }
  // the interior rows (4 .. n-5; the middle row is one when n >= 9) are iw[0] x the 8th
  // difference: the sweeps keep it by a cascade of differences
  static const int c8[9] = {1, -8, 28, -56, 70, -56, 28, -8, 1};
  if (t.n >= 9)
    for (int l = 0; l < 9; l++)
      if (iw[mid * 9 + l] != iw[mid * 9] * c8[l]) return false;
  return true;
}

// Upload the tables of every member, build the member-op arrays and
// allocate the workspaces.
int build_ctx(Ctx& c, const std::vector<GridInfo>& g, int precision, const char* who) {
  const int M = (int)g.size();
  c.precision = precision;
  c.nmem = M;
  for (int m = 1; m < M; m++)
    for (int d = 0; d < 3; d++) {
      if (g[m].periodic[d] != g[0].periodic[d] || (g[m].n[d] < 4) != (g[0].n[d] < 4) ||
          (g[m].n[d] == 1) != (g[0].n[d] == 1) || g[m].bc[d][0] != g[0].bc[d][0] ||
          g[m].bc[d][1] != g[0].bc[d][1] || g[m].coordsys != g[0].coordsys) {
        set_error("%s: member %d differs from member 0 in periodicity, boundary codes, coordinate system or "
                  "null directions", who, m);
        return PG_EINVAL;
      }
    }
  std::vector<long long> off(M + 1, 0);
  for (int m = 0; m < M; m++) off[m + 1] = off[m] + g[m].npts;
  for (int d = 0; d < 3; d++)
    for (int m = 0; m < M; m++) c.nmax[d] = std::max(c.nmax[d], g[m].n[d]);
  c.npts = off[M];
  // layout of the blob: [tables ...][member ops (variant x precision x kind x direction x member)];
  // variant 0 = the operators for symmetric fields, 1 = the antisymmetric variants
  auto align = [](size_t x) { return (x + 15) & ~(size_t)15; };
  size_t total = 0;
  for (int m = 0; m < M; m++)
    for (int k = 0; k < OPK_COUNT; k++)
      for (int d = 0; d < 3; d++) {
        const size_t n = (size_t)g[m].n[d];
        total += 2 * (align(n * 9 * 8) + align(n * 12 * 8) + align(n * 9 * 4) + align(n * 12 * 4) + align(n * 9 * 4));
      }
  const size_t ops_off = align(total);
  total = ops_off + sizeof(MemberOp) * (size_t)M * 2 * 2 * OPK_COUNT * 3;
  cudaError_t e = cudaMalloc(&c.blob, total);
  if (e != cudaSuccess) {
    set_error("%s: cudaMalloc tables: %s", who, cudaGetErrorString(e));
    return PG_ENOMEM;
  }
  std::vector<unsigned char> host(total, 0);
  size_t pos = 0;
  auto put = [&](const std::vector<double>& v, bool f32) -> const void* {
    pos = align(pos);
    const void* dptr = (unsigned char*)c.blob + pos;
    if (f32) {
      for (size_t i = 0; i < v.size(); i++) {
        const float x = (float)v[i];
        std::memcpy(&host[pos + i * 4], &x, 4);
      }
      pos += v.size() * 4;
    } else {
      std::memcpy(&host[pos], v.data(), v.size() * 8);
      pos += v.size() * 8;
    }
    return dptr;
  };
  auto put_i = [&](const std::vector<int>& v) -> const int* {
    pos = align(pos);
    const int* dptr = reinterpret_cast<const int*>((unsigned char*)c.blob + pos);
    std::memcpy(&host[pos], v.data(), v.size() * 4);
    pos += v.size() * 4;
    return dptr;
  };
  std::vector<MemberOp> mops((size_t)M * 2 * 2 * OPK_COUNT * 3);
  auto mindex = [&](int v, int p, int k, int d, int m) {
    return ((((size_t)v * 2 + p) * OPK_COUNT + k) * 3 + d) * M + m;
  };
  for (int v = 0; v < 2; v++)
  for (int m = 0; m < M; m++)
    for (int k = 0; k < OPK_COUNT; k++)
      for (int d = 0; d < 3; d++) {
        const OpTables& t = v == 0 ? g[m].tab[k][d] : g[m].tab_anti[k][d];
        std::vector<int> iw;
        double wsc = 0.0;
        const bool exact = integer_weights(t, iw, wsc);
        const int* rhs_i = put_i(exact ? iw : std::vector<int>((size_t)t.n * 9, 0));
        for (int p = 0; p < 2; p++) {
          MemberOp& o = mops[mindex(v, p, k, d, m)];
          o.rhs = put(t.rhs, p == PG_FP32);
          o.lu = put(t.lu, p == PG_FP32);
          o.n = g[m].n[d];
          o.nx = g[m].n[0];
          o.ny = g[m].n[1];
          o.bcl = t.bcl;
          o.lines = g[m].npts / g[m].n[d];
          o.off = off[m];
          const int mid = t.n / 2;
          for (int l = 0; l < 9; l++) o.ri[l] = t.null_op ? 0.0 : t.rhs[(size_t)mid * 9 + l];
          o.dm = g[m].dm[d];
          o.rhs_i = rhs_i;
          for (int l = 0; l < 9; l++) o.iw[l] = exact ? iw[(size_t)mid * 9 + l] : 0;
          o.exact = exact ? 1 : 0;
          o.wscale = (float)wsc;
          o.bch = t.bch;
        }
      }
  for (int v = 0; v < 2; v++)
  for (int p = 0; p < 2; p++)
    for (int k = 0; k < OPK_COUNT; k++)
      for (int d = 0; d < 3; d++) {
        long long line0 = 0;
        for (int m = 0; m < M; m++) {
          MemberOp& o = mops[mindex(v, p, k, d, m)];
          o.line0 = line0;
          line0 += o.lines;
        }
        OpRef& r = v == 0 ? c.ops[p][k][d] : c.anti[p][k][d];
        const OpTables& t = v == 0 ? g[0].tab[k][d] : g[0].tab_anti[k][d];
        r.exact = true;
        for (int m = 0; m < M; m++) r.exact = r.exact && mops[mindex(v, p, k, d, m)].exact;
        r.dev = reinterpret_cast<const MemberOp*>((unsigned char*)c.blob + ops_off) + mindex(v, p, k, d, 0);
        r.nops = M;
        r.nlines = line0;
        r.kind = k;
        r.periodic = t.periodic;
        r.implicit = t.implicit;
        r.addback = t.addback;
        r.null_op = t.null_op;
      }
  std::memcpy(&host[ops_off], mops.data(), sizeof(MemberOp) * mops.size());
  c.mops = mops;
  for (int d = 0; d < 3; d++) c.symm[d] = g[0].symm[d];
  c.coordsys = g[0].coordsys;
  e = cudaMemcpy(c.blob, host.data(), total, cudaMemcpyHostToDevice);
  const size_t nbytes = (size_t)c.npts * sizeof(double);
  if (e == cudaSuccess) e = cudaMalloc(&c.work, nbytes);
  if (e == cudaSuccess) e = cudaMalloc(&c.work2, nbytes);
  if (g[0].coordsys != PG_CARTESIAN)
    for (int q = 0; q < 3 && e == cudaSuccess; q++) e = cudaMalloc(&c.cyl[q], nbytes);
  if (g[0].coordsys >= PG_SPHERICAL && e == cudaSuccess) {  // mesh.f90:98-139: the fields each system keeps
    const int nf = g[0].coordsys == PG_CURVILINEAR ? MF_COUNT : MF_DET;
    e = cudaMalloc(&c.mf[0], nbytes * nf);
    for (int q = 1; q < nf && e == cudaSuccess; q++) c.mf[q] = c.mf[0] + (size_t)q * c.npts;
  }
  // two values per block for the two-pass diffusion limit (estimate, exact-point flag)
  const size_t npart = std::max((size_t)2 * kReduceBlocks, (size_t)M * kSegBlocks + 2 * (size_t)M);
  if (e == cudaSuccess) e = cudaMalloc(&c.partial, npart * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&c.status, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&c.emax, sizeof(int) * (size_t)M);
  if (e == cudaSuccess) e = cudaMemset(c.status, 0, sizeof(int));
  {  // per-member offsets and spacings (used by the ensemble reductions)
    std::vector<double> mc((size_t)M * 5);
    for (int m = 0; m < M; m++) {
      const double gl = std::min(std::min(g[m].dm[0], g[m].dm[1]), g[m].dm[2]);
      mc[(size_t)m * 5 + 0] = 1.0 / g[m].dm[0];
      mc[(size_t)m * 5 + 1] = 1.0 / g[m].dm[1];
      mc[(size_t)m * 5 + 2] = 1.0 / g[m].dm[2];
      mc[(size_t)m * 5 + 3] = 1.0 / gl;
      mc[(size_t)m * 5 + 4] = gl;
    }
    if (e == cudaSuccess) e = cudaMalloc(&c.moff, sizeof(long long) * (M + 1));
    if (e == cudaSuccess) e = cudaMemcpy(c.moff, off.data(), sizeof(long long) * (M + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&c.mconst, sizeof(double) * mc.size());
    if (e == cudaSuccess) e = cudaMemcpy(c.mconst, mc.data(), sizeof(double) * mc.size(), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    set_error("%s: %s", who, cudaGetErrorString(e));
    free_ctx(c);
    return PG_ENOMEM;
  }
  return PG_OK;
}

bool bad_dir(int d) { return d < 0 || d > 2; }

// The dense operator in terms of first differences.  Every operator here
// annihilates constants (D 1 = 0), so row i of D v equals
// sum_j D_ij (v_j - v_i), and each v_j - v_i is a sum of the differences
// w_m = v_m - v_{m-1} along the shorter way from i to j (w_0 = v_0 - v_{n-1}
// on periodic lines; on one-sided lines the path never wraps and w_0 is
// unused).  The result D' (OUT = D' w) is local around the diagonal in every
// row, including the rows next to a periodic wrap, so its products are of
// the size of the result and the FP32 accumulation sees no cancellation --
// the property the banded sweeps get from their difference-form stencils.
std::vector<double> difference_form(const std::vector<double>& D, int n, bool periodic) {
  std::vector<double> W((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) {
    const double* d = &D[(size_t)i * n];
    double* w = &W[(size_t)i * n];
    const int fwd = periodic ? n / 2 : n - 1 - i;        // forward partners i+1 .. i+fwd
    const int bwd = periodic ? n - 1 - n / 2 : i;        // backward partners i-1 .. i-bwd
    // v_{i+k} - v_i = sum_{l=1..k} w_{i+l}: w_{i+l} collects D_{i,i+k} for k >= l
    double acc = 0.0;
    for (int k = fwd; k >= 1; k--) {
      acc += d[(i + k) % n];
      w[(i + k) % n] += acc;
    }
    // v_{i-k} - v_i = -sum_{l=0..k-1} w_{i-l}: w_{i-l} collects -D_{i,i-k} for k > l
    acc = 0.0;
    for (int k = bwd; k >= 1; k--) {
      acc += d[(i - k + n) % n];
      w[(i - k + 1 + n) % n] -= acc;
    }
  }
  return W;
}

// Dense form of the d1, d8 and compact-filter operators of every member: D is
// the banded FP64 operator itself, applied to an identity (line k = e_k), so
// the dense and banded paths implement one matrix.  Members with identical
// tables share one split copy of D.
// Inverse of the n x n LHS of one line from its band rows (a, b, diag, c, d;
// periodic lines wrap), by Gauss-Jordan elimination with partial pivoting in
// FP64.  Empty when singular.
std::vector<double> invert_band(const std::vector<double>& band, int n, bool periodic) {
  std::vector<double> A((size_t)n * n, 0.0), X((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) {
    X[(size_t)i * n + i] = 1.0;
    for (int l = 0; l < 5; l++) {
      int j = i + l - 2;
      if (periodic) j = (j + n) % n;
      else if (j < 0 || j >= n) continue;
      A[(size_t)i * n + j] += band[(size_t)i * 5 + l];
    }
  }
  for (int col = 0; col < n; col++) {
    int piv = col;
    for (int r = col + 1; r < n; r++)
      if (std::fabs(A[(size_t)r * n + col]) > std::fabs(A[(size_t)piv * n + col])) piv = r;
    if (A[(size_t)piv * n + col] == 0.0) return {};
    if (piv != col)
      for (int j = 0; j < n; j++) {
        std::swap(A[(size_t)piv * n + j], A[(size_t)col * n + j]);
        std::swap(X[(size_t)piv * n + j], X[(size_t)col * n + j]);
      }
    const double inv = 1.0 / A[(size_t)col * n + col];
    for (int j = 0; j < n; j++) {
      A[(size_t)col * n + j] *= inv;
      X[(size_t)col * n + j] *= inv;
    }
    for (int r = 0; r < n; r++) {
      if (r == col) continue;
      const double f = A[(size_t)r * n + col];
      if (f == 0.0) continue;
      for (int j = 0; j < n; j++) {
        A[(size_t)r * n + j] -= f * A[(size_t)col * n + j];
        X[(size_t)r * n + j] -= f * X[(size_t)col * n + j];
      }
    }
  }
  return X;
}

int build_dense(Ctx& c, const std::vector<GridInfo>& g) {
  if (c.dense_built) return PG_OK;
  const int M = (int)g.size();
  const int kinds[4] = {OPK_D1, OPK_D8, OPK_SF, OPK_GF};
  struct Uniq {
    int k, d, m, rows, kchunks;
    std::vector<uint32_t> planes;
    size_t off;
  };
  std::vector<Uniq> uniq;
  std::vector<int> which((size_t)OPK_COUNT * 3 * M, -1);  // unique entry of (kind, dir, member)
  int nmax = 0;
  for (int k : kinds)
    for (int d = 0; d < 3; d++) {
      if (c.ops[PG_FP64][k][d].null_op) continue;
      // d8 with the exact fixed-point RHS: the dense form is A^-1 alone, applied to that RHS
      // (split TF32 products cannot hold the 8th difference's cancellation); without it, no dense d8
      if (k == OPK_D8 && !c.ops[PG_FP32][k][d].exact) continue;
      bool fits = true;
      for (int m = 0; m < M; m++) fits = fits && g[m].n[d] >= 16 && g[m].n[d] <= 1024;
      if (!fits) continue;
      for (int m = 0; m < M; m++) {
        const OpTables& t = g[m].tab[k][d];
        int u = -1;
        for (size_t q = 0; q < uniq.size() && u < 0; q++) {
          const Uniq& e = uniq[q];
          const OpTables& o = g[e.m].tab[k][d];
          if (e.k == k && e.d == d && o.n == t.n && o.rhs == t.rhs && o.lu == t.lu) u = (int)q;
        }
        if (u < 0) {
          uniq.push_back(Uniq{k, d, m, 0, 0, {}, 0});
          u = (int)uniq.size() - 1;
          nmax = std::max(nmax, t.n);
        }
        which[((size_t)k * 3 + d) * M + m] = u;
      }
    }
  if (uniq.empty()) {
    c.dense_built = true;
    return PG_OK;
  }
  // D of each unique operator: the FP64 banded sweep of an identity field
  const size_t nn = (size_t)nmax * nmax;
  double *ident = nullptr, *dout = nullptr, *scr = nullptr;
  MemberOp* tmp = nullptr;
  cudaError_t e = cudaMalloc(&ident, nn * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&dout, nn * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&scr, nn * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&tmp, sizeof(MemberOp));
  int rc = (e == cudaSuccess) ? PG_OK : PG_ENOMEM;
  if (rc) set_error("dense operators: %s", cudaGetErrorString(e));
  std::vector<double> eye, Dt, D;
  for (size_t q = 0; q < uniq.size() && rc == PG_OK; q++) {
    Uniq& u = uniq[q];
    const int n = g[u.m].n[u.d];
    if (u.k == OPK_D8) {  // A^-1 of the LHS band, in FP64 on the host
      D = invert_band(g[u.m].tab[u.k][u.d].lhs, n, c.ops[PG_FP64][u.k][u.d].periodic);
      if (D.empty()) {
        set_error("dense operators: singular d8 LHS");
        rc = PG_EINVAL;
        break;
      }
      split_dense(D, n, u.planes, u.rows, u.kchunks);
      continue;
    }
    eye.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) eye[(size_t)i * n + i] = 1.0;
    const size_t mi = ((((size_t)PG_FP64 * OPK_COUNT + u.k) * 3 + u.d) * M) + u.m;
    MemberOp mo = c.mops[mi];
    mo.nx = n;
    mo.ny = n;
    mo.lines = n;
    mo.line0 = 0;
    mo.off = 0;
    OpRef ref = c.ops[PG_FP64][u.k][u.d];
    ref.dev = tmp;
    ref.nops = 1;
    ref.nlines = n;
    e = cudaMemcpy(ident, eye.data(), eye.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(tmp, &mo, sizeof(MemberOp), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      set_error("dense operators: %s", cudaGetErrorString(e));
      rc = PG_ECUDA;
      break;
    }
    SweepLaunch s{ident, dout, scr, &ref, 0, EPI_STORE, 0};
    rc = launch_sweep(PG_FP64, s, nullptr);
    if (rc) break;
    Dt.resize((size_t)n * n);
    e = cudaMemcpy(Dt.data(), dout, Dt.size() * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      set_error("dense operators: %s", cudaGetErrorString(e));
      rc = PG_ECUDA;
      break;
    }
    // line k of the output is column k of D
    D.assign((size_t)n * n, 0.0);
    for (int k = 0; k < n; k++)
      for (int i = 0; i < n; i++) D[(size_t)i * n + k] = Dt[(size_t)k * n + i];
    if (ref.addback)
      for (int i = 0; i < n; i++) D[(size_t)i * n + i] -= 1.0;
    split_dense(difference_form(D, n, ref.periodic), n, u.planes, u.rows, u.kchunks);
  }
  cudaFree(ident);
  cudaFree(dout);
  cudaFree(scr);
  cudaFree(tmp);
  if (rc) return rc;
  // one blob: [planes ...][DenseOp arrays][DenseTile arrays]
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t total = 0;
  for (auto& u : uniq) {
    u.off = total;
    total = al(total + u.planes.size() * 4);
  }
  std::vector<DenseOp> dops;
  std::vector<DenseTile> dtiles;
  size_t set_ops[OPK_COUNT][3] = {}, set_tiles[OPK_COUNT][3] = {};
  int set_nt[OPK_COUNT][3] = {};
  for (int k : kinds)
    for (int d = 0; d < 3; d++) {
      if (which[((size_t)k * 3 + d) * M] < 0) continue;
      set_ops[k][d] = dops.size();
      set_tiles[k][d] = dtiles.size();
      for (int m = 0; m < M; m++) {
        const Uniq& u = uniq[which[((size_t)k * 3 + d) * M + m]];
        const int n = g[m].n[d];
        DenseOp o{};
        o.dsw = reinterpret_cast<const uint32_t*>(u.off);  // relocated below
        o.off = (long long)c.mops[(((size_t)PG_FP64 * OPK_COUNT + k) * 3 + d) * M + m].off;
        o.n = n;
        o.nx = g[m].n[0];
        o.ny = g[m].n[1];
        o.kchunks = u.kchunks;
        o.rows = u.rows;
        o.periodic = g[m].periodic[d];
        o.direct = (k == OPK_D8) ? 1 : 0;
        o.dm = g[m].dm[d];
        dops.push_back(o);
        const int lines = (int)(g[m].npts / n);
        const int lt = 128;                                  // lines per tile
        const int parts = (((n + 15) & ~15) + 255) / 256;    // 256 positions per tile
        for (int l0 = 0; l0 < lines; l0 += lt)
          for (int p = 0; p < parts; p++)
            dtiles.push_back(DenseTile{m, l0, std::min(lt, lines - l0), p});
      }
      set_nt[k][d] = (int)(dtiles.size() - set_tiles[k][d]);
    }
  const size_t ops_at = total;
  const size_t tiles_at = al(ops_at + dops.size() * sizeof(DenseOp));
  total = tiles_at + dtiles.size() * sizeof(DenseTile);
  e = cudaMalloc(&c.dense_blob, total);
  if (e != cudaSuccess) {
    set_error("dense operators: cudaMalloc: %s", cudaGetErrorString(e));
    return PG_ENOMEM;
  }
  unsigned char* base = (unsigned char*)c.dense_blob;
  for (auto& o : dops) o.dsw = reinterpret_cast<const uint32_t*>(base + (size_t)o.dsw);
  std::vector<unsigned char> host(total, 0);
  for (auto& u : uniq) std::memcpy(&host[u.off], u.planes.data(), u.planes.size() * 4);
  std::memcpy(&host[ops_at], dops.data(), dops.size() * sizeof(DenseOp));
  std::memcpy(&host[tiles_at], dtiles.data(), dtiles.size() * sizeof(DenseTile));
  e = cudaMemcpy(c.dense_blob, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_error("dense operators: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  for (int k : kinds)
    for (int d = 0; d < 3; d++) {
      if (which[((size_t)k * 3 + d) * M] < 0) continue;
      DenseSet& ds = c.dsets[k][d];
      ds.ops = reinterpret_cast<const DenseOp*>(base + ops_at) + set_ops[k][d];
      ds.tiles = reinterpret_cast<const DenseTile*>(base + tiles_at) + set_tiles[k][d];
      ds.ntiles = set_nt[k][d];
      ds.ok = true;
      ds.addback = c.ops[PG_FP64][k][d].addback;
      ds.direct = (k == OPK_D8);
    }
  c.dense_built = true;
  return PG_OK;
}

// Split-line tables of every (operator, direction) and member: segment
// starts, per-position coefficients, the reduced system's inverse rows and
// each segment's window of neighbouring segments (beyond which every entry of
// the inverse is below 2^-60 of its largest), one tile list per direction.
// Members with the same operator, extent and periodicity share one copy.
// A direction is left without split sweeps when a member needs more than 256
// segments or a tile more shared memory than a CTA has.
constexpr int kSplitMaxThreads = 256;
constexpr size_t kSplitMaxSmem = 227 * 1024;

int build_split_ctx(Ctx& c, const std::vector<GridInfo>& g) {
  if (c.split_built) return PG_OK;
  const int M = (int)g.size();
  struct Uniq {
    int k, n;
    bool per;
    std::vector<double> lhs;  // the band the tables factor (boundary codes change it at the ends)
    std::vector<int> start, win;
    std::vector<double> row, G;
    size_t off_row[2], off_G[2], off_start, off_win;
  };
  std::vector<Uniq> uniq;
  std::vector<int> which((size_t)OPK_COUNT * 3 * M, -1);
  bool dir_ok[OPK_COUNT][3];
  for (int k = 0; k < OPK_COUNT; k++)
    for (int d = 0; d < 3; d++) {
      dir_ok[k][d] = !c.ops[PG_FP64][k][d].null_op;
      for (int m = 0; m < M && dir_ok[k][d]; m++) {
        const OpTables& t = g[m].tab[k][d];
        const int n = t.n;
        if (n / kSplitSeg > kSplitMaxThreads) {
          dir_ok[k][d] = false;
          break;
        }
        int u = -1;
        for (size_t q = 0; q < uniq.size() && u < 0; q++)
          if (uniq[q].k == k && uniq[q].n == n && uniq[q].per == t.periodic && uniq[q].lhs == t.lhs) u = (int)q;
        if (u < 0) {
          Uniq e;
          e.k = k;
          e.n = n;
          e.per = t.periodic;
          e.lhs = t.lhs;
          const int rc = build_split(t.lhs, n, t.periodic, e.start, e.row, e.G);
          if (rc) return rc;
          const int S = (int)e.start.size() - 1, T = 4 * S;
          e.win.assign((size_t)2 * S, 0);
          if (!t.implicit) {
            e.row.clear();
            e.G.clear();
          } else {
            double gmax = 0.0;
            for (double v : e.G) gmax = std::max(gmax, std::fabs(v));
            const double thr = std::ldexp(gmax, -60);
            for (int j = 0; j < S; j++) {
              int w = 0;
              for (int js = 0; js < S; js++) {
                double mx = 0.0;
                for (int q = 0; q < 4; q++)
                  for (int cc = 0; cc < 4; cc++) mx = std::max(mx, std::fabs(e.G[((size_t)j * 4 + q) * T + 4 * js + cc]));
                if (mx <= thr) continue;
                int dist = std::abs(js - j);
                if (t.periodic) dist = std::min(dist, S - dist);
                w = std::max(w, dist);
              }
              int first, count;
              if (t.periodic) {
                if (2 * w + 1 >= S) {
                  first = 0;
                  count = S;
                } else {
                  first = ((j - w) % S + S) % S;
                  count = 2 * w + 1;
                }
              } else {
                first = std::max(0, j - w);
                count = std::min(S - 1, j + w) - first + 1;
              }
              e.win[(size_t)2 * j] = first;
              e.win[(size_t)2 * j + 1] = count;
            }
          }
          uniq.push_back(std::move(e));
          u = (int)uniq.size() - 1;
        }
        which[((size_t)k * 3 + d) * M + m] = u;
      }
    }
  // blob: [tables][SplitOp arrays 2 x OPK x 3 x M][tile arrays]
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t total = 0;
  for (auto& u : uniq) {
    u.off_row[0] = total;
    total = al(total + u.row.size() * 8);
    u.off_row[1] = total;
    total = al(total + u.row.size() * 4);
    u.off_G[0] = total;
    total = al(total + u.G.size() * 8);
    u.off_G[1] = total;
    total = al(total + u.G.size() * 4);
    u.off_start = total;
    total = al(total + u.start.size() * 4);
    u.off_win = total;
    total = al(total + u.win.size() * 4);
  }
  std::vector<SplitTile> tiles;
  size_t tile_at[OPK_COUNT][3] = {};
  int tile_n[OPK_COUNT][3] = {};
  size_t sm[3][OPK_COUNT][3] = {};  // fp32, fp64, mixed
  size_t smseg[OPK_COUNT][3] = {};   // register-resident FP32 form along the direction
  bool seg32[OPK_COUNT][3] = {};
  for (int k = 0; k < OPK_COUNT; k++)
    for (int d = 0; d < 3; d++) {
      if (!dir_ok[k][d]) continue;
      tile_at[k][d] = tiles.size();
      seg32[k][d] = true;
      for (int m = 0; m < M; m++) {
        const Uniq& u = uniq[which[((size_t)k * 3 + d) * M + m]];
        const int S = (int)u.start.size() - 1;
        const int nl = std::max(1, kSplitMaxThreads / S);
        const long long lines = g[m].npts / u.n;
        for (long long l0 = 0; l0 < lines; l0 += nl)
          tiles.push_back(SplitTile{m, (int)l0, (int)std::min<long long>(nl, lines - l0), 0});
        sm[0][k][d] = std::max(sm[0][k][d], split_smem_bytes(PG_FP32, false, u.n, S, nl));
        sm[1][k][d] = std::max(sm[1][k][d], split_smem_bytes(PG_FP64, false, u.n, S, nl));
        sm[2][k][d] = std::max(sm[2][k][d], split_smem_bytes(PG_FP32, true, u.n, S, nl));
        smseg[k][d] = std::max(smseg[k][d], seg_smem(d, u.n, S, nl));
        seg32[k][d] = seg32[k][d] && u.n % kSplitSeg == 0;
      }
      tile_n[k][d] = (int)(tiles.size() - tile_at[k][d]);
    }
  const size_t ops_at = al(total);
  const size_t tiles_at = al(ops_at + sizeof(SplitOp) * (size_t)2 * OPK_COUNT * 3 * M);
  total = tiles_at + tiles.size() * sizeof(SplitTile);
  cudaError_t e = cudaMalloc(&c.split_blob, std::max(total, (size_t)256));
  if (e != cudaSuccess) {
    set_error("split tables: cudaMalloc: %s", cudaGetErrorString(e));
    return PG_ENOMEM;
  }
  unsigned char* base = (unsigned char*)c.split_blob;
  std::vector<unsigned char> host(std::max(total, (size_t)256), 0);
  for (auto& u : uniq) {
    for (size_t i = 0; i < u.row.size(); i++) {
      std::memcpy(&host[u.off_row[0] + i * 8], &u.row[i], 8);
      const float f = (float)u.row[i];
      std::memcpy(&host[u.off_row[1] + i * 4], &f, 4);
    }
    for (size_t i = 0; i < u.G.size(); i++) {
      std::memcpy(&host[u.off_G[0] + i * 8], &u.G[i], 8);
      const float f = (float)u.G[i];
      std::memcpy(&host[u.off_G[1] + i * 4], &f, 4);
    }
    std::memcpy(&host[u.off_start], u.start.data(), u.start.size() * 4);
    std::memcpy(&host[u.off_win], u.win.data(), u.win.size() * 4);
  }
  std::vector<SplitOp> sops((size_t)2 * OPK_COUNT * 3 * M);
  auto sidx = [&](int p, int k, int d, int m) { return (((size_t)p * OPK_COUNT + k) * 3 + d) * M + m; };
  for (int p = 0; p < 2; p++)
    for (int k = 0; k < OPK_COUNT; k++)
      for (int d = 0; d < 3; d++) {
        if (!dir_ok[k][d]) continue;
        for (int m = 0; m < M; m++) {
          const Uniq& u = uniq[which[((size_t)k * 3 + d) * M + m]];
          SplitOp& o = sops[sidx(p, k, d, m)];
          o.row = base + u.off_row[p];
          o.G = base + u.off_G[p];
          o.start = reinterpret_cast<const int*>(base + u.off_start);
          o.win = reinterpret_cast<const int*>(base + u.off_win);
          o.S = (int)u.start.size() - 1;
          o.pad = 0;
        }
      }
  std::memcpy(&host[ops_at], sops.data(), sops.size() * sizeof(SplitOp));
  if (!tiles.empty()) std::memcpy(&host[tiles_at], tiles.data(), tiles.size() * sizeof(SplitTile));
  e = cudaMemcpy(c.split_blob, host.data(), host.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    set_error("split tables: %s", cudaGetErrorString(e));
    return PG_ECUDA;
  }
  for (int p = 0; p < 2; p++)
    for (int k = 0; k < OPK_COUNT; k++)
      for (int d = 0; d < 3; d++) {
        SplitSet& ss = c.splits[p][k][d];
        ss = SplitSet();
        if (!dir_ok[k][d]) continue;
        ss.sops = reinterpret_cast<const SplitOp*>(base + ops_at) + sidx(p, k, d, 0);
        ss.tiles = reinterpret_cast<const SplitTile*>(base + tiles_at) + tile_at[k][d];
        ss.ntiles = tile_n[k][d];
        ss.smem32 = sm[0][k][d];
        ss.smem64 = sm[1][k][d];
        ss.smem_mixed = sm[2][k][d];
        ss.seg32 = seg32[k][d];
        ss.smem_seg_x = ss.smem_seg_yz = smseg[k][d];
        const bool exact = (p == PG_FP32) && k == OPK_D8 && c.ops[PG_FP32][k][d].exact;
        size_t need = (p == PG_FP64) ? ss.smem64 : (exact ? ss.smem_mixed : ss.smem32);
        if (p == PG_FP32 && ss.seg32) need = smseg[k][d];  // launch_split's choice
        ss.ok = need <= kSplitMaxSmem;
      }
  c.split_built = true;
  return PG_OK;
}

// Split-line sweeps on (mode 1) or off (mode 0) for every operator and
// direction where they are built, in both precisions.
int set_line_split(Ctx& c, const std::vector<GridInfo>& g, int mode) {
  if (mode != 0 && mode != 1) {
    set_error("line split mode must be 0 or 1, not %d", mode);
    return PG_EINVAL;
  }
  if (mode == 1) {
    const int rc = build_split_ctx(c, g);
    if (rc) return rc;
  }
  for (int p = 0; p < 2; p++)
    for (int k = 0; k < OPK_COUNT; k++)
      for (int d = 0; d < 3; d++) c.use_split[p][k][d] = (mode == 1) && c.splits[p][k][d].ok;
  return PG_OK;
}

int dense_sweep(Ctx& c, int kind, int dir, const double* in, double* out, int epi, int scale_pow, void* st,
                bool emax_ready);

// Autotuning of PG_AUTO: for every (operator, direction), time each sweep
// form the grid has -- the dense tensor-core kernel, the FP32 banded sweep
// with one thread per line, the FP32 split-line sweep -- on this grid (CUDA
// events, median of 3 after one warm-up launch each) and keep the fastest.
int autotune_sweeps(Ctx& c) {
  double* out = nullptr;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&out, (size_t)c.npts * sizeof(double)) != cudaSuccess) {
    set_error("autotune: cudaMalloc failed");
    return PG_ENOMEM;
  }
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaMemset(c.work, 0, (size_t)c.npts * sizeof(double));
  int rc = PG_OK;
  for (int k = 0; k < OPK_COUNT && rc == PG_OK; k++)
    for (int d = 0; d < 3 && rc == PG_OK; d++) {
      const DenseSet& ds = c.dsets[k][d];
      const SplitSet& ss = c.splits[PG_FP32][k][d];
      const OpRef& op = c.ops[PG_FP32][k][d];
      c.use_dense[k][d] = false;
      c.use_split[PG_FP32][k][d] = false;
      if (op.null_op) continue;
      const bool have[3] = {ds.ok, true, c.split_built && ss.ok};
      if (!have[0] && !have[2]) continue;
      float t[3] = {INFINITY, INFINITY, INFINITY};
      for (int way = 0; way < 3 && rc == PG_OK; way++) {
        if (!have[way]) continue;
        float best[3];
        for (int rep = 0; rep < 4 && rc == PG_OK; rep++) {
          cudaEventRecord(e0, 0);
          if (way == 0) {
            rc = dense_sweep(c, k, d, c.work, out, EPI_STORE, 0, nullptr, false);
          } else if (way == 1) {
            SweepLaunch s{c.work, out, c.work2, &op, d, EPI_STORE, 0, c.emax, c.moff};
            rc = launch_sweep(PG_FP32, s, nullptr);
          } else {
            if (k == OPK_D8 && op.exact) rc = launch_max_exponent(c.work, c.moff, c.nmem, c.emax, nullptr);
            if (rc == PG_OK) rc = launch_split(PG_FP32, op, ss, c.work, out, d, EPI_STORE, 0, c.emax, nullptr);
          }
          cudaEventRecord(e1, 0);
          cudaEventSynchronize(e1);
          if (rep > 0) cudaEventElapsedTime(&best[rep - 1], e0, e1);
        }
        std::sort(best, best + 3);
        t[way] = best[1];
      }
      const int win = (t[0] <= t[1] && t[0] <= t[2]) ? 0 : (t[2] < t[1] ? 2 : 1);
      c.use_dense[k][d] = (win == 0);
      c.use_split[PG_FP32][k][d] = (win == 2);
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  cudaError_t e = cudaGetLastError();
  if (rc == PG_OK && e != cudaSuccess) {
    set_error("autotune: %s", cudaGetErrorString(e));
    rc = PG_ECUDA;
  }
  return rc;
}

// Arithmetic of later sweeps: PG_FP64 / PG_FP32 banded; PG_DENSE (dense
// split-TF32 operators wherever built, FP32 banded elsewhere); PG_AUTO (per
// operator and direction the fastest of dense, FP32 banded and FP32
// split-line, measured on this grid).
int set_precision(Ctx& c, const std::vector<GridInfo>& g, int precision) {
  if (precision == PG_DENSE || precision == PG_AUTO) {
    int rc = build_dense(c, g);
    if (rc) return rc;
    c.precision = PG_FP32;
    c.dense = true;
    if (precision == PG_AUTO) {
      rc = build_split_ctx(c, g);
      if (rc) return rc;
      return autotune_sweeps(c);
    }
    for (int k = 0; k < OPK_COUNT; k++)
      for (int d = 0; d < 3; d++) c.use_dense[k][d] = c.dsets[k][d].ok;
    return PG_OK;
  }
  if (precision != PG_FP64 && precision != PG_FP32) return PG_EINVAL;
  c.precision = precision;
  c.dense = false;
  return PG_OK;
}

// emax_ready: the exponents of `in` for the exact d8 RHS are already in c.emax
// One dense sweep.  d8 (direct): the exact fixed-point RHS of every point
// into work2, then A^-1 on the tensor cores.
int dense_sweep(Ctx& c, int kind, int dir, const double* in, double* out, int epi, int scale_pow, void* st,
                bool emax_ready) {
  const DenseSet& ds = c.dsets[kind][dir];
  if (ds.direct) {
    if (!emax_ready) {
      const int rc = launch_max_exponent(in, c.moff, c.nmem, c.emax, st);
      if (rc) return rc;
    }
    const int rc = launch_d8_rhs(c.ops[PG_FP32][kind][dir], in, c.work2, dir, c.emax, c.nmax[dir], st);
    if (rc) return rc;
    return launch_dense(ds, c.work2, out, dir, epi, scale_pow, c.status, st);
  }
  if (in == out) {  // tiles read whole lines that other tiles write: work on a copy
    int rc = launch_copy(c.work2, in, c.npts, st);
    if (rc) return rc;
    in = c.work2;
  }
  return launch_dense(ds, in, out, dir, epi, scale_pow, c.status, st);
}

// sym = -1: the variant for antisymmetric fields, where the direction has a
// symmetry plane (compact_operators.f90:30-35: bc = -1 selects operator 2);
// it runs the banded sweep with one thread per line.
int sweep(Ctx& c, int kind, int dir, const double* in, double* out, int epi, int scale_pow, void* st,
          bool emax_ready = false, int sym = 1) {
  if (sym == -1 && c.symm[dir]) {
    SweepLaunch s{in, out, c.work2, &c.anti[c.precision][kind][dir], dir, epi, scale_pow, c.emax, c.moff, emax_ready};
    return launch_sweep(c.precision, s, st);
  }
  if (c.dense && c.use_dense[kind][dir]) return dense_sweep(c, kind, dir, in, out, epi, scale_pow, st, emax_ready);
  if (c.use_split[c.precision][kind][dir]) {
    const OpRef& op = c.ops[c.precision][kind][dir];
    if (c.precision == PG_FP32 && kind == OPK_D8 && op.exact && !emax_ready) {
      const int rc = launch_max_exponent(in, c.moff, c.nmem, c.emax, st);
      if (rc) return rc;
    }
    return launch_split(c.precision, op, c.splits[c.precision][kind][dir], in, out, dir, epi, scale_pow, c.emax, st);
  }
  SweepLaunch s{in, out, c.work2, &c.ops[c.precision][kind][dir], dir, epi, scale_pow, c.emax, c.moff, emax_ready};
  return launch_sweep(c.precision, s, st);
}

// null-op semantics of compact_operators.f90: derivatives -> 0, filters -> copy
int apply_one(Ctx& c, int kind, int dir, const double* in, double* out, void* st, int sym = 1) {
  if (c.ops[c.precision][kind][dir].null_op) {
    if (kind == OPK_SF || kind == OPK_GF) return launch_copy(out, in, c.npts, st);
    return launch_fill(out, 0.0, c.npts, st);
  }
  return sweep(c, kind, dir, in, out, EPI_STORE, 0, st, false, sym);
}

// operators.f90:848-853 / :872-875: x -> y -> z, null directions copy
int filter_all(Ctx& c, int k, const double* in, double* out, void* st, const int* sym = nullptr) {
  int dirs[3], nd = 0;
  for (int d = 0; d < 3; d++)
    if (!c.ops[c.precision][k][d].null_op) dirs[nd++] = d;
  if (nd == 0) return launch_copy(out, in, c.npts, st);
  const double* src = in;
  for (int q = 0; q < nd; q++) {  // ping-pong so that the last sweep lands in `out`
    double* dst = ((nd - 1 - q) % 2 == 0) ? out : c.work;
    int rc = sweep(c, k, dirs[q], src, dst, EPI_STORE, 0, st, false, sym ? sym[dirs[q]] : 1);
    if (rc) return rc;
    src = dst;
  }
  return PG_OK;
}

// ringS with L = 2 (operators.f90:615-643); a direction of one point, or a
// null d8, contributes 0 and max(x, 0) = x for x >= 0 (operators.f90:701-753).
int ring(Ctx& c, const double* in, double* out, void* st) {
  bool first = true;
  for (int d = 0; d < 3; d++) {
    if (c.ops[c.precision][OPK_D8][d].null_op) continue;
    int rc = sweep(c, OPK_D8, d, in, out, first ? EPI_RING_SET : EPI_RING_MAX, 2, st, !first);
    if (rc) return rc;
    first = false;
  }
  if (first) return launch_fill(out, 0.0, c.npts, st);
  return PG_OK;
}

// ringV with L = 1 (operators.f90:645-699): max over components then times
// d equals max over (component, direction) of |d8| d, rounding being monotonic
int ringv(Ctx& c, const double* vx, const double* vy, const double* vz, double* out, void* st) {
  const double* src[3] = {vx, vy, vz};
  bool first = true;
  for (int q = 0; q < 3; q++) {  // component-major: the exponents of one input serve its three sweeps
    bool ready = false;
    for (int d = 0; d < 3; d++) {
      if (c.ops[c.precision][OPK_D8][d].null_op) continue;
      int rc = sweep(c, OPK_D8, d, src[q], out, first ? EPI_RING_SET : EPI_RING_MAX, 1, st, ready);
      if (rc) return rc;
      first = false;
      ready = true;
    }
  }
  if (first) return launch_fill(out, 0.0, c.npts, st);
  return PG_OK;
}

int grad(Ctx& c, const double* in, double* gx, double* gy, double* gz, void* st) {
  int rc = apply_one(c, OPK_D1, 0, in, gx, st);
  if (!rc) rc = apply_one(c, OPK_D1, 1, in, gy, st);
  if (!rc) rc = apply_one(c, OPK_D1, 2, in, gz, st);
  return rc;
}

// LapS, Cartesian (operators.f90:513-526): d2x + d2y + d2z, null directions contribute 0
int laplacian(Ctx& c, const double* in, double* out, void* st) {
  bool first = true;
  for (int d = 0; d < 3; d++) {
    if (c.ops[c.precision][OPK_D2][d].null_op) continue;
    int rc = sweep(c, OPK_D2, d, in, out, first ? EPI_STORE : EPI_ADD, 0, st);
    if (rc) return rc;
    first = false;
  }
  if (first) return launch_fill(out, 0.0, c.npts, st);
  return PG_OK;
}

// divV, Cartesian (operators.f90:38-53): df = fA + fB + fC
int divergence(Ctx& c, const double* fx, const double* fy, const double* fz, double* out, void* st) {
  const double* f[3] = {fx, fy, fz};
  bool first = true;
  for (int d = 0; d < 3; d++) {
    if (c.ops[c.precision][OPK_D1][d].null_op) continue;  // contributes exactly 0
    // a vector component normal to a symmetry plane is antisymmetric (operators.f90:48-50, isym = -1)
    int rc = sweep(c, OPK_D1, d, f[d], out, first ? EPI_STORE : EPI_ADD, 0, st, false, c.symm[d] ? -1 : 1);
    if (rc) return rc;
    first = false;
  }
  if (first) return launch_fill(out, 0.0, c.npts, st);
  return PG_OK;
}

int host_prepare(Ctx& c) {
  if (!c.stream) PG_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  if (!c.host_in) PG_CUDA(cudaMalloc(&c.host_in, (size_t)c.npts * sizeof(double)));
  if (!c.host_out) PG_CUDA(cudaMalloc(&c.host_out, (size_t)c.npts * sizeof(double)));
  return PG_OK;
}

template <typename F>
int host_call(Ctx& c, const double* in, double* out, F&& f) {
  if (!in || !out) return PG_EINVAL;
  int rc = host_prepare(c);
  if (rc) return rc;
  const size_t bytes = (size_t)c.npts * sizeof(double);
  PG_CUDA(cudaMemcpyAsync(c.host_in, in, bytes, cudaMemcpyHostToDevice, c.stream));
  rc = f(c.host_in, c.host_out, (void*)c.stream);
  if (rc) {
    cudaStreamSynchronize(c.stream);
    return rc;
  }
  PG_CUDA(cudaMemcpyAsync(out, c.host_out, bytes, cudaMemcpyDeviceToHost, c.stream));
  PG_CUDA(cudaStreamSynchronize(c.stream));
  return PG_OK;
}

int read_status(Ctx& c, int* status) {
  int v = 0;
  PG_CUDA(cudaMemcpy(&v, c.status, sizeof(int), cudaMemcpyDeviceToHost));
  if (v != 0) PG_CUDA(cudaMemset(c.status, 0, sizeof(int)));
  *status = v;
  return PG_OK;
}

}  // namespace
}  // namespace pg

using namespace pg;

struct pg_handle {
  GridInfo g;
  Ctx c;
};

struct pg_ensemble {
  std::vector<GridInfo> g;
  Ctx c;
};

extern "C" {

const char* pg_last_error(void) { return g_err; }

const char* pg_version(void) { return "pyranda_gb300 0.2 (sm_103a)"; }

uint64_t pg_launch_count(void) { return g_launches.load(); }

namespace pg {
namespace {

// isym^p of a direction (patch.f90:89-91): -1 for odd p where the direction has a SYMM end
int isym(const Ctx& c, int d, int p) { return (c.symm[d] && (p & 1)) ? -1 : 1; }

int cyl(const pg_handle* h, int op, const double* a, const double* b, const double* c_, const double* e,
        const double* f, double* out, void* st) {
  const GridInfo& g = h->g;
  return launch_cyl(op, g.npts, g.n[0], g.n[1], g.x1f[0], g.d[0], g.d[1], g.d[2], a, b, c_, e, f, out, st);
}

// divV, cylindrical (operators.f90:55-64): (d(r fx)/dr + dfy/dy) / r + dfz/dz
int divergence_cyl(pg_handle* h, const double* fx, const double* fy, const double* fz, double* out, void* st) {
  Ctx& c = h->c;
  int rc = cyl(h, CYL_MUL_R, fx, nullptr, nullptr, nullptr, nullptr, c.cyl[0], st);
  if (!rc) rc = apply_one(c, OPK_D1, 0, c.cyl[0], c.cyl[1], st, isym(c, 0, 2));
  if (!rc) rc = apply_one(c, OPK_D1, 1, fy, c.cyl[2], st, isym(c, 1, 1));
  if (!rc) rc = apply_one(c, OPK_D1, 2, fz, out, st, isym(c, 2, 1));
  if (!rc) rc = cyl(h, CYL_DIVV, c.cyl[1], c.cyl[2], out, nullptr, nullptr, out, st);
  return rc;
}

// divT (operators.f90:97-146): Cartesian and cylindrical (spherical and
// curvilinear: divt_metric).  f = {fxx, fxy, fxz,
// fyx, fyy, fyz, fzx, fzy, fzz}; out = {dfx, dfy, dfz}, distinct from f.
int divt(pg_handle* h, const double* const* f, double* const* out, void* st) {
  Ctx& c = h->c;
  const double *fxx = f[0], *fxy = f[1], *fxz = f[2], *fyx = f[3], *fyy = f[4], *fyz = f[5], *fzx = f[6],
               *fzy = f[7], *fzz = f[8];
  int rc = PG_OK;
  if (c.coordsys == PG_CARTESIAN) {  // :104-122: dfx = d(fxx)/dx + d(fyx)/dy + d(fzx)/dz ...
    const double* cols[3][3] = {{fxx, fyx, fzx}, {fxy, fyy, fzy}, {fxz, fyz, fzz}};
    for (int comp = 0; comp < 3 && !rc; comp++) {
      bool first = true;
      for (int d = 0; d < 3 && !rc; d++) {
        if (c.ops[c.precision][OPK_D1][d].null_op) continue;
        rc = sweep(c, OPK_D1, d, cols[comp][d], out[comp], first ? EPI_STORE : EPI_ADD, 0, st, false,
                   isym(c, d, d == comp ? 2 : 1));
        first = false;
      }
      if (!rc && first) rc = launch_fill(out[comp], 0.0, c.npts, st);
    }
    return rc;
  }
  // cylindrical (:123-146)
  rc = cyl(h, CYL_MUL_R, fxx, nullptr, nullptr, nullptr, nullptr, c.cyl[0], st);
  if (!rc) rc = apply_one(c, OPK_D1, 0, c.cyl[0], c.cyl[1], st, isym(c, 0, 3));
  if (!rc) rc = apply_one(c, OPK_D1, 1, fyx, c.cyl[2], st, isym(c, 1, 1));
  if (!rc) rc = apply_one(c, OPK_D1, 2, fzx, out[0], st, isym(c, 2, 1));
  if (!rc) rc = cyl(h, CYL_DIVT_X, c.cyl[1], c.cyl[2], out[0], fyy, nullptr, out[0], st);
  if (!rc) rc = cyl(h, CYL_MUL_R2, fxy, nullptr, nullptr, nullptr, nullptr, c.cyl[0], st);
  if (!rc) rc = apply_one(c, OPK_D1, 0, c.cyl[0], c.cyl[1], st, isym(c, 0, 3));
  if (!rc) rc = apply_one(c, OPK_D1, 1, fyy, c.cyl[2], st, isym(c, 1, 2));
  if (!rc) rc = apply_one(c, OPK_D1, 2, fzy, out[1], st, isym(c, 2, 1));
  if (!rc) rc = cyl(h, CYL_DIVT_Y, c.cyl[1], c.cyl[2], out[1], fyx, fxy, out[1], st);
  if (!rc) rc = cyl(h, CYL_MUL_R, fxz, nullptr, nullptr, nullptr, nullptr, c.cyl[0], st);
  if (!rc) rc = apply_one(c, OPK_D1, 0, c.cyl[0], c.cyl[1], st, isym(c, 0, 2));
  if (!rc) rc = apply_one(c, OPK_D1, 1, fyz, c.cyl[2], st, isym(c, 1, 1));
  if (!rc) rc = apply_one(c, OPK_D1, 2, fzz, out[2], st, isym(c, 2, 2));
  if (!rc) rc = cyl(h, CYL_DIVV, c.cyl[1], c.cyl[2], out[2], nullptr, nullptr, out[2], st);
  return rc;
}

// ---------------------------------------------------------------------------
// Spherical and curvilinear grids: the derivative sweeps of the handle joined
// by the pointwise metric forms of pg_metric.cu (operators.f90:54-209).
// ---------------------------------------------------------------------------
MetricArgs margs(const pg_handle* h, int op) {
  const GridInfo& g = h->g;
  MetricArgs A;
  A.op = op;
  A.n = g.npts;
  A.nx = g.n[0];
  A.ny = g.n[1];
  A.nz = g.n[2];
  A.coordsys = g.coordsys;
  for (int d = 0; d < 3; d++) {
    A.x1f[d] = g.x1f[d];
    A.d[d] = g.d[d];
    A.x1[d] = g.x1[d];
    A.xn[d] = g.xn[d];
  }
  for (int q = 0; q < MF_COUNT; q++) A.mf[q] = h->c.mf[q];
  return A;
}

int metric(const pg_handle* h, int op, std::initializer_list<const double*> in, std::initializer_list<double*> out,
           void* st, int L = 0) {
  MetricArgs A = margs(h, op);
  int q = 0;
  for (const double* p : in) A.in[q++] = p;
  q = 0;
  for (double* p : out) A.out[q++] = p;
  A.L = L;
  return launch_metric(A, st);
}

bool sph(const Ctx& c) { return c.coordsys == PG_SPHERICAL || c.coordsys == PG_SPHERICAL_RATIO; }

// gradS (operators.f90:197-209): the derivatives along the grid lines, then the metric factors
int grad_metric(pg_handle* h, const double* in, double* gx, double* gy, double* gz, void* st) {
  int rc = grad(h->c, in, gx, gy, gz, st);
  if (!rc) rc = metric(h, sph(h->c) ? MET_SPH_GRAD : MET_CURV_GRAD, {}, {gx, gy, gz}, st);
  return rc;
}

// divV (operators.f90:64-90)
int div_metric(pg_handle* h, const double* fx, const double* fy, const double* fz, double* out, void* st) {
  Ctx& c = h->c;
  double *w0 = c.cyl[0], *w1 = c.cyl[1], *w2 = c.cyl[2];
  int rc;
  if (sph(c)) {  // r^2 fx and fy sin(theta) (isymX^3, isymY^2, isymZ), then (fA dx/d1)/r^2 + (fB+fC)/(r sin)
    rc = metric(h, MET_SPH_DIV_PRE, {fx, fy}, {w0, w1}, st);
    if (!rc) rc = apply_one(c, OPK_D1, 0, w0, w2, st, isym(c, 0, 3));
    if (!rc) rc = apply_one(c, OPK_D1, 1, w1, w0, st, isym(c, 1, 2));
    if (!rc) rc = apply_one(c, OPK_D1, 2, fz, out, st, isym(c, 2, 1));
    if (!rc) rc = metric(h, MET_SPH_DIV_POST, {w2, w0, out}, {out}, st);
    return rc;
  }
  // curvilinear: the contravariant fluxes times det J along A, B, C, summed, over det J
  rc = metric(h, MET_CURV_DIV_PRE, {fx, fy, fz}, {w0, w1, w2}, st);
  if (!rc) rc = apply_one(c, OPK_D1, 0, w0, out, st);
  if (!rc) rc = apply_one(c, OPK_D1, 1, w1, w0, st);
  if (!rc) rc = apply_one(c, OPK_D1, 2, w2, w1, st);
  if (!rc) rc = metric(h, MET_CURV_DIV_POST, {out, w0, w1}, {out}, st);
  return rc;
}

// divT (operators.f90:147-177): spherical rows, or the divergence of each row on curvilinear grids
int divt_metric(pg_handle* h, const double* const* f, double* const* out, void* st) {
  Ctx& c = h->c;
  if (!sph(c)) {
    int rc = div_metric(h, f[0], f[1], f[2], out[0], st);
    if (!rc) rc = div_metric(h, f[3], f[4], f[5], out[1], st);
    if (!rc) rc = div_metric(h, f[6], f[7], f[8], out[2], st);
    return rc;
  }
  const double *fxx = f[0], *fxy = f[1], *fxz = f[2], *fyx = f[3], *fyy = f[4], *fyz = f[5], *fzx = f[6],
               *fzy = f[7], *fzz = f[8];
  double *w0 = c.cyl[0], *w1 = c.cyl[1], *w2 = c.cyl[2];
  // row: (r^k f_x, theta form of f_y, f_z) with the symmetry powers of each derivative, then the row's combination
  struct Row {
    const double *a, *b, *cz;
    int k, py, pz;
    const double *t0, *t1, *t2;
  };
  const Row rows[3] = {{fxx, fyx, fzx, 2, 2, 1, fyy, fzz, nullptr},
                       {fxy, fyy, fzy, 3, 3, 1, fyx, fxy, fzz},
                       {fxz, fyz, fzz, 3, 2, 2, fzx, fxz, fzy}};
  int rc = PG_OK;
  for (int r = 0; r < 3 && !rc; r++) {
    const Row& R = rows[r];
    rc = metric(h, MET_SPH_T_PRE, {R.a, R.b}, {w0, w1}, st, R.k);
    if (!rc) rc = apply_one(c, OPK_D1, 0, w0, w2, st, 1);  // isymX^4
    if (!rc) rc = apply_one(c, OPK_D1, 1, w1, w0, st, isym(c, 1, R.py));
    if (!rc) rc = apply_one(c, OPK_D1, 2, R.cz, w1, st, isym(c, 2, R.pz));
    if (!rc) rc = metric(h, MET_SPH_T_POST, {w2, w0, w1, R.t0, R.t1, R.t2}, {out[r]}, st, r);
  }
  return rc;
}

// filter('spectral') on spherical and curvilinear grids (operators.f90:884-889):
// filter CellVol f, divide by the filtered cell volume (CellVol itself when ratio-zoned)
int filter_metric(pg_handle* h, const double* in, double* out, void* st) {
  Ctx& c = h->c;
  int rc = metric(h, MET_VOL_MUL, {in}, {c.cyl[0]}, st);
  if (!rc) rc = filter_all(c, OPK_SF, c.cyl[0], out, st);
  if (!rc) rc = metric(h, MET_VOL_DIV, {out, c.mf[c.coordsys == PG_SPHERICAL_RATIO ? MF_CV : MF_CVS]}, {out}, st);
  return rc;
}

// ringS / ringV with mesh-field scales (operators.f90:615-699): the d8 of each
// (component, direction) into a workspace field, then max(out, |d8| d^L)
bool ring_fields(const Ctx& c, const GridInfo& g) {
  return c.coordsys >= PG_SPHERICAL || (c.coordsys == PG_CYLINDRICAL && g.n[1] > 1);
}

int ring_metric(pg_handle* h, const double* const* src, int ncomp, int L, double* out, void* st) {
  Ctx& c = h->c;
  bool first = true;
  int rc = PG_OK;
  for (int q = 0; q < ncomp && !rc; q++)
    for (int d = 0; d < 3 && !rc; d++) {
      if (c.ops[c.precision][OPK_D8][d].null_op) continue;
      rc = apply_one(c, OPK_D8, d, src[q], c.cyl[0], st);
      if (rc) break;
      MetricArgs A = margs(h, MET_RING);
      A.in[0] = c.cyl[0];
      A.out[0] = out;
      A.dir = d;
      A.L = L;
      A.first = first ? 1 : 0;
      rc = launch_metric(A, st);
      first = false;
    }
  if (!rc && first) rc = launch_fill(out, 0.0, c.npts, st);
  return rc;
}

// LapS, cylindrical and spherical (operators.f90:527-559)
int laplacian_metric(pg_handle* h, const double* in, double* out, void* st) {
  Ctx& c = h->c;
  double *w0 = c.cyl[0], *w1 = c.cyl[1];
  const int L = c.coordsys == PG_CYLINDRICAL ? 1 : 2;
  int rc = apply_one(c, OPK_D1, 0, in, w0, st);
  if (!rc) rc = metric(h, MET_LAP_MUL, {w0}, {w1}, st, L);   // r^L df/dr
  if (!rc) rc = apply_one(c, OPK_D1, 0, w1, w0, st);
  if (!rc) rc = metric(h, MET_LAP_X, {w0}, {out}, st, L);    // / r^L
  if (c.coordsys == PG_CYLINDRICAL) {
    if (!rc) rc = apply_one(c, OPK_D2, 1, in, w0, st);
  } else {
    if (!rc) rc = apply_one(c, OPK_D1, 1, in, w0, st);
    if (!rc) rc = metric(h, MET_LAP_SIN, {w0}, {w1}, st);     // sin(theta) df/dtheta
    if (!rc) rc = apply_one(c, OPK_D1, 1, w1, w0, st);
  }
  if (!rc) rc = metric(h, MET_LAP_ADD_Y, {w0}, {out}, st);
  if (!rc) rc = apply_one(c, OPK_D2, 2, in, w0, st);
  if (!rc) rc = metric(h, MET_LAP_ADD_Z, {w0}, {out}, st);
  return rc;
}

// The mesh fields of a spherical or curvilinear grid (mesh.f90:169-386), on
// FP64 Cartesian handles of the same extents: one with the grid's own ends
// (the stock operators) and, when the coordinates are not periodic, one with
// one-sided ends everywhere for the Jacobian (mesh.f90:246-307).
int mesh_setup(pg_handle* h, const double* x, const double* y, const double* z, int mesh_per, void* st) {
  Ctx& c = h->c;
  const GridInfo& g = h->g;
  pg_grid base{};
  for (int d = 0; d < 3; d++) {
    base.n[d] = g.n[d];
    base.periodic[d] = g.periodic[d];
    base.x1[d] = g.x1[d];
    base.xn[d] = g.xn[d];
    for (int e = 0; e < 2; e++) base.bc[d][e] = g.bc[d][e];
  }
  base.precision = PG_FP64;
  base.coordsys = PG_CARTESIAN;
  pg_handle *stock = nullptr, *custom = nullptr;
  int rc = pg_create(&base, &stock);
  if (!rc && c.coordsys == PG_CURVILINEAR && mesh_per) {
    pg_grid open = base;
    for (int d = 0; d < 3; d++) {
      open.periodic[d] = 0;
      open.bc[d][0] = open.bc[d][1] = PG_BC_NONE;
    }
    rc = pg_create(&open, &custom);
  }
  if (!rc && sph(c)) {
    MetricArgs A = margs(h, MET_SPH_MESH);
    if (c.coordsys == PG_SPHERICAL_RATIO) {  // mesh.f90:180-186
      A.s1 = std::log((double)(g.n[0] - 1) * g.d[0]) / (g.d[1] * (double)(g.n[0] - 1));  // Csp
      A.s0 = (g.x1f[0] + g.d[0] / 2.0) / std::exp(A.s1 * g.d[1]);                        // Asp
    }
    rc = launch_metric(A, st);
  }
  if (!rc && c.coordsys == PG_CURVILINEAR) {
    const size_t nbytes = (size_t)c.npts * sizeof(double);
    if (!x) {
      rc = launch_metric(margs(h, MET_NODES), st);
    } else {
      const double* src[3] = {x, y, z};
      for (int q = 0; q < 3 && !rc; q++)
        if (cudaMemcpyAsync(c.mf[MF_X + q], src[q], nbytes, cudaMemcpyDeviceToDevice, (cudaStream_t)st) !=
            cudaSuccess) {
          set_error("pg_set_mesh_coords: %s", cudaGetErrorString(cudaGetLastError()));
          rc = PG_ECUDA;
        }
    }
    pg_handle* jh = custom ? custom : stock;
    for (int q = 0; q < 3 && !rc; q++)  // J[3 q + d] = d(coordinate q) / d(direction d)
      for (int d = 0; d < 3 && !rc; d++) rc = pg_d1(jh, d, c.mf[MF_X + q], c.mf[MF_J0 + 3 * q + d], st);
    if (!rc) rc = launch_metric(margs(h, MET_CURV_METRIC), st);
  }
  if (!rc) {  // mesh.f90:373-386: the filtered cell volumes (spherical and curvilinear), else CellVol
    const size_t nbytes = (size_t)c.npts * sizeof(double);
    if (c.coordsys == PG_SPHERICAL || c.coordsys == PG_CURVILINEAR) {
      rc = pg_filter(stock, PG_SPECTRAL, PG_DIR_ALL, c.mf[MF_CV], c.mf[MF_CVS], st);
      if (!rc) rc = pg_filter(stock, PG_GAUSSIAN, PG_DIR_ALL, c.mf[MF_CV], c.mf[MF_CVG], st);
    } else {
      for (int q = MF_CVS; q <= MF_CVG && !rc; q++)
        if (cudaMemcpyAsync(c.mf[q], c.mf[MF_CV], nbytes, cudaMemcpyDeviceToDevice, (cudaStream_t)st) !=
            cudaSuccess)
          rc = PG_ECUDA;
    }
  }
  if (cudaStreamSynchronize((cudaStream_t)st) != cudaSuccess && !rc) {
    set_error("mesh set-up: %s", cudaGetErrorString(cudaGetLastError()));
    rc = PG_ECUDA;
  }
  if (custom) pg_destroy(custom);
  if (stock) pg_destroy(stock);
  return rc;
}

}  // namespace
}  // namespace pg

int pg_create(const pg_grid* grid, pg_handle** out) {
  if (!grid || !out) {
    set_error("pg_create: NULL argument");
    return PG_EINVAL;
  }
  *out = nullptr;
  if (grid->precision < PG_FP64 || grid->precision > PG_AUTO) {
    set_error("pg_create: bad precision %d", grid->precision);
    return PG_EINVAL;
  }
  pg_handle* h = new pg_handle();
  int rc = grid_info(grid, h->g, "pg_create");
  if (rc == PG_OK) rc = build_ctx(h->c, std::vector<GridInfo>{h->g}, PG_FP64, "pg_create");
  if (rc == PG_OK && grid->coordsys >= PG_SPHERICAL) rc = mesh_setup(h, nullptr, nullptr, nullptr, 1, nullptr);
  if (rc == PG_OK) rc = set_precision(h->c, std::vector<GridInfo>{h->g}, grid->precision);
  if (rc != PG_OK) {
    free_ctx(h->c);
    delete h;
    return rc;
  }
  *out = h;
  return PG_OK;
}

int pg_destroy(pg_handle* h) {
  if (!h) return PG_OK;
  free_ctx(h->c);
  delete h;
  return PG_OK;
}

int pg_device_status(pg_handle* h, int* status) {
  if (!h || !status) return PG_EINVAL;
  return read_status(h->c, status);
}

int pg_set_precision(pg_handle* h, int precision) {
  if (!h) return PG_EINVAL;
  return set_precision(h->c, std::vector<GridInfo>{h->g}, precision);
}

int pg_wait_selftest(pg_handle* h, unsigned limit_ms, void* stream) {
  if (!h || limit_ms == 0 || limit_ms > 10000) return PG_EINVAL;
  return launch_wait_selftest(h->c.status, limit_ms, stream);
}

int pg_set_line_split(pg_handle* h, int mode) {
  if (!h) return PG_EINVAL;
  return set_line_split(h->c, std::vector<GridInfo>{h->g}, mode);
}

int pg_sweep_plan(const pg_handle* h, int* plan) {
  if (!h || !plan) return PG_EINVAL;
  const Ctx& c = h->c;
  for (int k = 0; k < OPK_COUNT; k++)
    for (int d = 0; d < 3; d++)
      plan[k * 3 + d] = (c.dense && c.use_dense[k][d]) ? 1 : (c.use_split[c.precision][k][d] ? 2 : 0);
  return PG_OK;
}

// A plan as pg_sweep_plan writes it (per operator and direction: 0 FP32 banded,
// 1 dense, 2 FP32 split-line), applied without timing: the dense and split
// tables it needs are built, then the handle runs the FP32 path with it.
int pg_set_sweep_plan(pg_handle* h, const int* plan) {
  if (!h || !plan) return PG_EINVAL;
  Ctx& c = h->c;
  const std::vector<GridInfo> g{h->g};
  bool want_dense = false, want_split = false;
  for (int i = 0; i < OPK_COUNT * 3; i++) {
    if (plan[i] < 0 || plan[i] > 2) {
      set_error("pg_set_sweep_plan: entry %d = %d is not 0 (banded), 1 (dense) or 2 (split)", i, plan[i]);
      return PG_EINVAL;
    }
    want_dense = want_dense || plan[i] == 1;
    want_split = want_split || plan[i] == 2;
  }
  int rc = want_dense ? build_dense(c, g) : PG_OK;
  if (rc == PG_OK && want_split) rc = build_split_ctx(c, g);
  if (rc != PG_OK) return rc;
  for (int k = 0; k < OPK_COUNT; k++)
    for (int d = 0; d < 3; d++) {
      const int p = plan[k * 3 + d];
      if ((p == 1 && !c.dsets[k][d].ok) || (p == 2 && !c.splits[PG_FP32][k][d].ok)) {
        set_error("pg_set_sweep_plan: operator %d along %d has no %s form on this grid", k, d,
                  p == 1 ? "dense" : "split");
        return PG_EINVAL;
      }
    }
  c.precision = PG_FP32;
  c.dense = want_dense;
  for (int k = 0; k < OPK_COUNT; k++)
    for (int d = 0; d < 3; d++) {
      c.use_dense[k][d] = plan[k * 3 + d] == 1;
      c.use_split[PG_FP32][k][d] = plan[k * 3 + d] == 2;
    }
  return PG_OK;
}

int pg_dense_plan(const pg_handle* h, int* plan) {
  if (!h || !plan) return PG_EINVAL;
  for (int k = 0; k <= OPK_GF; k++)
    for (int d = 0; d < 3; d++) plan[k * 3 + d] = (h->c.dense && h->c.use_dense[k][d]) ? 1 : 0;
  return PG_OK;
}

int pg_get_spacing(const pg_handle* h, double* patch_d, double* mesh_d) {
  if (!h) return PG_EINVAL;
  for (int d = 0; d < 3; d++) {
    if (patch_d) patch_d[d] = h->g.d[d];
    if (mesh_d) mesh_d[d] = h->g.dm[d];
  }
  return PG_OK;
}

int pg_d1(pg_handle* h, int dir, const double* in, double* out, void* stream) {
  if (!h || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(h->c, OPK_D1, dir, in, out, stream);
}

int pg_d8(pg_handle* h, int dir, const double* in, double* out, void* stream) {
  if (!h || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(h->c, OPK_D8, dir, in, out, stream);
}

int pg_d2(pg_handle* h, int dir, const double* in, double* out, void* stream) {
  if (!h || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(h->c, OPK_D2, dir, in, out, stream);
}

int pg_d4(pg_handle* h, int dir, const double* in, double* out, void* stream) {
  if (!h || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(h->c, OPK_D4, dir, in, out, stream);
}

int pg_set_mesh_coords(pg_handle* h, const double* x, const double* y, const double* z, int mesh_periodic,
                       void* stream) {
  if (!h || !x || !y || !z) return PG_EINVAL;
  if (h->c.coordsys != PG_CURVILINEAR) {
    set_error("pg_set_mesh_coords: the grid is not curvilinear");
    return PG_EINVAL;
  }
  return mesh_setup(h, x, y, z, mesh_periodic ? 1 : 0, stream);
}

int pg_laplacian(pg_handle* h, const double* in, double* out, void* stream) {
  if (!h || !in || !out) return PG_EINVAL;
  if (in == out) {
    set_error("pg_laplacian: in and out must differ");
    return PG_EINVAL;
  }
  if (h->c.coordsys == PG_CURVILINEAR || h->c.coordsys == PG_SPHERICAL_RATIO) {
    set_error("pg_laplacian: no Laplacian on curvilinear or ratio-zoned spherical grids (operators.f90:513-559)");
    return PG_EINVAL;
  }
  if (h->c.coordsys != PG_CARTESIAN) return laplacian_metric(h, in, out, stream);
  return laplacian(h->c, in, out, stream);
}

int pg_filter(pg_handle* h, int kind, int dir, const double* in, double* out, void* stream) {
  if (!h || !in || !out || (kind != PG_SPECTRAL && kind != PG_GAUSSIAN) || dir < 0 || dir > 3) return PG_EINVAL;
  const int k = kind == PG_SPECTRAL ? OPK_SF : OPK_GF;
  if (dir < 3) return apply_one(h->c, k, dir, in, out, stream);
  if (h->c.coordsys >= PG_SPHERICAL && kind == PG_SPECTRAL) {
    if (in == out) {
      set_error("pg_filter: on a non-Cartesian grid out must not alias in");
      return PG_EINVAL;
    }
    return filter_metric(h, in, out, stream);
  }
  if (h->c.coordsys == PG_CYLINDRICAL && kind == PG_SPECTRAL) {
    // operators.f90:876-883: filter the volume-weighted field (CellVol is odd in r, so the radial
    // sweep takes the antisymmetric variant) and divide by the cell volume
    if (in == out) {
      set_error("pg_filter: on a cylindrical grid out must not alias in");
      return PG_EINVAL;
    }
    Ctx& c = h->c;
    const int sym[3] = {-1, 1, 1};
    int rc = cyl(h, CYL_CELLVOL_MUL, in, nullptr, nullptr, nullptr, nullptr, c.cyl[0], stream);
    if (!rc) rc = filter_all(c, k, c.cyl[0], out, stream, sym);
    if (!rc) rc = cyl(h, CYL_CELLVOL_DIV, out, nullptr, nullptr, nullptr, nullptr, out, stream);
    return rc;
  }
  return filter_all(h->c, k, in, out, stream);
}

int pg_d1_sym(pg_handle* h, int dir, int sym, const double* in, double* out, void* stream) {
  if (!h || !in || !out || bad_dir(dir) || (sym != 1 && sym != -1)) return PG_EINVAL;
  return apply_one(h->c, OPK_D1, dir, in, out, stream, sym);
}

int pg_d8_sym(pg_handle* h, int dir, int sym, const double* in, double* out, void* stream) {
  if (!h || !in || !out || bad_dir(dir) || (sym != 1 && sym != -1)) return PG_EINVAL;
  return apply_one(h->c, OPK_D8, dir, in, out, stream, sym);
}

int pg_filter_sym(pg_handle* h, int kind, int dir, const int* sym, const double* in, double* out, void* stream) {
  if (!h || !in || !out || !sym || (kind != PG_SPECTRAL && kind != PG_GAUSSIAN) || dir < 0 || dir > 3)
    return PG_EINVAL;
  for (int d = 0; d < 3; d++)
    if (sym[d] != 1 && sym[d] != -1) return PG_EINVAL;
  const int k = kind == PG_SPECTRAL ? OPK_SF : OPK_GF;
  if (dir < 3) return apply_one(h->c, k, dir, in, out, stream, sym[dir]);
  return filter_all(h->c, k, in, out, stream, sym);
}

int pg_ring(pg_handle* h, const double* in, double* out, void* stream) {
  if (!h || !in || !out) return PG_EINVAL;
  if (in == out) {
    set_error("pg_ring: in and out must differ");
    return PG_EINVAL;
  }
  if (ring_fields(h->c, h->g)) return ring_metric(h, &in, 1, 2, out, stream);
  return ring(h->c, in, out, stream);
}

int pg_ringv(pg_handle* h, const double* vx, const double* vy, const double* vz, double* out, void* stream) {
  if (!h || !vx || !vy || !vz || !out) return PG_EINVAL;
  if (out == vx || out == vy || out == vz) {
    set_error("pg_ringv: out must not alias an input");
    return PG_EINVAL;
  }
  if (ring_fields(h->c, h->g)) {
    const double* src[3] = {vx, vy, vz};
    return ring_metric(h, src, 3, 1, out, stream);
  }
  return ringv(h->c, vx, vy, vz, out, stream);
}

int pg_grad(pg_handle* h, const double* in, double* gx, double* gy, double* gz, void* stream) {
  if (!h || !in || !gx || !gy || !gz) return PG_EINVAL;
  if (h->c.coordsys >= PG_SPHERICAL) return grad_metric(h, in, gx, gy, gz, stream);
  int rc = grad(h->c, in, gx, gy, gz, stream);
  if (!rc && h->c.coordsys == PG_CYLINDRICAL)  // operators.f90:193-196: dfdy / r
    rc = cyl(h, CYL_DIV_R, gy, nullptr, nullptr, nullptr, nullptr, gy, stream);
  return rc;
}

int pg_divt(pg_handle* h, const double* const* f, double* const* out, void* stream) {
  if (!h || !f || !out) return PG_EINVAL;
  for (int q = 0; q < 9; q++)
    if (!f[q]) return PG_EINVAL;
  for (int q = 0; q < 3; q++) {
    if (!out[q]) return PG_EINVAL;
    for (int r = 0; r < 9; r++)
      if (out[q] == f[r]) {
        set_error("pg_divt: outputs must not alias inputs");
        return PG_EINVAL;
      }
  }
  if (h->c.coordsys >= PG_SPHERICAL) return divt_metric(h, f, out, stream);
  return divt(h, f, out, stream);
}

int pg_div(pg_handle* h, const double* fx, const double* fy, const double* fz, double* out, void* stream) {
  if (h && h->c.coordsys == PG_CYLINDRICAL) {
    if (!fx || !fy || !fz || !out) return PG_EINVAL;
    return divergence_cyl(h, fx, fy, fz, out, stream);
  }
  if (!h || !fx || !fy || !fz || !out) return PG_EINVAL;
  if (out == fy || out == fz) {
    set_error("pg_div: out must not alias fy or fz");
    return PG_EINVAL;
  }
  if (h->c.coordsys >= PG_SPHERICAL) return div_metric(h, fx, fy, fz, out, stream);
  return divergence(h->c, fx, fy, fz, out, stream);
}

int pg_mesh(pg_handle* h, int which, double* out, void* stream) {
  if (!h || !out || which < 0 || which > PG_MESH_DC_DZ) return PG_EINVAL;
  const GridInfo& g = h->g;
  if (g.coordsys >= PG_SPHERICAL) {
    if (which >= PG_MESH_DET && g.coordsys != PG_CURVILINEAR) {
      set_error("pg_mesh: det J and the inverse Jacobian exist on curvilinear grids only");
      return PG_EINVAL;
    }
    const cudaError_t e = cudaMemcpyAsync(out, h->c.mf[which], (size_t)h->c.npts * sizeof(double),
                                          cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
    if (e != cudaSuccess) {
      set_error("pg_mesh: %s", cudaGetErrorString(e));
      return PG_ECUDA;
    }
    return PG_OK;
  }
  if (which >= PG_MESH_DET) {
    set_error("pg_mesh: det J and the inverse Jacobian exist on curvilinear grids only");
    return PG_EINVAL;
  }
  if (which == PG_MESH_CELLVOL_S || which == PG_MESH_CELLVOL_G) which = PG_MESH_CELLVOL;  // mesh.f90:384-386
  if (g.coordsys == PG_CYLINDRICAL && (which == PG_MESH_D2 || which == PG_MESH_GRIDLEN || which == PG_MESH_CELLVOL)) {
    // mesh.f90:213-225: d2 = r dy, GridLen and CellVol vary with the radius
    const int op = which == PG_MESH_D2 ? CYL_D2 : (which == PG_MESH_GRIDLEN ? CYL_GRIDLEN : CYL_CELLVOL);
    return cyl(h, op, nullptr, nullptr, nullptr, nullptr, nullptr, out, stream);
  }
  if (g.coordsys == PG_CYLINDRICAL && (which == PG_MESH_D1 || which == PG_MESH_D3)) {
    const double dd[3] = {g.d[0], g.d[1], g.d[2]};  // d1 = dx, d3 = dz (mesh.f90:214-216)
    return launch_mesh(which, out, g.n[0], g.n[1], g.n[2], g.x1f, g.d, dd, stream);
  }
  return launch_mesh(which, out, g.n[0], g.n[1], g.n[2], g.x1f, g.d, g.dm, stream);
}

int pg_rk_stage(pg_handle* h, int nvar, double* const* U, double* const* PHI, const double* const* F,
                const double* dt, double A, double B, void* stream) {
  if (!h || nvar < 0 || (nvar > 0 && (!U || !PHI || !F || !dt))) return PG_EINVAL;
  if (nvar == 0) return PG_OK;
  return launch_rk_stage(nvar, U, PHI, F, dt, A, B, h->c.npts, 0, stream);
}

int pg_courant(pg_handle* h, const double* u, const double* v, const double* w, const double* c, double vconst,
               double wconst, double* out, void* stream) {
  if (!h || !u || !c || !out) return PG_EINVAL;
  const GridInfo& g = h->g;
  if (g.coordsys == PG_CYLINDRICAL && g.n[1] > 1) {
    set_error("pg_courant: cylindrical grids with more than one point in angle are not supported");
    return PG_EINVAL;
  }
  if (g.coordsys >= PG_SPHERICAL) {  // the rate on the mesh fields, its maximum, the reciprocal
    MetricArgs A = margs(h, MET_COURANT);
    A.in[0] = u;
    A.in[1] = v;
    A.in[2] = w;
    A.in[3] = c;
    A.s0 = vconst;
    A.s1 = wconst;
    A.out[0] = h->c.cyl[0];
    int rc = launch_metric(A, stream);
    if (!rc) rc = launch_reduce(1, h->c.cyl[0], h->c.npts, h->c.partial, out, stream);
    if (!rc) {
      MetricArgs R = margs(h, MET_RECIP);
      R.n = 1;
      R.out[0] = out;
      rc = launch_metric(R, stream);
    }
    return rc;
  }
  const double gl = std::min(std::min(g.dm[0], g.dm[1]), g.dm[2]);
  return launch_courant(u, v, w, c, vconst, wconst, g.dm, gl, h->c.npts, h->c.partial, out, stream);
}

int pg_diff(pg_handle* h, const double* bulk, const double* rho, double* out, void* stream) {
  if (!h || !bulk || !rho || !out) return PG_EINVAL;
  const GridInfo& g = h->g;
  if (g.coordsys == PG_CYLINDRICAL && g.n[1] > 1) {
    set_error("pg_diff: cylindrical grids with more than one point in angle are not supported");
    return PG_EINVAL;
  }
  if (g.coordsys >= PG_SPHERICAL) {  // the rate on the GridLen field, its minimum
    int rc = metric(h, MET_DIFF, {bulk, rho}, {h->c.cyl[0]}, stream);
    if (!rc) rc = launch_reduce(2, h->c.cyl[0], h->c.npts, h->c.partial, out, stream);
    return rc;
  }
  const double gl = std::min(std::min(g.dm[0], g.dm[1]), g.dm[2]);
  return launch_diff(bulk, rho, gl, h->c.npts, h->c.partial, out, stream);
}

int pg_reduce(pg_handle* h, int op, const double* in, int64_t n, double* out, void* stream) {
  if (!h || !in || !out || op < 0 || op > 2 || n <= 0) return PG_EINVAL;
  return launch_reduce(op, in, n, h->c.partial, out, stream);
}

int pg_check_finite(const double* in, int64_t n, int* flag, void* stream) {
  if (!in || !flag || n < 0) return PG_EINVAL;
  return launch_check_finite(in, n, flag, stream);
}

int pg_d1_host(pg_handle* h, int dir, const double* in, double* out) {
  if (!h) return PG_EINVAL;
  return host_call(h->c, in, out, [&](const double* a, double* b, void* s) { return pg_d1(h, dir, a, b, s); });
}

int pg_d8_host(pg_handle* h, int dir, const double* in, double* out) {
  if (!h) return PG_EINVAL;
  return host_call(h->c, in, out, [&](const double* a, double* b, void* s) { return pg_d8(h, dir, a, b, s); });
}

int pg_d2_host(pg_handle* h, int dir, const double* in, double* out) {
  if (!h) return PG_EINVAL;
  return host_call(h->c, in, out, [&](const double* a, double* b, void* s) { return pg_d2(h, dir, a, b, s); });
}

int pg_d4_host(pg_handle* h, int dir, const double* in, double* out) {
  if (!h) return PG_EINVAL;
  return host_call(h->c, in, out, [&](const double* a, double* b, void* s) { return pg_d4(h, dir, a, b, s); });
}

int pg_laplacian_host(pg_handle* h, const double* in, double* out) {
  if (!h) return PG_EINVAL;
  return host_call(h->c, in, out, [&](const double* a, double* b, void* s) { return pg_laplacian(h, a, b, s); });
}

int pg_filter_host(pg_handle* h, int kind, int dir, const double* in, double* out) {
  if (!h) return PG_EINVAL;
  return host_call(h->c, in, out,
                   [&](const double* a, double* b, void* s) { return pg_filter(h, kind, dir, a, b, s); });
}

int pg_ring_host(pg_handle* h, const double* in, double* out) {
  if (!h) return PG_EINVAL;
  return host_call(h->c, in, out, [&](const double* a, double* b, void* s) { return pg_ring(h, a, b, s); });
}

// ---------------------------------------------------------------------------
// ensembles
// ---------------------------------------------------------------------------
int pg_ens_create(int m, const pg_grid* grids, pg_ensemble** out) {
  if (m < 1 || !grids || !out) {
    set_error("pg_ens_create: bad argument");
    return PG_EINVAL;
  }
  *out = nullptr;
  pg_ensemble* e = new pg_ensemble();
  e->g.resize(m);
  for (int i = 0; i < m; i++) {
    if (grids[i].precision != grids[0].precision ||
        grids[i].precision < PG_FP64 || grids[i].precision > PG_AUTO) {
      delete e;
      set_error("pg_ens_create: members must share one valid precision");
      return PG_EINVAL;
    }
    if (grids[i].coordsys != PG_CARTESIAN) {
      set_error("pg_ens_create: ensembles are Cartesian");
      delete e;
      return PG_EINVAL;
    }
    int rc = grid_info(&grids[i], e->g[i], "pg_ens_create");
    if (rc != PG_OK) {
      delete e;
      return rc;
    }
  }
  int rc = build_ctx(e->c, e->g, PG_FP64, "pg_ens_create");
  if (rc == PG_OK) rc = set_precision(e->c, e->g, grids[0].precision);
  if (rc != PG_OK) {
    free_ctx(e->c);
    delete e;
    return rc;
  }
  *out = e;
  return PG_OK;
}

int pg_ens_destroy(pg_ensemble* e) {
  if (!e) return PG_OK;
  free_ctx(e->c);
  delete e;
  return PG_OK;
}

int64_t pg_ens_points(const pg_ensemble* e, int64_t* offsets) {
  if (!e) return -1;
  if (offsets) {
    int64_t o = 0;
    for (size_t i = 0; i < e->g.size(); i++) {
      offsets[i] = o;
      o += e->g[i].npts;
    }
    offsets[e->g.size()] = o;
  }
  return e->c.npts;
}

int pg_ens_set_line_split(pg_ensemble* e, int mode) {
  if (!e) return PG_EINVAL;
  return set_line_split(e->c, e->g, mode);
}

int pg_ens_set_precision(pg_ensemble* e, int precision) {
  if (!e) return PG_EINVAL;
  return set_precision(e->c, e->g, precision);
}

int pg_ens_spacing(const pg_ensemble* e, int member, double* patch_d, double* mesh_d) {
  if (!e || member < 0 || member >= (int)e->g.size()) return PG_EINVAL;
  for (int d = 0; d < 3; d++) {
    if (patch_d) patch_d[d] = e->g[member].d[d];
    if (mesh_d) mesh_d[d] = e->g[member].dm[d];
  }
  return PG_OK;
}

int pg_ens_d1(pg_ensemble* e, int dir, const double* in, double* out, void* stream) {
  if (!e || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(e->c, OPK_D1, dir, in, out, stream);
}

int pg_ens_d8(pg_ensemble* e, int dir, const double* in, double* out, void* stream) {
  if (!e || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(e->c, OPK_D8, dir, in, out, stream);
}

int pg_ens_d2(pg_ensemble* e, int dir, const double* in, double* out, void* stream) {
  if (!e || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(e->c, OPK_D2, dir, in, out, stream);
}

int pg_ens_d4(pg_ensemble* e, int dir, const double* in, double* out, void* stream) {
  if (!e || !in || !out || bad_dir(dir)) return PG_EINVAL;
  return apply_one(e->c, OPK_D4, dir, in, out, stream);
}

int pg_ens_laplacian(pg_ensemble* e, const double* in, double* out, void* stream) {
  if (!e || !in || !out || in == out) return PG_EINVAL;
  return laplacian(e->c, in, out, stream);
}

int pg_ens_filter(pg_ensemble* e, int kind, int dir, const double* in, double* out, void* stream) {
  if (!e || !in || !out || (kind != PG_SPECTRAL && kind != PG_GAUSSIAN) || dir < 0 || dir > 3) return PG_EINVAL;
  const int k = kind == PG_SPECTRAL ? OPK_SF : OPK_GF;
  if (dir < 3) return apply_one(e->c, k, dir, in, out, stream);
  return filter_all(e->c, k, in, out, stream);
}

int pg_ens_ring(pg_ensemble* e, const double* in, double* out, void* stream) {
  if (!e || !in || !out || in == out) return PG_EINVAL;
  return ring(e->c, in, out, stream);
}

int pg_ens_ringv(pg_ensemble* e, const double* vx, const double* vy, const double* vz, double* out, void* stream) {
  if (!e || !vx || !vy || !vz || !out || out == vx || out == vy || out == vz) return PG_EINVAL;
  return ringv(e->c, vx, vy, vz, out, stream);
}

int pg_ens_grad(pg_ensemble* e, const double* in, double* gx, double* gy, double* gz, void* stream) {
  if (!e || !in || !gx || !gy || !gz) return PG_EINVAL;
  return grad(e->c, in, gx, gy, gz, stream);
}

int pg_ens_div(pg_ensemble* e, const double* fx, const double* fy, const double* fz, double* out, void* stream) {
  if (!e || !fx || !fy || !fz || !out || out == fy || out == fz) return PG_EINVAL;
  return divergence(e->c, fx, fy, fz, out, stream);
}

int pg_ens_mesh(pg_ensemble* e, int which, double* out, void* stream) {
  if (!e || !out || which < 0 || which > 7) return PG_EINVAL;
  int64_t o = 0;
  for (const GridInfo& g : e->g) {
    int rc = launch_mesh(which, out + o, g.n[0], g.n[1], g.n[2], g.x1f, g.d, g.dm, stream);
    if (rc) return rc;
    o += g.npts;
  }
  return PG_OK;
}

int pg_ens_rk_stage(pg_ensemble* e, int nvar, double* const* U, double* const* PHI, const double* const* F,
                    const double* dt_field, double A, double B, void* stream) {
  if (!e || nvar < 0 || (nvar > 0 && (!U || !PHI || !F || !dt_field))) return PG_EINVAL;
  if (nvar == 0) return PG_OK;
  return launch_rk_stage(nvar, U, PHI, F, dt_field, A, B, e->c.npts, 1, stream);
}

int pg_ens_courant(pg_ensemble* e, const double* u, const double* v, const double* w, const double* c,
                   double vconst, double wconst, double* out_field, void* stream) {
  if (!e || !u || !c || !out_field) return PG_EINVAL;
  return launch_seg_courant(u, v, w, c, vconst, wconst, e->c.mconst, e->c.moff, e->c.nmem, e->c.npts,
                            e->c.partial, out_field, stream);
}

int pg_ens_diff(pg_ensemble* e, const double* bulk, const double* rho, double* out_field, void* stream) {
  if (!e || !bulk || !rho || !out_field) return PG_EINVAL;
  return launch_seg_diff(bulk, rho, e->c.mconst, e->c.moff, e->c.nmem, e->c.npts, e->c.partial, out_field, stream);
}

int pg_ens_reduce(pg_ensemble* e, int op, const double* in, double* out_field, double* out_member, void* stream) {
  if (!e || !in || (!out_field && !out_member) || op < 0 || op > 2) return PG_EINVAL;
  return launch_seg_reduce(op, in, e->c.moff, e->c.nmem, e->c.npts, e->c.partial, out_field, out_member, stream);
}

// ------------------------------------------------------------ learned LAD
namespace {
LadGrid lad_grid(const GridInfo& g) {
  LadGrid lg;
  for (int d = 0; d < 3; d++) {
    lg.n[d] = g.n[d];
    lg.per[d] = g.periodic[d];
  }
  lg.delta = std::max(std::max(g.dm[0], g.dm[1]), g.dm[2]);  // the largest mesh spacing
  for (int d = 0; d < 3; d++) lg.rd[d] = (float)(1.0 / g.d[d]);
  return lg;
}
}  // namespace

int pg_lad_closure(pg_handle* h, const pg_lad_model* m, const double* div, const double* gmag, const double* rho,
                   const double* dt, double cv, double* beta, double* kappa, int* flag, void* stream) {
  if (!h || !m || !m->wbf16 || !m->params || !m->xmean || !m->xinvstd || !div || !gmag || !rho || !dt || !beta ||
      !kappa || !flag)
    return PG_EINVAL;
  if (((uintptr_t)m->wbf16 & 15u) != 0) {  // the kernel stages the weights in 16-byte chunks
    set_error("pg_lad_closure: the BF16 weights must be 16-byte aligned");
    return PG_EINVAL;
  }
  LadInferArgs a{*m, lad_grid(h->g), div, gmag, rho, dt, cv, beta, kappa, flag, h->c.status};
  return launch_lad_infer(a, stream);
}

int pg_lad_grad_magnitude(pg_handle* h, const double* rho, double* out, void* stream) {
  if (!h || !rho || !out) return PG_EINVAL;
  if (rho == out) {
    set_error("pg_lad_grad_magnitude: in and out must differ");
    return PG_EINVAL;
  }
  return launch_lad_grad_magnitude(rho, lad_grid(h->g), out, stream);
}

int pg_lad_features(pg_handle* h, const double* div, const double* gmag, const int64_t* pts, int64_t ns,
                    float* raw, void* stream) {
  if (!h || !div || !gmag || !pts || !raw || ns < 0) return PG_EINVAL;
  if (ns == 0) return PG_OK;
  return launch_lad_features(div, gmag, lad_grid(h->g), pts, ns, raw, stream);
}

int pg_lad_normalize(const float* raw, int64_t ns, const float* xmean, const float* xinvstd, void* X,
                     void* stream) {
  if (!raw || !xmean || !xinvstd || !X || ns < 0) return PG_EINVAL;
  if (ns == 0) return PG_OK;
  return launch_lad_normalize(raw, ns, xmean, xinvstd, X, stream);
}

int pg_lad_train_step(const pg_lad_model* m, const void* X, const float* T, int64_t rows, float inv_count,
                      float* grad, float* loss, float* Y, void* stream) {
  if (!m || !m->wbf16 || !m->params || !X || !T || !grad || rows < 0) return PG_EINVAL;
  LadTrainArgs a{*m, X, T, rows, inv_count, grad, loss, Y};
  return launch_lad_train(a, stream);
}

int pg_lad_adam(float* params, float* m, float* v, const float* grad, int n, float lr, float beta1, float beta2,
                float eps, int step, void* pbf, int nbf, void* stream) {
  if (!params || !m || !v || !grad || n <= 0 || step < 1 || nbf < 0 || nbf > n || (nbf > 0 && !pbf))
    return PG_EINVAL;
  return launch_lad_adam(params, m, v, grad, n, lr, beta1, beta2, eps, step, pbf, nbf, stream);
}

int pg_ens_device_status(pg_ensemble* e, int* status) {
  if (!e || !status) return PG_EINVAL;
  return read_status(e->c, status);
}

}  // extern "C"
