// Internal declarations shared by the host assembly, the kernels and the C ABI.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/pyranda_gpu.h"

namespace pg {

// d1 (c10d1), d8 (c10d8), compact filter (c8ff8), Gaussian filter (cgfs4),
// d2 (c10d2, compact) and d4 (e4d4, explicit)
enum { OPK_D1 = 0, OPK_D8 = 1, OPK_SF = 2, OPK_GF = 3, OPK_D2 = 4, OPK_D4 = 5, OPK_COUNT = 6 };

// Host-side tables of one operator along one direction (built by pg_setup.cpp).
struct OpTables {
  int kind = 0, n = 0;
  bool periodic = false, implicit = false, addback = false, null_op = true;
  std::vector<double> rhs;  // n x 9 per-row RHS weights
  std::vector<double> lu;   // n x 12 per-row solve coefficients (pg_setup.cpp solve_tables)
  std::vector<double> lhs;  // n x 5 LHS band (a, b, diag, c, d) before factorisation
  int bcl = 0, bch = 0;     // boundary code of each end's rows: 0 one-sided, +1/-1 symmetry plane, 2 extended
};

// bc_lo / bc_hi: 0 one-sided (NONE), 1 symmetry plane (SYMM), 2 extended data (XTND);
// sym = +1 the operator for symmetric fields, -1 for antisymmetric ones.
int build_operator(int kind, int n, bool periodic, double scale, OpTables& t, int bc_lo = 0, int bc_hi = 0,
                   int sym = 1);

// Split-line (reduced-system) solve tables of one line's LHS band (n x 5):
// segment starts (S + 1), per-position rows (n x 12) and the per-segment rows
// of the reduced system's inverse (S x 4 x 4S).  pg_setup.cpp.
constexpr int kSplitSeg = 32;  // points per segment (the last takes the remainder)
int build_split(const std::vector<double>& band, int n, bool periodic, std::vector<int>& start,
                std::vector<double>& row, std::vector<double>& G);

// Epilogues fused into the store of a sweep.
enum {
  EPI_STORE = 0,     // out = r
  EPI_ADD = 1,       // out = out + r            (divergence accumulation)
  EPI_RING_SET = 2,  // out = |r| * s            (first direction of a ring)
  EPI_RING_MAX = 3,  // out = max(out, |r| * s)  (later directions / components)
  EPI_COUNT = 4
};
// Epilogues each operator is called with; the sweep kernels instantiate only
// these: d1 and d2 store or accumulate, d8 stores or keeps the ring's running
// max, d4 and the filters store.
constexpr unsigned kEpiStoreAdd = (1u << EPI_STORE) | (1u << EPI_ADD);
constexpr unsigned kEpiStore = (1u << EPI_STORE);
constexpr unsigned kEpiRing = (1u << EPI_STORE) | (1u << EPI_RING_SET) | (1u << EPI_RING_MAX);


// One operator of one grid along one direction, as the sweep kernels read it
// (device memory).  A single grid has one entry per (precision, kind,
// direction); an ensemble of grids has one per member, and one launch sweeps
// the lines of every member.
struct MemberOp {
  const void* rhs;  // n x 9 per-row RHS weights (T)
  const void* lu;   // n x 12 per-row solve coefficients (T), layout of pg_setup.cpp solve_tables
  int n;            // points per line
  int nx, ny;       // grid extents (to decode a line index)
  int bcl;          // boundary code of the lower end's rows (0, +1, -1, 2; OpTables::bcl)
  long long lines;  // lines of this grid along the direction
  long long line0;  // first global line of this grid (prefix over members)
  long long off;    // first point of this grid in the flat field
  double ri[9];     // interior RHS weights
  double dm;        // mesh spacing along the direction (ring scale)
  // d8 with integer weights (RHS weight = wscale x integer): the FP32 sweeps
  // evaluate its RHS exactly in 64-bit fixed point (the 8th difference
  // cancels ~40 bits of a smooth field)
  const int* rhs_i; // n x 9 per-row integer RHS weights
  int iw[9];        // interior integer weights
  int exact;        // 1: rhs_i / iw / wscale are valid
  float wscale;
  int bch;          // boundary code of the upper end's rows
};

// Host view of one (kind, direction, precision) operator of a grid or ensemble.
struct OpRef {
  const MemberOp* dev = nullptr;  // nops entries in device memory
  int nops = 0;
  long long nlines = 0;           // total lines over all members
  int kind = 0;
  bool periodic = false, implicit = false, addback = false, null_op = true;
  bool exact = false;             // every member's MemberOp::exact
};

struct SweepLaunch {
  const double* in;
  double* out;
  void* scratch;   // one field of forward-elimination values (workspace)
  const OpRef* op;
  int dir;
  int epi;         // EPI_*
  int scale_pow;   // ring epilogues scale |r| by dm^scale_pow
  // exact d8 RHS (FP32 sweeps): per member the largest binary exponent of `in`
  int* emax = nullptr;              // nops ints
  const long long* moff = nullptr;  // member point offsets (nops + 1)
  bool emax_ready = false;          // emax already holds the exponents of `in`
};

// Launches one directional sweep over every member.  Returns a pg_status.
int launch_sweep(int precision, const SweepLaunch& s, void* stream);
// The exact fixed-point RHS of the d8 sweeps (FP32 path) of every point along
// `dir`, rounded once to FP32 and stored as FP64 in `rhs`; emax holds the
// members' exponents (launch_max_exponent); nmax = the longest member line.
int launch_d8_rhs(const OpRef& op, const double* in, double* rhs, int dir, const int* emax, int nmax,
                  void* stream);

// Split-line sweeps (pg_split.cu): one member's tables along one direction
// (device memory; built by pg_setup.cpp build_split).
struct SplitOp {
  const void* row;   // n x 12 per-position coefficients (T)
  const void* G;     // S x 4 x 4S rows of the reduced system's inverse (T)
  const int* start;  // S + 1 segment starts
  const int* win;    // per segment: first segment of its reduced-solve window, segments in the window
  int S;
  int pad;
};
// One CTA's lines: [line0, line0 + nlines) of member op, nlines * S <= 256.
struct SplitTile {
  int op;
  int line0;
  int nlines;
  int pad;
};
struct SplitSet {
  const SplitOp* sops = nullptr;  // per member (this precision's tables)
  const SplitTile* tiles = nullptr;
  int ntiles = 0;
  bool ok = false;
  size_t smem32 = 0, smem64 = 0, smem_mixed = 0;  // dynamic shared memory of the FP32 / FP64 / exact-d8 kernels
  // every member's lines a multiple of kSplitSeg points: the FP32 sweeps take the
  // register-resident form (seg_kernel), with this shared memory along x and along y / z
  bool seg32 = false;
  size_t smem_seg_x = 0, smem_seg_yz = 0;
};
// Shared memory of one split tile (precision PG_FP32 / PG_FP64; exact: FP32 d8 with the raw FP64 values).
size_t split_smem_bytes(int precision, bool exact, int n, int S, int nl);
size_t seg_smem(int dir, int n, int S, int nl);
int launch_split(int precision, const OpRef& op, const SplitSet& ss, const double* in, double* out, int dir, int epi,
                 int scale_pow, const int* emax, void* stream);

// Dense operator of one member along one direction (device memory): the
// difference form D' of D (OUT = D' w, w_k = v_k - v_{k-1}) split into TF32
// hi/lo planes laid out as [kchunk][hi, lo][rows][32] words, each 8-row
// group 128B-swizzled (the shared-memory layout the MMA reads).
struct DenseOp {
  const uint32_t* dsw;
  long long off;    // first point of the member in the flat field
  int n;            // points per line
  int nx, ny;       // member extents (to decode a line index)
  int kchunks;      // ceil(n / 32)
  int rows;         // rows of each plane: n padded to a multiple of 128
  int periodic;     // 1: w_0 = v_0 - v_{n-1} (the wrap difference)
  int direct;       // 1: the planes hold D itself, applied to v (no differences)
  double dm;        // mesh spacing along the direction (ring scale)
};
// One CTA's output tile: lines [line0, line0 + nlines) of member `op`
// (at most 128); part = which 256 positions of the lines.
struct DenseTile {
  int op;
  int line0;
  int nlines;
  int part;
};
// Host view of the dense form of one (kind, direction) operator.
struct DenseSet {
  const DenseOp* ops = nullptr;
  const DenseTile* tiles = nullptr;
  int ntiles = 0;
  bool ok = false;       // dense form built (every member has 16 <= n <= 1024)
  bool addback = false;  // filters: out = v + D v with D = A^-1 (B - A)
  bool direct = false;   // d8: D = A^-1 applied to the exact fixed-point RHS (launch_d8_rhs)
};
// Split a row-major n x n FP64 matrix into the DenseOp plane layout.
void split_dense(const std::vector<double>& D, int n, std::vector<uint32_t>& out, int& rows, int& kchunks);
// A bounded wait that is never satisfied: records PG_ETIMEOUT after limit_ms.
int launch_wait_selftest(int* status, unsigned limit_ms, void* stream);
// One dense sweep (tcgen05 split-TF32 GEMM) with a fused epilogue.
int launch_dense(const DenseSet& ds, const double* in, double* out, int dir, int epi, int scale_pow, int* status,
                 void* stream);
int launch_fill(double* out, double value, int64_t n, void* stream);
int launch_copy(double* out, const double* in, int64_t n, void* stream);
// dt_is_field = 0: dt is one device scalar; 1: dt is a field (one value per point)
int launch_rk_stage(int nvar, double* const* U, double* const* PHI, const double* const* F,
                    const double* dt, double A, double B, int64_t n, int dt_is_field, void* stream);
int launch_courant(const double* u, const double* v, const double* w, const double* c,
                   double vconst, double wconst, const double d[3], double gridlen, int64_t n,
                   double* partial, double* out, void* stream);
int launch_diff(const double* bulk, const double* rho, double gl2, int64_t n, double* partial,
                double* out, void* stream);
int launch_reduce(int op, const double* in, int64_t n, double* partial, double* out, void* stream);
int launch_check_finite(const double* in, int64_t n, int* flag, void* stream);
// Per member m, the largest biased binary exponent of in[moff[m] .. moff[m+1]) (0 for an all-zero member).
int launch_max_exponent(const double* in, const long long* moff, int nmem, int* emax, void* stream);
int launch_mesh(int which, double* out, int nx, int ny, int nz, const double x1f[3],
                const double d[3], const double dm[3], void* stream);
// Cylindrical pointwise forms (r = the radius of the point's x index):
enum {
  CYL_MUL_R = 0,        // out = r a
  CYL_MUL_R2 = 1,       // out = r^2 a
  CYL_DIV_R = 2,        // out = a / r
  CYL_DIVV = 3,         // out = (a + b) / r + c
  CYL_DIVT_X = 4,       // out = (a + b - e) / r + c
  CYL_DIVT_Y = 5,       // out = a / r^2 + (b + e - f) / r + c
  CYL_CELLVOL_MUL = 6,  // out = a CellVol
  CYL_CELLVOL_DIV = 7,  // out = a / CellVol
  CYL_CELLVOL = 8,      // out = CellVol
  CYL_D2 = 9,           // out = r dy
  CYL_GRIDLEN = 10      // out = GridLen
};
int launch_cyl(int op, int64_t n, int nx, int ny, double x1, double dx, double dy, double dz, const double* a,
               const double* b, const double* c, const double* e, const double* f, double* out, void* stream);

// Mesh fields of spherical and curvilinear grids (mesh.f90:35-50), in this
// order in the handle: native coordinates, d1 d2 d3, GridLen, CellVol, the
// filtered cell volumes, det J and the inverse Jacobian rows dA/dx dA/dy dA/dz,
// dB/.., dC/.. (curvilinear grids only; they hold d(x,y,z)/d(A,B,C) until the
// metric form inverts them).  The indices equal pg_mesh_var's.
enum { MF_X, MF_Y, MF_Z, MF_D1, MF_D2, MF_D3, MF_GL, MF_CV, MF_CVS, MF_CVG, MF_DET, MF_J0, MF_COUNT = MF_J0 + 9 };

// Pointwise forms of the non-Cartesian grids (pg_metric.cu).
enum {
  MET_SPH_MESH,       // spherical mesh fields from the point indices (s0 = Asp, s1 = Csp when ratio-zoned)
  MET_NODES,          // node coordinates x1 + i (xn - x1) / (n - 1) into the coordinate fields
  MET_CURV_METRIC,    // J slots -> inverse Jacobian, det J, d1 d2 d3, CellVol, GridLen
  MET_SPH_GRAD,       // out[0..2] in place: (dx / d1) gx, gy / r, gz / (r sin(theta))
  MET_CURV_GRAD,      // out[0..2] in place: (d/dA, d/dB, d/dC) -> (d/dx, d/dy, d/dz)
  MET_SPH_DIV_PRE,    // out0 = r^2 in0, out1 = in1 sin(theta)
  MET_SPH_DIV_POST,   // out0 = (in0 dx / d1) / r^2 + (in1 + in2) / (r sin(theta))
  MET_CURV_DIV_PRE,   // out[r] = (in . grad of coordinate r) det J
  MET_CURV_DIV_POST,  // out0 = (in0 + in1 + in2) / det J
  MET_SPH_T_PRE,      // L = 2: out0 = r^2 in0, out1 = in1 / (1 / sin(theta)); L = 3: r^3 in0, in1 sin(theta)
  MET_SPH_T_POST,     // spherical divT row L (0, 1, 2) from fA fB fC and three tensor components
  MET_LAP_MUL,        // out0 = r^L in0
  MET_LAP_X,          // out0 = in0 / r^L
  MET_LAP_SIN,        // out0 = sin(theta) in0
  MET_LAP_ADD_Y,      // out0 += in0 / r^2 (cylindrical) or in0 / (r^2 sin(theta)) (spherical)
  MET_LAP_ADD_Z,      // out0 += in0 (cylindrical) or in0 / (r sin(theta))^2 (spherical)
  MET_VOL_MUL,        // out0 = in0 CellVol
  MET_VOL_DIV,        // out0 = in0 / in1
  MET_RING,           // out0 = (first ? : max(out0, )) |in0| d_dir^L
  MET_COURANT,        // out0 = the courant rate (in0..2 velocity, NULL = s0 / s1; in3 sound speed)
  MET_DIFF,           // out0 = in1 GridLen^2 / max(1e-12, in0)
  MET_RECIP,          // out0 = 1 / out0
  MET_COUNT
};
struct MetricArgs {
  int op = 0;
  int64_t n = 0;
  int nx = 1, ny = 1, nz = 1;
  int coordsys = 0;
  int dir = 0, L = 0, first = 0;
  double x1f[3] = {0, 0, 0}, d[3] = {0, 0, 0};  // face coordinates and patch spacings
  double x1[3] = {0, 0, 0}, xn[3] = {0, 0, 0};  // node extents
  double s0 = 0.0, s1 = 0.0;
  const double* in[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  double* out[3] = {nullptr, nullptr, nullptr};
  double* mf[MF_COUNT] = {};
};
int launch_metric(const MetricArgs& A, void* stream);

// Number of blocks used by the two-pass reductions (partial buffer length).
constexpr int kReduceBlocks = 1024;
// Reduction blocks per member of an ensemble.
constexpr int kSegBlocks = 32;

// Ensemble reductions: one value per member, written per member to
// out_member (if not NULL) and broadcast to every point of the member in
// out_field (if not NULL).  moff holds the nmem+1 point offsets; mconst the
// per-member 1/d1 1/d2 1/d3 1/GridLen GridLen; partial at least
// nmem*kSegBlocks + 2*nmem doubles.
int launch_seg_reduce(int op, const double* in, const long long* moff, int nmem, int64_t npts, double* partial,
                      double* out_field, double* out_member, void* stream);
int launch_seg_courant(const double* u, const double* v, const double* w, const double* c, double vconst,
                       double wconst, const double* mconst, const long long* moff, int nmem, int64_t npts,
                       double* partial, double* out_field, void* stream);
int launch_seg_diff(const double* bulk, const double* rho, const double* mconst, const long long* moff, int nmem,
                    int64_t npts, double* partial, double* out_field, void* stream);

// Learned LAD closure (pg_lad.cu).
struct LadGrid {
  int n[3];
  int per[3];
  double delta;  // largest mesh spacing
  float rd[3];   // 1 / mesh spacing per direction (FP32)
};
struct LadInferArgs {
  pg_lad_model model;
  LadGrid grid;
  const double *div, *gmag, *rho, *dt;
  double cv;
  double *beta, *kappa;
  int* flag;
  int* status;  // device status word (PG_ETIMEOUT when a tensor-core wait runs out)
};
struct LadTrainArgs {
  pg_lad_model model;
  const void* X;     // BF16 [rows][PG_LAD_K]
  const float* T;    // [rows][PG_LAD_OUT]
  long long rows;
  float inv_count;
  float* grad;       // parameter layout
  float* loss;
  float* Y;
};
int launch_lad_infer(const LadInferArgs& a, void* stream);
int launch_lad_features(const double* div, const double* gmag, const LadGrid& g, const int64_t* pts, int64_t ns,
                        float* raw, void* stream);
int launch_lad_grad_magnitude(const double* rho, const LadGrid& g, double* out, void* stream);
int launch_lad_normalize(const float* raw, int64_t ns, const float* xm, const float* xs, void* X, void* stream);
int launch_lad_train(const LadTrainArgs& a, void* stream);
int launch_lad_adam(float* p, float* m, float* v, const float* g, int n, float lr, float b1, float b2, float eps,
                    int step, void* pbf, int nbf, void* stream);

void set_error(const char* fmt, ...);
void count_launch(uint64_t k = 1);

}  // namespace pg
