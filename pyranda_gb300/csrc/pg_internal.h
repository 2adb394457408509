// Internal declarations shared by the host assembly, the kernels and the C ABI.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/pyranda_gpu.h"

namespace pg {

enum { OPK_D1 = 0, OPK_D8 = 1, OPK_SF = 2, OPK_GF = 3, OPK_COUNT = 4 };

// Host-side tables of one operator along one direction (built by pg_setup.cpp).
struct OpTables {
  int kind = 0, n = 0;
  bool periodic = false, implicit = false, addback = false, null_op = true;
  std::vector<double> rhs;  // n x 9 per-row RHS weights
  std::vector<double> lu;   // n x 9 per-row solve coefficients
};

int build_operator(int kind, int n, bool periodic, double scale, OpTables& t);

// Epilogues fused into the store of a sweep.
enum {
  EPI_STORE = 0,     // out = r
  EPI_ADD = 1,       // out = out + r            (divergence accumulation)
  EPI_RING_SET = 2,  // out = |r| * s            (first direction of a ring)
  EPI_RING_MAX = 3,  // out = max(out, |r| * s)  (later directions / components)
  EPI_COUNT = 4
};

// One operator of one grid along one direction, as the sweep kernels read it
// (device memory).  A single grid has one entry per (precision, kind,
// direction); an ensemble of grids has one per member, and one launch sweeps
// the lines of every member.
struct MemberOp {
  const void* rhs;  // n x 9 per-row RHS weights (T)
  const void* lu;   // n x 12 per-row solve coefficients (T)
  int n;            // points per line
  int nx, ny;       // grid extents (to decode a line index)
  int pad;
  long long lines;  // lines of this grid along the direction
  long long line0;  // first global line of this grid (prefix over members)
  long long off;    // first point of this grid in the flat field
  double ri[9];     // interior RHS weights
  double dm;        // mesh spacing along the direction (ring scale)
};

// Host view of one (kind, direction, precision) operator of a grid or ensemble.
struct OpRef {
  const MemberOp* dev = nullptr;  // nops entries in device memory
  int nops = 0;
  long long nlines = 0;           // total lines over all members
  int kind = 0;
  bool periodic = false, implicit = false, addback = false, null_op = true;
};

struct SweepLaunch {
  const double* in;
  double* out;
  void* scratch;   // one field of forward-elimination values (workspace)
  const OpRef* op;
  int dir;
  int epi;         // EPI_*
  int scale_pow;   // ring epilogues scale |r| by dm^scale_pow
};

// Launches one directional sweep over every member.  Returns a pg_status.
int launch_sweep(int precision, const SweepLaunch& s, void* stream);
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
int launch_mesh(int which, double* out, int nx, int ny, int nz, const double x1f[3],
                const double d[3], const double dm[3], void* stream);

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

void set_error(const char* fmt, ...);
void count_launch(uint64_t k = 1);

}  // namespace pg
