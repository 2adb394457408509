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

// Device-resident operator (one kind, one direction, one precision).
struct DevOp {
  int kind = 0, n = 0;
  bool periodic = false, implicit = false, addback = false, null_op = true;
  const void* rhs = nullptr;  // n x 9 (double or float)
  const void* lu = nullptr;   // n x 9 (double or float)
  double rhs_in[9] = {0};     // interior RHS weights (kernel parameters)
};

struct SweepLaunch {
  const double* in;
  double* out;
  int nx, ny, nz;
  int dir;
  double epi_scale;  // ring scale
  int epi;           // EPI_*
  int* status;       // device status word of the handle
  void* scratch;     // one field of forward-elimination values (handle workspace)
};

// Launches one directional sweep.  Returns a pg_status.
int launch_sweep(const DevOp& op, int precision, const SweepLaunch& s, void* stream);
int launch_fill(double* out, double value, int64_t n, void* stream);
int launch_copy(double* out, const double* in, int64_t n, void* stream);
int launch_rk_stage(int nvar, double* const* U, double* const* PHI, const double* const* F,
                    const double* dt, double A, double B, int64_t n, void* stream);
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

void set_error(const char* fmt, ...);
void count_launch(uint64_t k = 1);

}  // namespace pg
