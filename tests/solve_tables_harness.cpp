// Host harness of the solve tables (compiled by tests/test_solve_tables_cpu.py
// together with pyranda_gb300/csrc/pg_setup.cpp): for one operator it applies
// the banded / Schur-complement tables (OpTables::lu, the layout documented in
// pg_setup.cpp) and the split-line tables (build_split) to a random right-hand
// side the way the sweeps do, in FP64, and returns each result's residual
// ||A x - r|| / ||r|| against the assembled LHS band.
#include <cmath>
#include <random>
#include <vector>

#include "../pyranda_gb300/csrc/pg_internal.h"

using pg::OpTables;

namespace {

double residual(const std::vector<double>& band, int n, bool per, const std::vector<double>& x,
                const std::vector<double>& r) {
  double num = 0.0, den = 0.0;
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int l = 0; l < 5; l++) {
      int c = i + l - 2;
      if (per) c = ((c % n) + n) % n;
      else if (c < 0 || c >= n) continue;
      s += band[(size_t)i * 5 + l] * x[c];
    }
    num += (s - r[i]) * (s - r[i]);
    den += r[i] * r[i];
  }
  return std::sqrt(num / den);
}

}  // namespace

extern "C" int pg_test_solve_residual(int kind, int n, int per, int bl, int bh, int sym, int seed,
                                      double* res_banded, double* res_split) {
  OpTables t;
  int rc = pg::build_operator(kind, n, per != 0, 1.0, t, bl, bh, sym);
  if (rc) return rc;
  if (!t.implicit) return -1;
  std::mt19937 gen((unsigned)seed);
  std::normal_distribution<double> nd;
  std::vector<double> r(n), x(n, 0.0), z(n, 0.0);
  for (auto& v : r) v = nd(gen);
  const double* L = t.lu.data();
  auto row = [&](int i, int k) { return L[(size_t)i * 12 + k]; };
  // banded / Schur-complement tables: [rho alpha beta G0 | u1 u2 F0 F1 | G1 ...]
  const int m = per ? n - 2 : n;
  double t0 = 0.0, t1 = 0.0;
  for (int i = 0; i < m; i++) {
    double v = row(i, 0) * r[i];
    if (i >= 1) v -= row(i, 1) * z[i - 1];
    if (i >= 2) v -= row(i, 2) * z[i - 2];
    z[i] = v;
    t0 += row(i, 3) * v;
    t1 += row(i, 8) * v;
  }
  double xb0 = 0.0, xb1 = 0.0;
  if (per) {  // x_B = S^-1 (r_B - G z_I), S^-1 in row n - 2
    const double b0 = r[n - 2] - t0, b1 = r[n - 1] - t1;
    xb0 = row(n - 2, 0) * b0 + row(n - 2, 1) * b1;
    xb1 = row(n - 2, 2) * b0 + row(n - 2, 3) * b1;
    x[n - 2] = xb0;
    x[n - 1] = xb1;
  }
  for (int i = m - 1; i >= 0; i--) {
    double v = z[i];
    if (i + 1 < m) v -= row(i, 4) * x[i + 1];
    if (i + 2 < m) v -= row(i, 5) * x[i + 2];
    if (per) v -= row(i, 6) * xb0 + row(i, 7) * xb1;
    x[i] = v;
  }
  *res_banded = residual(t.lhs, n, per != 0, x, r);
  // split-line tables: segment blocks, tips, the reduced system's inverse rows
  std::vector<int> start;
  std::vector<double> srow, G;
  rc = pg::build_split(t.lhs, n, per != 0, start, srow, G);
  if (rc) return rc;
  const int S = (int)start.size() - 1, T = 4 * S;
  std::vector<double> y(n), tips(T), xs(n);
  for (int j = 0; j < S; j++) {
    const int a = start[j], b = start[j + 1];
    double z1 = 0.0, z2 = 0.0;
    for (int i = a; i < b; i++) {
      const double* f = &srow[(size_t)i * 12];
      double v = f[0] * r[i] - f[2] * z2 - f[1] * z1;
      z2 = z1;
      z1 = v;
      y[i] = v;
    }
    double y1 = 0.0, y2 = 0.0;
    for (int i = b - 1; i >= a; i--) {
      const double* f = &srow[(size_t)i * 12 + 4];
      double v = y[i] - f[1] * y2 - f[0] * y1;
      y[i] = v;
      y2 = y1;
      y1 = v;
    }
    tips[4 * j] = y[a];
    tips[4 * j + 1] = y[a + 1];
    tips[4 * j + 2] = y[b - 2];
    tips[4 * j + 3] = y[b - 1];
  }
  for (int j = 0; j < S; j++) {
    double q[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = 0; c < 4; c++)
      for (int idx = 0; idx < T; idx++) q[c] += G[(size_t)j * 16 * S + (size_t)c * T + idx] * tips[idx];
    for (int i = start[j]; i < start[j + 1]; i++) {
      const double* sp = &srow[(size_t)i * 12 + 8];
      xs[i] = y[i] - sp[0] * q[0] - sp[1] * q[1] - sp[2] * q[2] - sp[3] * q[3];
    }
  }
  *res_split = residual(t.lhs, n, per != 0, xs, r);
  return 0;
}
