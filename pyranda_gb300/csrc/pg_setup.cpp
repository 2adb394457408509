// Host-side operator assembly for the GB300 compact-operator library.
//
// Builds, once per grid and direction, the per-row coefficient tables that the
// sweep kernels read:
//   - the weight tables of pyranda/parcop/stencils.f90 (c10d1 :207-277,
//     c10d2 :358-428, e4d4 :430-513, c10d8 :515-621, c8ff8 :713-835,
//     cgfs4 :1387-1476), boundary code 0 (one-sided closures) and periodic;
//   - the global LHS/RHS assembly of compact_basetype.f90:124-148 (np = 1);
//   - the solve tables of the sweeps: a Crout band factorisation, and for
//     periodic lines a Schur-complement (Sherman-Morrison-Woodbury) treatment
//     of the wrap (the reference factors the same matrices with its own
//     bordered LU, pentadiagonal.f90:18-135; any stable factorisation gives
//     the same operator to rounding).
#include "pg_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace pg {

namespace {

// One stencil family.  Rows are 0-based (row j = Fortran boundary point j+1);
// lhs[] has `ncl` entries, rhs[] has `ncr` entries.
struct Stencil {
  int ncl, ncr, nbc;
  bool implicit, addback;  // addback = null_option 1 (filters)
  double lhs[5], rhs[9];
  double lhs_lo[4][5], rhs_lo[4][9];  // one-sided rows (boundary code 0)
  double lhs_hi[4][5], rhs_hi[4][9];
  // rows for extended boundary data (boundary code 2, XTND), where the reference defines them
  bool has_xt;
  double xt_lhs_lo[4][5], xt_rhs_lo[4][9];
  double xt_lhs_hi[4][5], xt_rhs_hi[4][9];
  // signs of the symmetric variant's folds (LHS, RHS): a first derivative of a
  // symmetric field is antisymmetric, so its LHS folds with the opposite sign
  double fold_lhs, fold_rhs;
  bool diff_form;  // filters store RHS - LHS (stencils.f90:832-834, :1472-1475)
};

// Upper boundary rows mirror the lower ones: row j of the upper block is the
// reversed row (nbc-1-j) of the lower block (stencils.f90, e.g. :241-244).
void mirror(Stencil& s, double rhs_sign) {
  for (int j = 0; j < s.nbc; j++) {
    for (int l = 0; l < s.ncl; l++) s.lhs_hi[j][l] = s.lhs_lo[s.nbc - 1 - j][s.ncl - 1 - l];
    for (int l = 0; l < s.ncr; l++) s.rhs_hi[j][l] = rhs_sign * s.rhs_lo[s.nbc - 1 - j][s.ncr - 1 - l];
    for (int l = 0; l < s.ncl; l++) s.xt_lhs_hi[j][l] = s.xt_lhs_lo[s.nbc - 1 - j][s.ncl - 1 - l];
    for (int l = 0; l < s.ncr; l++) s.xt_rhs_hi[j][l] = rhs_sign * s.xt_rhs_lo[s.nbc - 1 - j][s.ncr - 1 - l];
  }
}

// Extended-data rows from tables (upper rows mirrored by `mirror`).
void set_xt(Stencil& s, const double (*L)[5], const double (*R)[9]) {
  s.has_xt = true;
  for (int j = 0; j < s.nbc; j++) {
    for (int l = 0; l < s.ncl; l++) s.xt_lhs_lo[j][l] = L ? L[j][l] : s.lhs[l];
    for (int l = 0; l < s.ncr; l++) s.xt_rhs_lo[j][l] = R ? R[j][l] : s.rhs[l];
  }
}

// Difference form used by the filters: the stored RHS is RHS - LHS on the
// overlapping entries (stencils.f90:832-834 and :1472-1475).
void to_difference_form(const Stencil& s, const double* lhs, double* rhs) {
  const int off = (s.ncr - s.ncl) / 2;
  for (int l = 0; l < s.ncl; l++) rhs[off + l] -= lhs[l];
}

// Rows of a symmetry plane (boundary code +-1): the interior stencil with the
// entries that fall on points beyond the end moved onto their mirror images.
// The plane lies half a spacing outside the end point (pyranda's grid points
// are cell centres), so the point p = -1 - q beyond the lower end mirrors
// point q; sign = +1 folds a symmetric field, -1 an antisymmetric one.
// Row j is the j-th point from the end; `upper` mirrors about the upper end.
void fold_row(const double* interior, int width, int j, bool upper, double sign, double* row) {
  const int c = width / 2;
  for (int l = 0; l < width; l++) row[l] = interior[l];
  for (int l = 0; l < width; l++) {
    const int off = l - c;                 // offset of entry l from the row's point
    const int beyond = upper ? off - j : -(j + off);  // > 0: this many points past the end
    if (beyond <= 0) continue;
    const int mirror_off = upper ? j - (beyond - 1) : -j + (beyond - 1);  // the mirror point's offset
    row[mirror_off + c] += sign * row[l];
    row[l] = 0.0;
  }
}

Stencil stencil_d1() {  // c10d1
  Stencil s{};
  s.ncl = 5; s.ncr = 7; s.nbc = 4; s.implicit = true; s.addback = false;
  const double L[5] = {0.45, 4.5, 9.0, 4.5, 0.45};
  const double R[7] = {-0.015, -1.515, -6.375, 0.0, 6.375, 1.515, 0.015};
  const double LB[4][5] = {{0.0, 0.0, 4.725, 9.45, 0.0},
                           {0.0, 1.94578125, 7.783125, 1.94578125, 0.0},
                           {0.2964375, 4.743, 10.67175, 4.743, 0.2964375},
                           {0.451390625, 4.63271875, 9.38146875, 4.63271875, 0.451390625}};
  const double RB[4][7] = {{0.0, 0.0, 0.0, -11.8125, 9.45, 2.3625, 0.0},
                           {0.0, 0.0, -5.83734375, 0.0, 5.83734375, 0.0, 0.0},
                           {0.0, -1.23515625, -7.905, 0.0, 7.905, 1.23515625, 0.0},
                           {-0.015, -1.53, -6.66984375, 0.0, 6.66984375, 1.53, 0.015}};
  std::memcpy(s.lhs, L, sizeof L);
  std::memcpy(s.rhs, R, sizeof R);
  for (int j = 0; j < 4; j++) {
    std::memcpy(s.lhs_lo[j], LB[j], sizeof LB[j]);
    std::memcpy(s.rhs_lo[j], RB[j], sizeof RB[j]);
  }
  // extended boundary data rows (stencils.f90:261-276)
  const double XL[4][5] = {{0.0, 0.0, 6.0, 0.0, 0.0},
                           {0.0, 2.25, 6.0, 2.25, 0.0},
                           {0.3, 3.0, 6.0, 3.0, 0.3},
                           {0.3, 3.0, 6.0, 3.0, 0.3}};
  const double XR[4][9] = {{-0.1, 0.9, -4.5, 0.0, 4.5, -0.9, 0.1},
                           {0.0125, -0.3, -4.6875, 0.0, 4.6875, 0.3, -0.0125},
                           {-0.01, -1.01, -4.25, 0.0, 4.25, 1.01, 0.01},
                           {-0.01, -1.01, -4.25, 0.0, 4.25, 1.01, 0.01}};
  set_xt(s, XL, XR);
  s.fold_lhs = -1.0;  // symmetric field, antisymmetric derivative (stencils.f90:256-259)
  s.fold_rhs = 1.0;
  mirror(s, -1.0);  // antisymmetric operator
  return s;
}

Stencil stencil_d2() {  // c10d2: compact 10th-order second derivative
  Stencil s{};
  s.ncl = 5; s.ncr = 7; s.nbc = 4; s.implicit = true; s.addback = false;
  const double L[5] = {387.0, 6012.0, 16182.0, 6012.0, 387.0};
  const double R[7] = {79.0, 4671.0, 9585.0, -28670.0, 9585.0, 4671.0, 79.0};
  const double LB[4][5] = {{0.0, 0.0, 1.0, 11.0, 0.0},
                           {0.0, 1.0, 10.0, 1.0, 0.0},
                           {23.0, 688.0, 2358.0, 688.0, 23.0},
                           {387.0, 6012.0, 16182.0, 6012.0, 387.0}};
  const double RB[4][7] = {{0.0, 0.0, 0.0, 13.0, -27.0, 15.0, -1.0},
                           {0.0, 0.0, 12.0, -24.0, 12.0, 0.0, 0.0},
                           {0.0, 465.0, 1920.0, -4770.0, 1920.0, 465.0, 0.0},
                           {79.0, 4671.0, 9585.0, -28670.0, 9585.0, 4671.0, 79.0}};
  std::memcpy(s.lhs, L, sizeof L);
  std::memcpy(s.rhs, R, sizeof R);
  for (int j = 0; j < 4; j++) {
    std::memcpy(s.lhs_lo[j], LB[j], sizeof LB[j]);
    std::memcpy(s.rhs_lo[j], RB[j], sizeof RB[j]);
  }
  // extended boundary data rows (stencils.f90:411-427)
  const double XL[4][5] = {{0.0, 0.0, 18.0, 0.0, 0.0},
                           {0.0, 4.05, 17.1, 4.05, 0.0},
                           {0.387, 6.012, 16.182, 6.012, 0.387},
                           {0.387, 6.012, 16.182, 6.012, 0.387}};
  const double XR[4][9] = {{0.2, -2.7, 27.0, -49.0, 27.0, -2.7, 0.2},
                           {-0.0575, 2.295, 16.5375, -37.55, 16.5375, 2.295, -0.0575},
                           {0.079, 4.671, 9.585, -28.670, 9.585, 4.671, 0.079},
                           {0.079, 4.671, 9.585, -28.670, 9.585, 4.671, 0.079}};
  set_xt(s, XL, XR);
  s.fold_lhs = s.fold_rhs = 1.0;
  mirror(s, 1.0);
  return s;
}

// e4d4: explicit 4th-order fourth derivative, no metric.  The reference
// defines three one-sided rows per end (stencils.f90:480-489) but declares
// four (nbc1 = nbc2 = 4), leaving its fourth lower row and its last upper row
// unset; here the three defined rows close each end (the upper ones mirrored)
// and every other row is interior.
Stencil stencil_d4() {
  Stencil s{};
  s.ncl = 1; s.ncr = 7; s.nbc = 3; s.implicit = false; s.addback = false;
  const double a = 28.0 / 3.0, b = -6.5, c = 2.0, d = -1.0 / 6.0;
  const double R[7] = {d, c, b, a, b, c, d};
  const double RB[3][7] = {{0.0, 0.0, 0.0, a + b, b + c, c + d, d},
                           {0.0, 0.0, b + c, a + d, b, 0.0, 0.0},
                           {0.0, c + d, b, a, b, c, 0.0}};
  s.lhs[0] = 1.0;
  std::memcpy(s.rhs, R, sizeof R);
  for (int j = 0; j < 3; j++) {
    s.lhs_lo[j][0] = 1.0;
    std::memcpy(s.rhs_lo[j], RB[j], sizeof RB[j]);
  }
  set_xt(s, nullptr, nullptr);  // extended data: interior rows (stencils.f90:500-512)
  s.fold_lhs = s.fold_rhs = 1.0;
  mirror(s, 1.0);
  return s;
}

Stencil stencil_d8() {  // c10d8
  Stencil s{};
  s.ncl = 5; s.ncr = 9; s.nbc = 4; s.implicit = true; s.addback = false;
  const double z = 29.0, al = 14.0, be = 1.5;
  const double a = 4200.0, b = -3360.0, c = 1680.0, d = -480.0, e = 60.0;
  const double L[5] = {be, al, z, al, be};
  const double R[9] = {e, d, c, b, a, b, c, d, e};
  const double LB[4][5] = {{0.0, 0.0, al + z, be + al, be},
                           {0.0, be + al, z, al, be},
                           {be, al, z, al, be},
                           {be, al, z, al, be}};
  const double RB[4][9] = {{0.0, 0.0, 0.0, 0.0, b + a, c + b, d + c, e + d, e},
                           {0.0, 0.0, 0.0, c + b, d + a, e + b, c, d, e},
                           {0.0, 0.0, d + c, e + b, a, b, c, d, e},
                           {0.0, e + d, c, b, a, b, c, d, e}};
  std::memcpy(s.lhs, L, sizeof L);
  std::memcpy(s.rhs, R, sizeof R);
  for (int j = 0; j < 4; j++) {
    std::memcpy(s.lhs_lo[j], LB[j], sizeof LB[j]);
    std::memcpy(s.rhs_lo[j], RB[j], sizeof RB[j]);
  }
  // extended boundary data (stencils.f90:604-620): LHS rows 1-2 given, RHS interior
  const double XL[4][5] = {{0.0, 0.0, 60.0, 0.0, 0.0}, {0.0, 20.0, 20.0, 20.0, 0.0}, {be, al, z, al, be},
                           {be, al, z, al, be}};
  set_xt(s, XL, nullptr);
  s.fold_lhs = s.fold_rhs = 1.0;
  mirror(s, 1.0);
  return s;
}

Stencil stencil_sf() {  // c8ff8, 9/10 dealiasing filter with telescoped ends
  Stencil s{};
  s.ncl = 5; s.ncr = 9; s.nbc = 4; s.implicit = true; s.addback = true;
  const double be = 1.6688e-1, al = 6.6624e-1, z = 1.0;
  const double a = 9.9965e-1, b = 6.6652e-1, c = 1.6674e-1, d = 4.0e-5, e = -5.0e-6;
  const double L[5] = {be, al, z, al, be};
  const double R[9] = {e, d, c, b, a, b, c, d, e};
  const double LB[4][5] = {{0.0, 0.0, 1.0, 0.0, 0.0},
                           {0.0, 4.997e-1, 1.0, 4.997e-1, 0.0},
                           {1.6688e-1, 6.6624e-1, 1.0, 6.6624e-1, 1.6688e-1},
                           {1.6688e-1, 6.6624e-1, 1.0, 6.6624e-1, 1.6688e-1}};
  const double RB[4][9] = {
      {0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 4.9985e-1, 9.997e-1, 4.9985e-1, 0.0, 0.0, 0.0},
      {0.0, 0.0, 1.668e-1, 6.6656e-1, 9.9952e-1, 6.6656e-1, 1.668e-1, 0.0, 0.0},
      {0.0, 4.0e-5, 1.6672e-1, 6.6652e-1, 9.9968e-1, 6.6652e-1, 1.6672e-1, 4.0e-5, 0.0}};
  std::memcpy(s.lhs, L, sizeof L);
  std::memcpy(s.rhs, R, sizeof R);
  for (int j = 0; j < 4; j++) {
    std::memcpy(s.lhs_lo[j], LB[j], sizeof LB[j]);
    std::memcpy(s.rhs_lo[j], RB[j], sizeof RB[j]);
  }
  // the reference leaves this filter's extended-data rows unset (stencils.f90:814-826 are
  // commented out); an XTND end takes the one-sided rows here
  s.has_xt = false;
  s.fold_lhs = s.fold_rhs = 1.0;
  mirror(s, 1.0);
  s.diff_form = true;
  return s;
}

Stencil stencil_gf() {  // cgfs4, explicit 9-point Gaussian
  Stencil s{};
  s.ncl = 1; s.ncr = 9; s.nbc = 4; s.implicit = false; s.addback = true;
  const double a = 3565.0 / 10368.0, b = 3091.0 / 12960.0, c = 1997.0 / 25920.0,
               d = 149.0 / 12960.0, e = 107.0 / 103680.0;
  const double R[9] = {e, d, c, b, a, b, c, d, e};
  // one-sided ends fold the stencil onto itself (stencils.f90:1444-1447)
  const double RB[4][9] = {{0.0, 0.0, 0.0, 0.0, a + b, b + c, c + d, d + e, e},
                           {0.0, 0.0, 0.0, b + c, a + d, b + e, c, d, e},
                           {0.0, 0.0, c + d, b + e, a, b, c, d, e},
                           {0.0, d + e, c, b, a, b, c, d, e}};
  s.lhs[0] = 1.0;
  std::memcpy(s.rhs, R, sizeof R);
  for (int j = 0; j < 4; j++) {
    s.lhs_lo[j][0] = 1.0;
    std::memcpy(s.rhs_lo[j], RB[j], sizeof RB[j]);
  }
  set_xt(s, nullptr, nullptr);  // extended data: interior rows (stencils.f90:1456-1467)
  s.fold_lhs = s.fold_rhs = 1.0;
  mirror(s, 1.0);
  // the reference's first upper extended row is the reversed fourth one-sided row
  // (stencils.f90:1468: arb2(:,1,2) = arb1(ncr:1:-1,4,0))
  for (int l = 0; l < s.ncr; l++) s.xt_rhs_hi[0][l] = s.rhs_lo[3][s.ncr - 1 - l];
  s.diff_form = true;
  return s;
}

// ---------------------------------------------------------------------------
// Solve tables.  The LHS of every implicit operator is a pentadiagonal matrix
// A (band rows (a, b, diag, c, d) = A[i][i-2 .. i+2]; periodic lines wrap the
// column index).  The sweeps solve A x = r in one forward and one backward
// pass per line, from these per-row coefficients:
//
//  * non-periodic lines: the Crout factorisation A = L U, L lower triangular
//    with two subdiagonals, U unit upper triangular with two superdiagonals.
//    Forward:  z_i = rho_i r_i - alpha_i z_{i-1} - beta_i z_{i-2}
//              (rho = 1 / L_ii, alpha = L_i,i-1 rho, beta = L_i,i-2 rho);
//    backward: x_i = z_i - u1_i x_{i+1} - u2_i x_{i+2}.
//  * periodic lines: the wrap couples the first and the last unknowns.  The
//    last two unknowns x_B = (x_{n-2}, x_{n-1}) are split off; the other
//    m = n-2 form a plain banded block A_II = L U (the wrap only reaches
//    A_IB, A_BI).  Eliminating x_I (the Schur complement on x_B, i.e. the
//    Sherman-Morrison-Woodbury form of the rank-4 wrap correction):
//       F = L^-1 A_IB (m x 2),  G = A_BI U^-1 (2 x m),  S = A_BB - G F (2 x 2)
//       forward  z_I = L^-1 r_I, accumulating t = G z_I
//       x_B = S^-1 (r_B - t)
//       backward x_i = z_i - u1_i x_{i+1} - u2_i x_{i+2} - F_i0 x_{n-2} - F_i1 x_{n-1}
//    so the wrap costs two fused multiply-adds per point in each pass and the
//    line is still read once forward and once backward.
// Per-row layout (12 values, two 16-byte groups the sweeps load at once):
//   [0] rho  [1] alpha  [2] beta  [3] G_0i | [4] u1  [5] u2  [6] F_i0  [7] F_i1 | [8] G_1i
// and for periodic lines row n-2 holds S^-1 = (s00, s01, s10, s11) in [0..3].
// Entries a row does not use are zero, so the first and last rows need no
// special cases in the sweeps.
constexpr int kSolveStride = 12;

// Crout factorisation of an m x m matrix of lower and upper bandwidth 2
// (entry(i, j) gives A_ij for |i - j| <= 2), without pivoting: every LHS here
// is diagonally dominant.  Lw[i*3 + k] = L_i,i-k (k = 0..2), Uw[i*3 + k] =
// U_i,i+k (k = 1, 2).
template <class Entry>
bool crout_banded(int m, Entry entry, std::vector<double>& Lw, std::vector<double>& Uw) {
  Lw.assign((size_t)m * 3, 0.0);
  Uw.assign((size_t)m * 3, 0.0);
  auto Lij = [&](int i, int j) -> double { return (j <= i && i - j <= 2 && j >= 0) ? Lw[(size_t)i * 3 + (i - j)] : 0.0; };
  auto Uij = [&](int i, int j) -> double {
    if (i == j) return 1.0;
    return (j > i && j - i <= 2 && j < m) ? Uw[(size_t)i * 3 + (j - i)] : 0.0;
  };
  for (int i = 0; i < m; i++) {
    for (int j = std::max(0, i - 2); j <= i; j++) {  // row i of L
      double s = entry(i, j);
      for (int k = std::max(0, std::max(i, j) - 2); k < j; k++) s -= Lij(i, k) * Uij(k, j);
      Lw[(size_t)i * 3 + (i - j)] = s;
    }
    const double lii = Lw[(size_t)i * 3];
    if (lii == 0.0 || !std::isfinite(lii)) return false;
    for (int j = i + 1; j <= std::min(m - 1, i + 2); j++) {  // row i of U
      double s = entry(i, j);
      for (int k = std::max(0, j - 2); k < i; k++) s -= Lij(i, k) * Uij(k, j);
      Uw[(size_t)i * 3 + (j - i)] = s / lii;
    }
  }
  return true;
}

// The per-row solve coefficients of one line's LHS (band rows n x 5).
bool solve_tables(const std::vector<double>& band, int n, bool periodic, std::vector<double>& out) {
  out.assign((size_t)n * kSolveStride, 0.0);
  // A_ij of the full line matrix (periodic: columns taken modulo n)
  auto A = [&](int i, int j) -> double {
    double s = 0.0;
    for (int l = 0; l < 5; l++) {
      int c = i + l - 2;
      if (periodic) c = ((c % n) + n) % n;
      if (c == j) s += band[(size_t)i * 5 + l];
    }
    return s;
  };
  const int m = periodic ? n - 2 : n;
  std::vector<double> Lw, Uw;
  if (!crout_banded(m, A, Lw, Uw)) return false;
  auto row = [&](int i) { return &out[(size_t)i * kSolveStride]; };
  for (int i = 0; i < m; i++) {
    double* r = row(i);
    const double rho = 1.0 / Lw[(size_t)i * 3];
    r[0] = rho;
    r[1] = Lw[(size_t)i * 3 + 1] * rho;
    r[2] = Lw[(size_t)i * 3 + 2] * rho;
    r[4] = Uw[(size_t)i * 3 + 1];
    r[5] = Uw[(size_t)i * 3 + 2];
  }
  if (!periodic) return true;
  // F = L^-1 A_IB: forward substitution of the two border columns
  std::vector<double> F((size_t)m * 2, 0.0), G((size_t)2 * m, 0.0);
  for (int c = 0; c < 2; c++)
    for (int i = 0; i < m; i++) {
      double s = A(i, m + c);
      if (i >= 1) s -= Lw[(size_t)i * 3 + 1] * F[(size_t)(i - 1) * 2 + c];
      if (i >= 2) s -= Lw[(size_t)i * 3 + 2] * F[(size_t)(i - 2) * 2 + c];
      F[(size_t)i * 2 + c] = s / Lw[(size_t)i * 3];
    }
  // G = A_BI U^-1: G U = A_BI, solved column by column (U unit upper)
  for (int b = 0; b < 2; b++)
    for (int j = 0; j < m; j++) {
      double s = A(m + b, j);
      if (j >= 1) s -= G[(size_t)b * m + j - 1] * Uw[(size_t)(j - 1) * 3 + 1];
      if (j >= 2) s -= G[(size_t)b * m + j - 2] * Uw[(size_t)(j - 2) * 3 + 2];
      G[(size_t)b * m + j] = s;
    }
  // S = A_BB - G F and its inverse
  double S[2][2];
  for (int b = 0; b < 2; b++)
    for (int c = 0; c < 2; c++) {
      double s = A(m + b, m + c);
      for (int i = 0; i < m; i++) s -= G[(size_t)b * m + i] * F[(size_t)i * 2 + c];
      S[b][c] = s;
    }
  const double det = S[0][0] * S[1][1] - S[0][1] * S[1][0];
  if (det == 0.0 || !std::isfinite(det)) return false;
  for (int i = 0; i < m; i++) {
    double* r = row(i);
    r[3] = G[i];
    r[8] = G[(size_t)m + i];
    r[6] = F[(size_t)i * 2];
    r[7] = F[(size_t)i * 2 + 1];
  }
  double* s = row(m);
  s[0] = S[1][1] / det;
  s[1] = -S[0][1] / det;
  s[2] = -S[1][0] / det;
  s[3] = S[0][0] / det;
  return true;
}

// Gauss-Jordan inverse with partial pivoting of a small dense matrix (row
// major k x k, FP64); false when singular.
bool invert_small(std::vector<double> a, int k, std::vector<double>& inv) {
  inv.assign((size_t)k * k, 0.0);
  for (int i = 0; i < k; i++) inv[(size_t)i * k + i] = 1.0;
  for (int c = 0; c < k; c++) {
    int piv = c;
    for (int r = c + 1; r < k; r++)
      if (std::fabs(a[(size_t)r * k + c]) > std::fabs(a[(size_t)piv * k + c])) piv = r;
    const double d = a[(size_t)piv * k + c];
    if (d == 0.0 || !std::isfinite(d)) return false;
    if (piv != c)
      for (int j = 0; j < k; j++) {
        std::swap(a[(size_t)piv * k + j], a[(size_t)c * k + j]);
        std::swap(inv[(size_t)piv * k + j], inv[(size_t)c * k + j]);
      }
    const double rd = 1.0 / d;
    for (int j = 0; j < k; j++) {
      a[(size_t)c * k + j] *= rd;
      inv[(size_t)c * k + j] *= rd;
    }
    for (int r = 0; r < k; r++) {
      if (r == c) continue;
      const double f = a[(size_t)r * k + c];
      if (f == 0.0) continue;
      for (int j = 0; j < k; j++) {
        a[(size_t)r * k + j] -= f * a[(size_t)c * k + j];
        inv[(size_t)r * k + j] -= f * inv[(size_t)c * k + j];
      }
    }
  }
  return true;
}

}  // namespace

// Split-line tables: the reduced-system form of the line solve (the
// reference's parallel solver, compact_basetype.f90:171-197 with
// pentadiagonal.f90:160-626 and compact_d1.f90:242-337, splits a line
// across MPI ranks the same way).  The line is cut into S segments of
// kSplitSeg points (the last one takes the remainder, up to 2 kSplitSeg - 1).
// Segment j = rows [a, b) couples to its neighbours only through its first
// two and last two rows:
//   A_jj x_j + C_j xbot_{j-1} + B_j xtop_{j+1} = r_j
// (xbot = the last two unknowns of the segment before, xtop = the first two
// of the segment after; periodic lines wrap, one-sided lines have no
// coupling at their ends).  With y_j = A_jj^-1 r_j and the spikes
// W_j = A_jj^-1 C_j, V_j = A_jj^-1 B_j (L x 2 each):
//   x_j = y_j - W_j xbot_{j-1} - V_j xtop_{j+1}.
// Taking the tip rows (0, 1, L-2, L-1) of every segment gives the reduced
// system R t = y_tips over the 4S tip unknowns; R is the same for every line
// of a grid, so its inverse is formed here once, and each segment keeps the
// four rows of R^-1 that give its xbot_{j-1} and xtop_{j+1}.
// Tables: row[p * 12 + ...] per position p (local Crout of its segment block
// and its spikes): [0] rho [1] alpha [2] beta | [4] u1 [5] u2 |
// [8] W_0 [9] W_1 [10] V_0 [11] V_1; G[(j * 4 + q) * 4S + i] for q = xbot 0,
// xbot 1, xtop 0, xtop 1.
int build_split(const std::vector<double>& band, int n, bool periodic, std::vector<int>& start,
                std::vector<double>& row, std::vector<double>& G) {
  const int S = std::max(1, n / kSplitSeg);
  start.assign((size_t)S + 1, 0);
  for (int j = 0; j < S; j++) start[j] = j * kSplitSeg;
  start[S] = n;
  auto A = [&](int i, int j) -> double {  // entry of the full line matrix
    double s = 0.0;
    for (int l = 0; l < 5; l++) {
      int c = i + l - 2;
      if (periodic) c = ((c % n) + n) % n;
      else if (c < 0 || c >= n) continue;
      if (c == j) s += band[(size_t)i * 5 + l];
    }
    return s;
  };
  row.assign((size_t)n * 12, 0.0);
  const int T = 4 * S;
  std::vector<double> R((size_t)T * T, 0.0);
  for (int j = 0; j < S; j++) {
    const int a = start[j], b = start[j + 1], L = b - a;
    if (L < 4) return PG_EBADSHAPE;
    std::vector<double> Lw, Uw;
    if (!crout_banded(L, [&](int i, int k) { return A(a + i, a + k); }, Lw, Uw)) return PG_EINVAL;
    // spike columns: right-hand sides C_j (rows 0, 1) and B_j (rows L-2, L-1)
    const bool left = periodic || j > 0, right = periodic || j < S - 1;
    const int pl = ((a - 2) % n + n) % n, pl1 = ((a - 1) % n + n) % n;  // xbot_{j-1} positions
    const int pr = b % n, pr1 = (b + 1) % n;                            // xtop_{j+1} positions
    std::vector<double> rhs((size_t)L * 4, 0.0);  // columns W0 W1 V0 V1
    if (left) {
      rhs[0 * 4 + 0] = A(a, pl);
      rhs[0 * 4 + 1] = A(a, pl1);
      rhs[1 * 4 + 1] = A(a + 1, pl1);
    }
    if (right) {
      rhs[(size_t)(L - 2) * 4 + 2] = A(b - 2, pr);
      rhs[(size_t)(L - 1) * 4 + 2] = A(b - 1, pr);
      rhs[(size_t)(L - 1) * 4 + 3] = A(b - 1, pr1);
    }
    // solve A_jj X = rhs for the 4 columns (forward with L, backward with unit U)
    for (int c = 0; c < 4; c++) {
      std::vector<double> z((size_t)L, 0.0);
      for (int i = 0; i < L; i++) {
        double v = rhs[(size_t)i * 4 + c];
        if (i >= 1) v -= Lw[(size_t)i * 3 + 1] * z[i - 1];
        if (i >= 2) v -= Lw[(size_t)i * 3 + 2] * z[i - 2];
        z[i] = v / Lw[(size_t)i * 3];
      }
      for (int i = L - 1; i >= 0; i--) {
        double v = z[i];
        if (i + 1 < L) v -= Uw[(size_t)i * 3 + 1] * z[i + 1];
        if (i + 2 < L) v -= Uw[(size_t)i * 3 + 2] * z[i + 2];
        z[i] = v;
      }
      for (int i = 0; i < L; i++) row[(size_t)(a + i) * 12 + 8 + c] = z[i];
    }
    for (int i = 0; i < L; i++) {
      double* r = &row[(size_t)(a + i) * 12];
      const double rho = 1.0 / Lw[(size_t)i * 3];
      r[0] = rho;
      r[1] = Lw[(size_t)i * 3 + 1] * rho;
      r[2] = Lw[(size_t)i * 3 + 2] * rho;
      r[4] = Uw[(size_t)i * 3 + 1];
      r[5] = Uw[(size_t)i * 3 + 2];
    }
    // reduced-system rows of the four tips
    const int jm = (j + S - 1) % S, jp = (j + 1) % S;
    const int li[4] = {0, 1, L - 2, L - 1};
    for (int q = 0; q < 4; q++) {
      const int rr = 4 * j + q;
      const double* w = &row[(size_t)(a + li[q]) * 12 + 8];
      R[(size_t)rr * T + rr] += 1.0;
      for (int c = 0; c < 2; c++) {
        R[(size_t)rr * T + 4 * jm + 2 + c] += w[c];
        R[(size_t)rr * T + 4 * jp + c] += w[2 + c];
      }
    }
  }
  std::vector<double> Ri;
  if (!invert_small(R, T, Ri)) return PG_EINVAL;
  G.assign((size_t)S * 4 * T, 0.0);
  for (int j = 0; j < S; j++) {
    const int jm = (j + S - 1) % S, jp = (j + 1) % S;
    const bool left = periodic || j > 0, right = periodic || j < S - 1;
    const int src[4] = {4 * jm + 2, 4 * jm + 3, 4 * jp, 4 * jp + 1};
    const bool use[4] = {left, left, right, right};
    for (int q = 0; q < 4; q++)
      if (use[q])
        for (int i = 0; i < T; i++) G[((size_t)j * 4 + q) * T + i] = Ri[(size_t)src[q] * T + i];
  }
  return PG_OK;
}

// Build the host tables of one operator along one direction.
// Output layout (all row-major, n rows):
//   rhs[n*9]   per-row RHS weights (d1, d2, d4 use the first 7), already divided
//              by the metric `scale` when scale != 0 (d1: dx, compact_operators.f90:41-46;
//              d2: dx^2, :149-152)
//   lu[n*12]   per-row solve coefficients (solve_tables above); empty rows
//              for explicit operators.
int build_operator(int kind, int n, bool periodic, double scale, OpTables& t, int bc_lo, int bc_hi, int sym) {
  Stencil s;
  switch (kind) {
    case OPK_D1: s = stencil_d1(); break;
    case OPK_D8: s = stencil_d8(); break;
    case OPK_SF: s = stencil_sf(); break;
    case OPK_GF: s = stencil_gf(); break;
    case OPK_D2: s = stencil_d2(); break;
    case OPK_D4: s = stencil_d4(); break;
    default: return PG_EINVAL;
  }
  if (bc_lo < 0 || bc_lo > 2 || bc_hi < 0 || bc_hi > 2 || (sym != 1 && sym != -1)) return PG_EINVAL;
  t.kind = kind;
  t.n = n;
  t.periodic = periodic;
  t.implicit = s.implicit;
  t.addback = s.addback;
  t.null_op = (n < 4);
  t.rhs.assign((size_t)n * 9, 0.0);
  t.lu.assign((size_t)n * kSolveStride, 0.0);
  // the boundary code each end's rows follow (compact.f90:77-91): 0 one-sided, +-1 the
  // symmetric / antisymmetric variant at a symmetry plane, 2 extended data
  auto code = [&](int bc) { return bc == 1 ? sym : (bc == 2 && s.has_xt ? 2 : 0); };
  t.bcl = periodic ? 0 : code(bc_lo);
  t.bch = periodic ? 0 : code(bc_hi);
  if (t.null_op) return PG_OK;
  if (n < 8) return PG_EBADSHAPE;  // the reference stencils index 8 points per line

  // global assembly (compact_basetype.f90:124-133)
  std::vector<double> band((size_t)n * 9, 0.0);  // band cols 0..4 = LHS (a,b,diag,c,d)
  const int offl = (5 - s.ncl) / 2;              // Gaussian: its single LHS weight is the diagonal
  auto put_row = [&](int i, const double* lhs, const double* rhs) {
    double l5[5] = {0, 0, 0, 0, 0}, r9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int l = 0; l < s.ncl; l++) l5[l] = lhs[l];
    for (int l = 0; l < s.ncr; l++) r9[l] = rhs[l];
    if (s.diff_form) to_difference_form(s, l5, r9);
    for (int l = 0; l < s.ncl; l++) band[(size_t)i * 9 + offl + l] = l5[l];
    for (int l = 0; l < s.ncr; l++) t.rhs[(size_t)i * 9 + l] = r9[l];
  };
  for (int i = 0; i < n; i++) put_row(i, s.lhs, s.rhs);
  if (s.ncr == 9) {  // the FP32 sweeps pair the 9-point interior weights about the centre
    const double* r = &t.rhs[(size_t)(n / 2) * 9];
    for (int k = 1; k <= 4; k++)
      if (r[4 - k] != r[4 + k]) return PG_EINVAL;
  }
  if (!periodic) {
    for (int end = 0; end < 2; end++) {
      const int c = end == 0 ? t.bcl : t.bch;
      for (int j = 0; j < s.nbc; j++) {
        const int i = end == 0 ? j : n - s.nbc + j;  // rows of the upper block are stored from n - nbc
        const int from_end = end == 0 ? j : s.nbc - 1 - j;
        double fl[5], fr[9];
        const double *L, *R;
        if (c == 0) {
          L = end == 0 ? s.lhs_lo[j] : s.lhs_hi[j];
          R = end == 0 ? s.rhs_lo[j] : s.rhs_hi[j];
        } else if (c == 2) {
          L = end == 0 ? s.xt_lhs_lo[j] : s.xt_lhs_hi[j];
          R = end == 0 ? s.xt_rhs_lo[j] : s.xt_rhs_hi[j];
        } else {  // symmetry plane: fold the interior stencil (stencils.f90:2390-2453)
          const double sl = (c == 1 ? s.fold_lhs : -s.fold_lhs), sr = (c == 1 ? s.fold_rhs : -s.fold_rhs);
          fold_row(s.lhs, s.ncl, from_end, end == 1, sl, fl);
          fold_row(s.rhs, s.ncr, from_end, end == 1, sr, fr);
          L = fl;
          R = fr;
        }
        put_row(i, L, R);
      }
    }
  }
  if (scale != 0.0)
    for (auto& v : t.rhs) v = v / scale;
  t.lhs.assign((size_t)n * 5, 0.0);
  for (int i = 0; i < n; i++)
    for (int l = 0; l < 5; l++) t.lhs[(size_t)i * 5 + l] = band[(size_t)i * 9 + l];

  if (s.implicit && !solve_tables(t.lhs, n, periodic, t.lu)) return PG_EINVAL;
  return PG_OK;
}

}  // namespace pg
