// Host-side operator assembly for the GB300 compact-operator library.
//
// Builds, once per grid and direction, the per-row coefficient tables that the
// sweep kernels read:
//   - the weight tables of pyranda/parcop/stencils.f90 (c10d1 :207-277,
//     c10d2 :358-428, e4d4 :430-513, c10d8 :515-621, c8ff8 :713-835,
//     cgfs4 :1387-1476), boundary code 0 (one-sided closures) and periodic;
//   - the global LHS/RHS assembly of compact_basetype.f90:124-148 (np = 1);
//   - the LU factorisations bpentLUD1 / ppentLUD1 of pentadiagonal.f90:18-135.
// The factorisation steps are kept as in the reference (the kernels replay the
// matching substitutions), so results agree with the reference to rounding.
#include "pg_internal.h"

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
  double lhs_lo[4][5], rhs_lo[4][9];
  double lhs_hi[4][5], rhs_hi[4][9];
};

// Upper boundary rows mirror the lower ones: row j of the upper block is the
// reversed row (nbc-1-j) of the lower block (stencils.f90, e.g. :241-244).
void mirror(Stencil& s, double rhs_sign) {
  for (int j = 0; j < s.nbc; j++) {
    for (int l = 0; l < s.ncl; l++) s.lhs_hi[j][l] = s.lhs_lo[s.nbc - 1 - j][s.ncl - 1 - l];
    for (int l = 0; l < s.ncr; l++) s.rhs_hi[j][l] = rhs_sign * s.rhs_lo[s.nbc - 1 - j][s.ncr - 1 - l];
  }
}

// Difference form used by the filters: the stored RHS is RHS - LHS on the
// overlapping entries (stencils.f90:832-834 and :1472-1475).
void to_difference_form(Stencil& s) {
  const int off = (s.ncr - s.ncl) / 2;
  for (int l = 0; l < s.ncl; l++) s.rhs[off + l] -= s.lhs[l];
  for (int j = 0; j < 4; j++)
    for (int l = 0; l < s.ncl; l++) {
      s.rhs_lo[j][off + l] -= s.lhs_lo[j][l];
      s.rhs_hi[j][off + l] -= s.lhs_hi[j][l];
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
  mirror(s, 1.0);
  to_difference_form(s);
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
  mirror(s, 1.0);
  to_difference_form(s);
  return s;
}

// LU factorisation of the non-periodic pentadiagonal matrix, band columns
// 0..4 = (a, b, diag, c, d); the diagonal is stored inverted
// (bpentLUD1, pentadiagonal.f90:18-39).
void factor_banded(std::vector<double>& c, int n) {
  auto C = [&](int i, int k) -> double& { return c[(size_t)i * 9 + k]; };
  for (int i = 0; i < n - 2; i++) {
    C(i + 1, 1) /= C(i, 2);
    C(i + 1, 2) -= C(i, 3) * C(i + 1, 1);
    C(i + 1, 3) -= C(i, 4) * C(i + 1, 1);
    C(i + 2, 0) /= C(i, 2);
    C(i + 2, 1) -= C(i, 3) * C(i + 2, 0);
    C(i + 2, 2) -= C(i, 4) * C(i + 2, 0);
  }
  C(n - 1, 1) /= C(n - 2, 2);
  C(n - 1, 2) -= C(n - 2, 3) * C(n - 1, 1);
  for (int i = 0; i < n; i++) C(i, 2) = 1.0 / C(i, 2);
}

// Bordered LU of the cyclic pentadiagonal matrix (ppentLUD1,
// pentadiagonal.f90:64-135).  Columns 5,6 hold the multipliers of the last two
// rows, columns 7,8 the fill of the last two columns.  0-based: row r here is
// Fortran row r+1, column k is Fortran column k+1.
void factor_cyclic(std::vector<double>& c, int N) {
  auto C = [&](int i1, int k1) -> double& { return c[(size_t)(i1 - 1) * 9 + (k1 - 1)]; };
  C(1, 8) = C(1, 1);
  C(1, 9) = C(1, 2);
  C(1, 3) = 1.0 / C(1, 3);
  C(1, 6) = C(N - 1, 5) * C(1, 3);
  C(1, 7) = C(N, 4) * C(1, 3);
  C(2, 2) = C(2, 2) * C(1, 3);
  C(2, 3) = C(2, 3) - C(2, 2) * C(1, 4);
  C(2, 4) = C(2, 4) - C(2, 2) * C(1, 5);
  C(2, 8) = -C(2, 2) * C(1, 8);
  C(2, 9) = C(2, 1) - C(2, 2) * C(1, 9);
  C(2, 3) = 1.0 / C(2, 3);
  C(2, 6) = -C(1, 6) * C(1, 4) * C(2, 3);
  C(2, 7) = (C(N, 5) - C(1, 7) * C(1, 4)) * C(2, 3);
  for (int k = 3; k <= N - 4; k++) {
    C(k, 1) = C(k, 1) * C(k - 2, 3);
    C(k, 2) = (C(k, 2) - C(k, 1) * C(k - 2, 4)) * C(k - 1, 3);
    C(k, 3) = C(k, 3) - (C(k, 2) * C(k - 1, 4) + C(k, 1) * C(k - 2, 5));
    C(k, 4) = C(k, 4) - C(k, 2) * C(k - 1, 5);
    C(k, 8) = -(C(k, 2) * C(k - 1, 8) + C(k, 1) * C(k - 2, 8));
    C(k, 9) = -(C(k, 2) * C(k - 1, 9) + C(k, 1) * C(k - 2, 9));
    C(k, 3) = 1.0 / C(k, 3);
    C(k, 6) = -(C(k - 1, 6) * C(k - 1, 4) + C(k - 2, 6) * C(k - 2, 5)) * C(k, 3);
    C(k, 7) = -(C(k - 1, 7) * C(k - 1, 4) + C(k - 2, 7) * C(k - 2, 5)) * C(k, 3);
  }
  int k = N - 3;
  C(k, 1) = C(k, 1) * C(k - 2, 3);
  C(k, 2) = (C(k, 2) - C(k, 1) * C(k - 2, 4)) * C(k - 1, 3);
  C(k, 3) = C(k, 3) - (C(k, 2) * C(k - 1, 4) + C(k, 1) * C(k - 2, 5));
  C(k, 4) = C(k, 4) - C(k, 2) * C(k - 1, 5);
  C(k, 8) = C(k, 5) - (C(k, 2) * C(k - 1, 8) + C(k, 1) * C(k - 2, 8));
  C(k, 9) = -(C(k, 2) * C(k - 1, 9) + C(k, 1) * C(k - 2, 9));
  C(k, 3) = 1.0 / C(k, 3);
  C(k, 6) = (C(N - 1, 1) - (C(k - 1, 6) * C(k - 1, 4) + C(k - 2, 6) * C(k - 2, 5))) * C(k, 3);
  C(k, 7) = -(C(k - 1, 7) * C(k - 1, 4) + C(k - 2, 7) * C(k - 2, 5)) * C(k, 3);
  k = N - 2;
  C(k, 1) = C(k, 1) * C(k - 2, 3);
  C(k, 2) = (C(k, 2) - C(k, 1) * C(k - 2, 4)) * C(k - 1, 3);
  C(k, 3) = C(k, 3) - (C(k, 2) * C(k - 1, 4) + C(k, 1) * C(k - 2, 5));
  C(k, 8) = C(k, 4) - (C(k, 2) * C(k - 1, 8) + C(k, 1) * C(k - 2, 8));
  C(k, 9) = C(k, 5) - (C(k, 2) * C(k - 1, 9) + C(k, 1) * C(k - 2, 9));
  C(k, 3) = 1.0 / C(k, 3);
  C(k, 6) = (C(N - 1, 2) - C(k - 1, 6) * C(k - 1, 4) - C(k - 2, 6) * C(k - 2, 5)) * C(k, 3);
  C(k, 7) = (C(N, 1) - C(k - 1, 7) * C(k - 1, 4) - C(k - 2, 7) * C(k - 2, 5)) * C(k, 3);
  for (int q = 1; q <= N - 2; q++) {
    C(N - 1, 3) = C(N - 1, 3) - C(q, 6) * C(q, 8);
    C(N - 1, 4) = C(N - 1, 4) - C(q, 6) * C(q, 9);
  }
  C(N - 1, 9) = C(N - 1, 4);
  for (int q = 1; q <= N - 2; q++) C(N, 2) = C(N, 2) - C(q, 7) * C(q, 8);
  C(N - 1, 3) = 1.0 / C(N - 1, 3);
  C(N - 1, 7) = C(N, 2) * C(N - 1, 3);
  for (int q = 1; q <= N - 1; q++) C(N, 3) = C(N, 3) - C(q, 7) * C(q, 9);
  C(N, 3) = 1.0 / C(N, 3);
}

}  // namespace

// Build the host tables of one operator along one direction.
// Output layout (all row-major, n rows):
//   rhs[n*9]   per-row RHS weights (d1, d2, d4 use the first 7), already divided
//              by the metric `scale` when scale != 0 (d1: dx, compact_operators.f90:41-46;
//              d2: dx^2, :149-152)
//   lu[n*9]    per-row solve coefficients in the order consumed by the kernels:
//              0:c1 1:c2 (forward) 2:c3 (inverse diagonal) 3:c4 4:c5 (backward)
//              5:c6 6:c7 (cyclic row multipliers) 7:c8 8:c9 (cyclic fill)
//              with entries the substitution does not use set to zero.
int build_operator(int kind, int n, bool periodic, double scale, OpTables& t) {
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
  t.kind = kind;
  t.n = n;
  t.periodic = periodic;
  t.implicit = s.implicit;
  t.addback = s.addback;
  t.null_op = (n < 4);
  t.rhs.assign((size_t)n * 9, 0.0);
  t.lu.assign((size_t)n * 9, 0.0);
  if (t.null_op) return PG_OK;
  if (n < 8) return PG_EBADSHAPE;  // the reference stencils index 8 points per line

  // global assembly (compact_basetype.f90:124-133)
  std::vector<double> band((size_t)n * 9, 0.0);  // band cols 0..4 = LHS (a,b,diag,c,d)
  const int offl = (5 - s.ncl) / 2;              // Gaussian: its single LHS weight is the diagonal
  for (int i = 0; i < n; i++) {
    for (int l = 0; l < s.ncl; l++) band[(size_t)i * 9 + offl + l] = s.lhs[l];
    for (int l = 0; l < s.ncr; l++) t.rhs[(size_t)i * 9 + l] = s.rhs[l];
  }
  if (!periodic) {
    for (int j = 0; j < s.nbc; j++) {
      for (int l = 0; l < s.ncl; l++) band[(size_t)j * 9 + offl + l] = s.lhs_lo[j][l];
      for (int l = 0; l < s.ncr; l++) t.rhs[(size_t)j * 9 + l] = s.rhs_lo[j][l];
    }
    for (int j = 0; j < s.nbc; j++) {
      const int i = n - s.nbc + j;
      for (int l = 0; l < s.ncl; l++) band[(size_t)i * 9 + offl + l] = s.lhs_hi[j][l];
      for (int l = 0; l < s.ncr; l++) t.rhs[(size_t)i * 9 + l] = s.rhs_hi[j][l];
    }
  }
  if (scale != 0.0)
    for (auto& v : t.rhs) v = v / scale;
  t.lhs.assign((size_t)n * 5, 0.0);
  for (int i = 0; i < n; i++)
    for (int l = 0; l < 5; l++) t.lhs[(size_t)i * 5 + l] = band[(size_t)i * 9 + l];

  if (s.implicit) {
    auto L = [&](int i, int k) -> double& { return t.lu[(size_t)i * 9 + k]; };
    if (periodic) {
      factor_cyclic(band, n);
      auto B = [&](int i, int k) { return band[(size_t)i * 9 + k]; };
      for (int i = 0; i < n; i++) {
        L(i, 0) = B(i, 0); L(i, 1) = B(i, 1); L(i, 2) = B(i, 2);
        L(i, 3) = B(i, 3); L(i, 4) = B(i, 4); L(i, 5) = B(i, 5);
        L(i, 6) = B(i, 6); L(i, 7) = B(i, 7); L(i, 8) = B(i, 8);
      }
      // forward: row 0 has no multipliers, row 1 only c2 (ppentLUS3x :664-666)
      L(0, 0) = 0.0; L(0, 1) = 0.0; L(1, 0) = 0.0;
      // backward: row N-2 (Fortran N-1) uses only its fill column c9; rows
      // N-3 and N-4 (Fortran N-2, N-3) have their c4/c5 folded into c8/c9
      L(n - 3, 3) = 0.0; L(n - 3, 4) = 0.0; L(n - 4, 4) = 0.0;
    } else {
      factor_banded(band, n);
      auto B = [&](int i, int k) { return band[(size_t)i * 9 + k]; };
      for (int i = 0; i < n; i++) {
        L(i, 0) = B(i, 0); L(i, 1) = B(i, 1); L(i, 2) = B(i, 2);
        L(i, 3) = B(i, 3); L(i, 4) = B(i, 4);
      }
      L(0, 0) = 0.0; L(0, 1) = 0.0; L(1, 0) = 0.0;
      L(n - 2, 4) = 0.0; L(n - 1, 3) = 0.0; L(n - 1, 4) = 0.0;
    }
  }
  return PG_OK;
}

}  // namespace pg
