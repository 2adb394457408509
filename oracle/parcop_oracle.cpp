// ORACLE — test infrastructure only.
//
// A plain FP64 CPU restatement of pyranda's parcop compact-operator path, used
// by the test-suite and by smoke() as the expected answer for the CUDA library,
// and by bench.py as the timed CPU baseline.  Nothing in the product links or
// calls this file.
//
// Every routine names the reference Fortran it restates (paths relative to the
// pyranda project).  The arithmetic follows the reference loop by loop (same
// operand order, same summation grouping) so that results agree to rounding.
//
// Scope: np = 1 (no MPI decomposition); boundary codes PERI (periodic), NONE
// (one-sided closures, mbc = 0), SYMM (symmetry planes, mbc = +-1, both
// operator variants) and XTND (extended-data rows, mbc = 2, without supplied
// data); Cartesian, cylindrical, spherical (with and without ratio zoning in
// the radius) and general curvilinear coordinates (mesh.f90:169-386).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Weight tables: pyranda/parcop/stencils.f90
// Rows are stored 0-based: alb1[j][l] is Fortran alb1(l+1, j+1, 0).
// ---------------------------------------------------------------------------
struct Weight {
  int nol, nor, ncl, ncr, nbc1, nbc2, null_option;
  bool implicit_op;
  double ali[5], ari[9];
  double alb1[4][5], alb2[4][5], arb1[4][9], arb2[4][9];  // boundary code 0 (one-sided)
  // rows of boundary codes -1, +1 (symmetry planes) and 2 (extended data): [code + 1]
  // (code 0 is the arrays above; index 1 unused)
  double xlb1[4][4][5], xlb2[4][4][5], xrb1[4][4][9], xrb2[4][4][9];
  bool has_xtnd;
};

// lower_symm_weights_int / upper_symm_weights_int: stencils.f90:2390-2453.
// alb/arb are 0-based [row][entry] copies of the Fortran alb(entry, row).
void lower_symm(double (*alb)[5], double (*arb)[9], const Weight& w, int syml, int symr) {
  for (int i = 0; i < w.nbc1; i++) {
    for (int l = 0; l < w.ncl; l++) alb[i][l] = w.ali[l];
    for (int l = 0; l < w.ncr; l++) arb[i][l] = w.ari[l];
  }
  for (int j = 1; j <= w.nol; j++) {
    const int k = w.nol - j + 1;
    for (int i = 1; i <= k; i++) {
      const int i1 = k - i + 1, i2 = k + i;
      alb[j - 1][i2 - 1] = alb[j - 1][i2 - 1] + (double)syml * alb[j - 1][i1 - 1];
      alb[j - 1][i1 - 1] = 0.0;
    }
  }
  for (int j = 1; j <= w.nor; j++) {
    const int k = w.nor - j + 1;
    for (int i = 1; i <= k; i++) {
      const int i1 = k - i + 1, i2 = k + i;
      arb[j - 1][i2 - 1] = arb[j - 1][i2 - 1] + (double)symr * arb[j - 1][i1 - 1];
      arb[j - 1][i1 - 1] = 0.0;
    }
  }
}
void upper_symm(double (*alb)[5], double (*arb)[9], const Weight& w, int syml, int symr) {
  const int n = w.nbc2;
  for (int i = 0; i < n; i++) {
    for (int l = 0; l < w.ncl; l++) alb[i][l] = w.ali[l];
    for (int l = 0; l < w.ncr; l++) arb[i][l] = w.ari[l];
  }
  for (int j = 1; j <= w.nol; j++) {
    const int jj = n + 1 - j, k = w.nol - j + 1, noff = w.ncl - k;
    for (int i = 1; i <= k; i++) {
      alb[jj - 1][noff - i] = alb[jj - 1][noff - i] + (double)syml * alb[jj - 1][noff + i - 1];
      alb[jj - 1][noff + i - 1] = 0.0;
    }
  }
  for (int j = n - w.nor + 1; j <= n; j++) {
    const int k = j - n + w.nor, noff = w.ncr - k;
    for (int i = 1; i <= k; i++) {
      arb[j - 1][noff - i] = arb[j - 1][noff - i] + (double)symr * arb[j - 1][noff + i - 1];
      arb[j - 1][noff + i - 1] = 0.0;
    }
  }
}

// The symmetric (+1) and antisymmetric (-1) rows of one operator, with the
// (LHS, RHS) fold signs of its +1 variant (e.g. stencils.f90:256-259 for d1,
// :600-603 for d8).
void set_symm_rows(Weight& w, int syml1, int symr1) {
  lower_symm(w.xlb1[2], w.xrb1[2], w, syml1, symr1);
  lower_symm(w.xlb1[0], w.xrb1[0], w, -syml1, -symr1);
  upper_symm(w.xlb2[2], w.xrb2[2], w, syml1, symr1);
  upper_symm(w.xlb2[0], w.xrb2[0], w, -syml1, -symr1);
}

// Extended-data rows (code 2): lower rows given, upper rows the lower ones
// reversed (alb2(:,j,2) = alb1(ncl:1:-1, nbc+1-j, 2); arb2 likewise times rsign).
void set_xtnd_rows(Weight& w, const double (*L)[5], const double (*R)[9], double rsign) {
  w.has_xtnd = true;
  for (int j = 0; j < w.nbc1; j++) {
    for (int l = 0; l < w.ncl; l++) w.xlb1[3][j][l] = L ? L[j][l] : w.ali[l];
    for (int l = 0; l < w.ncr; l++) w.xrb1[3][j][l] = R ? R[j][l] : w.ari[l];
  }
  for (int j = 0; j < w.nbc2; j++) {
    for (int l = 0; l < w.ncl; l++) w.xlb2[3][j][l] = w.xlb1[3][w.nbc1 - 1 - j][w.ncl - 1 - l];
    for (int l = 0; l < w.ncr; l++) w.xrb2[3][j][l] = rsign * w.xrb1[3][w.nbc1 - 1 - j][w.ncr - 1 - l];
  }
}

void mirror_rows(Weight& w, double rsign) {
  // alb2(:,j) = alb1(ncl:1:-1, 5-j) ; arb2(:,j) = rsign*arb1(ncr:1:-1, 5-j)
  for (int j = 0; j < 4; j++) {
    for (int l = 0; l < w.ncl; l++) w.alb2[j][l] = w.alb1[3 - j][w.ncl - 1 - l];
    for (int l = 0; l < w.ncr; l++) w.arb2[j][l] = rsign * w.arb1[3 - j][w.ncr - 1 - l];
  }
}

// c10d1: stencils.f90:207-277 (interior :236-237, one-sided rows :239-254)
Weight make_c10d1() {
  Weight w{};
  w.nol = 2; w.nor = 3; w.ncl = 5; w.ncr = 7; w.nbc1 = 4; w.nbc2 = 4;
  w.null_option = 0; w.implicit_op = true;
  const double ali[5] = {0.45, 4.5, 9.0, 4.5, 0.45};
  const double ari[7] = {-0.015, -1.515, -6.375, 0.0, 6.375, 1.515, 0.015};
  std::memcpy(w.ali, ali, sizeof ali); std::memcpy(w.ari, ari, sizeof ari);
  const double alb1[4][5] = {{0.0, 0.0, 4.725, 9.45, 0.0},
                             {0.0, 1.94578125, 7.783125, 1.94578125, 0.0},
                             {0.2964375, 4.743, 10.67175, 4.743, 0.2964375},
                             {0.451390625, 4.63271875, 9.38146875, 4.63271875, 0.451390625}};
  const double arb1[4][7] = {{0.0, 0.0, 0.0, -11.8125, 9.45, 2.3625, 0.0},
                             {0.0, 0.0, -5.83734375, 0.0, 5.83734375, 0.0, 0.0},
                             {0.0, -1.23515625, -7.905, 0.0, 7.905, 1.23515625, 0.0},
                             {-0.015, -1.53, -6.66984375, 0.0, 6.66984375, 1.53, 0.015}};
  for (int j = 0; j < 4; j++) {
    for (int l = 0; l < 5; l++) w.alb1[j][l] = alb1[j][l];
    for (int l = 0; l < 7; l++) w.arb1[j][l] = arb1[j][l];
  }
  mirror_rows(w, -1.0);
  set_symm_rows(w, -1, +1);  // :256-259
  const double XL[4][5] = {{0.0, 0.0, 6.0, 0.0, 0.0}, {0.0, 2.25, 6.0, 2.25, 0.0}, {0.3, 3.0, 6.0, 3.0, 0.3},
                           {0.3, 3.0, 6.0, 3.0, 0.3}};  // :261-264
  const double XR[4][9] = {{-0.1, 0.9, -4.5, 0.0, 4.5, -0.9, 0.1},
                           {0.0125, -0.3, -4.6875, 0.0, 4.6875, 0.3, -0.0125},
                           {-0.01, -1.01, -4.25, 0.0, 4.25, 1.01, 0.01},
                           {-0.01, -1.01, -4.25, 0.0, 4.25, 1.01, 0.01}};  // :269-272
  set_xtnd_rows(w, XL, XR, -1.0);
  return w;
}

// c10d8: stencils.f90:515-621 (interior :519-526,:573-574, one-sided :576-591)
Weight make_c10d8() {
  Weight w{};
  w.nol = 2; w.nor = 4; w.ncl = 5; w.ncr = 9; w.nbc1 = 4; w.nbc2 = 4;
  w.null_option = 0; w.implicit_op = true;
  const double zeta = 29.0, alpha = 14.0, beta = 1.5;
  const double aa = 4200.0, bb = -3360.0, cc = 1680.0, dd = -480.0, ee = 60.0;
  const double alpha2 = beta + alpha, zeta1 = alpha + zeta, alpha1 = beta + alpha;
  const double dd4 = ee + dd, cc3 = dd + cc, bb3 = ee + bb, bb2 = cc + bb, aa2 = dd + aa,
               b22 = ee + bb, aa1 = bb + aa, bb1 = cc + bb, cc1 = dd + cc, dd1 = ee + dd;
  const double ali[5] = {beta, alpha, zeta, alpha, beta};
  const double ari[9] = {ee, dd, cc, bb, aa, bb, cc, dd, ee};
  std::memcpy(w.ali, ali, sizeof ali); std::memcpy(w.ari, ari, sizeof ari);
  const double alb1[4][5] = {{0.0, 0.0, zeta1, alpha1, beta},
                             {0.0, alpha2, zeta, alpha, beta},
                             {beta, alpha, zeta, alpha, beta},
                             {beta, alpha, zeta, alpha, beta}};
  const double arb1[4][9] = {{0.0, 0.0, 0.0, 0.0, aa1, bb1, cc1, dd1, ee},
                             {0.0, 0.0, 0.0, bb2, aa2, b22, cc, dd, ee},
                             {0.0, 0.0, cc3, bb3, aa, bb, cc, dd, ee},
                             {0.0, dd4, cc, bb, aa, bb, cc, dd, ee}};
  for (int j = 0; j < 4; j++) {
    for (int l = 0; l < 5; l++) w.alb1[j][l] = alb1[j][l];
    for (int l = 0; l < 9; l++) w.arb1[j][l] = arb1[j][l];
  }
  mirror_rows(w, 1.0);
  set_symm_rows(w, +1, +1);  // :600-603
  const double XL[4][5] = {{0.0, 0.0, 60.0, 0.0, 0.0}, {0.0, 20.0, 20.0, 20.0, 0.0},
                           {beta, alpha, zeta, alpha, beta}, {beta, alpha, zeta, alpha, beta}};  // :605-608
  set_xtnd_rows(w, XL, nullptr, 1.0);  // arb1(:,1:4,2) = ari (:613-616)
  return w;
}

// c8ff8 (sfspec = 2): stencils.f90:713-835, stored as RHS - LHS (:832-834)
Weight make_c8ff8() {
  Weight w{};
  w.nol = 2; w.nor = 4; w.ncl = 5; w.ncr = 9; w.nbc1 = 4; w.nbc2 = 4;
  w.null_option = 1; w.implicit_op = true;
  const double beta = 1.6688e-1, alpha = 6.6624e-1, zeta = 1.0;
  const double aa = 9.9965e-1, bb = 6.6652e-1, cc = 1.6674e-1, dd = 4.0e-5, ee = -5.0e-6;
  const double ali[5] = {beta, alpha, zeta, alpha, beta};
  const double ari[9] = {ee, dd, cc, bb, aa, bb, cc, dd, ee};
  std::memcpy(w.ali, ali, sizeof ali); std::memcpy(w.ari, ari, sizeof ari);
  const double alb1[4][5] = {{0.0, 0.0, 1.0, 0.0, 0.0},
                             {0.0, 4.997e-1, 1.0, 4.997e-1, 0.0},
                             {1.6688e-1, 6.6624e-1, 1.0, 6.6624e-1, 1.6688e-1},
                             {1.6688e-1, 6.6624e-1, 1.0, 6.6624e-1, 1.6688e-1}};
  const double arb1[4][9] = {
      {0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0},
      {0.0, 0.0, 0.0, 4.9985e-1, 9.997e-1, 4.9985e-1, 0.0, 0.0, 0.0},
      {0.0, 0.0, 1.668e-1, 6.6656e-1, 9.9952e-1, 6.6656e-1, 1.668e-1, 0.0, 0.0},
      {0.0, 4.0e-5, 1.6672e-1, 6.6652e-1, 9.9968e-1, 6.6652e-1, 1.6672e-1, 4.0e-5, 0.0}};
  for (int j = 0; j < 4; j++) {
    for (int l = 0; l < 5; l++) w.alb1[j][l] = alb1[j][l];
    for (int l = 0; l < 9; l++) w.arb1[j][l] = arb1[j][l];
  }
  mirror_rows(w, 1.0);
  set_symm_rows(w, +1, +1);  // :810-813
  // the extended-data rows are commented out in the reference (:814-826), so
  // its code-2 rows are never set; this restatement gives them the one-sided
  // rows (the product does the same)
  for (int j = 0; j < 4; j++) {
    for (int l = 0; l < 5; l++) { w.xlb1[3][j][l] = w.alb1[j][l]; w.xlb2[3][j][l] = w.alb2[j][l]; }
    for (int l = 0; l < 9; l++) { w.xrb1[3][j][l] = w.arb1[j][l]; w.xrb2[3][j][l] = w.arb2[j][l]; }
  }
  // difference form: ari(3:7) -= ali(1:5), same for every boundary row (:832-834)
  for (int l = 0; l < 5; l++) w.ari[2 + l] -= w.ali[l];
  for (int j = 0; j < 4; j++)
    for (int l = 0; l < 5; l++) {
      w.arb1[j][2 + l] -= w.alb1[j][l];
      w.arb2[j][2 + l] -= w.alb2[j][l];
      for (int c = 0; c < 4; c++) {
        w.xrb1[c][j][2 + l] -= w.xlb1[c][j][l];
        w.xrb2[c][j][2 + l] -= w.xlb2[c][j][l];
      }
    }
  return w;
}

// cgfs4 (gfspec = 6): stencils.f90:1387-1476, explicit, difference form (:1472-1475)
Weight make_cgfs4() {
  Weight w{};
  w.nol = 0; w.nor = 4; w.ncl = 1; w.ncr = 9; w.nbc1 = 4; w.nbc2 = 4;
  w.null_option = 1; w.implicit_op = false;
  const double agau = 3565.0 / 10368.0, bgau = 3091.0 / 12960.0, cgau = 1997.0 / 25920.0,
               dgau = 149.0 / 12960.0, egau = 107.0 / 103680.0;
  const double dg14 = dgau + egau, cg13 = cgau + dgau, bg23 = bgau + egau, bg12 = bgau + cgau,
               ag22 = agau + dgau, bg32 = bgau + egau, ag11 = agau + bgau, bg21 = bgau + cgau,
               cg31 = cgau + dgau, dg41 = dgau + egau;
  w.ali[0] = 1.0;
  const double ari[9] = {egau, dgau, cgau, bgau, agau, bgau, cgau, dgau, egau};
  std::memcpy(w.ari, ari, sizeof ari);
  const double arb1[4][9] = {{0.0, 0.0, 0.0, 0.0, ag11, bg21, cg31, dg41, egau},
                             {0.0, 0.0, 0.0, bg12, ag22, bg32, cgau, dgau, egau},
                             {0.0, 0.0, cg13, bg23, agau, bgau, cgau, dgau, egau},
                             {0.0, dg14, cgau, bgau, agau, bgau, cgau, dgau, egau}};
  for (int j = 0; j < 4; j++) {
    w.alb1[j][0] = 1.0;
    for (int l = 0; l < 9; l++) w.arb1[j][l] = arb1[j][l];
  }
  mirror_rows(w, 1.0);
  set_symm_rows(w, +1, +1);  // :1451-1454
  set_xtnd_rows(w, nullptr, nullptr, 1.0);  // :1456-1467: LHS 1, RHS interior
  // :1468 takes the first upper row from the reversed fourth one-sided row
  for (int l = 0; l < 9; l++) w.xrb2[3][0][l] = w.arb1[3][8 - l];
  // difference form (:1472-1475)
  w.ari[4] -= w.ali[0];
  for (int j = 0; j < 4; j++) {
    w.arb1[j][4] -= w.alb1[j][0];
    w.arb2[j][4] -= w.alb2[j][0];
    for (int c = 0; c < 4; c++) {
      w.xrb1[c][j][4] -= w.xlb1[c][j][0];
      w.xrb2[c][j][4] -= w.xlb2[c][j][0];
    }
  }
  return w;
}

// c10d2: stencils.f90:358-428 (compact 10th-order second derivative)
Weight make_c10d2() {
  Weight w{};
  w.nol = 2; w.nor = 3; w.ncl = 5; w.ncr = 7; w.nbc1 = 4; w.nbc2 = 4; w.null_option = 0;
  w.implicit_op = true;
  const double ali[5] = {387.0, 6012.0, 16182.0, 6012.0, 387.0};
  const double ari[7] = {79.0, 4671.0, 9585.0, -28670.0, 9585.0, 4671.0, 79.0};
  const double alb1[4][5] = {{0.0, 0.0, 1.0, 11.0, 0.0},
                             {0.0, 1.0, 10.0, 1.0, 0.0},
                             {23.0, 688.0, 2358.0, 688.0, 23.0},
                             {387.0, 6012.0, 16182.0, 6012.0, 387.0}};
  const double arb1[4][7] = {{0.0, 0.0, 0.0, 13.0, -27.0, 15.0, -1.0},
                             {0.0, 0.0, 12.0, -24.0, 12.0, 0.0, 0.0},
                             {0.0, 465.0, 1920.0, -4770.0, 1920.0, 465.0, 0.0},
                             {79.0, 4671.0, 9585.0, -28670.0, 9585.0, 4671.0, 79.0}};
  for (int l = 0; l < 5; l++) w.ali[l] = ali[l];
  for (int l = 0; l < 7; l++) w.ari[l] = ari[l];
  for (int j = 0; j < 4; j++) {
    for (int l = 0; l < 5; l++) w.alb1[j][l] = alb1[j][l];
    for (int l = 0; l < 7; l++) w.arb1[j][l] = arb1[j][l];
  }
  mirror_rows(w, 1.0);  // alb2(:,j) = alb1(ncl:1:-1, 5-j), arb2 likewise (:391-398, :404-411)
  set_symm_rows(w, +1, +1);  // :407-410
  const double XL[4][5] = {{0.0, 0.0, 18.0, 0.0, 0.0}, {0.0, 4.05, 17.1, 4.05, 0.0},
                           {0.387, 6.012, 16.182, 6.012, 0.387}, {0.387, 6.012, 16.182, 6.012, 0.387}};
  const double XR[4][9] = {{0.2, -2.7, 27.0, -49.0, 27.0, -2.7, 0.2},
                           {-0.0575, 2.295, 16.5375, -37.55, 16.5375, 2.295, -0.0575},
                           {0.079, 4.671, 9.585, -28.670, 9.585, 4.671, 0.079},
                           {0.079, 4.671, 9.585, -28.670, 9.585, 4.671, 0.079}};  // :412-427
  set_xtnd_rows(w, XL, XR, 1.0);
  return w;
}

// e4d4: stencils.f90:430-513 (explicit 4th-order fourth derivative).  The
// reference sets three one-sided rows per end (:480-492) while declaring
// nbc1 = nbc2 = 4, so its fourth lower row and last upper row are never set;
// this restatement closes each end with the three defined rows (the upper
// ones are alb2/arb2(:,1..3) of :483-485, :491-493, reversed rows 3, 2, 1).
Weight make_e4d4() {
  Weight w{};
  w.nol = 0; w.nor = 3; w.ncl = 1; w.ncr = 7; w.nbc1 = 3; w.nbc2 = 3; w.null_option = 0;
  w.implicit_op = false;
  const double agau = 28.0 / 3.0, bgau = -6.5, cgau = 2.0, dgau = -1.0 / 6.0;
  const double cgau13 = cgau + dgau, bgau12 = bgau + cgau, agau22 = agau + dgau;
  const double agau11 = agau + bgau, bgau21 = bgau + cgau, cgau31 = cgau + dgau;
  const double ari[7] = {dgau, cgau, bgau, agau, bgau, cgau, dgau};
  const double arb1[3][7] = {{0.0, 0.0, 0.0, agau11, bgau21, cgau31, dgau},
                             {0.0, 0.0, bgau12, agau22, bgau, 0.0, 0.0},
                             {0.0, cgau13, bgau, agau, bgau, cgau, 0.0}};
  w.ali[0] = 1.0;
  for (int l = 0; l < 7; l++) w.ari[l] = ari[l];
  for (int j = 0; j < 3; j++) {
    w.alb1[j][0] = 1.0;
    w.alb2[j][0] = 1.0;
    for (int l = 0; l < 7; l++) w.arb1[j][l] = arb1[j][l];
  }
  for (int j = 0; j < 3; j++)
    for (int l = 0; l < 7; l++) w.arb2[j][l] = w.arb1[2 - j][6 - l];
  // symmetric rows (:496-499); n = size(alb,2) = 4 rows are set there, the
  // fourth (interior) one falls outside this restatement's three boundary rows
  set_symm_rows(w, +1, +1);
  set_xtnd_rows(w, nullptr, nullptr, 1.0);  // :501-512: LHS 1, RHS interior
  return w;
}

// ---------------------------------------------------------------------------
// One operator along one direction: compact_basetype.f90:65-209 (np = 1)
// ---------------------------------------------------------------------------
struct Op1 {
  bool null_op = true, periodic = false, implicit_op = false;
  int kind = 0;  // 1 = d1 evaluator (compact_d1.f90), 3 = r3 (compact_r3.f90), 4 = r4 (compact_r4.f90)
  int null_option = 0, n = 0, nal = 0;
  std::vector<double> al;  // al(i, c) -> al[(c-1)*n + (i-1)], factored
  std::vector<double> ar;  // ar(l, i) -> ar[(i-1)*ncr + (l-1)]
  int ncr = 0;
  int bc1 = 0, bc2 = 0;  // op%bc: boundary codes of the lower and upper end (-1, 0, 1, 2)
  double& AL(int i, int c) { return al[(size_t)(c - 1) * n + (i - 1)]; }
  double AL(int i, int c) const { return al[(size_t)(c - 1) * n + (i - 1)]; }
  double AR(int l, int i) const { return ar[(size_t)(i - 1) * ncr + (l - 1)]; }
};

// bpentLUD1: pentadiagonal.f90:18-39
void bpentLUD1(Op1& o) {
  const int n = o.n;
  for (int i = 1; i <= n - 2; i++) {
    o.AL(i + 1, 2) = o.AL(i + 1, 2) / o.AL(i, 3);
    o.AL(i + 1, 3) = o.AL(i + 1, 3) - o.AL(i, 4) * o.AL(i + 1, 2);
    o.AL(i + 1, 4) = o.AL(i + 1, 4) - o.AL(i, 5) * o.AL(i + 1, 2);
    o.AL(i + 2, 1) = o.AL(i + 2, 1) / o.AL(i, 3);
    o.AL(i + 2, 2) = o.AL(i + 2, 2) - o.AL(i, 4) * o.AL(i + 2, 1);
    o.AL(i + 2, 3) = o.AL(i + 2, 3) - o.AL(i, 5) * o.AL(i + 2, 1);
  }
  o.AL(n, 2) = o.AL(n, 2) / o.AL(n - 1, 3);
  o.AL(n, 3) = o.AL(n, 3) - o.AL(n - 1, 4) * o.AL(n, 2);
  for (int i = 1; i <= n; i++) o.AL(i, 3) = 1.0 / o.AL(i, 3);
}

// ppentLUD1: pentadiagonal.f90:64-135 (cyclic pentadiagonal, bordered LU)
void ppentLUD1(Op1& o) {
  const int N = o.n;
  auto c = [&](int i, int j) -> double& { return o.AL(i, j); };
  const double one = 1.0;
  c(1, 8) = c(1, 1);
  c(1, 9) = c(1, 2);
  c(1, 3) = one / c(1, 3);
  c(1, 6) = c(N - 1, 5) * c(1, 3);
  c(1, 7) = c(N, 4) * c(1, 3);
  c(2, 2) = c(2, 2) * c(1, 3);
  c(2, 3) = c(2, 3) - c(2, 2) * c(1, 4);
  c(2, 4) = c(2, 4) - c(2, 2) * c(1, 5);
  c(2, 8) = -c(2, 2) * c(1, 8);
  c(2, 9) = c(2, 1) - c(2, 2) * c(1, 9);
  c(2, 3) = one / c(2, 3);
  c(2, 6) = -c(1, 6) * c(1, 4) * c(2, 3);
  c(2, 7) = (c(N, 5) - c(1, 7) * c(1, 4)) * c(2, 3);
  for (int K = 3; K <= N - 4; K++) {
    c(K, 1) = c(K, 1) * c(K - 2, 3);
    c(K, 2) = (c(K, 2) - c(K, 1) * c(K - 2, 4)) * c(K - 1, 3);
    c(K, 3) = c(K, 3) - (c(K, 2) * c(K - 1, 4) + c(K, 1) * c(K - 2, 5));
    c(K, 4) = c(K, 4) - c(K, 2) * c(K - 1, 5);
    c(K, 8) = -(c(K, 2) * c(K - 1, 8) + c(K, 1) * c(K - 2, 8));
    c(K, 9) = -(c(K, 2) * c(K - 1, 9) + c(K, 1) * c(K - 2, 9));
    c(K, 3) = one / c(K, 3);
    c(K, 6) = -(c(K - 1, 6) * c(K - 1, 4) + c(K - 2, 6) * c(K - 2, 5)) * c(K, 3);
    c(K, 7) = -(c(K - 1, 7) * c(K - 1, 4) + c(K - 2, 7) * c(K - 2, 5)) * c(K, 3);
  }
  c(N - 3, 1) = c(N - 3, 1) * c(N - 5, 3);
  c(N - 3, 2) = (c(N - 3, 2) - c(N - 3, 1) * c(N - 5, 4)) * c(N - 4, 3);
  c(N - 3, 3) = c(N - 3, 3) - (c(N - 3, 2) * c(N - 4, 4) + c(N - 3, 1) * c(N - 5, 5));
  c(N - 3, 4) = c(N - 3, 4) - c(N - 3, 2) * c(N - 4, 5);
  c(N - 3, 8) = c(N - 3, 5) - (c(N - 3, 2) * c(N - 4, 8) + c(N - 3, 1) * c(N - 5, 8));
  c(N - 3, 9) = -(c(N - 3, 2) * c(N - 4, 9) + c(N - 3, 1) * c(N - 5, 9));
  c(N - 3, 3) = one / c(N - 3, 3);
  c(N - 3, 6) = (c(N - 1, 1) - (c(N - 4, 6) * c(N - 4, 4) + c(N - 5, 6) * c(N - 5, 5))) * c(N - 3, 3);
  c(N - 3, 7) = -(c(N - 4, 7) * c(N - 4, 4) + c(N - 5, 7) * c(N - 5, 5)) * c(N - 3, 3);
  c(N - 2, 1) = c(N - 2, 1) * c(N - 4, 3);
  c(N - 2, 2) = (c(N - 2, 2) - c(N - 2, 1) * c(N - 4, 4)) * c(N - 3, 3);
  c(N - 2, 3) = c(N - 2, 3) - (c(N - 2, 2) * c(N - 3, 4) + c(N - 2, 1) * c(N - 4, 5));
  c(N - 2, 8) = c(N - 2, 4) - (c(N - 2, 2) * c(N - 3, 8) + c(N - 2, 1) * c(N - 4, 8));
  c(N - 2, 9) = c(N - 2, 5) - (c(N - 2, 2) * c(N - 3, 9) + c(N - 2, 1) * c(N - 4, 9));
  c(N - 2, 3) = one / c(N - 2, 3);
  c(N - 2, 6) = (c(N - 1, 2) - c(N - 3, 6) * c(N - 3, 4) - c(N - 4, 6) * c(N - 4, 5)) * c(N - 2, 3);
  c(N - 2, 7) = (c(N, 1) - c(N - 3, 7) * c(N - 3, 4) - c(N - 4, 7) * c(N - 4, 5)) * c(N - 2, 3);
  for (int K = 1; K <= N - 2; K++) {
    c(N - 1, 3) = c(N - 1, 3) - c(K, 6) * c(K, 8);
    c(N - 1, 4) = c(N - 1, 4) - c(K, 6) * c(K, 9);
  }
  c(N - 1, 9) = c(N - 1, 4);
  for (int K = 1; K <= N - 2; K++) c(N, 2) = c(N, 2) - c(K, 7) * c(K, 8);
  c(N - 1, 3) = one / c(N - 1, 3);
  c(N - 1, 7) = c(N, 2) * c(N - 1, 3);
  for (int K = 1; K <= N - 1; K++) c(N, 3) = c(N, 3) - c(K, 7) * c(K, 9);
  c(N, 3) = one / c(N, 3);
}

// setup_compact_op1: compact_basetype.f90:65-170 for np = 1; bc1 / bc2 are
// the op%bc codes of the two ends (compact.f90:77-91)
Op1 setup_op(const Weight& w, int kind, int n, bool periodic, int bc1 = 0, int bc2 = 0) {
  Op1 o;
  o.kind = kind;
  o.bc1 = periodic ? 0 : bc1;
  o.bc2 = periodic ? 0 : bc2;
  o.n = n;
  o.periodic = periodic;
  o.null_option = w.null_option;
  o.implicit_op = w.implicit_op;
  o.ncr = w.ncr;
  o.null_op = (n < 4);  // compact.f90:95-97, compact_basetype.f90:100-104
  if (o.null_op) return o;
  o.nal = periodic ? w.ncl + 4 : w.ncl;
  // gal(1:ncl, i) = ali, gar(:, i) = ari; one-sided rows patched at the ends
  std::vector<double> gal((size_t)o.nal * n, 0.0), gar((size_t)w.ncr * n, 0.0);
  for (int i = 0; i < n; i++) {
    for (int l = 0; l < w.ncl; l++) gal[(size_t)i * o.nal + l] = w.ali[l];
    for (int l = 0; l < w.ncr; l++) gar[(size_t)i * w.ncr + l] = w.ari[l];
  }
  if (!periodic) {  // alb1(:,:,bc(1)) / alb2(:,:,bc(2)) (compact_basetype.f90:126-131)
    for (int j = 0; j < w.nbc1; j++) {
      const double* L = o.bc1 == 0 ? w.alb1[j] : w.xlb1[o.bc1 + 1][j];
      const double* R = o.bc1 == 0 ? w.arb1[j] : w.xrb1[o.bc1 + 1][j];
      for (int l = 0; l < w.ncl; l++) gal[(size_t)j * o.nal + l] = L[l];
      for (int l = 0; l < w.ncr; l++) gar[(size_t)j * w.ncr + l] = R[l];
    }
    for (int j = 0; j < w.nbc2; j++) {
      const int i = n - w.nbc2 + j;
      const double* L = o.bc2 == 0 ? w.alb2[j] : w.xlb2[o.bc2 + 1][j];
      const double* R = o.bc2 == 0 ? w.arb2[j] : w.xrb2[o.bc2 + 1][j];
      for (int l = 0; l < w.ncl; l++) gal[(size_t)i * o.nal + l] = L[l];
      for (int l = 0; l < w.ncr; l++) gar[(size_t)i * w.ncr + l] = R[l];
    }
  }
  o.al.assign((size_t)n * o.nal, 0.0);
  for (int i = 1; i <= n; i++)
    for (int c = 1; c <= o.nal; c++) o.AL(i, c) = gal[(size_t)(i - 1) * o.nal + (c - 1)];
  o.ar = gar;
  if (o.implicit_op) {
    if (periodic) ppentLUD1(o);
    else bpentLUD1(o);
  }
  return o;
}

// ---------------------------------------------------------------------------
// Line evaluators.  v and dv are 1-based views of one line (v[1..n]).
// ---------------------------------------------------------------------------

// d1 RHS: compact_d1.f90:100-193 (periodic halo or one-sided bc = 0 ends)
void rhs_d1(const Op1& o, const double* v, double* dv) {
  const int ax = o.n;
  auto a = [&](int l, int i) { return o.AR(l, i); };
  if (o.periodic) {
    // vbr1(1:3) = v(ax-2:ax), vbr2(1:3) = v(1:3)  (:100-110)
    const double b11 = v[ax - 2], b12 = v[ax - 1], b13 = v[ax];
    const double b21 = v[1], b22 = v[2], b23 = v[3];
    dv[1] = a(5, 1) * (v[2] - b13) + a(6, 1) * (v[3] - b12) + a(7, 1) * (v[4] - b11);
    dv[2] = a(5, 2) * (v[3] - v[1]) + a(6, 2) * (v[4] - b13) + a(7, 2) * (v[5] - b12);
    dv[3] = a(5, 3) * (v[4] - v[2]) + a(6, 3) * (v[5] - v[1]) + a(7, 3) * (v[6] - b13);
    for (int i = 4; i <= ax - 3; i++)
      dv[i] = a(5, i) * (v[i + 1] - v[i - 1]) + a(6, i) * (v[i + 2] - v[i - 2]) + a(7, i) * (v[i + 3] - v[i - 3]);
    dv[ax - 2] = a(5, ax - 2) * (v[ax - 1] - v[ax - 3]) + a(6, ax - 2) * (v[ax] - v[ax - 4]) + a(7, ax - 2) * (b21 - v[ax - 5]);
    dv[ax - 1] = a(5, ax - 1) * (v[ax] - v[ax - 2]) + a(6, ax - 1) * (b21 - v[ax - 3]) + a(7, ax - 1) * (b22 - v[ax - 4]);
    dv[ax] = a(5, ax) * (b21 - v[ax - 1]) + a(6, ax) * (b22 - v[ax - 2]) + a(7, ax) * (b23 - v[ax - 3]);
    return;
  }
  if (o.bc1 == -1) {  // antisymmetric (:121-128)
    double s = 0.0;
    for (int l = 4; l <= 7; l++) s += a(l, 1) * v[l - 3];
    dv[1] = s;
    s = 0.0;
    for (int l = 3; l <= 7; l++) s += a(l, 2) * v[l - 2];
    dv[2] = s;
    s = 0.0;
    for (int l = 2; l <= 7; l++) s += a(l, 3) * v[l - 1];
    dv[3] = s;
  } else {  // one-sided / symmetric / extended: difference form (:131-139)
    double s = 0.0;
    for (int l = 5; l <= 7; l++) s += a(l, 1) * (v[l - 3] - v[1]);
    dv[1] = s;
    s = 0.0;
    for (int l = 4; l <= 7; l++) s += a(l, 2) * (v[l - 2] - v[1]);
    dv[2] = s;
    dv[3] = a(5, 3) * (v[4] - v[2]) + a(6, 3) * (v[5] - v[1]) + a(7, 3) * (v[6] - v[1]);
  }
  for (int i = 4; i <= ax - 3; i++)
    dv[i] = a(5, i) * (v[i + 1] - v[i - 1]) + a(6, i) * (v[i + 2] - v[i - 2]) + a(7, i) * (v[i + 3] - v[i - 3]);
  if (o.bc2 == -1) {  // antisymmetric (:163-170)
    double s = 0.0;
    for (int l = 1; l <= 6; l++) s += a(l, ax - 2) * v[ax - 6 + l];
    dv[ax - 2] = s;
    s = 0.0;
    for (int l = 1; l <= 5; l++) s += a(l, ax - 1) * v[ax - 5 + l];
    dv[ax - 1] = s;
    s = 0.0;
    for (int l = 1; l <= 4; l++) s += a(l, ax) * v[ax - 4 + l];
    dv[ax] = s;
  } else {
    dv[ax - 2] = a(1, ax - 2) * (v[ax - 5] - v[ax]) + a(2, ax - 2) * (v[ax - 4] - v[ax]) + a(3, ax - 2) * (v[ax - 3] - v[ax - 1]);
    double s = 0.0;
    for (int l = 1; l <= 4; l++) s += a(l, ax - 1) * (v[ax - 5 + l] - v[ax]);
    dv[ax - 1] = s;
    s = 0.0;
    for (int l = 1; l <= 3; l++) s += a(l, ax) * (v[ax - 4 + l] - v[ax]);
    dv[ax] = s;
  }
}

// r4 RHS: compact_r4.f90:77-193 (9-point difference form)
void rhs_r4(const Op1& o, const double* v, double* dv) {
  const int ax = o.n;
  auto a = [&](int l, int i) { return o.AR(l, i); };
  if (o.periodic) {
    // vbr1(1:4) = v(ax-3:ax), vbr2(1:4) = v(1:4)  (:97-104)
    double b1[5], b2[5];
    for (int q = 1; q <= 4; q++) { b1[q] = v[ax - 4 + q]; b2[q] = v[q]; }
    for (int i = 1; i <= 4; i++) {
      // sum(ar(1:5-i,i)*(vbr1(i:4)-v(i))) + sum(ar(6-i:9,i)*(v(1:4+i)-v(i)))
      double s1 = 0.0, s2 = 0.0;
      for (int l = 1; l <= 5 - i; l++) s1 += a(l, i) * (b1[i - 1 + l] - v[i]);
      for (int l = 6 - i; l <= 9; l++) s2 += a(l, i) * (v[l + i - 5] - v[i]);
      dv[i] = s1 + s2;
    }
  } else if (o.bc1 == -1) {
    for (int i = 1; i <= 4; i++) {
      // sum(ar(6-i:9,i)*v(1:4+i))  (:108-117, antisymmetric)
      double s = 0.0;
      for (int l = 6 - i; l <= 9; l++) s += a(l, i) * v[l + i - 5];
      dv[i] = s;
    }
  } else {
    for (int i = 1; i <= 4; i++) {
      // sum(ar(7-i:9,i)*(v(2:4+i)-v(1)))  (:120-125)
      double s = 0.0;
      for (int l = 7 - i; l <= 9; l++) s += a(l, i) * (v[l + i - 5] - v[1]);
      dv[i] = s;
    }
  }
  for (int i = 5; i <= ax - 4; i++) {
    double s = 0.0;
    const double vc = v[i];
    for (int l = 1; l <= 9; l++) s = s + (v[l + i - 5] - vc) * a(l, i);
    dv[i] = s;
  }
  if (o.periodic) {
    double b2[5];
    for (int q = 1; q <= 4; q++) b2[q] = v[q];
    for (int q = 3; q >= 0; q--) {
      const int i = ax - q;
      // sum(ar(1:5+q,i)*(v(i-4:ax)-v(i))) + sum(ar(6+q:9,i)*(vbr2(1:4-q)-v(i)))  (:180-189)
      double s1 = 0.0, s2 = 0.0;
      for (int l = 1; l <= 5 + q; l++) s1 += a(l, i) * (v[i - 5 + l] - v[i]);
      for (int l = 6 + q; l <= 9; l++) s2 += a(l, i) * (b2[l - 5 - q] - v[i]);
      dv[i] = s1 + s2;
    }
  } else if (o.bc2 == -1) {
    for (int q = 3; q >= 0; q--) {
      const int i = ax - q;
      // sum(ar(1:5+q,i)*v(i-4:ax))  (:154-163, antisymmetric)
      double s = 0.0;
      for (int l = 1; l <= 5 + q; l++) s += a(l, i) * v[i - 5 + l];
      dv[i] = s;
    }
  } else {
    for (int q = 3; q >= 0; q--) {
      const int i = ax - q;
      // sum(ar(1:4+q,i)*(v(i-4:ax-1)-v(ax)))  (:166-171)
      double s = 0.0;
      for (int l = 1; l <= 4 + q; l++) s += a(l, i) * (v[i - 5 + l] - v[ax]);
      dv[i] = s;
    }
  }
}

// bpentLUS3x for one line: pentadiagonal.f90:629-651
void solve_b(const Op1& o, double* r) {
  const int n = o.n;
  for (int i = 1; i <= n - 2; i++) {
    r[i + 1] = r[i + 1] - r[i] * o.AL(i + 1, 2);
    r[i + 2] = r[i + 2] - r[i] * o.AL(i + 2, 1);
  }
  r[n] = (r[n] - r[n - 1] * o.AL(n, 2)) * o.AL(n, 3);
  r[n - 1] = (r[n - 1] - o.AL(n - 1, 4) * r[n]) * o.AL(n - 1, 3);
  for (int i = n - 2; i >= 1; i--)
    r[i] = (r[i] - o.AL(i, 4) * r[i + 1] - o.AL(i, 5) * r[i + 2]) * o.AL(i, 3);
}

// ppentLUS3x for one line: pentadiagonal.f90:654-684
void solve_p(const Op1& o, double* r) {
  const int N = o.n;
  auto c = [&](int i, int j) { return o.AL(i, j); };
  r[2] = r[2] - c(2, 2) * r[1];
  double tmp1 = c(1, 6) * r[1] + c(2, 6) * r[2];
  double tmp2 = c(1, 7) * r[1] + c(2, 7) * r[2];
  for (int i = 3; i <= N - 2; i++) {
    r[i] = r[i] - (c(i, 2) * r[i - 1] + c(i, 1) * r[i - 2]);
    tmp1 = tmp1 + c(i, 6) * r[i];
    tmp2 = tmp2 + c(i, 7) * r[i];
  }
  r[N - 1] = r[N - 1] - tmp1;
  r[N] = (r[N] - tmp2 - c(N - 1, 7) * r[N - 1]) * c(N, 3);
  r[N - 1] = (r[N - 1] - c(N - 1, 9) * r[N]) * c(N - 1, 3);
  r[N - 2] = (r[N - 2] - c(N - 2, 8) * r[N - 1] - c(N - 2, 9) * r[N]) * c(N - 2, 3);
  r[N - 3] = (r[N - 3] - (c(N - 3, 4) * r[N - 2] + c(N - 3, 8) * r[N - 1] + c(N - 3, 9) * r[N])) * c(N - 3, 3);
  for (int i = N - 4; i >= 1; i--)
    r[i] = (r[i] - (c(i, 4) * r[i + 1] + c(i, 5) * r[i + 2] + c(i, 8) * r[N - 1] + c(i, 9) * r[N])) * c(i, 3);
}

// r3 RHS: compact_r3.f90:72-157 (np = 1).  Periodic lines take the wrapped
// points as ghost data (:86-89); non-periodic ones take zeros (:90-105), whose
// closure weights vanish.  Fortran SUM adds left to right.
void rhs_r3(const Op1& o, const double* v, double* dv) {
  const int ax = o.n;
  auto a = [&](int l, int i) { return o.AR(l, i); };
  double vbr1[4] = {0.0, 0.0, 0.0, 0.0}, vbr2[4] = {0.0, 0.0, 0.0, 0.0};  // 1-based
  if (o.periodic) {
    for (int q = 1; q <= 3; q++) {
      vbr1[q] = v[ax - 3 + q];
      vbr2[q] = v[q];
    }
  }
  auto part = [&](int i, int l0, int l1, auto val) {  // sum(ar(l0:l1, i) * (val(l) - v(i)))
    double s = 0.0;
    for (int l = l0; l <= l1; l++) s += a(l, i) * (val(l) - v[i]);
    return s;
  };
  auto sumr = [&](int i) {  // sum(op%ar, dim=1) (:106)
    double t = 0.0;
    for (int l = 1; l <= 7; l++) t += a(l, i);
    return t;
  };
  // :109-112 (antisymmetric: + sumr(i) v(i)), :116-119
  dv[1] = part(1, 1, 3, [&](int l) { return vbr1[l]; }) + part(1, 4, 7, [&](int l) { return v[l - 3]; });
  dv[2] = part(2, 1, 2, [&](int l) { return vbr1[l + 1]; }) + part(2, 3, 7, [&](int l) { return v[l - 2]; });
  dv[3] = part(3, 1, 1, [&](int l) { return vbr1[l + 2]; }) + part(3, 2, 7, [&](int l) { return v[l - 1]; });
  if (!o.periodic && o.bc1 == -1)
    for (int i = 1; i <= 3; i++) dv[i] = dv[i] + sumr(i) * v[i];
  for (int i = 4; i <= ax - 3; i++) dv[i] = part(i, 1, 7, [&](int l) { return v[i - 4 + l]; });  // :137-143
  // :154-156
  dv[ax - 2] = part(ax - 2, 1, 6, [&](int l) { return v[ax - 6 + l]; }) +
               part(ax - 2, 7, 7, [&](int l) { return vbr2[l - 6]; });
  dv[ax - 1] = part(ax - 1, 1, 5, [&](int l) { return v[ax - 5 + l]; }) +
               part(ax - 1, 6, 7, [&](int l) { return vbr2[l - 5]; });
  dv[ax] = part(ax, 1, 4, [&](int l) { return v[ax - 4 + l]; }) + part(ax, 5, 7, [&](int l) { return vbr2[l - 4]; });
  if (!o.periodic && o.bc2 == -1)  // :146-151
    for (int i = ax - 2; i <= ax; i++) dv[i] = dv[i] + sumr(i) * v[i];
}

// Full line evaluation (eval_compact_op1x_d1 / _r3 / _r4), np = 1, then the
// metric scale when scale != 0 (d1: dx, compact_operators.f90:41-46; d2: dx**2, :149-152).
void eval_line(const Op1& o, const double* v, double* dv, double scale) {
  if (o.kind == 1) rhs_d1(o, v, dv);
  else if (o.kind == 3) rhs_r3(o, v, dv);
  else rhs_r4(o, v, dv);
  if (o.implicit_op) {
    if (o.periodic) solve_p(o, dv);
    else solve_b(o, dv);
  }
  if (o.null_option == 1)
    for (int i = 1; i <= o.n; i++) dv[i] = dv[i] + v[i];
  if (scale != 0.0)
    for (int i = 1; i <= o.n; i++) dv[i] = dv[i] / scale;
}

}  // namespace

// ---------------------------------------------------------------------------
// Handle: one grid (one pyranda patch), all operators for x, y, z.
// ---------------------------------------------------------------------------
// Mesh fields of spherical and curvilinear grids (mesh.f90:35-50): coordinates,
// d1 d2 d3, GridLen, CellVol, the filtered cell volumes, det J and the inverse
// Jacobian rows dA/dx dA/dy dA/dz, dB/.., dC/.. (curvilinear only).
enum { MF_X, MF_Y, MF_Z, MF_D1, MF_D2, MF_D3, MF_GL, MF_CV, MF_CVS, MF_CVG, MF_DET, MF_J0, MF_COUNT = MF_J0 + 9 };

struct og_handle {
  int n[3];
  int periodic[3];
  double d[3];     // patch spacing dx, dy, dz (patch.f90:83-85)
  double dmesh[3]; // mesh d1, d2, d3 (mesh.f90:192-209)
  double x1f[3];   // lower face coordinates (parcop.f90:51-56)
  int bc[3][2];    // 0 NONE, 1 SYMM, 2 XTND per end (pyrandaMPI.py:101-131)
  int symm[3];     // isym = -1 where a direction has a SYMM end (patch.f90:89-91)
  int coordsys;    // 0 Cartesian, 1 cylindrical, 2 spherical, 3 curvilinear, 4 spherical ratio-zoned
  Op1 d1[3], d8[3], sf[3], gf[3], d2[3], d4[3];
  Op1 anti[6][3];  // operator n = 2 of a SYMM direction (mbc = -1, compact.f90:80-85)
  std::vector<double> mf[MF_COUNT];  // coordsys 2, 3, 4
};

namespace {

enum { OP_D1 = 0, OP_D8 = 1, OP_SF = 2, OP_GF = 3, OP_D2 = 4, OP_D4 = 5 };

const Op1& pick(const og_handle* h, int op, int dir, int sym = 1) {
  if (sym == -1 && h->symm[dir]) return h->anti[op][dir];
  switch (op) {
    case OP_D1: return h->d1[dir];
    case OP_D8: return h->d8[dir];
    case OP_SF: return h->sf[dir];
    case OP_D2: return h->d2[dir];
    case OP_D4: return h->d4[dir];
    default: return h->gf[dir];
  }
}

// Apply one operator along direction dir over a Fortran-ordered (nx,ny,nz) field.
// Null ops follow compact_operators.f90: derivatives give 0 (:24-29, :288-294),
// filters copy (:396-401).
void apply_op(const og_handle* h, const Op1& o, int op, int dir, const double* in, double* out) {
  const int nx = h->n[0], ny = h->n[1], nz = h->n[2];
  const size_t npts = (size_t)nx * ny * nz;
  if (o.null_op) {
    if (op == OP_SF || op == OP_GF) std::memcpy(out, in, npts * sizeof(double));
    else std::memset(out, 0, npts * sizeof(double));
    return;
  }
  const double scale = (op == OP_D1) ? h->d[dir] : ((op == OP_D2) ? h->d[dir] * h->d[dir] : 0.0);
  const int n = h->n[dir];
  size_t stride, nlines;
  if (dir == 0) { stride = 1; nlines = (size_t)ny * nz; }
  else if (dir == 1) { stride = nx; nlines = (size_t)nx * nz; }
  else { stride = (size_t)nx * ny; nlines = (size_t)nx * ny; }
  const int B = 8;  // lines gathered together for the strided directions
  const long nblk = (long)((nlines + B - 1) / B);
#pragma omp parallel
  {
    std::vector<double> vb((size_t)B * (n + 1)), db((size_t)B * (n + 1));
#pragma omp for schedule(static)
    for (long blk = 0; blk < nblk; blk++) {
      const size_t l0 = (size_t)blk * B;
      const int nb = (int)std::min<size_t>(B, nlines - l0);
      size_t base[8];
      for (int b = 0; b < nb; b++) {
        const size_t L = l0 + b;
        if (dir == 0) base[b] = L * nx;
        else if (dir == 1) base[b] = (L / nx) * (size_t)nx * ny + (L % nx);
        else base[b] = L;
      }
      for (int i = 0; i < n; i++)
        for (int b = 0; b < nb; b++) vb[(size_t)b * (n + 1) + i + 1] = in[base[b] + i * stride];
      for (int b = 0; b < nb; b++) eval_line(o, &vb[(size_t)b * (n + 1)], &db[(size_t)b * (n + 1)], scale);
      for (int i = 0; i < n; i++)
        for (int b = 0; b < nb; b++) out[base[b] + i * stride] = db[(size_t)b * (n + 1) + i + 1];
    }
  }
}

void apply_dir(const og_handle* h, int op, int dir, const double* in, double* out, int sym = 1) {
  apply_op(h, pick(h, op, dir, sym), op, dir, in, out);
}

}  // namespace

namespace {
// mesh.f90:172-175: xgrid(i) = x1 + REAL(2*i-1)*half*dx (the radius on cylindrical grids)
double xgrid(const og_handle* h, size_t p) {
  const int i = (int)(p % (size_t)h->n[0]) + 1;
  return h->x1f[0] + (double)(2 * i - 1) * 0.5 * h->d[0];
}
// mesh.f90:213-225: CellVol of a cylindrical grid (d1 = dx, d2 = r dy, d3 = dz)
double cellvol_cyl(const og_handle* h, size_t p) {
  const double pi = std::acos(-1.0), r = xgrid(h, p);
  if (h->n[1] == 1) return h->d[0] * 2.0 * pi * r * h->d[2];
  return h->d[0] * (r * h->d[1]) * h->d[2];
}
int isym_pow(const og_handle* h, int d, int p) { return (h->symm[d] && (p & 1)) ? -1 : 1; }

size_t npts_of(const og_handle* h) { return (size_t)h->n[0] * h->n[1] * h->n[2]; }

// mesh d1, d2, d3 at point p (the ring scales, mesh.f90:192-358): constants on
// Cartesian grids, d2 = r dy on cylindrical grids, fields otherwise
double mesh_d(const og_handle* h, int dir, size_t p) {
  if (h->coordsys == 0) return h->dmesh[dir];
  if (h->coordsys == 1) return dir == 1 ? xgrid(h, p) * h->d[1] : h->d[dir];
  return h->mf[MF_D1 + dir][p];
}

// mesh.f90:373-386: the filtered cell volumes that divide a filtered
// volume-weighted field (spherical and curvilinear grids; CellVol otherwise)
void cell_bar(og_handle* h) {
  const size_t np = npts_of(h);
  h->mf[MF_CVS].assign(np, 0.0);
  h->mf[MF_CVG].assign(np, 0.0);
  if (h->coordsys == 2 || h->coordsys == 3) {
    std::vector<double> tmp(np);
    apply_dir(h, OP_SF, 0, h->mf[MF_CV].data(), h->mf[MF_CVS].data());
    apply_dir(h, OP_SF, 1, h->mf[MF_CVS].data(), tmp.data());
    apply_dir(h, OP_SF, 2, tmp.data(), h->mf[MF_CVS].data());
    apply_dir(h, OP_GF, 0, h->mf[MF_CV].data(), h->mf[MF_CVG].data());
    apply_dir(h, OP_GF, 1, h->mf[MF_CVG].data(), tmp.data());
    apply_dir(h, OP_GF, 2, tmp.data(), h->mf[MF_CVG].data());
  } else {
    h->mf[MF_CVS] = h->mf[MF_CV];
    h->mf[MF_CVG] = h->mf[MF_CV];
  }
}

// Spherical grids, x = radius, y = theta, z = phi (mesh.f90:169-186, :227-244);
// coordsys 4 zones the radius by a constant ratio (:180-186, :231)
void sph_mesh(og_handle* h) {
  const int nx = h->n[0], ny = h->n[1], nz = h->n[2];
  const size_t np = npts_of(h);
  for (int q = MF_X; q <= MF_CV; q++) h->mf[q].assign(np, 0.0);
  const double pi = std::acos(-1.0), dx = h->d[0], dy = h->d[1], dz = h->d[2];
  double Csp = 0.0, Asp = 0.0;
  if (h->coordsys == 4) {
    Csp = std::log((double)(nx - 1) * dx) / (dy * (double)(nx - 1));
    Asp = (h->x1f[0] + dx / 2.0) / std::exp(Csp * dy);
  }
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const size_t p = ((size_t)k * ny + j) * nx + i;
        double r = h->x1f[0] + (double)(2 * (i + 1) - 1) * 0.5 * dx;
        const double th = h->x1f[1] + (double)(2 * (j + 1) - 1) * 0.5 * dy;
        const double ph = h->x1f[2] + (double)(2 * (k + 1) - 1) * 0.5 * dz;
        if (h->coordsys == 4) r = Asp * std::exp(Csp * dy * (double)(i + 1));
        double d1 = dx;
        const double d2 = r * dy, d3 = r * std::sin(th) * dz;
        if (h->coordsys == 4) d1 = Csp * r * dy;
        double cv = d1 * d2 * d3, gl = std::min(std::min(d1, d2), d3);
        if (ny == 1 && nz == 1) {
          cv = d1 * 4.0 * pi * (r * r);
          gl = d1;
        }
        h->mf[MF_X][p] = r;
        h->mf[MF_Y][p] = th;
        h->mf[MF_Z][p] = ph;
        h->mf[MF_D1][p] = d1;
        h->mf[MF_D2][p] = d2;
        h->mf[MF_D3][p] = d3;
        h->mf[MF_GL][p] = gl;
        h->mf[MF_CV][p] = cv;
      }
  cell_bar(h);
}

// General curvilinear grids (mesh.f90:245-358): the Jacobian of the supplied
// coordinates by the first-derivative operator (a non-periodic one with
// one-sided ends when the coordinates are not periodic, mesh.f90:246-307),
// its determinant and inverse, the physical spacings, CellVol and GridLen.
void curv_mesh(og_handle* h, const double* x, const double* y, const double* z, int mesh_per) {
  const size_t np = npts_of(h);
  for (int q = 0; q < MF_COUNT; q++) h->mf[q].assign(np, 0.0);
  std::memcpy(h->mf[MF_X].data(), x, np * sizeof(double));
  std::memcpy(h->mf[MF_Y].data(), y, np * sizeof(double));
  std::memcpy(h->mf[MF_Z].data(), z, np * sizeof(double));
  // J[c][d] = d(coordinate c)/d(direction d), stored in the inverse-Jacobian slots first
  const Weight wd1 = make_c10d1();
  const double* xs[3] = {x, y, z};
  for (int d = 0; d < 3; d++) {
    Op1 custom;
    if (mesh_per) custom = setup_op(wd1, 1, h->n[d], false, 0, 0);
    for (int c = 0; c < 3; c++) {
      double* dst = h->mf[MF_J0 + 3 * c + d].data();
      if (mesh_per) apply_op(h, custom, OP_D1, d, xs[c], dst);
      else apply_dir(h, OP_D1, d, xs[c], dst);
    }
  }
  const double dA = h->d[0], dB = h->d[1], dC = h->d[2];
  for (size_t p = 0; p < np; p++) {
    double J[9];
    for (int q = 0; q < 9; q++) J[q] = h->mf[MF_J0 + q][p];
    double &dxdA = J[0], &dxdB = J[1], &dxdC = J[2], &dydA = J[3], &dydB = J[4], &dydC = J[5], &dzdA = J[6],
           &dzdB = J[7], &dzdC = J[8];
    if (h->n[0] == 1) dxdA = 1.0;
    if (h->n[1] == 1) dydB = 1.0;
    if (h->n[2] == 1) dzdC = 1.0;
    const double det = -dxdC * dydB * dzdA + dxdB * dydC * dzdA + dxdC * dydA * dzdB - dxdA * dydC * dzdB -
                       dxdB * dydA * dzdC + dxdA * dydB * dzdC;
    double* o[9];
    for (int q = 0; q < 9; q++) o[q] = &h->mf[MF_J0 + q][p];
    *o[0] = (-dydC * dzdB + dydB * dzdC) / det;  // dA/dx
    *o[1] = (dxdC * dzdB - dxdB * dzdC) / det;   // dA/dy
    *o[2] = (-dxdC * dydB + dxdB * dydC) / det;  // dA/dz
    *o[3] = (dydC * dzdA - dydA * dzdC) / det;   // dB/dx
    *o[4] = (-dxdC * dzdA + dxdA * dzdC) / det;  // dB/dy
    *o[5] = (dxdC * dydA - dxdA * dydC) / det;   // dB/dz
    *o[6] = (-dydB * dzdA + dydA * dzdB) / det;  // dC/dx
    *o[7] = (dxdB * dzdA - dxdA * dzdB) / det;   // dC/dy
    *o[8] = (-dxdB * dydA + dxdA * dydB) / det;  // dC/dz
    const double d1 = std::sqrt((dxdA * dA) * (dxdA * dA) + (dydA * dA) * (dydA * dA) + (dzdA * dA) * (dzdA * dA));
    const double d2 = std::sqrt((dxdB * dB) * (dxdB * dB) + (dydB * dB) * (dydB * dB) + (dzdB * dB) * (dzdB * dB));
    const double d3 = std::sqrt((dxdC * dC) * (dxdC * dC) + (dydC * dC) * (dydC * dC) + (dzdC * dC) * (dzdC * dC));
    h->mf[MF_DET][p] = det;
    h->mf[MF_D1][p] = d1;
    h->mf[MF_D2][p] = d2;
    h->mf[MF_D3][p] = d3;
    h->mf[MF_CV][p] = d1 * d2 * d3;
    h->mf[MF_GL][p] = std::min(std::min(d1, d2), d3);
  }
  cell_bar(h);
}

// pyrandaMesh.py:96-108: the coordinates of a curvilinear grid before a mapping
// is supplied are the nodes numpy.linspace(x1, xn, nn) of every direction
void curv_default(og_handle* h, const double* x1, const double* xn) {
  const int nx = h->n[0], ny = h->n[1], nz = h->n[2];
  const size_t np = npts_of(h);
  std::vector<double> c[3];
  for (int q = 0; q < 3; q++) c[q].resize(np);
  auto lin = [&](int d, int i) {
    const int n = h->n[d];
    if (n == 1) return x1[d];
    if (i == n - 1) return xn[d];
    return x1[d] + (double)i * ((xn[d] - x1[d]) / (double)(n - 1));
  };
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const size_t p = ((size_t)k * ny + j) * nx + i;
        c[0][p] = lin(0, i);
        c[1][p] = lin(1, j);
        c[2][p] = lin(2, k);
      }
  curv_mesh(h, c[0].data(), c[1].data(), c[2].data(), 1);
}
}  // namespace

extern "C" {

int og_create2(const int* n, const int* periodic, const int* bc, int coordsys, const double* x1, const double* xn,
               og_handle** out);

// parcop.f90:23-61 (setup: node extents -> faces) + patch.f90:83-85 + mesh.f90:169-211
int og_create(const int* n, const int* periodic, const double* x1, const double* xn, og_handle** out) {
  const int bc[6] = {0, 0, 0, 0, 0, 0};
  return og_create2(n, periodic, bc, 0, x1, xn, out);
}

// The same with the boundary codes of every end (bc[2 d + e]: 0 NONE, 1 SYMM,
// 2 XTND) and the coordinate system (0 Cartesian, 1 cylindrical).
int og_create2(const int* n, const int* periodic, const int* bc, int coordsys, const double* x1, const double* xn,
               og_handle** out) {
  if (!n || !periodic || !bc || !x1 || !xn || !out || coordsys < 0 || coordsys > 4) return 1;
  og_handle* h = new og_handle();
  h->coordsys = coordsys;
  for (int d = 0; d < 3; d++) {
    for (int e = 0; e < 2; e++) h->bc[d][e] = periodic[d] ? 0 : bc[2 * d + e];
    h->symm[d] = (h->bc[d][0] == 1 || h->bc[d][1] == 1) ? 1 : 0;
  }
  for (int d = 0; d < 3; d++) {
    if (n[d] < 1) { delete h; return 1; }
    h->n[d] = n[d];
    h->periodic[d] = periodic[d] ? 1 : 0;
    const double dn = (xn[d] - x1[d]) / (double)std::max(n[d] - 1, 1);
    const double f1 = x1[d] - dn / 2.0, fn = xn[d] + dn / 2.0;
    h->x1f[d] = f1;
    h->d[d] = (fn - f1) / (double)n[d];
  }
  for (int d = 0; d < 3; d++) {
    if (h->n[d] == 1) {
      const int a = (d + 1) % 3, b = (d + 2) % 3;
      const int lo = std::min(a, b), hi = std::max(a, b);
      h->dmesh[d] = std::max(h->d[lo], h->d[hi]);
    } else {
      h->dmesh[d] = h->d[d];
    }
  }
  static const Weight wd1 = make_c10d1(), wd8 = make_c10d8(), wsf = make_c8ff8(), wgf = make_cgfs4();
  static const Weight wd2 = make_c10d2(), wd4 = make_e4d4();
  for (int d = 0; d < 3; d++) {
    const bool per = h->periodic[d] != 0;
    // mbc of operator n (compact.f90:77-91): SYMM ends +1 for n = 1, -1 for n = 2; XTND 2
    int c1[2], c2[2];
    for (int v = 0; v < 2; v++) {
      const int sgn = v == 0 ? 1 : -1;
      c1[v] = h->bc[d][0] == 1 ? sgn : (h->bc[d][0] == 2 ? 2 : 0);
      c2[v] = h->bc[d][1] == 1 ? sgn : (h->bc[d][1] == 2 ? 2 : 0);
    }
    h->d2[d] = setup_op(wd2, 3, h->n[d], per, c1[0], c2[0]);
    h->d4[d] = setup_op(wd4, 3, h->n[d], per, c1[0], c2[0]);
    h->d1[d] = setup_op(wd1, 1, h->n[d], per, c1[0], c2[0]);
    h->d8[d] = setup_op(wd8, 4, h->n[d], per, c1[0], c2[0]);
    h->sf[d] = setup_op(wsf, 4, h->n[d], per, c1[0], c2[0]);
    h->gf[d] = setup_op(wgf, 4, h->n[d], per, c1[0], c2[0]);
    const Weight* ws[6] = {&wd1, &wd8, &wsf, &wgf, &wd2, &wd4};
    const int kinds[6] = {1, 4, 4, 4, 3, 3};
    for (int op = 0; op < 6; op++) h->anti[op][d] = setup_op(*ws[op], kinds[op], h->n[d], per, c1[1], c2[1]);
  }
  if (coordsys == 2 || coordsys == 4) sph_mesh(h);
  if (coordsys == 3) curv_default(h, x1, xn);
  *out = h;
  return 0;
}

// setup_mesh_x3 (parcop.f90:73-81, mesh.f90:163-168 and :245-358): the
// coordinates of a curvilinear grid; mesh_per is pyranda's 'periodicGrid'
// option (the Jacobian by a non-periodic first derivative)
int og_set_mesh_x3(og_handle* h, const double* x, const double* y, const double* z, int mesh_per) {
  if (!h || !x || !y || !z || h->coordsys != 3) return 1;
  curv_mesh(h, x, y, z, mesh_per ? 1 : 0);
  return 0;
}

void og_destroy(og_handle* h) { delete h; }

int og_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void og_set_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

// op: 0 = d1 (ddx/ddy/ddz), 1 = d8 (dd8x..), 2 = compact filter c8ff8, 3 = gaussian cgfs4,
// 4 = d2 (c10d2), 5 = d4 (e4d4, dd4x..)
int og_apply(const og_handle* h, int op, int dir, const double* in, double* out) {
  if (!h || op < 0 || op > 5 || dir < 0 || dir > 2) return 1;
  apply_dir(h, op, dir, in, out);
  return 0;
}

// d1x / d8x / filterx with the bc argument (compact_operators.f90:30-35,
// :403-409): sym = -1 takes operator 2 on a direction with a SYMM end.
int og_apply_sym(const og_handle* h, int op, int dir, int sym, const double* in, double* out) {
  if (!h || op < 0 || op > 5 || dir < 0 || dir > 2 || (sym != 1 && sym != -1)) return 1;
  apply_dir(h, op, dir, in, out, sym);
  return 0;
}

// filter x -> y -> z with one bc per direction (operators.f90:873-875)
int og_filter3_sym(const og_handle* h, int op, const int* sym, const double* in, double* out) {
  if (!h || (op != 2 && op != 3) || !sym) return 1;
  const size_t np = (size_t)h->n[0] * h->n[1] * h->n[2];
  std::vector<double> tmp(np);
  apply_dir(h, op, 0, in, out, sym[0]);
  apply_dir(h, op, 1, out, tmp.data(), sym[1]);
  apply_dir(h, op, 2, tmp.data(), out, sym[2]);
  return 0;
}

// LapS: operators.f90:513-526 (Cartesian: Lapf = Lapf + tmp + dum), :527-543
// (cylindrical), :544-559 (spherical, coordsys 2).  The reference has no
// branch for coordsys 3 and 4 (its output is left unset): an error here.
int og_laplacian(const og_handle* h, const double* in, double* out) {
  if (!h || h->coordsys > 2) return 1;
  const size_t npts = (size_t)h->n[0] * h->n[1] * h->n[2];
  std::vector<double> tmp(npts), dum(npts);
  if (h->coordsys == 1) {
    apply_dir(h, OP_D1, 0, in, tmp.data());
    for (size_t p = 0; p < npts; p++) dum[p] = xgrid(h, p) * tmp[p];
    apply_dir(h, OP_D1, 0, dum.data(), tmp.data());
    for (size_t p = 0; p < npts; p++) out[p] = tmp[p] / xgrid(h, p);
    apply_dir(h, OP_D2, 1, in, tmp.data());
    for (size_t p = 0; p < npts; p++) {
      const double r = xgrid(h, p);
      dum[p] = tmp[p] / (r * r);
      out[p] = out[p] + dum[p];
    }
    apply_dir(h, OP_D2, 2, in, tmp.data());
    for (size_t p = 0; p < npts; p++) out[p] = out[p] + tmp[p];
    return 0;
  }
  if (h->coordsys == 2) {
    const double *R = h->mf[MF_X].data(), *T = h->mf[MF_Y].data();
    apply_dir(h, OP_D1, 0, in, tmp.data());
    for (size_t p = 0; p < npts; p++) dum[p] = (R[p] * R[p]) * tmp[p];
    apply_dir(h, OP_D1, 0, dum.data(), tmp.data());
    for (size_t p = 0; p < npts; p++) out[p] = tmp[p] / (R[p] * R[p]);
    apply_dir(h, OP_D1, 1, in, tmp.data());
    for (size_t p = 0; p < npts; p++) dum[p] = std::sin(T[p]) * tmp[p];
    apply_dir(h, OP_D1, 1, dum.data(), tmp.data());
    for (size_t p = 0; p < npts; p++) {
      dum[p] = tmp[p] / ((R[p] * R[p]) * std::sin(T[p]));
      out[p] = out[p] + dum[p];
    }
    apply_dir(h, OP_D2, 2, in, tmp.data());
    for (size_t p = 0; p < npts; p++) {
      const double q = R[p] * std::sin(T[p]);
      dum[p] = tmp[p] / (q * q);
      out[p] = out[p] + dum[p];
    }
    return 0;
  }
  apply_dir(h, OP_D2, 0, in, out);
  apply_dir(h, OP_D2, 1, in, tmp.data());
  apply_dir(h, OP_D2, 2, in, dum.data());
  for (size_t p = 0; p < npts; p++) out[p] = out[p] + tmp[p] + dum[p];
  return 0;
}

// sFilter / gFilter: operators.f90:848-853, :860-875 (x -> y -> z with a temporary)
int og_filter3(const og_handle* h, int op, const double* in, double* out) {
  if (!h || (op != 2 && op != 3)) return 1;
  const size_t np = (size_t)h->n[0] * h->n[1] * h->n[2];
  std::vector<double> tmp(np);
  if (h->coordsys >= 2 && op == 2) {  // 'spectral', spherical and curvilinear: operators.f90:884-889
    const double* cv = h->mf[MF_CV].data();
    const double* bar = h->mf[h->coordsys == 4 ? MF_CV : MF_CVS].data();  // CellVolS = CellVol for coordsys 4
    std::vector<double> fv(np);
    for (size_t p = 0; p < np; p++) fv[p] = in[p] * cv[p];
    apply_dir(h, op, 0, fv.data(), out);
    apply_dir(h, op, 1, out, tmp.data());
    apply_dir(h, op, 2, tmp.data(), out);
    for (size_t p = 0; p < np; p++) out[p] = out[p] / bar[p];
    return 0;
  }
  if (h->coordsys == 1 && op == 2) {  // 'spectral' on a cylindrical grid: operators.f90:876-883
    std::vector<double> fv(np);
    for (size_t p = 0; p < np; p++) fv[p] = in[p] * cellvol_cyl(h, p);
    apply_dir(h, op, 0, fv.data(), out, -1);  // xasym = -xasym: CellVol is odd in r
    apply_dir(h, op, 1, out, tmp.data(), 1);
    apply_dir(h, op, 2, tmp.data(), out, 1);
    for (size_t p = 0; p < np; p++) out[p] = out[p] / cellvol_cyl(h, p);
    return 0;
  }
  apply_dir(h, op, 0, in, out);
  apply_dir(h, op, 1, out, tmp.data());
  apply_dir(h, op, 2, tmp.data(), out);
  return 0;
}

// ringS: operators.f90:615-643 with ringx/y/z (:701-753); L = 0, 1 or 2
int og_ring(const og_handle* h, const double* f, double* out, int L) {
  if (!h) return 1;
  const size_t np = (size_t)h->n[0] * h->n[1] * h->n[2];
  std::vector<double> r1(np), r2(np), r3(np);
  double* rs[3] = {r1.data(), r2.data(), r3.data()};
  for (int d = 0; d < 3; d++) {
    if (h->n[d] == 1) std::memset(rs[d], 0, np * sizeof(double));
    else apply_dir(h, OP_D8, d, f, rs[d]);
  }
  // the mesh d1, d2, d3 are fields on non-Cartesian grids (d2 = r dy when cylindrical)
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)np; i++) {
    double a, b, c;
    if (L == 0) { a = std::fabs(r1[i]); b = std::fabs(r2[i]); c = std::fabs(r3[i]); }
    else {
      double s[3];
      for (int d = 0; d < 3; d++) {
        const double m = mesh_d(h, d, (size_t)i);
        s[d] = L == 1 ? m : m * m;
      }
      a = std::fabs(r1[i]) * s[0]; b = std::fabs(r2[i]) * s[1]; c = std::fabs(r3[i]) * s[2];
    }
    out[i] = std::max(std::max(a, b), c);
  }
  return 0;
}

// ringV: operators.f90:645-699
int og_ringv(const og_handle* h, const double* f, const double* g, const double* q, double* out, int L) {
  if (!h) return 1;
  const size_t np = (size_t)h->n[0] * h->n[1] * h->n[2];
  std::vector<double> r(9 * np);
  const double* src[3] = {f, g, q};
  for (int c = 0; c < 3; c++)
    for (int d = 0; d < 3; d++) {
      double* dst = &r[(size_t)(c * 3 + d) * np];
      if (h->n[d] == 1) std::memset(dst, 0, np * sizeof(double));
      else apply_dir(h, OP_D8, d, src[c], dst);
    }
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)np; i++) {
    double m[3];
    for (int d = 0; d < 3; d++) {
      const double a = std::fabs(r[(size_t)(0 + d) * np + i]), b = std::fabs(r[(size_t)(3 + d) * np + i]),
                   c = std::fabs(r[(size_t)(6 + d) * np + i]);
      m[d] = std::max(std::max(a, b), c);
      const double md = mesh_d(h, d, (size_t)i);
      if (L != 0) m[d] = m[d] * (L == 1 ? md : md * md);
    }
    out[i] = std::max(std::max(m[0], m[1]), m[2]);
  }
  return 0;
}

// gradS: operators.f90:184-212 (cylindrical: dfdy = dfdy/xgrid, :193-196)
int og_grad(const og_handle* h, const double* f, double* gx, double* gy, double* gz) {
  if (!h) return 1;
  apply_dir(h, OP_D1, 0, f, gx);
  apply_dir(h, OP_D1, 1, f, gy);
  apply_dir(h, OP_D1, 2, f, gz);
  const size_t np = (size_t)h->n[0] * h->n[1] * h->n[2];
  if (h->coordsys == 1) {
    for (size_t p = 0; p < np; p++) gy[p] = gy[p] / xgrid(h, p);
  } else if (h->coordsys == 2 || h->coordsys == 4) {  // operators.f90:197-201
    const double *R = h->mf[MF_X].data(), *T = h->mf[MF_Y].data(), *D1 = h->mf[MF_D1].data();
    for (size_t p = 0; p < np; p++) {
      gx[p] = gx[p] * h->d[0] / D1[p];
      gy[p] = gy[p] / R[p];
      gz[p] = gz[p] / (R[p] * std::sin(T[p]));
    }
  } else if (h->coordsys == 3) {  // operators.f90:202-209
    for (size_t p = 0; p < np; p++) {
      double m[9];
      for (int q = 0; q < 9; q++) m[q] = h->mf[MF_J0 + q][p];
      const double a = gx[p], b = gy[p], c = gz[p];
      gx[p] = a * m[0] + b * m[3] + c * m[6];
      gy[p] = a * m[1] + b * m[4] + c * m[7];
      gz[p] = a * m[2] + b * m[5] + c * m[8];
    }
  }
  return 0;
}

namespace {
// divV on spherical grids (operators.f90:64-76)
void div_sph(const og_handle* h, const double* fx, const double* fy, const double* fz, double* out) {
  const size_t np = npts_of(h);
  const double *R = h->mf[MF_X].data(), *T = h->mf[MF_Y].data(), *D1 = h->mf[MF_D1].data();
  std::vector<double> tmp(np), fA(np), fB(np), fC(np);
  for (size_t p = 0; p < np; p++) {
    tmp[p] = (R[p] * R[p]) * fx[p];
    out[p] = fy[p] * std::sin(T[p]);
  }
  apply_dir(h, OP_D1, 0, tmp.data(), fA.data(), isym_pow(h, 0, 3));
  for (size_t p = 0; p < np; p++) fA[p] = fA[p] * h->d[0] / D1[p];
  apply_dir(h, OP_D1, 1, out, fB.data(), isym_pow(h, 1, 2));
  apply_dir(h, OP_D1, 2, fz, fC.data(), isym_pow(h, 2, 1));
  for (size_t p = 0; p < np; p++) out[p] = fA[p] / (R[p] * R[p]) + (fB[p] + fC[p]) / (R[p] * std::sin(T[p]));
}

// divV on curvilinear grids (operators.f90:77-90): the contravariant fluxes
// times det J, differentiated along A, B, C, summed and divided by det J
void div_curv(const og_handle* h, const double* fx, const double* fy, const double* fz, double* out) {
  const size_t np = npts_of(h);
  std::vector<double> fA(np), fB(np), fC(np), tmp(np);
  const double* det = h->mf[MF_DET].data();
  for (size_t p = 0; p < np; p++) {
    double m[9];
    for (int q = 0; q < 9; q++) m[q] = h->mf[MF_J0 + q][p];
    fA[p] = (fx[p] * m[0] + fy[p] * m[1] + fz[p] * m[2]) * det[p];
    fB[p] = (fx[p] * m[3] + fy[p] * m[4] + fz[p] * m[5]) * det[p];
    fC[p] = (fx[p] * m[6] + fy[p] * m[7] + fz[p] * m[8]) * det[p];
  }
  apply_dir(h, OP_D1, 0, fA.data(), out);
  apply_dir(h, OP_D1, 1, fB.data(), tmp.data());
  for (size_t p = 0; p < np; p++) out[p] = out[p] + tmp[p];
  apply_dir(h, OP_D1, 2, fC.data(), tmp.data());
  for (size_t p = 0; p < np; p++) out[p] = (out[p] + tmp[p]) / det[p];
}

// divT on spherical grids (operators.f90:148-173), with iR = 1/r,
// isinY = 1/sin(theta), itanY = 1/tan(theta) as mesh.f90:241-243 stores them
void divt_sph(const og_handle* h, const double* const* f, double* const* out) {
  const size_t np = npts_of(h);
  const double *R = h->mf[MF_X].data(), *T = h->mf[MF_Y].data(), *D1 = h->mf[MF_D1].data();
  const double *fxx = f[0], *fxy = f[1], *fxz = f[2], *fyx = f[3], *fyy = f[4], *fyz = f[5], *fzx = f[6],
               *fzy = f[7], *fzz = f[8];
  std::vector<double> tmp(np), fA(np), fB(np), fC(np);
  const double dx = h->d[0];
  for (size_t p = 0; p < np; p++) tmp[p] = (R[p] * R[p]) * fxx[p];
  apply_dir(h, OP_D1, 0, tmp.data(), fA.data(), 1);
  for (size_t p = 0; p < np; p++) {
    fA[p] = fA[p] * dx / D1[p];
    tmp[p] = fyx[p] / (1.0 / std::sin(T[p]));
  }
  apply_dir(h, OP_D1, 1, tmp.data(), fB.data(), 1);
  apply_dir(h, OP_D1, 2, fzx, fC.data(), isym_pow(h, 2, 1));
  for (size_t p = 0; p < np; p++) {
    const double iR = 1.0 / R[p], isinY = 1.0 / std::sin(T[p]);
    out[0][p] = fA[p] * (iR * iR) + (fB[p] + fC[p]) * iR * isinY - (fyy[p] + fzz[p]) * iR;
    tmp[p] = (R[p] * R[p] * R[p]) * fxy[p];
  }
  apply_dir(h, OP_D1, 0, tmp.data(), fA.data(), 1);
  for (size_t p = 0; p < np; p++) {
    fA[p] = fA[p] * dx / D1[p];
    tmp[p] = fyy[p] * std::sin(T[p]);
  }
  apply_dir(h, OP_D1, 1, tmp.data(), fB.data(), isym_pow(h, 1, 3));
  apply_dir(h, OP_D1, 2, fzy, fC.data(), isym_pow(h, 2, 1));
  for (size_t p = 0; p < np; p++) {
    const double iR = 1.0 / R[p], isinY = 1.0 / std::sin(T[p]), itanY = 1.0 / std::tan(T[p]);
    out[1][p] = fA[p] * (iR * iR * iR) + (fB[p] + fC[p]) * iR * isinY + (fyx[p] - fxy[p] - fzz[p] * itanY) * iR;
    tmp[p] = (R[p] * R[p] * R[p]) * fxz[p];
  }
  apply_dir(h, OP_D1, 0, tmp.data(), fA.data(), 1);
  for (size_t p = 0; p < np; p++) {
    fA[p] = fA[p] * dx / D1[p];
    tmp[p] = fyz[p] * std::sin(T[p]);
  }
  apply_dir(h, OP_D1, 1, tmp.data(), fB.data(), 1);
  apply_dir(h, OP_D1, 2, fzz, fC.data(), 1);
  for (size_t p = 0; p < np; p++) {
    const double iR = 1.0 / R[p], isinY = 1.0 / std::sin(T[p]), itanY = 1.0 / std::tan(T[p]);
    out[2][p] = fA[p] * (iR * iR * iR) + (fB[p] + fC[p]) * iR * isinY + (fzx[p] - fxz[p] + fzy[p] * itanY) * iR;
  }
}
}  // namespace

// divT: operators.f90:97-181 (Cartesian :104-122, cylindrical :123-146,
// spherical :147-173, curvilinear :174-177).
// f: fxx fxy fxz fyx fyy fyz fzx fzy fzz; out: dfx dfy dfz
int og_divt(const og_handle* h, const double* const* f, double* const* out) {
  if (!h) return 1;
  const size_t np = (size_t)h->n[0] * h->n[1] * h->n[2];
  std::vector<double> tmp(np), fA(np), fB(np), fC(np);
  const double *fxx = f[0], *fxy = f[1], *fxz = f[2], *fyx = f[3], *fyy = f[4], *fyz = f[5], *fzx = f[6],
               *fzy = f[7], *fzz = f[8];
  if (h->coordsys == 2 || h->coordsys == 4) {
    divt_sph(h, f, out);
    return 0;
  }
  if (h->coordsys == 3) {  // the divergence of each row
    div_curv(h, fxx, fxy, fxz, out[0]);
    div_curv(h, fyx, fyy, fyz, out[1]);
    div_curv(h, fzx, fzy, fzz, out[2]);
    return 0;
  }
  if (h->coordsys == 0) {
    const double* cols[3][3] = {{fxx, fyx, fzx}, {fxy, fyy, fzy}, {fxz, fyz, fzz}};
    for (int c = 0; c < 3; c++) {
      apply_dir(h, OP_D1, 0, cols[c][0], fA.data(), isym_pow(h, 0, c == 0 ? 2 : 1));
      apply_dir(h, OP_D1, 1, cols[c][1], fB.data(), isym_pow(h, 1, c == 1 ? 2 : 1));
      apply_dir(h, OP_D1, 2, cols[c][2], fC.data(), isym_pow(h, 2, c == 2 ? 2 : 1));
      for (size_t p = 0; p < np; p++) out[c][p] = fA[p] + fB[p] + fC[p];
    }
    return 0;
  }
  for (size_t p = 0; p < np; p++) tmp[p] = xgrid(h, p) * fxx[p];
  apply_dir(h, OP_D1, 0, tmp.data(), fA.data(), isym_pow(h, 0, 3));
  apply_dir(h, OP_D1, 1, fyx, fB.data(), isym_pow(h, 1, 1));
  apply_dir(h, OP_D1, 2, fzx, fC.data(), isym_pow(h, 2, 1));
  for (size_t p = 0; p < np; p++) {
    const double r = xgrid(h, p);
    out[0][p] = (fA[p] + fB[p] - fyy[p]) / r + fC[p];
    tmp[p] = r * r * fxy[p];
  }
  apply_dir(h, OP_D1, 0, tmp.data(), fA.data(), isym_pow(h, 0, 3));
  apply_dir(h, OP_D1, 1, fyy, fB.data(), isym_pow(h, 1, 2));
  apply_dir(h, OP_D1, 2, fzy, fC.data(), isym_pow(h, 2, 1));
  for (size_t p = 0; p < np; p++) {
    const double r = xgrid(h, p);
    out[1][p] = fA[p] / (r * r) + (fB[p] + fyx[p] - fxy[p]) / r + fC[p];
    tmp[p] = r * fxz[p];
  }
  apply_dir(h, OP_D1, 0, tmp.data(), fA.data(), isym_pow(h, 0, 2));
  apply_dir(h, OP_D1, 1, fyz, fB.data(), isym_pow(h, 1, 1));
  apply_dir(h, OP_D1, 2, fzz, fC.data(), isym_pow(h, 2, 2));
  for (size_t p = 0; p < np; p++) out[2][p] = (fA[p] + fB[p]) / xgrid(h, p) + fC[p];
  return 0;
}

// divV: operators.f90:38-90 (Cartesian :47-53, cylindrical :55-64, spherical
// :64-76 and curvilinear :77-90 in div_sph / div_curv)
int og_div(const og_handle* h, const double* fx, const double* fy, const double* fz, double* out) {
  if (!h) return 1;
  const size_t np = (size_t)h->n[0] * h->n[1] * h->n[2];
  std::vector<double> a(np), b(np);
  if (h->coordsys == 2 || h->coordsys == 4) {
    div_sph(h, fx, fy, fz, out);
    return 0;
  }
  if (h->coordsys == 3) {
    div_curv(h, fx, fy, fz, out);
    return 0;
  }
  if (h->coordsys == 1) {  // operators.f90:55-64
    std::vector<double> tmp(np), c(np);
    for (size_t p = 0; p < np; p++) tmp[p] = xgrid(h, p) * fx[p];
    apply_dir(h, OP_D1, 0, tmp.data(), a.data(), isym_pow(h, 0, 2));
    apply_dir(h, OP_D1, 1, fy, b.data(), isym_pow(h, 1, 1));
    apply_dir(h, OP_D1, 2, fz, c.data(), isym_pow(h, 2, 1));
    for (size_t p = 0; p < np; p++) out[p] = (a[p] + b[p]) / xgrid(h, p) + c[p];
    return 0;
  }
  // ddx(fx, fA, isymX) ... (operators.f90:47-50)
  apply_dir(h, OP_D1, 0, fx, out, h->symm[0] ? -1 : 1);
  apply_dir(h, OP_D1, 1, fy, a.data(), h->symm[1] ? -1 : 1);
  apply_dir(h, OP_D1, 2, fz, b.data(), h->symm[2] ? -1 : 1);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)np; i++) out[i] = out[i] + a[i] + b[i];
  return 0;
}

// Mesh quantities (mesh.f90:169-386):
// which = 0,1,2 -> x,y,z grid; 3,4,5 -> d1,d2,d3; 6 -> GridLen; 7 -> CellVol;
// 8, 9 -> CellVolS, CellVolG; 10 -> det J; 11..19 -> dA/dx dA/dy dA/dz dB/dx .. dC/dz
// (curvilinear grids only)
int og_mesh(const og_handle* h, int which, double* out) {
  if (!h || which < 0 || which > 19) return 1;
  if (h->coordsys >= 2) {
    if (which >= MF_DET && h->coordsys != 3) return 1;
    std::memcpy(out, h->mf[which].data(), npts_of(h) * sizeof(double));
    return 0;
  }
  if (which >= 10) return 1;
  if (which == 8 || which == 9) which = 7;  // CellVolS = CellVolG = CellVol (mesh.f90:384-386)
  const int nx = h->n[0], ny = h->n[1], nz = h->n[2];
  const double gl = std::min(std::min(h->dmesh[0], h->dmesh[1]), h->dmesh[2]);
  const double cv = h->d[0] * h->d[1] * h->d[2];
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        const size_t p = ((size_t)k * ny + j) * nx + i;
        double v = 0.0;
        if (h->coordsys == 1 && which >= 3) {  // mesh.f90:213-225
          const double r = h->x1f[0] + (double)(2 * (i + 1) - 1) * 0.5 * h->d[0];
          const double d2 = r * h->d[1];
          switch (which) {
            case 3: v = h->d[0]; break;
            case 4: v = d2; break;
            case 5: v = h->d[2]; break;
            case 6: v = (ny == 1) ? std::min(h->d[0], h->d[2]) : std::min(std::min(h->d[0], d2), h->d[2]); break;
            default: v = cellvol_cyl(h, p); break;
          }
          out[p] = v;
          continue;
        }
        switch (which) {
          case 0: v = h->x1f[0] + (double)(2 * (i + 1) - 1) * 0.5 * h->d[0]; break;
          case 1: v = h->x1f[1] + (double)(2 * (j + 1) - 1) * 0.5 * h->d[1]; break;
          case 2: v = h->x1f[2] + (double)(2 * (k + 1) - 1) * 0.5 * h->d[2]; break;
          case 3: case 4: case 5: v = h->dmesh[which - 3]; break;
          case 6: v = gl; break;
          default: v = cv; break;
        }
        out[p] = v;
      }
  return 0;
}

// Spacing used by the d1 metric (patch dx), and the mesh d1..d3.
int og_spacing(const og_handle* h, double* patch_d, double* mesh_d) {
  if (!h) return 1;
  for (int d = 0; d < 3; d++) {
    if (patch_d) patch_d[d] = h->d[d];
    if (mesh_d) mesh_d[d] = h->dmesh[d];
  }
  return 0;
}

// Dense operator matrix D (n x n, row-major, D[i][j] = d out_i / d in_j) of one
// operator along one direction, formed by applying the line evaluator to unit
// vectors (the same matrix compact_basetype.f90:199-205 stores as sm).
int og_dense(const og_handle* h, int op, int dir, double* D) {
  if (!h || op < 0 || op > 3 || dir < 0 || dir > 2) return 1;
  const Op1& o = pick(h, op, dir);
  const int n = h->n[dir];
  if (o.null_op) return 2;
  const double scale = (op == OP_D1) ? h->d[dir] : 0.0;
  std::vector<double> v(n + 1), dv(n + 1);
  for (int j = 0; j < n; j++) {
    std::fill(v.begin(), v.end(), 0.0);
    v[j + 1] = 1.0;
    eval_line(o, v.data(), dv.data(), scale);
    for (int i = 0; i < n; i++) D[(size_t)i * n + j] = dv[i + 1];
  }
  return 0;
}

}  // extern "C"
