// Pointwise forms of the non-Cartesian grids: the spherical and curvilinear
// mesh fields (mesh.f90:169-358), the metric factors of grad / div / divT /
// the Laplacian (operators.f90:54-209, :527-559), the volume weighting of the
// spectral filter (:876-889), the mesh-field scales of ring (:615-699) and the
// courant / diffusion rates on mesh fields (pyrandaTimestep.py:42-77).
//
// Every form is one grid-stride pass over the points (HBM-bound, 8 B per
// operand); the derivative sweeps between them are the library's own.  This
// file is compiled without FMA contraction, so each form rounds operation by
// operation in the reference's order.
#include <cuda_runtime.h>

#include "pg_internal.h"

namespace pg {
namespace {

constexpr int kThreads = 256;

// grid-stride launches of at most 8 CTAs of 256 threads per SM
int grid_for(int64_t n) {
  const int64_t b = (n + kThreads - 1) / kThreads, cap = 152 * 8;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

__device__ __forceinline__ void point_ijk(int64_t p, int nx, int ny, int& i, int& j, int& k) {
  i = (int)(p % nx);
  const int64_t q = p / nx;
  j = (int)(q % ny);
  k = (int)(q / ny);
}

// the radius of a cylindrical grid (x index i): x1 + (2 i - 1) dx / 2, i from 1
__device__ __forceinline__ double cyl_r(const MetricArgs& A, int64_t p) {
  const int i = (int)(p % A.nx);
  return A.x1f[0] + (double)(2 * (i + 1) - 1) * 0.5 * A.d[0];
}

// the radius of a cylindrical or spherical grid at point p
__device__ __forceinline__ double radius(const MetricArgs& A, int64_t p) {
  return A.coordsys == PG_CYLINDRICAL ? cyl_r(A, p) : A.mf[MF_X][p];
}

// mesh d1 d2 d3 at point p: d2 = r dy on cylindrical grids, fields on spherical and curvilinear ones
__device__ __forceinline__ double mesh_d(const MetricArgs& A, int dir, int64_t p) {
  if (A.coordsys == PG_CYLINDRICAL) return dir == 1 ? cyl_r(A, p) * A.d[1] : A.d[dir];
  return A.mf[MF_D1 + dir][p];
}

__global__ void metric_kernel(const MetricArgs A) {
  const double pi = 3.141592653589793;  // acos(-1) in FP64
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < A.n; p += (int64_t)gridDim.x * blockDim.x) {
    switch (A.op) {
      case MET_SPH_MESH: {  // mesh.f90:169-186, :227-244
        int i, j, k;
        point_ijk(p, A.nx, A.ny, i, j, k);
        double r = A.x1f[0] + (double)(2 * (i + 1) - 1) * 0.5 * A.d[0];
        const double th = A.x1f[1] + (double)(2 * (j + 1) - 1) * 0.5 * A.d[1];
        const double ph = A.x1f[2] + (double)(2 * (k + 1) - 1) * 0.5 * A.d[2];
        if (A.coordsys == PG_SPHERICAL_RATIO) r = A.s0 * exp(A.s1 * A.d[1] * (double)(i + 1));  // Asp exp(Csp dy i)
        double d1 = A.d[0];
        const double d2 = r * A.d[1], d3 = r * sin(th) * A.d[2];
        if (A.coordsys == PG_SPHERICAL_RATIO) d1 = A.s1 * r * A.d[1];  // Csp xgrid dy
        double cv = d1 * d2 * d3, gl = fmin(fmin(d1, d2), d3);
        if (A.ny == 1 && A.nz == 1) {
          cv = d1 * 4.0 * pi * (r * r);
          gl = d1;
        }
        A.mf[MF_X][p] = r;
        A.mf[MF_Y][p] = th;
        A.mf[MF_Z][p] = ph;
        A.mf[MF_D1][p] = d1;
        A.mf[MF_D2][p] = d2;
        A.mf[MF_D3][p] = d3;
        A.mf[MF_GL][p] = gl;
        A.mf[MF_CV][p] = cv;
        break;
      }
      case MET_NODES: {  // numpy.linspace(x1, xn, n) per direction (pyrandaMesh.py:96-108)
        int idx[3];
        point_ijk(p, A.nx, A.ny, idx[0], idx[1], idx[2]);
        const int n[3] = {A.nx, A.ny, A.nz};
        for (int d = 0; d < 3; d++) {
          double v;
          if (n[d] == 1) v = A.x1[d];
          else if (idx[d] == n[d] - 1) v = A.xn[d];
          else v = A.x1[d] + (double)idx[d] * ((A.xn[d] - A.x1[d]) / (double)(n[d] - 1));
          A.mf[MF_X + d][p] = v;
        }
        break;
      }
      case MET_CURV_METRIC: {  // mesh.f90:310-358; the J slots hold d(x,y,z)/d(A,B,C) on entry
        double J[9];
        for (int q = 0; q < 9; q++) J[q] = A.mf[MF_J0 + q][p];
        if (A.nx == 1) J[0] = 1.0;  // dxdA
        if (A.ny == 1) J[4] = 1.0;  // dydB
        if (A.nz == 1) J[8] = 1.0;  // dzdC
        const double dxdA = J[0], dxdB = J[1], dxdC = J[2], dydA = J[3], dydB = J[4], dydC = J[5], dzdA = J[6],
                     dzdB = J[7], dzdC = J[8];
        const double det = -dxdC * dydB * dzdA + dxdB * dydC * dzdA + dxdC * dydA * dzdB - dxdA * dydC * dzdB -
                           dxdB * dydA * dzdC + dxdA * dydB * dzdC;
        A.mf[MF_J0 + 0][p] = (-dydC * dzdB + dydB * dzdC) / det;
        A.mf[MF_J0 + 1][p] = (dxdC * dzdB - dxdB * dzdC) / det;
        A.mf[MF_J0 + 2][p] = (-dxdC * dydB + dxdB * dydC) / det;
        A.mf[MF_J0 + 3][p] = (dydC * dzdA - dydA * dzdC) / det;
        A.mf[MF_J0 + 4][p] = (-dxdC * dzdA + dxdA * dzdC) / det;
        A.mf[MF_J0 + 5][p] = (dxdC * dydA - dxdA * dydC) / det;
        A.mf[MF_J0 + 6][p] = (-dydB * dzdA + dydA * dzdB) / det;
        A.mf[MF_J0 + 7][p] = (dxdB * dzdA - dxdA * dzdB) / det;
        A.mf[MF_J0 + 8][p] = (-dxdB * dydA + dxdA * dydB) / det;
        const double dA = A.d[0], dB = A.d[1], dC = A.d[2];
        const double d1 = sqrt((dxdA * dA) * (dxdA * dA) + (dydA * dA) * (dydA * dA) + (dzdA * dA) * (dzdA * dA));
        const double d2 = sqrt((dxdB * dB) * (dxdB * dB) + (dydB * dB) * (dydB * dB) + (dzdB * dB) * (dzdB * dB));
        const double d3 = sqrt((dxdC * dC) * (dxdC * dC) + (dydC * dC) * (dydC * dC) + (dzdC * dC) * (dzdC * dC));
        A.mf[MF_DET][p] = det;
        A.mf[MF_D1][p] = d1;
        A.mf[MF_D2][p] = d2;
        A.mf[MF_D3][p] = d3;
        A.mf[MF_CV][p] = d1 * d2 * d3;
        A.mf[MF_GL][p] = fmin(fmin(d1, d2), d3);
        break;
      }
      case MET_SPH_GRAD: {  // operators.f90:197-201, in place on out[0..2]
        const double r = A.mf[MF_X][p], t = A.mf[MF_Y][p];
        A.out[0][p] = A.out[0][p] * A.d[0] / A.mf[MF_D1][p];
        A.out[1][p] = A.out[1][p] / r;
        A.out[2][p] = A.out[2][p] / (r * sin(t));
        break;
      }
      case MET_CURV_GRAD: {  // operators.f90:202-209, in place: (d/dA, d/dB, d/dC) -> (d/dx, d/dy, d/dz)
        double m[9];
        for (int q = 0; q < 9; q++) m[q] = A.mf[MF_J0 + q][p];
        const double a = A.out[0][p], b = A.out[1][p], c = A.out[2][p];
        A.out[0][p] = a * m[0] + b * m[3] + c * m[6];
        A.out[1][p] = a * m[1] + b * m[4] + c * m[7];
        A.out[2][p] = a * m[2] + b * m[5] + c * m[8];
        break;
      }
      case MET_SPH_DIV_PRE: {  // operators.f90:67-68: r^2 fx, fy sin(theta)
        const double r = A.mf[MF_X][p];
        A.out[0][p] = (r * r) * A.in[0][p];
        A.out[1][p] = A.in[1][p] * sin(A.mf[MF_Y][p]);
        break;
      }
      case MET_SPH_DIV_POST: {  // operators.f90:71-75: (fA dx / d1) / r^2 + (fB + fC) / (r sin(theta))
        const double r = A.mf[MF_X][p];
        const double fA = A.in[0][p] * A.d[0] / A.mf[MF_D1][p];
        A.out[0][p] = fA / (r * r) + (A.in[1][p] + A.in[2][p]) / (r * sin(A.mf[MF_Y][p]));
        break;
      }
      case MET_CURV_DIV_PRE: {  // operators.f90:79-81: (f . grad A) det J, (f . grad B) det J, (f . grad C) det J
        const double fx = A.in[0][p], fy = A.in[1][p], fz = A.in[2][p], det = A.mf[MF_DET][p];
        for (int r = 0; r < 3; r++) {
          A.out[r][p] = (fx * A.mf[MF_J0 + 3 * r][p] + fy * A.mf[MF_J0 + 3 * r + 1][p] +
                         fz * A.mf[MF_J0 + 3 * r + 2][p]) * det;
        }
        break;
      }
      case MET_CURV_DIV_POST:  // operators.f90:83-89: ((dA + dB) + dC) / det J
        A.out[0][p] = (A.in[0][p] + A.in[1][p] + A.in[2][p]) / A.mf[MF_DET][p];
        break;
      case MET_SPH_T_PRE: {  // operators.f90:150-168: r^k f (out 0) and the theta form (out 1)
        const double r = A.mf[MF_X][p], t = A.mf[MF_Y][p];
        const double rk = A.L == 2 ? r * r : r * r * r;
        A.out[0][p] = rk * A.in[0][p];
        A.out[1][p] = A.L == 2 ? A.in[1][p] / (1.0 / sin(t)) : A.in[1][p] * sin(t);  // fyx / isinY, f sin(theta)
        break;
      }
      case MET_SPH_T_POST: {  // operators.f90:156-172, row L (0 x, 1 y, 2 z): in = fA fB fC and three tensor parts
        const double r = A.mf[MF_X][p], t = A.mf[MF_Y][p];
        const double iR = 1.0 / r, isinY = 1.0 / sin(t);
        const double fA = A.in[0][p] * A.d[0] / A.mf[MF_D1][p];
        const double fBC = (A.in[1][p] + A.in[2][p]) * iR * isinY;
        double v;
        if (A.L == 0) {  // dfx = fA iR^2 + (fB+fC) iR isinY - (fyy+fzz) iR
          v = fA * (iR * iR) + fBC - (A.in[3][p] + A.in[4][p]) * iR;
        } else {
          const double itanY = 1.0 / tan(t);
          const double tail = A.L == 1 ? (A.in[3][p] - A.in[4][p] - A.in[5][p] * itanY)   // fyx - fxy - fzz itanY
                                       : (A.in[3][p] - A.in[4][p] + A.in[5][p] * itanY);  // fzx - fxz + fzy itanY
          v = fA * (iR * iR * iR) + fBC + tail * iR;
        }
        A.out[0][p] = v;
        break;
      }
      case MET_LAP_MUL: {  // out = r^L in (cylindrical L = 1, spherical L = 2)
        const double r = radius(A, p);
        A.out[0][p] = (A.L == 1 ? r : r * r) * A.in[0][p];
        break;
      }
      case MET_LAP_X: {  // out = in / r^L
        const double r = radius(A, p);
        A.out[0][p] = A.in[0][p] / (A.L == 1 ? r : r * r);
        break;
      }
      case MET_LAP_SIN:  // out = sin(theta) in
        A.out[0][p] = sin(A.mf[MF_Y][p]) * A.in[0][p];
        break;
      case MET_LAP_ADD_Y: {  // out += in / r^2 (cylindrical), in / (r^2 sin(theta)) (spherical)
        const double r = radius(A, p);
        const double q = A.coordsys == PG_CYLINDRICAL ? r * r : (r * r) * sin(A.mf[MF_Y][p]);
        A.out[0][p] = A.out[0][p] + A.in[0][p] / q;
        break;
      }
      case MET_LAP_ADD_Z: {  // out += in (cylindrical), in / (r sin(theta))^2 (spherical)
        if (A.coordsys == PG_CYLINDRICAL) {
          A.out[0][p] = A.out[0][p] + A.in[0][p];
        } else {
          const double q = A.mf[MF_X][p] * sin(A.mf[MF_Y][p]);
          A.out[0][p] = A.out[0][p] + A.in[0][p] / (q * q);
        }
        break;
      }
      case MET_VOL_MUL:  // operators.f90:886: fun CellVol
        A.out[0][p] = A.in[0][p] * A.mf[MF_CV][p];
        break;
      case MET_VOL_DIV:  // operators.f90:890: bar / CellBar (CellBar = in[1])
        A.out[0][p] = A.in[0][p] / A.in[1][p];
        break;
      case MET_RING: {  // operators.f90:636-639 / :683-695: |d8| d^L, the first direction sets, the others max
        const double m = mesh_d(A, A.dir, p);
        const double v = fabs(A.in[0][p]) * (A.L == 1 ? m : m * m);
        A.out[0][p] = A.first ? v : fmax(A.out[0][p], v);
        break;
      }
      case MET_COURANT: {  // pyrandaTimestep.py:42-63: the rate whose maximum sets dt
        const double u = A.in[0][p], v = A.in[1] ? A.in[1][p] : A.s0, w = A.in[2] ? A.in[2][p] : A.s1;
        double vrate;
        if (A.coordsys == PG_CURVILINEAR) {
          const double dAdx = A.mf[MF_J0 + 0][p], dAdy = A.mf[MF_J0 + 1][p];
          const double dBdx = A.mf[MF_J0 + 3][p], dBdy = A.mf[MF_J0 + 4][p];
          const double magA = sqrt(dAdx * dAdx + dAdy * dAdy), magB = sqrt(dBdx * dBdx + dBdy * dBdy);
          const double uA = (u * dAdx + v * dAdy) / magA, uB = (u * dBdx + v * dBdy) / magB;
          vrate = fabs(uA) / A.mf[MF_D1][p] + fabs(uB) / A.mf[MF_D2][p];
        } else {
          vrate = fabs(u) / A.mf[MF_D1][p] + fabs(v) / A.mf[MF_D2][p] + fabs(w) / A.mf[MF_D3][p];
        }
        A.out[0][p] = vrate + fabs(A.in[3][p]) / A.mf[MF_GL][p];
        break;
      }
      case MET_DIFF: {  // pyrandaTimestep.py:71-77: rho GridLen^2 / max(1e-12, bulk)
        const double b = A.in[0][p], gl = A.mf[MF_GL][p];
        const double den = (b != b) ? b : fmax(1.0e-12, b);  // numpy.maximum propagates NaN
        A.out[0][p] = A.in[1][p] * gl * gl / den;
        break;
      }
      case MET_RECIP:  // 1 / max(rate) (n = 1)
        A.out[0][p] = 1.0 / A.out[0][p];
        break;
      default:
        break;
    }
  }
}

}  // namespace

int launch_metric(const MetricArgs& A, void* stream) {
  if (A.op < 0 || A.op >= MET_COUNT || A.n <= 0) {
    set_error("metric form %d: bad arguments", A.op);
    return PG_EINVAL;
  }
  metric_kernel<<<grid_for(A.n), kThreads, 0, (cudaStream_t)stream>>>(A);
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("metric form %d: %s", A.op, cudaGetErrorString(e));
    return PG_ECUDA;
  }
  return PG_OK;
}

}  // namespace pg
