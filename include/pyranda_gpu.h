/*
 * pyranda_gpu.h — C ABI of the GB300 compact-operator library.
 *
 * Drop-in replacement for the f2py module `pyranda.parcop.parcop`
 * (pyranda/parcop/parcop.f90) on one GPU with no MPI decomposition.
 *
 * Conventions
 *  - A field is a contiguous FP64 array of nx*ny*nz values in Fortran order
 *    (x fastest), i.e. the memory of numpy's F-ordered (nx,ny,nz) array that
 *    parcop receives (pyranda/pyrandaMPI.py:249-250).
 *  - Pointers are DEVICE pointers unless the function name ends in `_host`.
 *  - The caller owns inputs and outputs; the library never allocates per call
 *    (parcop's f2py wrappers allocated a new output on every call,
 *    parcop.f90:225-253 `intent(out)`).  Workspaces belong to the handle.
 *  - `stream` is a cudaStream_t passed as void*; NULL is the legacy stream.
 *    Calls are stream-ordered and never synchronise, so they can be recorded
 *    into a CUDA graph.
 *  - Every call returns a pg_status.  The library never exits the process
 *    (parcop printed and called `stop` on a size mismatch,
 *    pyranda/parcop/compact_d1.f90:65-72).
 *  - Null operators keep parcop's semantics: a direction with fewer than 4
 *    points yields zero for derivatives and a copy for filters
 *    (pyranda/parcop/compact.f90:95-97, compact_operators.f90:24-29,396-401).
 */
#ifndef PYRANDA_GPU_H
#define PYRANDA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PG_OK = 0,
  PG_EBADSHAPE = 1, /* unsupported extent (e.g. 4 <= n < 8 on a non-null direction) */
  PG_ENULLOP = 2,   /* operator requested on a null direction where no result exists */
  PG_ECUDA = 3,     /* a CUDA runtime call failed; see pg_last_error() */
  PG_ENAN = 4,      /* a non-finite value was found by pg_check_finite */
  PG_ETIMEOUT = 5,  /* a bounded device wait gave up */
  PG_EINVAL = 6,    /* bad argument (NULL pointer, bad enum) */
  PG_ENOMEM = 7     /* allocation of handle workspace failed */
} pg_status;

/* Arithmetic of the compact sweeps.  PG_FP64 follows the reference
 * arithmetic; PG_FP32 evaluates the sweeps in single precision on FP64
 * inputs/outputs (the fast path; FP64 state is kept by the caller), except
 * the d8 RHS, which is evaluated exactly in 64-bit fixed point (its 8th
 * difference cancels more bits than FP32 holds) before an FP32 solve.
 * PG_DENSE applies d1 and the two filters as dense n x n operators
 * D = A^-1 B (the reference's `sm`, compact_basetype.f90:199-205) on the
 * tensor cores in split TF32 (hi.hi + hi.lo + lo.hi, FP32 accumulation) for
 * directions of 16..1024 points, and d8 as A^-1 applied to its exact
 * fixed-point RHS; the FP32 banded sweeps elsewhere; the filters' add-back
 * of v stays in FP64.  PG_AUTO builds the same tables and
 * then, per operator and direction, times the dense kernel against the FP32
 * banded sweep and the FP32 split-line sweep (pg_set_line_split) on the
 * handle's own grid and keeps the fastest.  Selecting either builds the
 * tables once (allocates and synchronises). */
typedef enum { PG_FP64 = 0, PG_FP32 = 1, PG_DENSE = 2, PG_AUTO = 3 } pg_precision;

typedef enum { PG_SPECTRAL = 0, PG_GAUSSIAN = 1 } pg_filter_kind;

enum { PG_DIR_X = 0, PG_DIR_Y = 1, PG_DIR_Z = 2, PG_DIR_ALL = 3 };

/* Mesh quantities for pg_mesh (parcop.f90:84-191; mesh.f90:35-50).  The
 * coordinates are the native ones (radius, angle, ... on cylindrical and
 * spherical grids).  CELLVOL_S / _G are the filtered cell volumes that divide
 * a filtered volume-weighted field (CellVol itself on Cartesian, cylindrical
 * and ratio-zoned spherical grids); DET and the inverse Jacobian rows
 * DA_DX .. DC_DZ exist on curvilinear grids only (getVar 'dtJ', 'dAx' ..). */
typedef enum {
  PG_MESH_X = 0, PG_MESH_Y = 1, PG_MESH_Z = 2,
  PG_MESH_D1 = 3, PG_MESH_D2 = 4, PG_MESH_D3 = 5,
  PG_MESH_GRIDLEN = 6, PG_MESH_CELLVOL = 7,
  PG_MESH_CELLVOL_S = 8, PG_MESH_CELLVOL_G = 9, PG_MESH_DET = 10,
  PG_MESH_DA_DX = 11, PG_MESH_DA_DY = 12, PG_MESH_DA_DZ = 13,
  PG_MESH_DB_DX = 14, PG_MESH_DB_DY = 15, PG_MESH_DB_DZ = 16,
  PG_MESH_DC_DX = 17, PG_MESH_DC_DY = 18, PG_MESH_DC_DZ = 19
} pg_mesh_var;

/* Boundary codes of a non-periodic end (pyrandaMPI.py:101-131,
 * compact.f90:77-91). */
typedef enum { PG_BC_NONE = 0, PG_BC_SYMM = 1, PG_BC_XTND = 2 } pg_bc;
/* Coordinate systems (patch.f90 coordsys; mesh.f90:169-386): cylindrical
 * (x = radius, y = angle, z = axis), spherical (x = radius, y = polar angle,
 * z = azimuth; RATIO zones the radius by a constant ratio, mesh.f90:180-186),
 * and general curvilinear (coordinates supplied by pg_set_mesh_coords). */
typedef enum {
  PG_CARTESIAN = 0, PG_CYLINDRICAL = 1, PG_SPHERICAL = 2, PG_CURVILINEAR = 3, PG_SPHERICAL_RATIO = 4
} pg_coordsys;

typedef struct {
  int n[3];        /* nx, ny, nz (global = local: one GPU) */
  int periodic[3]; /* 1 = PERI, 0 = non-periodic (ends per bc below) */
  double x1[3];    /* first node coordinate per direction */
  double xn[3];    /* last node coordinate per direction */
  int precision;   /* pg_precision */
  int bc[3][2];    /* pg_bc of the lower and upper end of each non-periodic
                    * direction: NONE = one-sided closures; SYMM = a symmetry
                    * plane half a spacing outside the end point (operators
                    * for symmetric fields by default, the antisymmetric
                    * variants through the *_sym calls); XTND = the
                    * extended-data rows (the compact filter, whose reference
                    * rows are unset, keeps its one-sided rows there) */
  int coordsys;    /* pg_coordsys */
} pg_grid;

typedef struct pg_handle pg_handle;

/* setup (parcop.f90:23-61) + setup_mesh (parcop.f90:64-70):
 * node extents -> face extents, operator assembly and LU factorisation
 * for d1 (c10d1), d8 (c10d8), compact filter (c8ff8) and Gaussian (cgfs4). */
int pg_create(const pg_grid* grid, pg_handle** out);
/* Frees the handle and its device workspace. */
int pg_destroy(pg_handle* h);
/* Reads and clears the handle's device status word (synchronises with the
 * device).  *status is PG_OK, or PG_ETIMEOUT when a kernel's bounded wait on
 * an asynchronous copy gave up (the affected output is then not valid). */
int pg_device_status(pg_handle* h, int* status);
/* Switch the arithmetic of later sweeps on this handle (pg_precision). */
int pg_set_precision(pg_handle* h, int precision);
/* Failure-detection self-test: launches one CTA that waits on a barrier
 * nothing arrives at; after limit_ms (1..10000) the wait gives up and the
 * handle's status word reads PG_ETIMEOUT (pg_device_status), as after a
 * dense sweep whose copies or MMAs never complete.  The context stays usable. */
int pg_wait_selftest(pg_handle* h, unsigned limit_ms, void* stream);
/* Line solves of the banded sweeps (both precisions): mode 0 = one thread
 * streams a whole line (forward values through a workspace field); mode 1 =
 * split lines: each line is cut into segments of 32 points, one thread per
 * segment, joined by the reduced system of the segments' end unknowns -- the
 * reference's parallel solver across MPI ranks (compact_basetype.f90:171-197,
 * pentadiagonal.f90:160-626, compact_d1.f90:242-337) run across the threads
 * of one CTA, with the tile of lines staged in shared memory.  Lines of up to
 * 8192 points; directions beyond that keep mode 0.  Builds its tables on the
 * first call (allocates and synchronises). */
int pg_set_line_split(pg_handle* h, int mode);
/* The form of every sweep: plan[op * 3 + dir] = 0 (banded, one thread per
 * line), 1 (dense tensor-core kernel) or 2 (split-line banded), for op 0 d1,
 * 1 d8, 2 compact filter, 3 Gaussian filter, 4 d2, 5 d4. */
int pg_sweep_plan(const pg_handle* h, int* plan);
/* Applies a plan in pg_sweep_plan's layout (0 FP32 banded, 1 dense, 2 FP32
 * split-line per operator and direction) without timing it: builds the dense
 * and split tables the plan needs (allocates and synchronises) and runs the
 * FP32 path with it.  PG_EINVAL if an entry names a form the grid lacks.
 * No counterpart in the reference (an autotuner's cached result). */
int pg_set_sweep_plan(pg_handle* h, const int* plan);
/* The sweep plan of PG_DENSE / PG_AUTO: plan[op * 3 + dir] = 1 where the
 * dense kernel runs (op 0 d1, 1 d8, 2 compact filter, 3 Gaussian filter). */
int pg_dense_plan(const pg_handle* h, int* plan);
/* Patch spacing (used by the d1 metric) and mesh spacing d1..d3. */
int pg_get_spacing(const pg_handle* h, double* patch_d, double* mesh_d);
/* Text of the last error on this thread (static storage). */
const char* pg_last_error(void);
/* Library version string. */
const char* pg_version(void);

/* ddx / ddy / ddz (parcop.f90:225-253 -> compact_operators.f90:13-128):
 * 10th-order Pade first derivative, divided by the grid spacing. */
int pg_d1(pg_handle* h, int dir, const double* in, double* out, void* stream);
/* dd8x / dd8y / dd8z (parcop.f90:279-301 -> compact_operators.f90:280-383):
 * 8th derivative, no metric. */
int pg_d8(pg_handle* h, int dir, const double* in, double* out, void* stream);
/* d2x / d2y / d2z (compact_operators.f90:130-206): 10th-order compact second
 * derivative (c10d2), divided by the grid spacing squared. */
int pg_d2(pg_handle* h, int dir, const double* in, double* out, void* stream);
/* dd4x / dd4y / dd4z (parcop.f90:255-277 -> compact_operators.f90:208-278):
 * explicit 4th-order fourth derivative (e4d4), no metric.  On non-periodic
 * lines the three one-sided rows of each end close the stencil (the
 * reference declares a fourth row it never sets). */
int pg_d4(pg_handle* h, int dir, const double* in, double* out, void* stream);
/* plaplacian (parcop.f90:303-311 -> operators.f90:513-559): Cartesian
 * d2x + d2y + d2z (a direction of fewer than 4 points contributes 0);
 * cylindrical d(r df/dr)/dr / r + d2y / r^2 + d2z; spherical (coordsys 2)
 * d(r^2 df/dr)/dr / r^2 + d(sin(theta) df/dtheta)/dtheta / (r^2 sin(theta))
 * + d2z / (r sin(theta))^2.  The reference has no Laplacian on curvilinear
 * and ratio-zoned spherical grids: PG_EINVAL.  out must differ from in. */
int pg_laplacian(pg_handle* h, const double* in, double* out, void* stream);
/* sFilter / gFilter / gFilterDir (parcop.f90:337-368 -> operators.f90:755-896).
 * dir = PG_DIR_ALL gives the x->y->z sweep sequence of `filter`; on a
 * non-Cartesian grid the spectral filter acts on the field times the cell
 * volume and divides by the cell volume (cylindrical, :876-883) or by the
 * filtered cell volume (spherical and curvilinear, :884-889); out must differ
 * from in there. */
int pg_filter(pg_handle* h, int kind, int dir, const double* in, double* out, void* stream);
/* The operators of a direction with a symmetry plane come in two variants
 * (compact.f90:80-85): sym = +1 for fields symmetric about the plane (what
 * pg_d1 / pg_d8 / pg_filter apply), sym = -1 for antisymmetric ones -- the
 * bc argument of d1x / d8x / filterx (compact_operators.f90:13-50,
 * :280-313, :385-421).  Elsewhere both variants are the same operator.
 * pg_filter_sym takes one sign per direction (dir = PG_DIR_ALL sweeps x, y,
 * z with sym[0..2]). */
int pg_d1_sym(pg_handle* h, int dir, int sym, const double* in, double* out, void* stream);
int pg_d8_sym(pg_handle* h, int dir, int sym, const double* in, double* out, void* stream);
int pg_filter_sym(pg_handle* h, int kind, int dir, const int* sym, const double* in, double* out, void* stream);
/* pRing (parcop.f90:313-322 -> operators.f90:615-643 with L = 2); the
 * scales d1 d2 d3 are the mesh fields on non-Cartesian grids (d2 = r dy on
 * cylindrical ones). */
int pg_ring(pg_handle* h, const double* in, double* out, void* stream);
/* pRingV (parcop.f90:324-333 -> operators.f90:645-699 with L = 1). */
int pg_ringv(pg_handle* h, const double* vx, const double* vy, const double* vz, double* out,
             void* stream);
/* gradS (parcop.f90:371-379 -> operators.f90:184-212); cylindrical grids
 * divide the angular component by the radius, spherical grids the angular
 * ones by r and r sin(theta), curvilinear grids apply the inverse Jacobian. */
int pg_grad(pg_handle* h, const double* in, double* gx, double* gy, double* gz, void* stream);
/* divergence (parcop.f90:202-211 -> operators.f90:38-64): on a direction with
 * a symmetry plane the component along it is taken as antisymmetric
 * (isym = -1, patch.f90:89-91); cylindrical grids take (d(r fx)/dr +
 * dfy/dtheta) / r + dfz/dz, spherical and curvilinear grids the forms of
 * operators.f90:64-90.  Non-Cartesian grids use workspace fields of the
 * handle. */
int pg_div(pg_handle* h, const double* fx, const double* fy, const double* fz, double* out,
           void* stream);
/* divergenceTensor (parcop.f90:213-224 -> operators.f90:97-146): f holds the
 * nine device fields fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz; out the
 * three results dfx, dfy, dfz (distinct from f).  Every coordinate system
 * (curvilinear: the divergence of each row, operators.f90:174-177); the
 * symmetry multipliers isym^p of the reference select each derivative's
 * variant on directions with a symmetry plane. */
int pg_divt(pg_handle* h, const double* const* f, double* const* out, void* stream);
/* xGrid/yGrid/zGrid/dxGrid/.../mesh_getGridLen/mesh_getCellVol and getVar
 * (parcop.f90:84-191 -> mesh.f90:169-386); which is a pg_mesh_var. */
int pg_mesh(pg_handle* h, int which, double* out, void* stream);
/* setup_mesh_x3 (parcop.f90:73-81 -> mesh.f90:163-168, :245-386): the
 * coordinates of a curvilinear grid (device fields), the Jacobian by the
 * first-derivative operator -- a non-periodic one with one-sided ends when
 * mesh_periodic is set (pyranda's 'periodicGrid' option, mesh.f90:246-307),
 * else the grid's own -- its determinant and inverse, d1 d2 d3, CellVol,
 * GridLen and the filtered cell volumes.  A curvilinear handle starts from
 * the node coordinates x1 + i (xn - x1) / (n - 1) (pyrandaMesh.py:96-108)
 * with mesh_periodic set.  Allocates and synchronises (setup, not a step). */
int pg_set_mesh_coords(pg_handle* h, const double* x, const double* y, const double* z, int mesh_periodic,
                       void* stream);

/* One stage of the LSRK(5,4) update of pyranda.py:797-804 for nvar conserved
 * fields, fused:  PHI = A*PHI + dt*F ;  U = U + B*PHI.
 * U, PHI, F are arrays of nvar device pointers (host arrays of pointers);
 * dt is a device scalar so the step can be captured in a CUDA graph. */
int pg_rk_stage(pg_handle* h, int nvar, double* const* U, double* const* PHI,
                const double* const* F, const double* dt, double A, double B, void* stream);

/* pyrandaTimestep.courant (pyranda/pyrandaTimestep.py:42-67):
 * out[0] = 1 / max(|u|/d1 + |v|/d2 + |w|/d3 + |c|/GridLen), with the mesh
 * fields d1 d2 d3 GridLen on spherical and curvilinear grids; curvilinear
 * grids take the speeds along the A and B grid lines,
 * |u dA/dx + v dA/dy| / |grad A| / d1 + |u dB/dx + v dB/dy| / |grad B| / d2
 * (:45-56).  v or w may be NULL, meaning the constant vconst/wconst (scripts
 * pass 0.0).  Cylindrical grids with more than one point in angle return
 * PG_EINVAL. */
int pg_courant(pg_handle* h, const double* u, const double* v, const double* w, const double* c,
               double vconst, double wconst, double* out, void* stream);
/* pyrandaTimestep.diff (pyranda/pyrandaTimestep.py:71-77):
 * out[0] = min(rho * GridLen^2 / max(1e-12, bulk)) (GridLen the mesh field on
 * spherical and curvilinear grids). */
int pg_diff(pg_handle* h, const double* bulk, const double* rho, double* out, void* stream);
/* Global reductions (pyrandaMPI.py:307-326 sum3D/max3D/min3D on one GPU):
 * op 0 = sum, 1 = max, 2 = min over n values; out is a device scalar. */
int pg_reduce(pg_handle* h, int op, const double* in, int64_t n, double* out, void* stream);
/* Writes 1 to *flag (device int) if any of n values is not finite, else
 * leaves it unchanged (pyranda.py:359-369 checked for NaN on the host). */
int pg_check_finite(const double* in, int64_t n, int* flag, void* stream);

/* ---------------------------------------------------------------------------
 * Ensembles: many independent grids advanced together.  No counterpart in
 * parcop, which holds one patch per (patch, level) and runs them one at a time.
 * The members' fields are stored back to back in one flat FP64 buffer (member
 * m occupies points [offsets[m], offsets[m+1]) in its own Fortran order), and
 * every operator is one launch over the lines of all members, so small grids
 * fill the GPU together.  Members may differ in size but must share
 * periodicity and null directions.  Reductions give one value per member,
 * broadcast to the member's points (a per-point field) so that expressions
 * and the RK update can use them pointwise. */
typedef struct pg_ensemble pg_ensemble;
int pg_ens_create(int m, const pg_grid* grids, pg_ensemble** out);
int pg_ens_destroy(pg_ensemble* e);
/* Total points; fills offsets[0..m] when not NULL. */
int64_t pg_ens_points(const pg_ensemble* e, int64_t* offsets);
int pg_ens_set_precision(pg_ensemble* e, int precision);
int pg_ens_set_line_split(pg_ensemble* e, int mode);
int pg_ens_spacing(const pg_ensemble* e, int member, double* patch_d, double* mesh_d);
int pg_ens_d1(pg_ensemble* e, int dir, const double* in, double* out, void* stream);
int pg_ens_d8(pg_ensemble* e, int dir, const double* in, double* out, void* stream);
int pg_ens_d2(pg_ensemble* e, int dir, const double* in, double* out, void* stream);
int pg_ens_d4(pg_ensemble* e, int dir, const double* in, double* out, void* stream);
int pg_ens_laplacian(pg_ensemble* e, const double* in, double* out, void* stream);
int pg_ens_filter(pg_ensemble* e, int kind, int dir, const double* in, double* out, void* stream);
int pg_ens_ring(pg_ensemble* e, const double* in, double* out, void* stream);
int pg_ens_ringv(pg_ensemble* e, const double* vx, const double* vy, const double* vz, double* out,
                 void* stream);
int pg_ens_grad(pg_ensemble* e, const double* in, double* gx, double* gy, double* gz, void* stream);
int pg_ens_div(pg_ensemble* e, const double* fx, const double* fy, const double* fz, double* out,
               void* stream);
int pg_ens_mesh(pg_ensemble* e, int which, double* out, void* stream);
/* The LSRK stage with dt_field holding each point's time step. */
int pg_ens_rk_stage(pg_ensemble* e, int nvar, double* const* U, double* const* PHI,
                    const double* const* F, const double* dt_field, double A, double B, void* stream);
int pg_ens_courant(pg_ensemble* e, const double* u, const double* v, const double* w, const double* c,
                   double vconst, double wconst, double* out_field, void* stream);
int pg_ens_diff(pg_ensemble* e, const double* bulk, const double* rho, double* out_field, void* stream);
/* out_field (per point) and/or out_member (m values) may be NULL. */
int pg_ens_reduce(pg_ensemble* e, int op, const double* in, double* out_field, double* out_member,
                  void* stream);
int pg_ens_device_status(pg_ensemble* e, int* status);

/* ---------------------------------------------------------------------------
 * Learned LAD closure (no counterpart in the reference, which evaluates the
 * plain LAD operators of examples/ISSW_cyl.py:101-104 every stage).  A small
 * MLP predicts the artificial bulk viscosity beta and conductivity kappa from
 * the 27-point stencils of div(u)*D and |grad rho|*D plus D (D = the largest
 * mesh spacing):
 * PG_LAD_IN inputs padded to PG_LAD_K, three hidden layers of PG_LAD_HIDDEN
 * (ReLU), PG_LAD_OUT outputs; BF16 weights and activations, FP32 accumulation.
 * Outputs y are normalised:  beta = max(0, y0*ys0 + ym0) * rho * D  and
 * kappa = max(0, y1*ys1 + ym1) * rho * cv * D^2 / dt.
 * Parameters: one FP32 buffer of PG_LAD_NPARAM values laid out
 * [w1 64x64 | w2 64x64 | w3 64x64 | w4 2x64 | b1 64 | b2 64 | b3 64 | b4 2]
 * (weights row = output unit), and BF16 copies of its first PG_LAD_NWEIGHT
 * values (the weights, same order). */
#define PG_LAD_IN 55
#define PG_LAD_K 64
#define PG_LAD_HIDDEN 64
#define PG_LAD_OUT 2
#define PG_LAD_NWEIGHT (3 * 64 * 64 + 2 * 64)
#define PG_LAD_NPARAM (PG_LAD_NWEIGHT + 3 * 64 + 2)
typedef struct pg_lad_model {
  const void* wbf16;     /* PG_LAD_NWEIGHT BF16 weights (device, 16-byte aligned) */
  const float* params;   /* PG_LAD_NPARAM FP32 parameters (device; biases read here) */
  const float* xmean;    /* PG_LAD_K input means (device) */
  const float* xinvstd;  /* PG_LAD_K input 1/std (device) */
  float ym[2], ys[2];    /* output de-normalisation */
  float ylo[2], yhi[2];  /* accepted range of the raw outputs (training range + margin) */
} pg_lad_model;
/* beta and kappa of every point of the grid.  dt is a device scalar; *flag
 * (device int) is set to 1 when any raw output leaves [ylo, yhi], i.e. the
 * closure was asked outside its training range and the caller should fall
 * back to the plain LAD operators. */
int pg_lad_closure(pg_handle* h, const pg_lad_model* m, const double* div, const double* gmag, const double* rho,
                   const double* dt, double cv, double* beta, double* kappa, int* flag, void* stream);
/* The closure's |grad rho| input: second-order central differences along
 * every direction of more than one point (periodic lines wrap; the end points
 * of non-periodic lines take one-sided first differences), in FP32
 * arithmetic, stored as FP64. */
int pg_lad_grad_magnitude(pg_handle* h, const double* rho, double* out, void* stream);
/* Raw (unnormalised) feature rows of ns points (flat indices pts): raw[ns][PG_LAD_K]. */
int pg_lad_features(pg_handle* h, const double* div, const double* gmag, const int64_t* pts, int64_t ns,
                    float* raw, void* stream);
/* X[ns][PG_LAD_K] (BF16) = (raw - xmean) * xinvstd. */
int pg_lad_normalize(const float* raw, int64_t ns, const float* xmean, const float* xinvstd, void* X,
                     void* stream);
/* Adds the gradient of  mean((y - T)^2)  over rows x outputs of one batch
 * (X BF16 [rows][PG_LAD_K], T FP32 [rows][PG_LAD_OUT]) to grad (FP32,
 * parameter layout); adds the loss to *loss and writes outputs to Y when
 * those are not NULL.  inv_count is 1 / (rows of the whole batch * PG_LAD_OUT). */
int pg_lad_train_step(const pg_lad_model* m, const void* X, const float* T, int64_t rows, float inv_count,
                      float* grad, float* loss, float* Y, void* stream);
/* One Adam step on n FP32 parameters (moments m, v), then BF16 copies of the
 * first nbf of them into pbf. */
int pg_lad_adam(float* params, float* m, float* v, const float* grad, int n, float lr, float beta1, float beta2,
                float eps, int step, void* pbf, int nbf, void* stream);

/* Allocation-free reduction.  No counterpart in the reference.
 * For callers that cannot allocate device memory (a host framework whose
 * allocator forbids cudaMalloc, or code that never creates a pg_handle and so
 * owns no workspace): same result as pg_reduce (op 0 = sum, 1 = max, 2 = min
 * of n values into the device scalar *out) with its per-block partials kept in
 * a static device array of PG_NOALLOC_MAX_BLOCKS doubles (32 KiB) that every
 * GPU holds from library load to process exit.  n is limited to
 * PG_NOALLOC_MAX_VALUES; larger n returns PG_EBADSHAPE without launching.
 * Each call outside a stream capture looks up the array's address on the
 * current device (so a device reset between calls is harmless); a call inside
 * a capture reuses the address of an earlier call, so make one call on each
 * device before capturing.  All calls share the array: calls that overlap on
 * the GPU race and must be serialised by the caller. */
#define PG_NOALLOC_CHUNK 8192
#define PG_NOALLOC_MAX_BLOCKS 4096
#define PG_NOALLOC_MAX_VALUES ((int64_t)PG_NOALLOC_CHUNK * PG_NOALLOC_MAX_BLOCKS)
int pg_reduce_noalloc(int op, const double* in, int64_t n, double* out, void* stream);

/* Host-pointer variants: copy in, run on an internal stream, copy out,
 * synchronise.  For tests and for callers that hold host arrays. */
int pg_d1_host(pg_handle* h, int dir, const double* in, double* out);
int pg_d8_host(pg_handle* h, int dir, const double* in, double* out);
int pg_d2_host(pg_handle* h, int dir, const double* in, double* out);
int pg_d4_host(pg_handle* h, int dir, const double* in, double* out);
int pg_laplacian_host(pg_handle* h, const double* in, double* out);
int pg_filter_host(pg_handle* h, int kind, int dir, const double* in, double* out);
int pg_ring_host(pg_handle* h, const double* in, double* out);

/* Number of kernels this library has launched since load (for accounting). */
uint64_t pg_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* PYRANDA_GPU_H */
