/*
 * bcm_oracle.h -- CPU restatement of the BCMTools ghost-update and stencil
 * path.  TEST INFRASTRUCTURE ONLY: the GPU product never links, loads or calls
 * this code.  Tests, the smoke check and the bench's CPU-baseline leg use it as
 * the checker.
 *
 * Every routine restates a reference routine (file:line given beside it) with
 * the reference's loop order and the same floating-point operation order; the
 * library is compiled with -ffp-contract=off so no multiply-add is fused.
 *
 * Data layout (the reference's Scalar3D<T>, Scalar3D.h:58-68, Index3D.h:46-58):
 * a field is nb padded bricks stored back to back, each brick
 * (nx+2vc)*(ny+2vc)*(nz+2vc) elements, x fastest; cell (i,j,k), i in
 * [-vc, nx+vc), sits at  i + nx0*j + nx0*ny0*k + (1+nx0+nx0*ny0)*vc.
 * `bstride` is the element distance between consecutive bricks (>= brick size).
 */
#ifndef BCM_ORACLE_H
#define BCM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Face / subface numbering of BCMTools.h:48-51. */
enum { BCMO_X_M, BCMO_X_P, BCMO_Y_M, BCMO_Y_P, BCMO_Z_M, BCMO_Z_P };

/* Boundary types of examples Utils/include/BoundaryInfo.h:32-37. */
enum { BCMO_BC_INNER = 0, BCMO_BC_DIRICHLET = 1, BCMO_BC_NEUMANN = 2,
       BCMO_BC_PERIODIC = 3 };

/* Dirichlet ghost forms.
 *  SOR: one ghost layer, g = 2v - f         (sor1/Solver.cpp:232-294)
 *  BCX: as SOR plus the second layer = v    (SolverTest/bcx.f90:18-76)
 *       written only when vc >= 2 (the reference writes it out of bounds
 *       for vc = 1). */
enum { BCMO_DIRICHLET_SOR = 0, BCMO_DIRICHLET_BCX = 1 };

/* One rank's block table: the flattened NeighborInfo[6] of every block
 * (NeighborInfo.h:36-56).  nbr_id[(b*6+f)*4+s] is the neighbour block id
 * (-1: none), nbr_ld[b*6+f] the level difference (neighbour - self),
 * nbr_sf[b*6+f] the neighbour's subface (used when the level difference
 * is -1). */
typedef struct {
  int nb, nx, ny, nz, vc;
  long bstride;
  const int* nbr_id;
  const int* nbr_ld;
  const int* nbr_sf;
} bcmo_mesh;

/* Ghost update of all local faces, reference semantics
 * (BlockManager.cpp:471-530 face lists, :715-743 loop,
 *  VCUpdater.h:65-82 dispatch, Scalar3DUpdater.h:180-266,321-373,519-708).
 * axis_mask bit a selects faces of axis a (0:x 1:y 2:z);
 * ld_mask bit (ld+1) selects level difference ld in {-1,0,+1}. */
void bcmo_vc_update_f32(const bcmo_mesh* m, float* data, int axis_mask, int ld_mask);
void bcmo_vc_update_f64(const bcmo_mesh* m, double* data, int axis_mask, int ld_mask);

/* Dirichlet ghosts on faces with bc_type == BCMO_BC_DIRICHLET
 * (sor1/Solver.cpp:201-294; SolverTest/bcx.f90:18-76) and Neumann ghosts on
 * faces with BCMO_BC_NEUMANN (SolverTest/bcx.f90:198-376; bc_value the ghost
 * increment per layer, the outward derivative times the cell size). */
/* Boundary folding of a coefficient-brick operator A[7] = {Ap, Aw, Ae, As,
 * An, Ab, At} and right-hand side b (SolverTest bca.f90:12-394,
 * LocalScalar3D.h:260-285): outer Dirichlet / Neumann faces only. */
void bcmo_fold_f32(const bcmo_mesh* m, float* const* A, float* b, const int* bc_type,
                   const double* bc_value);
void bcmo_fold_f64(const bcmo_mesh* m, double* const* A, double* b, const int* bc_type,
                   const double* bc_value);

void bcmo_dirichlet_f32(const bcmo_mesh* m, float* data, const int* bc_type,
                        const double* bc_value, int form);
void bcmo_dirichlet_f64(const bcmo_mesh* m, double* data, const int* bc_type,
                        const double* bc_value, int form);

/* One red-black SOR pass in every block (both colours, stale ghosts).
 *  form 1 (sor1/Solver.cpp:132-153): f = c0 f + cx(fW+fE) + cy(fS+fN) + cz(fB+fT),
 *          coef[b*4..] = {c0, cx, cy, cz}
 *  form 2 (sor2/Solver.cpp:136-160): fNew = c (cx(..)+cy(..)+cz(..) - s),
 *          f = omega fNew + (1-omega) f,  coef[b*4..] = {c, cx, cy, cz}   */
void bcmo_sor_rb_f64(const bcmo_mesh* m, double* f, const double* s,
                     const double* coef, double omega, int form);
void bcmo_sor_rb_f32(const bcmo_mesh* m, float* f, const float* s,
                     const double* coef, double omega, int form);

/* Stencil operator: either per-block constant coefficients
 * cc[b*7 + {0:Ap,1:Aw,2:Ae,3:As,4:An,5:Ab,6:At}] (cc != NULL), or seven
 * coefficient fields A[0..6] in the same order (SolverTest layout). */
typedef struct {
  const double* cc;
  const void* A[7];
} bcmo_op;

/* jacobi_smoother (blas.f90:452-502): x1 = x0 - omega (x0 - r/Ap),
 * r = b - Aw xW - Ae xE - As xS - An xN - Ab xB - At xT, all in T. */
void bcmo_jacobi_f32(const bcmo_mesh* m, const bcmo_op* op, float* x1,
                     const float* x0, const float* b, float omega);
void bcmo_jacobi_f64(const bcmo_mesh* m, const bcmo_op* op, double* x1,
                     const double* x0, const double* b, double omega);

/* calc_ax (blas.f90:556-600), calc_r (:602-648). */
void bcmo_calc_ax_f32(const bcmo_mesh* m, const bcmo_op* op, float* ax, const float* x);
void bcmo_calc_ax_f64(const bcmo_mesh* m, const bcmo_op* op, double* ax, const double* x);
void bcmo_calc_r_f32(const bcmo_mesh* m, const bcmo_op* op, float* r, const float* x, const float* b);
void bcmo_calc_r_f64(const bcmo_mesh* m, const bcmo_op* op, double* r, const double* x, const double* b);
/* calc_r2 (blas.f90:650-698) summed over blocks in double (ILS3D.h:211-270). */
double bcmo_calc_r2_f32(const bcmo_mesh* m, const bcmo_op* op, const float* x, const float* b);
double bcmo_calc_r2_f64(const bcmo_mesh* m, const bcmo_op* op, const double* x, const double* b);
/* dot (blas.f90:379-412) per block in T, blocks summed in double (ILS3D.h:272-311). */
double bcmo_dot_f32(const bcmo_mesh* m, const float* x, const float* y);
double bcmo_dot_f64(const bcmo_mesh* m, const double* x, const double* y);

/* BLAS-1 on interiors (blas.f90:242-377) and whole bricks (fill :18-46, copy :82-110). */
void bcmo_axpy_f32(const bcmo_mesh* m, float* y, const float* x, float a);
void bcmo_axpy_f64(const bcmo_mesh* m, double* y, const double* x, double a);
void bcmo_xpay_f32(const bcmo_mesh* m, float* y, const float* x, float a);
void bcmo_xpay_f64(const bcmo_mesh* m, double* y, const double* x, double a);
void bcmo_axpyz_f32(const bcmo_mesh* m, float* z, const float* x, const float* y, float a);
void bcmo_axpyz_f64(const bcmo_mesh* m, double* z, const double* x, const double* y, double a);
void bcmo_axpbypz_f32(const bcmo_mesh* m, float* z, const float* x, const float* y, float a, float b);
void bcmo_axpbypz_f64(const bcmo_mesh* m, double* z, const double* x, const double* y, double a, double b);
void bcmo_fill_f32(const bcmo_mesh* m, float* x, float a);
void bcmo_fill_f64(const bcmo_mesh* m, double* x, double a);
void bcmo_copy_f32(const bcmo_mesh* m, float* y, const float* x);
void bcmo_copy_f64(const bcmo_mesh* m, double* y, const double* x);

/* Boundary imposition as LocalScalar3D::ImposeBoundaryCondition
 * (LocalScalar3D.h:228-258): all-at-once VC update, then Dirichlet ghosts. */
typedef struct {
  const int* bc_type;     /* [nb*6] */
  const double* bc_value; /* [nb*6] */
  int form;               /* BCMO_DIRICHLET_* */
} bcmo_bc;

/* Jacobi solver (ILS3D.h:478-529): returns iterations, residual^2 ratio in *res.
 * x, x0 are both work bricks; on return x holds the solution. */
int bcmo_jacobi_solve_f64(const bcmo_mesh* m, const bcmo_op* op, const bcmo_bc* bc,
                          double* x, double* x0, const double* b, double omega,
                          int max_iter, double eps, double* res);
int bcmo_jacobi_solve_f32(const bcmo_mesh* m, const bcmo_op* op, const bcmo_bc* bc,
                          float* x, float* x0, const float* b, float omega,
                          int max_iter, double eps, double* res);

/* Jacobi-preconditioned BiCGSTAB (ILS3D.h:663-844).  work must hold 9 fields
 * (r, r0, p, p_, q_, s, s_, t_, x0) of m->nb * m->bstride elements each.
 * Scalars follow the reference: dots summed in double, stored in T.
 * Returns the iteration count (0 when b = 0), *res = |r|^2/|b|^2. */
int bcmo_bicgstab_f64(const bcmo_mesh* m, const bcmo_op* op, const bcmo_bc* bc,
                      double* x, const double* b, double* work, double omega,
                      int n_pre, int max_iter, double eps, double* res);
int bcmo_bicgstab_f32(const bcmo_mesh* m, const bcmo_op* op, const bcmo_bc* bc,
                      float* x, const float* b, float* work, float omega,
                      int n_pre, int max_iter, double eps, double* res);

/* Red-black SOR driver, sor1/sor2 Solver::run (sor1/Solver.cpp:74-129,
 * sor2/Solver.cpp:77-133): per outer iteration, n_inner x (SOR pass + block
 * Dirichlet), then VC update + Dirichlet. */
void bcmo_sor_run_f64(const bcmo_mesh* m, const bcmo_bc* bc, double* f, const double* s,
                      const double* coef, double omega, int form, int n_inner, int n_outer);
void bcmo_sor_run_f32(const bcmo_mesh* m, const bcmo_bc* bc, float* f, const float* s,
                      const double* coef, double omega, int form, int n_inner, int n_outer);

/* Number of threads the OpenMP loops use (for the CPU baseline report). */
int bcmo_num_threads(void);
void bcmo_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
