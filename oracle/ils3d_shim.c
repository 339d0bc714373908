/*
 * ils3d_shim.c -- the Fortran symbols that SolverTest's ILS3D.h calls
 * (examples/SolverTest/blas.h, comm.h), for real = double, implemented on the
 * oracle's restatement of blas.f90 applied to one block.  TEST INFRASTRUCTURE
 * ONLY: it lets the reference's ILS3D::Jacobi and ILS3D::BiCGSTAB run here
 * (oracle/refils3d.cpp) with the oracle's loop bodies, so that their control
 * flow -- step order, scalar recurrences, reductions across blocks,
 * convergence test -- is compared with the oracle's own solvers.  The
 * image has no Fortran compiler, so the loop bodies themselves stay the
 * oracle's restatement.
 */
#include "bcm_oracle.h"

/* One block of sz[0] x sz[1] x sz[2] cells and *g ghost layers, its brick
 * at the pointers the caller passes (no neighbour table: the routines below
 * do not read one). */
static bcmo_mesh one_block(const int* sz, const int* g) {
  bcmo_mesh m;
  m.nb = 1;
  m.nx = sz[0];
  m.ny = sz[1];
  m.nz = sz[2];
  m.vc = *g;
  m.bstride = (long)(sz[0] + 2 * *g) * (sz[1] + 2 * *g) * (sz[2] + 2 * *g);
  m.nbr_id = 0;
  m.nbr_ld = 0;
  m.nbr_sf = 0;
  return m;
}

static bcmo_op fields(double* Ap, double* Aw, double* Ae, double* As, double* An, double* Ab,
                      double* At) {
  bcmo_op o;
  o.cc = 0;
  o.A[0] = Ap; o.A[1] = Aw; o.A[2] = Ae; o.A[3] = As;
  o.A[4] = An; o.A[5] = Ab; o.A[6] = At;
  return o;
}

/* blas.f90:18-46 */
void fill_(double* x, double* a, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_fill_f64(&m, x, *a);
}
/* blas.f90:82-110 */
void copy_(double* y, double* x, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_copy_f64(&m, y, x);
}
/* blas.f90:242-274: y = y + a x */
void axpy_(double* y, double* x, double* a, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_axpy_f64(&m, y, x, *a);
}
/* blas.f90:276-308: y = x + a y */
void xpay_(double* y, double* x, double* a, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_xpay_f64(&m, y, x, *a);
}
/* blas.f90:310-343: z = a x + y */
void axpyz_(double* z, double* x, double* y, double* a, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_axpyz_f64(&m, z, x, y, *a);
}
/* blas.f90:345-377: z = a x + b y + z */
void axpbypz_(double* z, double* x, double* y, double* a, double* b, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_axpbypz_f64(&m, z, x, y, *a, *b);
}
/* blas.f90:379-412: the block's inner product */
void dot_(double* xy, double* y, double* x, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  *xy = bcmo_dot_f64(&m, x, y);
}
/* blas.f90:452-502 */
void jacobi_smoother_(double* x1, double* x0, double* Ap, double* Aw, double* Ae, double* As,
                      double* An, double* Ab, double* At, double* b, double* omega, int* sz,
                      int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_op o = fields(Ap, Aw, Ae, As, An, Ab, At);
  bcmo_jacobi_f64(&m, &o, x1, x0, b, *omega);
}
/* blas.f90:556-600 */
void calc_ax_(double* ax, double* Ap, double* Aw, double* Ae, double* As, double* An,
              double* Ab, double* At, double* x, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_op o = fields(Ap, Aw, Ae, As, An, Ab, At);
  bcmo_calc_ax_f64(&m, &o, ax, x);
}
/* blas.f90:602-648 */
void calc_r_(double* r, double* Ap, double* Aw, double* Ae, double* As, double* An,
             double* Ab, double* At, double* x, double* b, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_op o = fields(Ap, Aw, Ae, As, An, Ab, At);
  bcmo_calc_r_f64(&m, &o, r, x, b);
}
/* blas.f90:650-698: the block's sum of squared residuals */
void calc_r2_(double* r2, double* Ap, double* Aw, double* Ae, double* As, double* An,
              double* Ab, double* At, double* x, double* b, int* sz, int* g) {
  bcmo_mesh m = one_block(sz, g);
  bcmo_op o = fields(Ap, Aw, Ae, As, An, Ab, At);
  *r2 = bcmo_calc_r2_f64(&m, &o, x, b);
}
/* comm.f90:18-55 on one rank: the sum over ranks is the local value */
void allreduce_(double* total, double* a) { *total = *a; }
