/*
 * bcmg.h -- C ABI of bcmtools_gb300, the GB300 (sm_103a) implementation of
 * the BCMTools ghost-update (virtual cell, "VC") and 7-point stencil path.
 *
 * Plain C: opaque handles, integer ids, raw pointers and sizes; no C++ or
 * PyTorch types cross this boundary.  Every call returns an int status whose
 * values mirror the reference's ExitStatus (BCMTools.h:54-63); failures never
 * exit the process, and bcmg_last_error() gives the message.
 *
 * Each entry point names the reference interface it replaces (file:line in
 * the BCMTools 1.0.5 sources).  Streams are cudaStream_t passed as void*;
 * NULL means the context's own stream.  Asynchronous calls return once the
 * work is queued; *_end / bcmg_sync wait for it.
 *
 * Field data layout is the reference's Scalar3D<T> brick (Scalar3D.h:58-68,
 * Index3D.h:46-58): per block (nx+2vc)(ny+2vc)(nz+2vc) elements, x fastest,
 * cell (i,j,k) at i + nx0*j + nx0*ny0*k + (1+nx0+nx0*ny0)*vc.  On the device
 * the bricks of a field sit in one allocation, block b at element offset
 * b*block_stride (block_stride is the brick size rounded up to 256 bytes).
 * Host-side upload/download use bricks packed back to back, which is the
 * reference's contiguous setDataClass<D,U,T> layout (BlockManager.h:253-283).
 */
#ifndef BCMG_H
#define BCMG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define BCMG_API __attribute__((visibility("default")))
#else
#define BCMG_API
#endif

/* ---- status codes: ExitStatus (BCMTools.h:54-63) plus device-side ones ---- */
enum {
  BCMG_SUCCESS = 0,        /* EX_SUCCESS */
  BCMG_FAILURE = 1,        /* EX_FAILURE: invalid mesh, 2:1 violation, bad id */
  BCMG_USAGE = 16,         /* EX_USAGE: bad argument */
  BCMG_MEMORY = 17,        /* EX_MEMORY: device allocation failed / over budget */
  BCMG_READ_DATA = 20,     /* EX_READ_DATA */
  BCMG_WRITE_DATA = 21,    /* EX_WRITE_DATA */
  BCMG_NO_DEVICE = 40,     /* no usable CUDA device */
  BCMG_CUDA_ERROR = 41,    /* a CUDA runtime call failed */
  BCMG_DIVERGED = 42,      /* NaN/Inf residual (ILS3D.h:53-59 exits there) */
  BCMG_NOT_CONVERGED = 43, /* iteration limit reached (informational) */
  BCMG_BREAKDOWN = 44,     /* Krylov breakdown: rho or omega underflow */
  BCMG_SCRATCH_LIMIT = 45  /* more blocks than bcmg_dot_noalloc's fixed scratch holds */
};

enum { BCMG_F32 = 0, BCMG_F64 = 1 };

/* Face / subface numbering (BCMTools.h:48-51). */
enum { BCMG_X_M = 0, BCMG_X_P, BCMG_Y_M, BCMG_Y_P, BCMG_Z_M, BCMG_Z_P };

/* VCUpdateMethod::Type (BlockManager.h:40-47). */
enum { BCMG_VC_AT_ONCE = 0, BCMG_VC_SEPARATE_XYZ = 1, BCMG_VC_SEPARATE_XYZ_LEVELDIFF = 2 };

/* BoundaryInfo::Type (Utils/include/BoundaryInfo.h:32-37). */
enum { BCMG_BC_INNER = 0, BCMG_BC_DIRICHLET = 1, BCMG_BC_NEUMANN = 2, BCMG_BC_PERIODIC = 3 };

/* Dirichlet ghost forms: SOR = one layer g = 2v - f (sor1/Solver.cpp:232-294);
 * BCX = SOR plus second layer = v when vc >= 2 (SolverTest/bcx.f90:18-76). */
enum { BCMG_DIRICHLET_SOR = 0, BCMG_DIRICHLET_BCX = 1 };

/* Octree leaf orderings (BCMOctree.h:44-49). */
enum { BCMG_ORDER_Z = 0, BCMG_ORDER_HILBERT = 1, BCMG_ORDER_RANDOM = 2, BCMG_ORDER_PEDIGREE = 3 };

/* Dividers: Flat and Simple follow SimpleDivider.h:30-153; SPHERE follows
 * SphereDivider.h:28-150 (blocks inside the sphere become inactive leaves,
 * which are not blocks; the ripple margin of MultiRootDivider.h:56-100;
 * float arithmetic); CYLINDER follows CylinderDivider.h:28-153 (the same on
 * x, y around an axis along z, blocks outside inactive); SPHERE_SURFACE refines every block whose box meets a
 * sphere's surface, BALLS every block whose box meets one of a set of balls
 * (the seeded refinement used by the benchmark meshes); those two keep every
 * leaf active. */
enum { BCMG_DIV_FLAT = 0, BCMG_DIV_SIMPLE = 1, BCMG_DIV_SPHERE_SURFACE = 2, BCMG_DIV_BALLS = 3,
       BCMG_DIV_SPHERE = 4, BCMG_DIV_CYLINDER = 5 };

/* ======================= octree (host side, no device) =====================
 * Replaces BCMOctree (Utils/include/BCMOctree.h:39-219, BCMOctree.cpp) with
 * RootGrid (RootGrid.h) and the Divider family; adds 2:1 face balancing, which
 * the reference does not do (BCMOctree.cpp:462-468 exits instead). */
typedef struct bcmg_octree_s* bcmg_octree;

typedef struct {
  int nx, ny, nz;        /* root blocks per axis (RootGrid(nx,ny,nz)) */
  int periodic_mask;     /* bit0 x, bit1 y, bit2 z (RootGrid::setPeriodicX..) */
  double origin[3];      /* position of root 0 (BlockFactory rootOrigin) */
  double root_length;    /* edge of one root block (BlockFactory rootLength) */
} bcmg_rootgrid;

typedef struct {
  int kind;              /* BCMG_DIV_* */
  int min_level, max_level;
  int direction_mask;    /* SIMPLE: SimpleDivider::Direction bits (0 = ALL) */
  double center[3], radius;   /* SPHERE, CYLINDER (x, y): in root-index units (unit root
                                 blocks, root 0 at (0,0,0)) whatever the root grid's origin
                                 and root_length are, as the reference builds these
                                 dividers (SphereDivider.h:72, CylinderDivider.h:69);
                                 SPHERE_SURFACE; BALLS radius: physical coordinates */
  const double* points;  /* BALLS: npoints * 3 coordinates */
  int npoints;
  int balance;           /* nonzero: enforce 2:1 across faces */
  double margin_ratio;   /* SPHERE, CYLINDER: extraMarginRatio (SphereDivider.h:57-68) */
} bcmg_divider;

/* BCMOctree(RootGrid*, Divider*, Ordering) (BCMOctree.cpp:23-41). */
BCMG_API int bcmg_octree_build(bcmg_octree* out, const bcmg_rootgrid* rg,
                               const bcmg_divider* div, int ordering, uint64_t seed);
/* BCMOctree(RootGrid*, const vector<Pedigree>&) (BCMOctree.cpp:66-96);
 * pedigrees use the 64-bit packing of Pedigree.h (x:16 y:16 z:16 root:12 level:4). */
BCMG_API int bcmg_octree_from_pedigrees(bcmg_octree* out, const bcmg_rootgrid* rg,
                                        const uint64_t* pedigrees, int n);
BCMG_API int bcmg_octree_num_leaves(bcmg_octree t, int* n);
/* Leaf list in block-id order: pedigree, level, origin[3], block size. */
BCMG_API int bcmg_octree_leaves(bcmg_octree t, uint64_t* pedigree, int* level,
                                double* origin, double* block_size);
/* NeighborInfo[6] of every leaf (BCMOctree::makeNeighborInfo, BCMOctree.cpp:423-478):
 * ld[b*6+f] level difference, id[(b*6+f)*4+s] neighbour ids (-1 none),
 * sf[b*6+f] neighbour subface, outer[b*6+f] face on the domain boundary
 * (checkOnOuterBoundary, BCMOctree.cpp:368-396; periodic faces included). */
BCMG_API int bcmg_octree_neighbors(bcmg_octree t, int* ld, int* id, int* sf, int* outer);
BCMG_API void bcmg_octree_destroy(bcmg_octree t);

/* ============================ context / mesh =============================== */
typedef struct bcmg_ctx_s* bcmg_ctx;

/* BlockManager::getInstance (BlockManager.h:153-156), one per host thread;
 * binds CUDA device `device` and creates the context stream. */
BCMG_API int bcmg_ctx_create(bcmg_ctx* out, int device);
BCMG_API void bcmg_ctx_destroy(bcmg_ctx c);
BCMG_API const char* bcmg_last_error(bcmg_ctx c);
BCMG_API int bcmg_sync(bcmg_ctx c, void* stream);
/* Device memory budget for fields and work vectors (0 = unlimited); an
 * allocation beyond it fails with BCMG_MEMORY before touching the device. */
BCMG_API int bcmg_set_memory_budget(bcmg_ctx c, size_t bytes);
BCMG_API int bcmg_memory_in_use(bcmg_ctx c, size_t* bytes);

/* BlockManager::registerBlock + endRegisterBlock (BlockManager.cpp:28-59):
 * nb blocks of nx*ny*nz cells (even, equal for all blocks, BlockBase.h:68-79),
 * with their flattened NeighborInfo tables (format of bcmg_octree_neighbors).
 * Builds the face table on the device (setFaceLists, BlockManager.cpp:471-530). */
BCMG_API int bcmg_register_blocks(bcmg_ctx c, int nb, int nx, int ny, int nz,
                                  const int* ld, const int* id, const int* sf);

/* Device-side mesh set-up: the octree, its 2:1 balance, the neighbour table
 * and the face tables made on the context's GPU, then the blocks registered
 * as bcmg_register_blocks does (BCMOctree.cpp:23-41, 66-96, 423-478 and
 * BlockManager.cpp:63-114 on the device).
 * bcmg_mesh_build: the octree of `div` over `rg`, 2:1 balanced when
 *   div->balance, blocks = its active leaves in Z order: the leaves, order
 *   and neighbour table of bcmg_octree_build(..., BCMG_ORDER_Z, 0) followed
 *   by bcmg_octree_neighbors.
 * bcmg_mesh_register_pedigrees: blocks = the listed leaves in list order,
 *   neighbours as bcmg_octree_from_pedigrees gives them (regions the list
 *   leaves out are inactive); with `balance`, the list is first refined 2:1
 *   (those regions taking part as inactive leaves) and the blocks are the
 *   balanced active leaves in Z order.  BCMG_USAGE for a leaf listed twice or
 *   listed above another, BCMG_FAILURE when a face spans two levels or more.
 * bcmg_mesh_pedigrees: the registered leaves' pedigrees (nb of them);
 * bcmg_mesh_neighbors: the registered neighbour table (ld[nb*6],
 *   id[nb*24], sf[nb*6]; outer[nb*6] for meshes of the device set-up, else
 *   pass null). */
BCMG_API int bcmg_mesh_build(bcmg_ctx c, const bcmg_rootgrid* rg, const bcmg_divider* div, int nx,
                             int ny, int nz);
BCMG_API int bcmg_mesh_register_pedigrees(bcmg_ctx c, const bcmg_rootgrid* rg,
                                          const uint64_t* pedigrees, int n, int balance, int nx,
                                          int ny, int nz);
/* bcmg_mesh_build_batch: k meshes (rgs[i], divs[i]) built on the device and
 * registered as one block set, mesh i's blocks from first[i] on (no face
 * joins two meshes); each as bcmg_mesh_build makes it alone. */
BCMG_API int bcmg_mesh_build_batch(bcmg_ctx c, int k, const bcmg_rootgrid* rgs,
                                   const bcmg_divider* divs, int nx, int ny, int nz, int* first);
BCMG_API int bcmg_mesh_pedigrees(bcmg_ctx c, uint64_t* pedigrees);
/* Ghost exchange with blocks of another process: the reference's
 * communication buffers (Scalar3DUpdater::copyToCommBuffer*,
 * copyFromCommBuffer*, Scalar3DUpdater.h:377-515, 711-901) packed and
 * unpacked on the device.  An entry names one receiving face: `face` the
 * receiver's face, `kind` BCMG_XCH_COPY (same level), BCMG_XCH_F2C (the
 * sender is finer; `subface` the quarter of the receiver's face) or
 * BCMG_XCH_C2F (the sender is coarser; `subface` the receiver's position on
 * the sender's face, NeighborInfo's neighbour subface), `block` the local
 * block -- the sender for bcmg_xch_pack, the receiver for bcmg_xch_unpack.
 * The sender computes the ghost values (copy, F2C average, C2F
 * interpolation, as the local update does) into `buf` (device memory),
 * entry after entry, each in the reference's buffer order (the receiving
 * ghost box, x fastest; vc*n*n values, vc*(n/2)^2 for F2C); the receiver
 * copies them into its ghosts.  bcmg_xch_bytes: the buffer size of a list. */
enum { BCMG_XCH_COPY = 0, BCMG_XCH_F2C = 1, BCMG_XCH_C2F = 2 };
typedef struct {
  int block, face, subface, kind;
} bcmg_xch_entry;
BCMG_API int bcmg_xch_bytes(bcmg_ctx c, int field, const bcmg_xch_entry* e, int n,
                            size_t* bytes);
BCMG_API int bcmg_xch_pack(bcmg_ctx c, int field, const bcmg_xch_entry* e, int n, void* buf,
                           void* stream);
BCMG_API int bcmg_xch_unpack(bcmg_ctx c, int field, const bcmg_xch_entry* e, int n,
                             const void* buf, void* stream);
/* Number of registered blocks (0 before registration). */
BCMG_API int bcmg_num_blocks(bcmg_ctx c, int* nb);
BCMG_API int bcmg_mesh_neighbors(bcmg_ctx c, int* ld, int* id, int* sf, int* outer);
/* Per-block boundary conditions: BoundaryInfo (Utils/include/BoundaryInfo.h)
 * with its values (sor1/main.cpp:141-143), bc_type[b*6+f] in BCMG_BC_*,
 * bc_value[b*6+f], Dirichlet ghost form BCMG_DIRICHLET_*.  A Neumann face's
 * value is the ghost increment per layer, the outward derivative times the
 * cell size (SolverTest/bcx.f90:198-376): ghost 1 = interior -/+ value in the
 * field's type, ghost 2 (vc >= 2) = interior -/+ 2*value in double, minus
 * faces subtracting.  Neumann faces run the Jacobi and BiCGSTAB iterations
 * as separate sweep and ghost launches; bcmg_sor_run rejects them with
 * BCMG_FAILURE, as sor1/Solver.cpp:214-221 does. */
BCMG_API int bcmg_set_boundary(bcmg_ctx c, const int* bc_type, const double* bc_value, int form);

/* ================================ fields ===================================
 * BlockManager::setDataClass<Scalar3D<T>, U>(vc) (BlockManager.h:226-247):
 * one Scalar3D<T> brick per block; ghosts start at 0. */
BCMG_API int bcmg_field_create(bcmg_ctx c, int dtype, int vc, int* field);
/* The same field in page-locked host memory mapped into the device's address
 * space (one pointer for host and device): the storage behind the C++
 * drop-in's Scalar3D<T> (include/bcmtools/BlockManager.h), whose host code
 * keeps sweeping its bricks as the reference does (Scalar3D.h:75-85, the
 * contiguous setDataClass<D,U,T> of BlockManager.h:253-283) while the ghost
 * update, Dirichlet ghosts, fills, copies and reductions run on the device.
 * The sweep and solver entry points (SOR, Jacobi, BiCGSTAB, coefficient
 * fields) refuse host fields with BCMG_USAGE.  Not counted in the budget. */
BCMG_API int bcmg_field_create_host(bcmg_ctx c, int dtype, int vc, int* field);
BCMG_API int bcmg_field_destroy(bcmg_ctx c, int field);
/* Scalar3D::getData / getIndex (Scalar3D.h:93-98): device pointer, element
 * stride between bricks, elements per brick. */
BCMG_API int bcmg_field_layout(bcmg_ctx c, int field, void** dptr, int64_t* block_stride,
                               int64_t* brick_elems);
BCMG_API int bcmg_field_upload(bcmg_ctx c, int field, const void* host, void* stream);
BCMG_API int bcmg_field_download(bcmg_ctx c, int field, void* host, void* stream);
/* fill (SolverTest/blas.f90:18-46): every cell of every brick, ghosts included. */
BCMG_API int bcmg_field_fill(bcmg_ctx c, int field, double value, void* stream);
/* Seeded uniform values in [lo, hi) on the interior cells of blocks
 * [first_block, first_block + nblocks), ghosts untouched; the value of a cell
 * depends only on (seed, block - first_block, cell), so a block range gets the
 * same values in any mesh it is part of (synthetic right-hand sides of the
 * batched and served workloads). */
BCMG_API int bcmg_field_fill_random(bcmg_ctx c, int field, int first_block, int nblocks,
                                    uint64_t seed, double lo, double hi, void* stream);
/* copy (blas.f90:82-110): whole bricks, same dtype and vc. */
BCMG_API int bcmg_field_copy(bcmg_ctx c, int dst, int src, void* stream);
/* LSSwap (LocalScalar3D.h:132-136): exchange the storage of two fields. */
BCMG_API int bcmg_field_swap(bcmg_ctx c, int a, int b);

/* ============================ ghost (VC) update ============================ */
/* BlockManager::prepareForVCUpdate (BlockManager.cpp:63-114). */
BCMG_API int bcmg_prepare_vc(bcmg_ctx c, int field, int tag, int method);
/* beginUpdateVC / endUpdateVC (BlockManager.h:449-455, 593-598) and their
 * per-axis / per-level-difference variants (BlockManager.h:461-726):
 * axis_mask bit a selects faces normal to axis a, ld_mask bit (ld+1) selects
 * level difference ld (bit0: C2F faces, bit1: same level, bit2: F2C faces).
 * begin launches one gather kernel over the selected entries; end waits. */
BCMG_API int bcmg_vc_begin(bcmg_ctx c, int field, int axis_mask, int ld_mask, void* stream);
BCMG_API int bcmg_vc_end(bcmg_ctx c, int field);
/* Dirichlet ghosts of all outer faces (sor1 Solver::setBoundaryCondition,
 * sor1/Solver.cpp:186-294; LocalScalar3D::ImposeBlockBoundaryCondition). */
BCMG_API int bcmg_bc_apply(bcmg_ctx c, int field, void* stream);
/* ImposeBoundaryCondition (LocalScalar3D.h:228-258): VC update of all faces
 * and the Dirichlet ghosts fused into one launch. */
BCMG_API int bcmg_impose_bc(bcmg_ctx c, int field, void* stream);

/* ================================ sweeps ==================================== */
/* sor1/sor2 Solver::run (sor1/Solver.cpp:74-129, sor2/Solver.cpp:77-133):
 * n_outer x { per block n_inner x (red-black SOR pass + block Dirichlet),
 *             then VC update + Dirichlet }.
 * form 1: coef[b*4..] = {c0, cx, cy, cz} of sor1; form 2: {c, cx, cy, cz} of
 * sor2 with source field s (s < 0 for none).  Coefficients are per block,
 * computed by the caller as the reference does. */
BCMG_API int bcmg_sor_run(bcmg_ctx c, int f, int s, const double* coef, double omega,
                          int form, int n_inner, int n_outer, void* stream);
/* Fused sweeps (default on): each outer iteration is one launch that writes
 * the next iterate and all its ghosts from shared memory (ping-pong with a
 * work copy of the field).  0 selects the separate sweep + gather launches of
 * the reference's order; results are identical. */
BCMG_API int bcmg_set_fusion(bcmg_ctx c, int enable);
/* Ghost form of the fused sweeps.  BCMG_GHOST_PULL: each launch first fills
 * its block's first ghost layer from the neighbours' interiors (ghosts on a
 * coarser block interpolated by the reader, F2C averages through a side
 * buffer their source CTAs write) and its Dirichlet ghosts from its own,
 * writes only its own brick, and a ghost update closes the run.  32^3 blocks
 * have the push form only.  BCMG_GHOST_PUSH: each launch writes every ghost value its interior
 * feeds into the neighbours' bricks.  BCMG_GHOST_AUTO (default): tuned or by
 * mesh size.  Results are identical; the forms differ in HBM traffic and in
 * the length of each CTA's chain of dependent loads. */
enum { BCMG_GHOST_PULL = 0, BCMG_GHOST_PUSH = 1, BCMG_GHOST_AUTO = 2 };
BCMG_API int bcmg_set_ghost_form(bcmg_ctx c, int form);
/* Kernel shape of the pull-form fused Jacobi sweep: 0 automatic (1), 1 one
 * CTA per block, 2 persistent CTAs double-buffering the next block.  Results
 * are identical. */
BCMG_API int bcmg_set_jacobi_shape(bcmg_ctx c, int shape);
/* Times the fused-Jacobi choices (1 push form, 2 pull form one CTA per
 * block, 3 pull form pipelined) on a copy of x (x is left unchanged) --
 * per sweep, as a run of 2*iters sweeps less a run of iters, so that a run's
 * fixed costs do not count -- and keeps the fastest for this (dtype, block
 * edge, vc); returns it (0 when the fused sweep does not apply) and its
 * time per sweep. */
BCMG_API int bcmg_autotune_jacobi(bcmg_ctx c, int op, int x, int b, double omega, int iters,
                                  int* best, double* best_us);
/* Kernel shape of the fused SOR sweep for cubic 8/16/32-cell blocks with
 * vc <= 2: 0 automatic (tuned if bcmg_autotune_sor ran, else 7 where it
 * applies, else 1); 1 one CTA per block, source staged in shared memory; 2
 * source read through L1; 3, 4 the same with 512 threads; 5 persistent CTAs
 * double-buffering the next block with bulk asynchronous copies; 6 the pull
 * ghost form, persistent CTAs double-buffering the next block (8/16-cell
 * blocks); 7 the pull ghost form, one CTA per block.  Results are identical. */
BCMG_API int bcmg_set_sor_variant(bcmg_ctx c, int variant);
/* Times every shape for `iters` outer iterations on a copy of field f (f is
 * left unchanged) and keeps the fastest for this (dtype, block edge, vc,
 * scheme) in the context; returns it and its time per iteration. */
BCMG_API int bcmg_autotune_sor(bcmg_ctx c, int f, int s, const double* coef, double omega,
                               int form, int iters, int* best, double* best_us);

/* 7-point operator: per-block constants cc[b*7+{Ap,Aw,Ae,As,An,Ab,At}], or
 * seven coefficient fields (SolverTest's Ap..At bricks, ILS3D.h:65-126). */
BCMG_API int bcmg_op_create_const(bcmg_ctx c, const double* cc, int* op);
BCMG_API int bcmg_op_create_fields(bcmg_ctx c, const int* fields7, int* op);
BCMG_API int bcmg_op_destroy(bcmg_ctx c, int op);
/* LocalScalar3D::ImposeBoundaryCondition(Ap..At, b) (SolverTest
 * LocalScalar3D.h:260-285, bca.f90:12-394): folds the outer faces of the
 * boundary table (faces without a neighbour) into the seven coefficient
 * fields of `op` and the right-hand side b, per cell in the order Aw, Ae,
 * As, An, Ab, At.  Dirichlet: Ap -= A_nb, b -= 2 A_nb v (A_nb v rounded to
 * the field's type, the rest in double), A_nb = 0.  Neumann (v the ghost
 * increment per layer, as in bcmg_set_boundary): Ap += A_nb, b += A_nb v on
 * minus faces and -= on plus faces, A_nb = 0.  Needs an operator of
 * coefficient fields (BCMG_USAGE otherwise); returns after the fold has run. */
BCMG_API int bcmg_op_fold_boundary(bcmg_ctx c, int op, int b, void* stream);

/* jacobi_smoother (blas.f90:452-502): x1 interior from x0 (with ghosts). */
BCMG_API int bcmg_jacobi_sweep(bcmg_ctx c, int op, int x1, int x0, int b, double omega,
                               void* stream);
/* n_iter x Jacobi_Smoother (ILS3D.h:65-126): sweep, then ghost update and
 * Dirichlet ghosts of the new iterate, with no convergence test.  For
 * per-block constant operators on cubic 8/16/32 blocks with vc <= 2 each
 * iteration is one fused launch (ping-pong with a work copy); use_graph != 0
 * captures the whole run into a CUDA graph on first use (needs a non-default
 * stream) and replays it afterwards. */
BCMG_API int bcmg_jacobi_run(bcmg_ctx c, int op, int x, int b, double omega, int n_iter,
                             int use_graph, void* stream);
/* calc_ax (blas.f90:556-600), calc_r (:602-648). */
BCMG_API int bcmg_calc_ax(bcmg_ctx c, int op, int ax, int x, void* stream);
BCMG_API int bcmg_calc_r(bcmg_ctx c, int op, int r, int x, int b, void* stream);
/* calc_r2 summed over all blocks (ILS3D::CalcR2, ILS3D.h:211-270), FP64
 * accumulation; synchronises the stream. */
BCMG_API int bcmg_calc_r2(bcmg_ctx c, int op, int x, int b, double* rr, void* stream);
/* ILS3D::DOT (ILS3D.h:272-311, blas.f90:379-412), FP64 accumulation,
 * deterministic; synchronises the stream. */
BCMG_API int bcmg_dot(bcmg_ctx c, int x, int y, double* out, void* stream);
/* Inner product that allocates nothing.  No counterpart in the reference.
 * It serves callers that cannot call cudaMalloc: host code embedded in an
 * application or framework that owns every device allocation through its
 * own pool, where nothing else may allocate and the caller has no way to
 * size a scratch buffer for this library.  It needs no context: x and y
 * are device field arenas (nb bricks of (nx+2vc)(ny+2vc)(nz+2vc) elements
 * of `dtype`, block_stride elements apart, as bcmg_field_layout reports),
 * `result` is a device double, and the work is queued on `stream` on the
 * calling thread's current device.  It computes what bcmg_dot computes,
 * with the same kernels.
 *
 * Its scratch (one double per block) is a fixed array inside the library,
 * BCMG_NOALLOC_MAX_BLOCKS entries (512 KiB) that every GPU loading the
 * library holds until the process exits; more blocks return
 * BCMG_SCRATCH_LIMIT, and bricks or brick planes beyond int32 elements
 * BCMG_USAGE.  The first call on a device (and the first after its context
 * was re-created, e.g. by cudaDeviceReset) looks up the array's device
 * address, so that first call should come before any stream capture.  All
 * calls share the array and it keeps the last call's partial sums: two calls
 * whose work overlaps on the GPU (for instance on two streams) race and give
 * wrong results. */
#define BCMG_NOALLOC_MAX_BLOCKS 65536
BCMG_API int bcmg_dot_noalloc(int dtype, const void* x, const void* y, int nb, int nx, int ny,
                              int nz, int vc, int64_t block_stride, double* result, void* stream);
/* AXPY/XPAY/AXPYZ/AXPBYPZ (ILS3D.h:313-405, blas.f90:242-377) on interiors. */
BCMG_API int bcmg_axpy(bcmg_ctx c, int y, int x, double a, void* stream);
BCMG_API int bcmg_xpay(bcmg_ctx c, int y, int x, double a, void* stream);
BCMG_API int bcmg_axpyz(bcmg_ctx c, int z, int x, int y, double a, void* stream);
BCMG_API int bcmg_axpbypz(bcmg_ctx c, int z, int x, int y, double a, double b, void* stream);

/* ================================ solvers =================================== */
typedef struct {
  int iterations;       /* count as ILS3D returns it (0: b = 0 or rho = 0) */
  double residual;      /* |r|^2 / |b|^2 at exit (IsConverged, ILS3D.h:41-63) */
  int status;           /* BCMG_SUCCESS / BCMG_NOT_CONVERGED / BCMG_DIVERGED / ... */
  int refinements;      /* mixed precision: outer refinement steps */
  double true_residual; /* mixed precision: FP64 |b - Ax| / |b| at exit */
  int fp64_iterations;  /* mixed precision: iterations of the FP64 BiCGSTAB that finished
                           the solve when the FP32 corrections stalled (0: none) */
} bcmg_solve_info;

/* Independent systems in one mesh: blocks [seg_first[s], seg_first[s+1]) are
 * segment s (seg_first[0] = 0, seg_first[nseg] = the block count; no face
 * joins two segments, BCMG_USAGE otherwise).  The solvers below then solve
 * every segment as its own system -- own scalars, residuals and convergence
 * test, results identical to solving it alone -- with every launch advancing
 * all of them; their info argument holds one record per segment.  No
 * counterpart in the reference, where one BlockManager holds one system. */
BCMG_API int bcmg_set_segments(bcmg_ctx c, int nseg, const int* seg_first);

/* ILS3D::Jacobi (ILS3D.h:478-529): x, b fields; ghosts via VC + Dirichlet
 * after every sweep; convergence |r|^2/|b|^2 <= eps^2. */
BCMG_API int bcmg_jacobi_solve(bcmg_ctx c, int op, int x, int b, double omega, int max_iter,
                               double eps, bcmg_solve_info* info, void* stream);
/* ILS3D::BiCGSTAB (ILS3D.h:663-844), right Jacobi preconditioner with n_pre
 * passes; vectors in the dtype of x; scalars in FP64 on the device, inner
 * products reduced in FP64 (float fields: exact products summed in
 * float-float along block columns, FP64 beyond); the host reads the
 * segments' status only between chunks of queued iterations. */
BCMG_API int bcmg_bicgstab(bcmg_ctx c, int op, int x, int b, double omega, int n_pre,
                           int max_iter, double eps, bcmg_solve_info* info, void* stream);
/* Mixed precision: x, b FP64 fields; FP64 residual r = b - Ax recomputed on
 * the device, FP32 BiCGSTAB correction solves to eps_inner -- or to half
 * the reduction the target still asks for, when that is looser -- or
 * max_inner iterations (each keeps its iterate of smallest residual), FP64 correction
 * accumulation, until |b - Ax| / |b| <= eps; a correction that does not
 * reduce |b - Ax| is undone and the correction solves' iteration cap halved;
 * when it would drop below 10, or after max_outer rounds, the FP64 BiCGSTAB
 * finishes from x (at most max_outer * max_inner iterations, counted in
 * info->iterations and reported in info->fp64_iterations; its work vectors
 * are allocated then).  Per segment (bcmg_set_segments), each with its own
 * refinement history. */
BCMG_API int bcmg_bicgstab_mixed(bcmg_ctx c, int op, int x, int b, double omega, int n_pre,
                                 int max_inner, double eps_inner, int max_outer, double eps,
                                 bcmg_solve_info* info, void* stream);

/* Per-launch CUDA-event timing on the launching stream.  Between
 * bcmg_profile_begin and bcmg_profile_end every kernel launch of the context is
 * bracketed by two events; end synchronises the device and returns, per kernel
 * kind, the summed device time in ms and the launch count.  Kinds: 0 ghost
 * gather, 1 red-black SOR, 2 Jacobi, 3 residual/calc_ax, 4 dot/reduction,
 * 5 BLAS-1, 6 fill, 7 other (8 entries). */
BCMG_API int bcmg_profile_begin(bcmg_ctx c);
BCMG_API int bcmg_profile_end(bcmg_ctx c, double* ms_by_kind, int64_t* count_by_kind);

/* Kernel launches issued by this context since creation (all entry points). */
BCMG_API int bcmg_launch_count(bcmg_ctx c, int64_t* n);

/* Self-check of the sweeps' division (a / b from a precomputed RN(1/b), two
 * FMA corrections) against the division instruction sequence on n seeded
 * random operand pairs per type; returns the numbers of differing results.
 * Allocates 16 bytes of device memory; runs on the default stream. */
BCMG_API int bcmg_check_division(uint64_t seed, int64_t n, int64_t* bad_f32, int64_t* bad_f64);

#ifdef __cplusplus
}
#endif
#endif
