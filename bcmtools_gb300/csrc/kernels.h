// kernels.h -- internal launcher declarations shared by the C ABI and the
// kernel translation units.  Not part of the public interface.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "krylov.cuh"

namespace bcmg {

// Up to 12 contiguous slices of the face table (4 kinds x 3 axes) selected
// by one launch; prefix[q] is the first warp of slice q.
struct VcRanges {
  int start[12];
  int prefix[13];
  int n;
};

template <typename T>
cudaError_t launch_vc_gather(T* data, const Geom& g, const VcTable& tab, const VcRanges& rg,
                             cudaStream_t st);

// Block Dirichlet description for the SOR kernel.
struct BlockBc {
  const int* type;      // [nb*6] BCMG_BC_*
  const double* value;  // [nb*6]
  int bcx;              // second ghost layer = v when vc >= 2
  // [nb*8] 2v (v rounded to float first in the bcx form) as a float where
  // that is exact, else NaN: lets float sweeps form 2v - f in one float
  // subtraction (tile_dirichlet)
  const float* v2f;
};

// Incoming ghost source of one face of one block (the pull form): kind -1
// (no neighbour), VC_COPY / VC_C2F (src[0], sub = the neighbour's subface)
// or VC_F2C (src[s] the fine neighbour on subface s).
struct FaceIn {
  int src[4];
  int kind;
  int sub;
};

// Per-block descriptor of the pull-form sweeps.  csrc[f]: the same-level
// neighbour on face f; for a face fed by a coarser block (flag bit
// bi_c2f_bit(f)) coarse block * 4 + this block's subface on it (the reader
// interpolates those ghosts from the coarse interior); for a face fed by
// finer blocks its slot in the side buffer of first-layer F2C ghosts; or -1.
// flags: bit f the face is fed by a neighbour (BI_FED << f), bit 8+f by a
// same-level one (BI_COPY << f), bit 16+f it carries a Dirichlet condition,
// bits 24..30 the number of F2C entries this block feeds (listed from
// out_begin).
struct BlockInfo {
  int csrc[6];
  int flags;
  int out_begin;
};
enum : unsigned { BI_FED = 1u, BI_COPY = 1u << 8, BI_DIR_SHIFT = 16, BI_OUT_SHIFT = 24 };
constexpr int kMaxOutEntries = 24;  // 6 faces x 4 finer neighbours
// Flag bit of a face fed by a coarser block (bits 6-7, 14-15, 22-23 are free).
__host__ __device__ constexpr int bi_c2f_bit(int f) { return f < 2 ? 6 + f : f < 4 ? 12 + f : 18 + f; }

// Outgoing ghost entries of every block (face-table entries grouped by source
// block, CSR): the entries a fused sweep CTA writes from shared memory.
struct PushTable {
  const int* ptr;        // [nb+1]
  const VcTask* tasks;   // entries with src == block, destination's view
  const unsigned char* fed;  // [nb] bit f: some neighbour writes face f's ghosts
  const FaceIn* in;          // [nb*6] ghost sources of each face (pull form)
  const BlockInfo* info;     // [nb] descriptors of the pull form
  const VcTask* out_tasks;   // F2C entries by source block (pull form)
  const void* side_in;       // first-layer F2C ghosts of the input
  void* side_out;            // ... of the output, written by their sources
  // x-face layers of the pipelined pull form, 2*N*N per block: block b's
  // columns x = 0 and x = N-1 (cell (y, z) at z*N + y) as the input had them,
  // and as the output has them (written by the launch that writes b)
  const void* xf_in;
  void* xf_out;
};


constexpr size_t kSorMaxSmem = 200 * 1024;
// Dynamic shared memory one CTA may use (227 KB on sm_100-class GPUs).
constexpr size_t kPipeMaxSmem = 227 * 1024;

// Kernel shapes of the fused sweep, chosen per (dtype, N, VC, scheme) by the
// autotuner (bcmg_autotune_sor) or fixed with bcmg_set_sor_variant.
enum SorVariant : int {
  SV_AUTO = 0,       // tuned choice if any, else SV_TILE_SS_256
  SV_TILE_SS_256 = 1,  // one CTA per block, source staged in shared memory
  SV_TILE_GS_256 = 2,  // one CTA per block, source read from global (L1)
  SV_TILE_SS_512 = 3,
  SV_TILE_GS_512 = 4,
  SV_PIPE_256 = 5,     // persistent, bulk-copy double buffering
  SV_PULL = 6,         // pull-form ghosts, persistent CTAs, double-buffered bulk copies
  SV_PULL_TILE = 7,    // pull-form ghosts, one CTA per block, bulk copies
  SV_COUNT = 8
};

// Red-black SOR pass(es).  fused: read A, write B with all ghosts (needs
// `push`); otherwise in place on B (A == B).
template <typename T>
cudaError_t launch_sor(const T* A, T* B, const T* s, const Geom& g, const double* coef,
                       double omega, int form, int n_inner, BlockBc bc, PushTable push,
                       bool fused, int* err, int variant, int pull_now, cudaStream_t st,
                       bool s_packed = false);
// Interior cells of every block of `src` into `dst`, N^3 per block in the
// order the pull-form SOR kernels sweep them (their packed source).
template <typename T>
cudaError_t launch_pack_source(T* dst, const T* src, const Geom& g, cudaStream_t st);
// Whether the pipelined pull-form sweeps cover this shape: cubic 8^3 / 16^3
// blocks, vc 1 or 2, two stages (tile, second field if any, 640 B of block
// constants and entries) within one CTA's shared memory.
inline bool pipe_shape_ok(int dtype_bytes, int n, int vc, bool second_field) {
  if ((n != 8 && n != 16) || (vc != 1 && vc != 2)) return false;
  const size_t lx = (size_t)n + 2 * vc, es = (size_t)dtype_bytes;
  const size_t tile = (lx * (n + 2) * (n + 2) * es + 127) / 128 * 128;
  const bool compact = (vc * lx * es) % 16 == 0;
  const size_t s = second_field ? ((size_t)n * (compact ? n * lx : lx * lx) * es + 127) / 128 * 128 : 0;
  return 2 * (tile + s + 640) <= kPipeMaxSmem;
}
inline bool sor_pull_ok(int dtype_bytes, int n, int vc, int form) {
  return pipe_shape_ok(dtype_bytes, n, vc, form == 2);
}

// Seven-point operator: per-block constants cc[b*7+c] (double, rounded to T
// in the kernel) or seven coefficient fields.
template <typename T>
struct Op {
  const double* cc;
  const T* A[7];
  const T* cf8;  // per block {Ap..At, RN(1/Ap)} rounded to T (constant operators), or null
};

template <typename T>
cudaError_t launch_jacobi(T* x1, const T* x0, const T* b, Op<T> op, const Geom& g, T omega,
                          cudaStream_t st);
// Fused Jacobi sweep: x1 interior, Dirichlet ghosts and pushed VC ghosts from
// x0 (per-block constant operator: cf[b*8 + 0..6] the seven coefficients and
// cf[b*8 + 7] 1/Ap, all rounded to T); every other cell of x1 (edges,
// corners, ghost layers no neighbour or Dirichlet condition writes) takes
// x0's value.  partial[b] = sum of squared residuals of x0 when partial !=
// null.  cudaErrorInvalidValue for shapes it does not cover (cubic 8/16
// blocks, vc <= 2, tiles within shared memory).
// Ghost modes of the fused sweeps.  kGhostPush: x0's ghosts are read as
// they are and the launch writes every ghost x1 feeds (x1 leaves with all
// ghosts updated).  kGhostPull: the launch first fills x0's first ghost
// layer from its neighbours' interiors and its Dirichlet ghosts (the ghost
// update that follows a sweep, done by the reader), and writes no ghost of a
// fed face -- x1's ghosts need a ghost update before anything else reads
// them.  kGhostAsIs: the pull kernel on x0's ghosts as they are (the first
// launch of a run).
// kGhostPushZero: the push form on 32^3 blocks with x0 taken as zero
// everywhere (not read): the first pass of a preconditioner from zero.
enum : int { kGhostPush = 0, kGhostPull = 1, kGhostAsIs = 2, kGhostPushZero = 3 };
// Kernel shapes of the pull-form Jacobi sweep: one CTA per block, or the
// persistent double-buffered pipeline.
enum : int { kJacobiTile = 1, kJacobiPipe = 2 };
// The BiCGSTAB preconditioner's zero-start pass made in one launch with the
// vector update that produces its right-hand side b (32^3 blocks, streamed
// kernel): kind kPreP b = r + beta (b - gamma q) (kr_p), kPreS b = r -
// alpha q (kr_s), kPreCopy b = r; the new b is written back, the scalars
// come from the segments' records, blocks of finished segments are skipped.
enum : int { kPreNone = 0, kPreP = 1, kPreS = 2, kPreCopy = 3 };
template <typename T>
struct JacPre {
  int kind;
  const T* r;
  const T* q;
  KSegs segs;
};

template <typename T>
cudaError_t launch_jacobi_fused(const T* x0, T* x1, const T* b, const Geom& g, const T* cf,
                                T omega, BlockBc bc, PushTable push, int ghost_mode, int shape,
                                double* partial, int* err, const JacPre<T>* pre,
                                cudaStream_t st);
// mode 0: ax = A x;  mode 1: r = b - A x;  mode 2: partial[b] = sum r^2 (no store)
template <typename T>
cudaError_t launch_residual(T* out, const T* x, const T* b, Op<T> op, const Geom& g, int mode,
                            double* partial, cudaStream_t st);
// Per-block FP64 partial sums of x.y (interiors).
template <typename T>
cudaError_t launch_dot_partial(const T* x, const T* y, const Geom& g, double* partial,
                               cudaStream_t st);
// Sum n partials in a fixed order into *out (one CTA).
cudaError_t launch_reduce_final(const double* partial, int n, double* out, cudaStream_t st);

// Interior BLAS-1: kind 0 axpy y+=a x; 1 xpay y=x+a y; 2 axpyz z=a x+y;
// 3 axpbypz z=a x+b y+z; 4 scal z=a z.
template <typename T>
cudaError_t launch_blas1(int kind, T* z, const T* x, const T* y, T a, T b, const Geom& g,
                         cudaStream_t st);
// Folds the boundary faces of a coefficient-brick operator into its diagonal
// and the right-hand side (SolverTest bca.f90:12-394): code[b*6+f] 0 none,
// 1 Dirichlet, 2 Neumann; xc[b*6+f] the face value.  Three launches, x then
// y then z faces, so every cell sees the reference's Aw, Ae, As, An, Ab, At
// order.
template <typename T>
struct FoldPtrs {
  T* A[7];  // Ap, Aw, Ae, As, An, Ab, At
  T* b;
};
template <typename T>
cudaError_t launch_fold_boundary(FoldPtrs<T> p, const Geom& g, const int* code, const double* xc,
                                 cudaStream_t st);
// Exchange with other processes (exchange.cu): pack (values of each entry
// from its source block t.src into buf + off) or unpack (buf + off into the
// ghosts of t.dst).
template <typename T>
cudaError_t launch_xch(T* data, const Geom& g, const VcTask* ents, const int64_t* off, int n,
                       T* buf, bool pack, cudaStream_t st);

// Device-resident BiCGSTAB iteration (krylov.cu): see krylov.cuh.
template <typename T>
cudaError_t launch_kr_p(T* p, const T* r, const T* q, const Geom& g, KSegs S, cudaStream_t st);
template <typename T>
cudaError_t launch_kr_s(T* s, const T* r, const T* q, const Geom& g, KSegs S, cudaStream_t st);
template <typename T>
cudaError_t launch_kr_ax(T* out, const T* x, Op<T> op, const T* y0, int ndot, const Geom& g,
                         KSegs S, double* partial, int* err, cudaStream_t st);
template <typename T>
cudaError_t launch_kr_xr(T* x, T* r, const T* p_, const T* s_, const T* s, const T* t,
                         const T* r0, const Geom& g, KSegs S, double* partial, int* err, cudaStream_t st);
template <typename T>
cudaError_t launch_kr_dot2(const T* x, const T* y, const T* u, const T* v, const Geom& g,
                           double* partial, cudaStream_t st);
template <typename T>
cudaError_t launch_kr_best(T* xbest, const T* x, const Geom& g, KSegs S, cudaStream_t st);
cudaError_t launch_kr_scalar(const double* partial, int nb, KSegs S, int stage, int max_iter,
                             double eps2, int keep_best, cudaStream_t st);
cudaError_t launch_kr_segsum(const double* partial, int nb, KSegs S, double* out,
                             cudaStream_t st);
template <typename T>
cudaError_t launch_kr_seg_copy(T* dst, const T* src, const Geom& g, const int* seg_of,
                               const unsigned char* flag, cudaStream_t st);
cudaError_t launch_kr_seg_to32(float* r32, const double* r64, const Geom& g32, const Geom& g64,
                               const int* seg_of, const unsigned char* flag, const double* scale,
                               cudaStream_t st);
cudaError_t launch_kr_seg_acc(double* x64, const float* d32, const Geom& g32, const Geom& g64,
                              const int* seg_of, const unsigned char* flag, const double* scale,
                              cudaStream_t st);

template <typename T>
cudaError_t launch_fill(T* x, int64_t n, T v, cudaStream_t st);
template <typename T>
cudaError_t launch_fill_random(T* x, const Geom& g, int b0, int nb, uint64_t seed, double lo,
                               double hi, cudaStream_t st);

}  // namespace bcmg
