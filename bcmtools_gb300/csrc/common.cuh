// common.cuh -- shared device definitions for the bcmtools_gb300 kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bcmg {

// Brick geometry of one field (Scalar3D<T> layout, Scalar3D.h:58-68):
// cell (i,j,k), i in [-vc, nx+vc), lives at off0 + i + sy*j + sz*k of the
// block's brick, bricks `bstride` elements apart.
struct Geom {
  int nx, ny, nz, vc;
  int sy, sz;      // nx0, nx0*ny0
  int off0;        // (1 + nx0 + nx0*ny0) * vc
  int64_t bstride;
  int nb;
  __host__ __device__ __forceinline__ int at(int i, int j, int k) const {
    return off0 + i + sy * j + sz * k;
  }
};

// Arithmetic without multiply-add contraction, so that every rounding step
// matches a C compiler run with -ffp-contract=off (the oracle) and the
// reference's x86-64 build (-O3, no FMA).
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xdiv(double a, double b) { return __ddiv_rn(a, b); }

// Face-table entry kinds.
enum : uint8_t { VC_COPY = 0, VC_F2C = 1, VC_C2F = 2, VC_DIRICHLET = 3 };

// One entry of the device face table: one (block, face, subface) of the
// reference's local face list (BlockManager.cpp:477-510), or one Dirichlet
// outer face.  16 bytes.
struct VcTask {
  int dst;          // block whose ghosts are written
  int src;          // neighbour block read (VC_COPY/F2C/C2F)
  uint8_t face;     // BCMG_X_M..BCMG_Z_P of dst
  uint8_t kind;     // VC_*
  uint8_t subface;  // F2C: dst subface; C2F: neighbour subface
  uint8_t flags;    // bit0: Dirichlet BCX second layer; kTaskNeumann: Neumann ghosts
  int slot;         // pull form: side-buffer slot of (dst, face) for F2C/C2F entries
};

constexpr uint8_t kTaskNeumann = 2;  // VC_DIRICHLET entry of a Neumann face

struct VcTable {
  const VcTask* tasks;
  int ntasks;
  const double* bcval;  // [nb*6] Dirichlet values (VC_DIRICHLET)
};

}  // namespace bcmg
