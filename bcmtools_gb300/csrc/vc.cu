// vc.cu -- the ghost (virtual cell) gather kernel.
//
// One launch updates every selected face of every block of one field: the
// reference's per-face loop BlockManager::copyVCFromNeighbor
// (BlockManager.cpp:715-743) over Scalar3DUpdater<T>'s same-level copy, F2C
// average and C2F interpolation (Scalar3DUpdater.h:181-266, 321-373,
// 519-708), plus the Dirichlet ghosts of outer faces (sor1/Solver.cpp:232-294,
// SolverTest/bcx.f90:18-76).  Every read is an interior cell and every write a
// ghost cell, so entries are independent and run concurrently.
//
// Work decomposition: one warp per face-table entry, lanes walking the entry's
// ghost box x-fastest (coalesced along rows for Y and Z faces).
#include "ghost.cuh"
#include "kernels.h"
#include "tile.cuh"

namespace bcmg {

template <typename T>
__global__ void __launch_bounds__(256) vc_gather_kernel(T* __restrict__ data, Geom g,
                                                        VcTable tab, VcRanges rg) {
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= rg.prefix[rg.n]) return;
  int q = 0;
  while (w >= rg.prefix[q + 1]) q++;
  const VcTask t = tab.tasks[rg.start[q] + (w - rg.prefix[q])];
  T* __restrict__ dst = data + (int64_t)t.dst * g.bstride;
  const int sb = t.kind == VC_DIRICHLET ? t.dst : t.src;
  const Acc<T> src{data + (int64_t)sb * g.bstride, g.sy, g.sz, g.off0};
  const double bcv = t.kind == VC_DIRICHLET ? tab.bcval[t.dst * 6 + t.face] : 0.0;
  task_apply<T>(t, dst, g, src, bcv, lane, 32);
}

// Cubic 8^3 / 16^3 / 32^3 blocks with vc <= 2: the same entries with the
// entry's kind, axis, block edge and ghost width fixed at compile time,
// reading the source brick in place (push_entry over the brick layout).
// The compiler's register budget (64 a thread): at the 40 of 6 CTAs per SM
// the copies of 16 cells in flight spill, and the same-level update of the
// two-level sphere mesh measured 68 us against 54.
template <typename T, int N, int VC>
__global__ void __launch_bounds__(256)
    vc_gather_cubic_kernel(T* __restrict__ data, Geom g, VcTable tab, VcRanges rg) {
  using BL = BrickTile<T, N, VC>;
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= rg.prefix[rg.n]) return;
  int q = 0;
  while (w >= rg.prefix[q + 1]) q++;
  const VcTask t = tab.tasks[rg.start[q] + (w - rg.prefix[q])];
  T* dst = data + (int64_t)t.dst * g.bstride;
  if (t.kind == VC_DIRICHLET) {
    const Acc<T> src{dst, g.sy, g.sz, g.off0};
    task_apply<T>(t, dst, g, src, tab.bcval[t.dst * 6 + t.face], lane, 32);
    return;
  }
  const T* src = data + (int64_t)t.src * g.bstride;
  if constexpr (sizeof(T) == 8 && N <= 16) {
    // FP64 C2F in two stages (c2f_entry_sep): the double pipe is its bound
    __shared__ double scr[8][kC2fScratch];
    if (t.kind == VC_C2F) {
      c2f_sep_dispatch<N, VC, BL>(t, reinterpret_cast<double*>(dst), g,
                                  reinterpret_cast<const double*>(src), lane,
                                  scr[threadIdx.x >> 5]);
      return;
    }
  }
  // 16 cells in flight per lane up to 16^3 blocks (measured faster there),
  // 8 for 32^3 (register budget)
  push_dispatch<T, N, VC, BL, (N <= 16 ? 16 : 8)>(t, dst, g, src, lane);
}

template <typename T>
cudaError_t launch_vc_gather(T* data, const Geom& g, const VcTable& tab, const VcRanges& rg,
                             cudaStream_t st) {
  const int nw = rg.prefix[rg.n];
  if (nw == 0) return cudaSuccess;
  const int warps_per_cta = 8;
  const int grid = (nw + warps_per_cta - 1) / warps_per_cta;
  const bool cubic = g.nx == g.ny && g.ny == g.nz && (g.vc == 1 || g.vc == 2);
  const int key = cubic ? g.nx * 4 + g.vc : 0;
  switch (key) {
    case 8 * 4 + 1: vc_gather_cubic_kernel<T, 8, 1><<<grid, 256, 0, st>>>(data, g, tab, rg); break;
    case 8 * 4 + 2: vc_gather_cubic_kernel<T, 8, 2><<<grid, 256, 0, st>>>(data, g, tab, rg); break;
    case 16 * 4 + 1: vc_gather_cubic_kernel<T, 16, 1><<<grid, 256, 0, st>>>(data, g, tab, rg); break;
    case 16 * 4 + 2: vc_gather_cubic_kernel<T, 16, 2><<<grid, 256, 0, st>>>(data, g, tab, rg); break;
    case 32 * 4 + 1: vc_gather_cubic_kernel<T, 32, 1><<<grid, 256, 0, st>>>(data, g, tab, rg); break;
    case 32 * 4 + 2: vc_gather_cubic_kernel<T, 32, 2><<<grid, 256, 0, st>>>(data, g, tab, rg); break;
    default: vc_gather_kernel<T><<<grid, 32 * warps_per_cta, 0, st>>>(data, g, tab, rg); break;
  }
  return cudaGetLastError();
}

template cudaError_t launch_vc_gather<float>(float*, const Geom&, const VcTable&,
                                             const VcRanges&, cudaStream_t);
template cudaError_t launch_vc_gather<double>(double*, const Geom&, const VcTable&,
                                              const VcRanges&, cudaStream_t);

}  // namespace bcmg
