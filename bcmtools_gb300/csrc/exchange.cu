// exchange.cu -- ghost exchange with blocks of another process: the
// reference's communication buffers (Scalar3DUpdater::copyToCommBuffer*,
// copyFromCommBuffer*, Scalar3DUpdater.h:377-515, 711-901) packed and
// unpacked on the device.
//
// As in the reference, the sender computes the values the receiver's ghosts
// take -- a copy of its interior slab (same level), the averages of its fine
// cells (F2C), the interpolation of its coarse interior (C2F) -- and the
// receiver copies them into its ghost box.  A buffer holds the entries one
// after another, each as the reference's per-face buffer: the ghost box of
// the receiving face (its quarter for F2C) with x fastest, vc x n x n values
// for same-level and C2F faces, vc x n/2 x n/2 for F2C (getSendBufferByteSize
// and its F2C/C2F variants, Scalar3DUpdater.h:84-111).  The values are those
// the local ghost update computes (ghost.cuh, the reference's operation
// order), so a ghost filled through a buffer equals one filled in place.
#include <cstdint>

#include "bcmg.h"
#include "ghost.cuh"
#include "kernels.h"

namespace bcmg {

// One warp per entry: the ghost values of entry t computed from the local
// source block t.src, written to buf + off[entry].
template <typename T>
__global__ void __launch_bounds__(256) xch_pack_kernel(const T* __restrict__ data, Geom g,
                                                     const VcTask* __restrict__ ents,
                                                     const int64_t* __restrict__ off, int n,
                                                     T* __restrict__ buf) {
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const VcTask t = ents[w];
  const Acc<T> src{data + (int64_t)t.src * g.bstride, g.sy, g.sz, g.off0};
  task_apply<T, true>(t, buf + off[w], g, src, 0.0, lane, 32);
}

// One warp per entry: buf + off[entry] copied into the ghost box of the local
// receiving block t.dst.
template <typename T>
__global__ void __launch_bounds__(256) xch_unpack_kernel(T* __restrict__ data, Geom g,
                                                       const VcTask* __restrict__ ents,
                                                       const int64_t* __restrict__ off, int n,
                                                       const T* __restrict__ buf) {
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const VcTask t = ents[w];
  const Box B = task_box(t, g);
  const int cnt = B.b[0] * B.b[1] * B.b[2], bxy = B.b[0] * B.b[1];
  T* dst = data + (int64_t)t.dst * g.bstride;
  const T* src = buf + off[w];
  for (int e = lane; e < cnt; e += 32) {
    int k, r, j, i;
    divmod(e, bxy, k, r);
    divmod(r, B.b[0], j, i);
    dst[g.at(B.d[0] + i, B.d[1] + j, B.d[2] + k)] = src[e];
  }
}

template <typename T>
cudaError_t launch_xch(T* data, const Geom& g, const VcTask* ents, const int64_t* off, int n,
                       T* buf, bool pack, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int grid = (n + 7) / 8;
  if (pack)
    xch_pack_kernel<T><<<grid, 256, 0, st>>>(data, g, ents, off, n, buf);
  else
    xch_unpack_kernel<T><<<grid, 256, 0, st>>>(data, g, ents, off, n, buf);
  return cudaGetLastError();
}

template cudaError_t launch_xch<float>(float*, const Geom&, const VcTask*, const int64_t*, int,
                                       float*, bool, cudaStream_t);
template cudaError_t launch_xch<double>(double*, const Geom&, const VcTask*, const int64_t*, int,
                                        double*, bool, cudaStream_t);

}  // namespace bcmg
