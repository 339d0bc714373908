// vc.cu -- the ghost (virtual cell) gather kernel.
//
// One launch updates every selected face of every block of one field: the
// reference's per-face loop BlockManager::copyVCFromNeighbor
// (BlockManager.cpp:715-743) over Scalar3DUpdater<T>'s same-level copy
// (Scalar3DUpdater.h:321-347), fine-to-coarse average (:181-198, :519-612) and
// coarse-to-fine trilinear interpolation (:203-266, :615-708), plus the
// Dirichlet ghosts of outer faces (sor1/Solver.cpp:232-294,
// SolverTest/bcx.f90:18-76).  Every read is an interior cell and every write a
// ghost cell, so entries are independent and run concurrently.
//
// Work decomposition: one warp per face-table entry, lanes walking the entry's
// ghost box x-fastest (coalesced along rows for Y and Z faces).
#include "common.cuh"
#include "kernels.h"

namespace bcmg {

// ---- C2F arithmetic (Scalar3DUpdater.h:221-266) ----------------------------
// I = min(max(i/2 - 1 + i%2, 0), n-2), r = -0.25 + 0.5 i - I (exact).
__device__ __forceinline__ void lin_interp(int i, int n, int& I, double& r) {
  int v = i / 2 - 1 + (i & 1);
  v = max(0, min(v, n - 2));
  I = v;
  r = -0.25 + 0.5 * (double)i - (double)v;
}

// r * c in the reference's types: REAL_TYPE x T, i.e. a float product in the
// float build and a double product in the double build.
__device__ __forceinline__ double rprod(double r, float c) {
  return (double)__fmul_rn((float)r, c);
}
__device__ __forceinline__ double rprod(double r, double c) { return __dmul_rn(r, c); }

template <typename T>
__device__ __forceinline__ T to_t(double v);
template <>
__device__ __forceinline__ float to_t<float>(double v) { return __double2float_rn(v); }
template <>
__device__ __forceinline__ double to_t<double>(double v) { return v; }

template <typename T>
__device__ __forceinline__ T c2f_value(const T* __restrict__ c, const Geom& g, int i, int j,
                                       int k) {
  int I, J, K;
  double r, s, t;
  lin_interp(i, g.nx, I, r);
  lin_interp(j, g.ny, J, s);
  lin_interp(k, g.nz, K, t);
  const int p = g.at(I, J, K);
  const double r1 = 1.0 - r, s1 = 1.0 - s, t1 = 1.0 - t;
  double a00 = xadd(xmul(r1, (double)c[p]), rprod(r, c[p + 1]));
  double a10 = xadd(xmul(r1, (double)c[p + g.sy]), rprod(r, c[p + g.sy + 1]));
  double a01 = xadd(xmul(r1, (double)c[p + g.sz]), rprod(r, c[p + g.sz + 1]));
  double a11 = xadd(xmul(r1, (double)c[p + g.sy + g.sz]), rprod(r, c[p + g.sy + g.sz + 1]));
  double v = xadd(xmul(t1, xadd(xmul(s1, a00), xmul(s, a10))),
                  xmul(t, xadd(xmul(s1, a01), xmul(s, a11))));
  return to_t<T>(v);
}

// F2C (Scalar3DUpdater.h:190-198): 8-cell sum in T left to right, times 0.125
// in double, rounded to T.
template <typename T>
__device__ __forceinline__ T f2c_value(const T* __restrict__ f, const Geom& g, int i, int j,
                                       int k) {
  const int p = g.at(i, j, k);
  T sum = f[p];
  sum = xadd(sum, f[p + 1]);
  sum = xadd(sum, f[p + g.sy]);
  sum = xadd(sum, f[p + g.sy + 1]);
  sum = xadd(sum, f[p + g.sz]);
  sum = xadd(sum, f[p + g.sz + 1]);
  sum = xadd(sum, f[p + g.sy + g.sz]);
  sum = xadd(sum, f[p + g.sy + g.sz + 1]);
  return to_t<T>(xmul(0.125, (double)sum));
}

template <typename T>
__global__ void __launch_bounds__(256) vc_gather_kernel(T* __restrict__ data, Geom g,
                                                        VcTable tab, VcRanges rg) {
  const int w = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= rg.prefix[rg.n]) return;
  int q = 0;
  while (w >= rg.prefix[q + 1]) q++;
  const VcTask t = tab.tasks[rg.start[q] + (w - rg.prefix[q])];

  const int nx = g.nx, ny = g.ny, nz = g.nz, vc = g.vc;
  T* __restrict__ dst = data + (int64_t)t.dst * g.bstride;
  const int face = t.face, axis = face >> 1, minus = (face & 1) == 0;

  if (t.kind == VC_COPY) {
    // Box and offsets of Scalar3DUpdater::copyFromNeighbor (Scalar3DUpdater.h:321-347).
    const T* __restrict__ src = data + (int64_t)t.src * g.bstride;
    int bx = nx, by = ny, bz = nz, d0[3] = {0, 0, 0}, s0[3] = {0, 0, 0};
    const int nn = axis == 0 ? nx : axis == 1 ? ny : nz;
    if (axis == 0) bx = vc; else if (axis == 1) by = vc; else bz = vc;
    d0[axis] = minus ? -vc : nn;
    s0[axis] = minus ? nn - vc : 0;
    const int cnt = bx * by * bz;
    for (int e = lane; e < cnt; e += 32) {
      int i = e % bx, r = e / bx, j = r % by, k = r / by;
      dst[g.at(d0[0] + i, d0[1] + j, d0[2] + k)] = src[g.at(s0[0] + i, s0[1] + j, s0[2] + k)];
    }
  } else if (t.kind == VC_F2C) {
    // Coarse ghosts from one fine neighbour (copyFromNeighborF2C_0, :519-612).
    const T* __restrict__ src = data + (int64_t)t.src * g.bstride;
    const int o0 = t.subface & 1, o1 = (t.subface >> 1) & 1;
    int bx = nx / 2, by = ny / 2, bz = nz / 2, d[3] = {0, 0, 0}, fo[3] = {0, 0, 0};
    if (axis == 0) {
      bx = vc; d[1] = (ny / 2) * o0; d[2] = (nz / 2) * o1;
      d[0] = minus ? -vc : nx; fo[0] = minus ? nx / 2 - vc : 0;
    } else if (axis == 1) {
      by = vc; d[2] = (nz / 2) * o0; d[0] = (nx / 2) * o1;
      d[1] = minus ? -vc : ny; fo[1] = minus ? ny / 2 - vc : 0;
    } else {
      bz = vc; d[0] = (nx / 2) * o0; d[1] = (ny / 2) * o1;
      d[2] = minus ? -vc : nz; fo[2] = minus ? nz / 2 - vc : 0;
    }
    const int cnt = bx * by * bz;
    for (int e = lane; e < cnt; e += 32) {
      int i = e % bx, r = e / bx, j = r % by, k = r / by;
      dst[g.at(d[0] + i, d[1] + j, d[2] + k)] =
          f2c_value<T>(src, g, 2 * (i + fo[0]), 2 * (j + fo[1]), 2 * (k + fo[2]));
    }
  } else if (t.kind == VC_C2F) {
    // Fine ghosts from the coarse neighbour (copyFromNeighborC2F_0, :615-708);
    // the neighbour's subface fixes the quadrant (VCUpdater.h:74-77).
    const T* __restrict__ src = data + (int64_t)t.src * g.bstride;
    const int o0 = t.subface & 1, o1 = (t.subface >> 1) & 1;
    int bx = nx, by = ny, bz = nz, d[3] = {0, 0, 0}, c[3] = {0, 0, 0};
    if (axis == 0) {
      bx = vc; c[1] = ny * o0; c[2] = nz * o1;
      d[0] = minus ? -vc : nx; c[0] = minus ? 2 * nx - vc : 0;
    } else if (axis == 1) {
      by = vc; c[2] = nz * o0; c[0] = nx * o1;
      d[1] = minus ? -vc : ny; c[1] = minus ? 2 * ny - vc : 0;
    } else {
      bz = vc; c[0] = nx * o0; c[1] = ny * o1;
      d[2] = minus ? -vc : nz; c[2] = minus ? 2 * nz - vc : 0;
    }
    const int cnt = bx * by * bz;
    for (int e = lane; e < cnt; e += 32) {
      int i = e % bx, r = e / bx, j = r % by, k = r / by;
      dst[g.at(d[0] + i, d[1] + j, d[2] + k)] =
          c2f_value<T>(src, g, i + c[0], j + c[1], k + c[2]);
    }
  } else {
    // Dirichlet ghost layer: g = 2v - f(adjacent interior), computed in double
    // (sor1/Solver.cpp:242 and bcx.f90:37); BCX also sets the second layer to v.
    double v = tab.bcval[t.dst * 6 + face];
    const bool bcx = t.flags & 1;
    if (bcx) v = (double)(T)v;
    const bool second = bcx && vc >= 2;
    int bx = nx, by = ny, bz = nz, gi[3] = {0, 0, 0}, ii[3] = {0, 0, 0}, g2[3] = {0, 0, 0};
    const int nn = axis == 0 ? nx : axis == 1 ? ny : nz;
    if (axis == 0) bx = 1; else if (axis == 1) by = 1; else bz = 1;
    gi[axis] = minus ? -1 : nn;
    ii[axis] = minus ? 0 : nn - 1;
    g2[axis] = minus ? -2 : nn + 1;
    const int cnt = bx * by * bz;
    const double v2 = xmul(2.0, v);
    for (int e = lane; e < cnt; e += 32) {
      int i = e % bx, r = e / bx, j = r % by, k = r / by;
      T fin = dst[g.at(ii[0] + i, ii[1] + j, ii[2] + k)];
      dst[g.at(gi[0] + i, gi[1] + j, gi[2] + k)] = to_t<T>(xsub(v2, (double)fin));
      if (second) dst[g.at(g2[0] + i, g2[1] + j, g2[2] + k)] = (T)v;
    }
  }
}

template <typename T>
cudaError_t launch_vc_gather(T* data, const Geom& g, const VcTable& tab, const VcRanges& rg,
                             cudaStream_t st) {
  const int nw = rg.prefix[rg.n];
  if (nw == 0) return cudaSuccess;
  const int warps_per_cta = 8;
  const int grid = (nw + warps_per_cta - 1) / warps_per_cta;
  vc_gather_kernel<T><<<grid, 32 * warps_per_cta, 0, st>>>(data, g, tab, rg);
  return cudaGetLastError();
}

template cudaError_t launch_vc_gather<float>(float*, const Geom&, const VcTable&,
                                             const VcRanges&, cudaStream_t);
template cudaError_t launch_vc_gather<double>(double*, const Geom&, const VcTable&,
                                              const VcRanges&, cudaStream_t);

}  // namespace bcmg
