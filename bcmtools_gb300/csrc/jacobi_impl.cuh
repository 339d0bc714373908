// jacobi_impl.cuh -- the fused Jacobi sweep: jacobi_smoother
// (SolverTest/blas.f90:452-502) followed by the ghost update and Dirichlet
// ghosts of the new iterate (Jacobi_Smoother's LSSwap + ImposeBoundaryCondition,
// ILS3D.h:108-123) in one launch, optionally with calc_r2 of the input iterate
// (blas.f90:650-698) accumulated on the way.
//
// Ping-pong: block b's tile of x0 (interior + first ghost layer) and its right
// hand side are staged in shared memory; each thread computes x1 for its cells
// in the reference's `real` operation order and stores it over the b value it
// consumed, so the b tile becomes the x1 tile; the CTA then writes x1's
// interior, its Dirichlet ghosts and every ghost value x1's interior feeds in
// the neighbours' bricks of the output field.  Per-block constant operator
// coefficients (cc, rounded to T) only.
#pragma once
#include "ghost.cuh"
#include "kernels.h"
#include "tile.cuh"

namespace bcmg {

struct JacArgs {
  const double* cc;  // [nb*7] {Ap, Aw, Ae, As, An, Ab, At}
  double omega;
  BlockBc bc;        // Dirichlet faces and values of the output iterate
  PushTable push;
  double* partial;   // [nb] FP64 sum of squared residuals of x0 (or null)
};

template <typename T, int N, int VC, bool RES>
__global__ void __launch_bounds__(256) jacobi_tile_kernel(const T* __restrict__ X0,
                                                          T* __restrict__ X1,
                                                          const T* __restrict__ Bv, Geom g,
                                                          JacArgs a) {
  using TL = Tile<T, N, VC>;
  using V = typename VecOf<TL::VEC_BYTES>::type;
  constexpr int NV = TL::LX * (int)sizeof(T) / TL::VEC_BYTES;
  constexpr int N3 = N * N * N;
  constexpr int XOFF = (TL::SIZE * (int)sizeof(T) + 15) / 16 * 16 / (int)sizeof(T);
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double red[32];
  T* x0 = reinterpret_cast<T*>(smraw);
  // b tile: field-tile layout for planes k in [0,N), so that after the sweep
  // (x1 written over b) `bt - LXY` indexes x1 with TL::at.
  T* bt = x0 + XOFF;
  T* x1t = bt - TL::LXY;
  const int b = blockIdx.x, tid = threadIdx.x;
  const T* ab = X0 + (int64_t)b * g.bstride;
  const T* bb = Bv + (int64_t)b * g.bstride;
  T* fb = X1 + (int64_t)b * g.bstride;
  // x0: rows y, z in [-1, N] (padded VC-1 .. VC+N), whole brick rows
  for (int e = tid; e < NV * (N + 2) * (N + 2); e += 256) {
    const int v = e % NV, row = e / NV, y = row % (N + 2), z = row / (N + 2);
    reinterpret_cast<V*>(x0 + row * TL::LX)[v] =
        reinterpret_cast<const V*>(ab + (VC - 1 + y) * TL::LX + (VC - 1 + z) * TL::LX * TL::LX)[v];
  }
  // b: rows y, z in [0, N) into tile rows y+1 of planes z
  for (int e = tid; e < NV * N * N; e += 256) {
    const int v = e % NV, row = e / NV, y = row % N, z = row / N;
    reinterpret_cast<V*>(bt + z * TL::LXY + (y + 1) * TL::LX)[v] =
        reinterpret_cast<const V*>(bb + (VC + y) * TL::LX + (VC + z) * TL::LX * TL::LX)[v];
  }
  T cf[7];
#pragma unroll
  for (int c = 0; c < 7; c++) cf[c] = (T)a.cc[b * 7 + c];
  const T om = (T)a.omega;
  unsigned dmask = 0;
  if (a.bc.type) {
#pragma unroll
    for (int fc = 0; fc < 6; fc++)
      if (a.bc.type[b * 6 + fc] == 1) dmask |= 1u << fc;
  }
  __syncthreads();

  double acc = 0.0;
#pragma unroll 4
  for (int t = tid; t < N3; t += 256) {
    const int i = t % N, r0 = t / N, j = r0 % N, k = r0 / N;
    const int p = TL::at(i, j, k);
    T r = x1t[p];  // b
    r = xsub(r, xmul(cf[1], x0[p - 1]));
    r = xsub(r, xmul(cf[2], x0[p + 1]));
    r = xsub(r, xmul(cf[3], x0[p - TL::LX]));
    r = xsub(r, xmul(cf[4], x0[p + TL::LX]));
    r = xsub(r, xmul(cf[5], x0[p - TL::LXY]));
    r = xsub(r, xmul(cf[6], x0[p + TL::LXY]));
    const T xc = x0[p];
    if (RES) {
      const T rf = xsub(r, xmul(cf[0], xc));
      acc += (double)rf * (double)rf;
    }
    const T xt = xdiv(r, cf[0]);
    x1t[p] = xsub(xc, xmul(om, xsub(xc, xt)));
  }
  if (RES) {
    // deterministic block sum of the squared residuals of x0
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
  }
  __syncthreads();
  if (RES && tid < 32) {
    double v = tid < 8 ? red[tid] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (tid == 0) a.partial[b] = v;
  }
  store_interior<T, N, VC>(x1t, fb, g, tid, 256);
  if (dmask) {
    // Dirichlet ghosts of x1 from its interior (sor1/Solver.cpp:232-294;
    // bcx.f90 second layer when requested)
    const double* dval = a.bc.value + b * 6;
    for (int fc = 0; fc < 6; fc++) {
      if (!((dmask >> fc) & 1)) continue;
      double v = dval[fc];
      if (a.bc.bcx) v = (double)(T)v;
      const double v2 = xmul(2.0, v);
      const int ax = fc >> 1;
      const bool minus = (fc & 1) == 0;
      const bool second = a.bc.bcx && VC >= 2;
      for (int e = tid; e < N * N; e += 256) {
        const int p = e % N, q = e / N;
        const int l1 = minus ? -1 : N, l0 = minus ? 0 : N - 1, l2 = minus ? -2 : N + 1;
        int gi, ii, g2;
        if (ax == 0) { gi = g.at(l1, p, q); ii = TL::at(l0, p, q); g2 = g.at(l2, p, q); }
        else if (ax == 1) { gi = g.at(p, l1, q); ii = TL::at(p, l0, q); g2 = g.at(p, l2, q); }
        else { gi = g.at(p, q, l1); ii = TL::at(p, q, l0); g2 = g.at(p, q, l2); }
        fb[gi] = to_t<T>(xsub(v2, (double)x1t[ii]));
        if (second) fb[g2] = (T)v;
      }
    }
  }
  const int lane = tid & 31, warp = tid >> 5;
  const int p0 = a.push.ptr[b], p1 = a.push.ptr[b + 1];
  for (int q = p0 + warp; q < p1; q += 8) {
    const VcTask t = a.push.tasks[q];
    push_dispatch<T, N, VC>(t, X1 + (int64_t)t.dst * g.bstride, g, x1t, lane);
  }
}

template <typename T, int N, int VC>
static cudaError_t jacobi_tile_launch(const T* x0, T* x1, const T* b, const Geom& g,
                                      const JacArgs& a, cudaStream_t st) {
  using TL = Tile<T, N, VC>;
  const size_t xb = (size_t)(TL::SIZE * sizeof(T) + 15) / 16 * 16;
  const size_t smem = xb + (size_t)TL::LXY * N * sizeof(T);
  if (smem > kSorMaxSmem) return cudaErrorInvalidValue;
  auto kern = a.partial ? jacobi_tile_kernel<T, N, VC, true> : jacobi_tile_kernel<T, N, VC, false>;
  // set once per process (it is not a stream operation, and runs before any
  // CUDA-graph capture of these launches)
  static bool attr_set[2] = {false, false};
  if (!attr_set[a.partial ? 1 : 0]) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSorMaxSmem);
    if (e != cudaSuccess) return e;
    attr_set[a.partial ? 1 : 0] = true;
  }
  kern<<<g.nb, 256, smem, st>>>(x0, x1, b, g, a);
  return cudaGetLastError();
}

template <typename T>
static bool jacobi_tile_ok(const Geom& g) {
  if (g.nx != g.ny || g.ny != g.nz || (g.vc != 1 && g.vc != 2)) return false;
  if (g.nx != 8 && g.nx != 16 && g.nx != 32) return false;
  const int n = g.nx, lx = n + 2 * g.vc;
  const size_t xb = ((size_t)lx * (n + 2) * (n + 2) * sizeof(T) + 15) / 16 * 16;
  return xb + (size_t)lx * (n + 2) * n * sizeof(T) <= kSorMaxSmem;
}

template <typename T>
cudaError_t launch_jacobi_fused_impl(const T* x0, T* x1, const T* b, const Geom& g,
                                     const double* cc, double omega, BlockBc bc, PushTable push,
                                     double* partial, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  if (!jacobi_tile_ok<T>(g)) return cudaErrorInvalidValue;
  JacArgs a{cc, omega, bc, push, partial};
  if (g.nx == 16)
    return g.vc == 1 ? jacobi_tile_launch<T, 16, 1>(x0, x1, b, g, a, st)
                     : jacobi_tile_launch<T, 16, 2>(x0, x1, b, g, a, st);
  if (g.nx == 8)
    return g.vc == 1 ? jacobi_tile_launch<T, 8, 1>(x0, x1, b, g, a, st)
                     : jacobi_tile_launch<T, 8, 2>(x0, x1, b, g, a, st);
  return g.vc == 1 ? jacobi_tile_launch<T, 32, 1>(x0, x1, b, g, a, st)
                   : jacobi_tile_launch<T, 32, 2>(x0, x1, b, g, a, st);
}

}  // namespace bcmg
