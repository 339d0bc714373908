// jacobi_impl.cuh -- the fused Jacobi sweep: jacobi_smoother
// (SolverTest/blas.f90:452-502) followed by the ghost update and Dirichlet
// ghosts of the new iterate (Jacobi_Smoother's LSSwap + ImposeBoundaryCondition,
// ILS3D.h:108-123) in one launch, optionally with calc_r2 of the input iterate
// (blas.f90:650-698) accumulated on the way.
//
// One CTA per block, one thread per (i,j) column.  The first warp starts bulk
// copies (the TMA engine's non-tensor form) at once: the whole x0 brick (one
// copy) and the interior rows of each interior plane of b (one per plane),
// completing on one mbarrier; nothing passes through registers, so every CTA
// resident on an SM keeps its whole tile in flight.  Each thread then walks
// its column in k with x0(k-1), x0(k), x0(k+1) in registers (five shared loads
// per cell), computes x1 in the reference's `real` operation order, stores it
// to HBM and over the b value it consumed; the CTA then writes the cells of
// x1's brick no neighbour writes (Dirichlet ghosts, edges, unfed faces) and
// every ghost value x1's interior feeds in the neighbours' bricks of the
// output field, reading x1 from shared memory.
#pragma once
#include "bulk.cuh"
#include "ghost.cuh"
#include "kernels.h"
#include "tile.cuh"

namespace bcmg {

template <typename T>
struct JacArgs {
  const T* cf;       // [nb*8] {Ap, Aw, Ae, As, An, Ab, At, 1/Ap} rounded to T
  T omega;
  BlockBc bc;        // Dirichlet faces and values of the output iterate
  PushTable push;     // ghost entries grouped by source block (push form)
  const FaceIn* in;   // [nb*6] ghost sources of each face (pull form)
  int pull_now;       // pull form: fill x0's ghosts from its neighbours first
  double* partial;   // [nb] sum of squared residuals of x0 (or null)
  int* err;          // device error word (bounded-wait timeouts)
};

// Shared-memory layout: mbarrier, x0 brick, b planes [VC, VC+N) (which the
// sweep turns into x1 planes in place).
template <typename T, int N, int VC>
struct JacLayout {
  using BL = BrickTile<T, N, VC>;
  static constexpr int NT = N * N;
  static constexpr unsigned X_BYTES = BL::SIZE * sizeof(T);
  static constexpr unsigned B_BYTES = N * BL::LXY * sizeof(T);
  static constexpr unsigned X_OFF = 16;
  static constexpr unsigned B_OFF = X_OFF + X_BYTES;
  static constexpr size_t SMEM = B_OFF + B_BYTES;
  static_assert(X_BYTES % 16 == 0 && B_BYTES % 16 == 0 && (VC * BL::LXY * sizeof(T)) % 16 == 0,
                "bulk copies need 16-byte sizes and offsets");
  // Rows j and j+D share a warp (N = 16): D*LX = 16 (mod 32) puts the two
  // half-warps of a float access on disjoint banks.
  static constexpr int pair_d() {
    for (int d = 1; d <= N / 2; d *= 2)
      if ((d * BL::LX) % 32 == 16) return d;
    return 1;
  }
  static constexpr int D = sizeof(T) == 4 ? pair_d() : 1;
  // CTAs per SM to plan registers for: as many as shared memory admits
  // (228 KB per SM, 1 KB reserved per CTA), but no fewer than 48 registers
  static constexpr int MIN_BLOCKS_SMEM = (int)(233472 / (SMEM + 1024));
  static constexpr int MIN_BLOCKS_REGS = 65536 / (NT * 48);
  static constexpr int MIN_BLOCKS =
      MIN_BLOCKS_SMEM < MIN_BLOCKS_REGS ? (MIN_BLOCKS_SMEM > 0 ? MIN_BLOCKS_SMEM : 1)
                                        : MIN_BLOCKS_REGS;
  // b: rows [VC, VC+N) of each interior plane, widened to 16-byte bounds
  // (same offsets in shared memory as in the brick)
  static constexpr unsigned ROW_LO = VC * BL::LX * sizeof(T) / 16 * 16;
  static constexpr unsigned ROW_HI = ((VC + N) * BL::LX * sizeof(T) + 15) / 16 * 16;
  static constexpr unsigned B_PLANE = ROW_HI - ROW_LO;
  static constexpr unsigned TX_BYTES = X_BYTES + N * B_PLANE;
  static_assert((BL::LXY * sizeof(T)) % 16 == 0 && ROW_HI <= BL::LXY * sizeof(T),
                "plane copies need 16-byte plane pitch");
};

// Index of the out-of-range coordinate u in [0, 2VC): -VC..-1, then N..N+VC-1.
template <int N, int VC>
__device__ __forceinline__ int shell_coord(int u) { return u < VC ? u - VC : N + u - VC; }

// Sum of squares in float-float for float sweeps (error-free product and
// Knuth's two-sum; one FP64 conversion per warp) and in double for double.
template <typename T>
struct SqAcc;
template <>
struct SqAcc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void merge(float hs, float hc) {
    const float t = __fadd_rn(s, hs);
    const float bv = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bv)), __fsub_rn(hs, bv));
    s = t;
    c = __fadd_rn(c, __fadd_rn(hc, e));
  }
  __device__ __forceinline__ void add(float r) {
    const float p = __fmul_rn(r, r);
    merge(p, __fmaf_rn(r, r, -p));
  }
  __device__ __forceinline__ void warp_reduce() {
    for (int o = 16; o > 0; o >>= 1) {
      const float hs = __shfl_down_sync(0xffffffffu, s, o);
      const float hc = __shfl_down_sync(0xffffffffu, c, o);
      merge(hs, hc);
    }
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};
template <>
struct SqAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double r) { s = __dadd_rn(s, __dmul_rn(r, r)); }
  __device__ __forceinline__ void warp_reduce() {
    for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(0xffffffffu, s, o));
  }
  __device__ __forceinline__ double value() const { return s; }
};

template <typename T, int N, int VC, bool RES, bool PULL>
__global__ void __launch_bounds__(N * N, (JacLayout<T, N, VC>::MIN_BLOCKS)) jacobi_tile_kernel(const T* __restrict__ X0,
                                                            T* __restrict__ X1,
                                                            const T* __restrict__ Bv, Geom g,
                                                            JacArgs<T> a) {
  using L = JacLayout<T, N, VC>;
  using BL = typename L::BL;
  constexpr int NT = L::NT, NW = NT / 32, LX = BL::LX, LXY = BL::LXY;
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ double red[NW];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  T* xs = reinterpret_cast<T*>(smraw + L::X_OFF);
  T* bs = reinterpret_cast<T*>(smraw + L::B_OFF);
  T* x1s = bs - VC * LXY;  // x1 (planes [0,N)) indexed by BL::at
  const int b = blockIdx.x, tid = threadIdx.x;
  const FaceIn* fin = PULL ? a.in + (int64_t)b * 6 : nullptr;
  if (tid < 32) {
    if (tid == 0) {
      mbar_init(bar, 1);
      mbar_fence_init();
      const unsigned char* xsrc = reinterpret_cast<const unsigned char*>(X0 + (int64_t)b * g.bstride);
      unsigned char* xdst = smraw + L::X_OFF;
      if (!PULL) {
        mbar_expect_tx(bar, L::TX_BYTES);
        bulk_g2s(xdst, xsrc, L::X_BYTES, bar);
      } else {
        // planes [0,N); the ghost planes -1 and N only where nothing else fills them
        constexpr unsigned PB = LXY * sizeof(T);
        const bool lo = !a.pull_now || fin[4].kind < 0, hi = !a.pull_now || fin[5].kind < 0;
        mbar_expect_tx(bar, L::TX_BYTES - L::X_BYTES + (N + lo + hi) * PB);
        bulk_g2s(xdst + VC * PB, xsrc + VC * PB, N * PB, bar);
        if (lo) bulk_g2s(xdst + (VC - 1) * PB, xsrc + (VC - 1) * PB, PB, bar);
        if (hi) bulk_g2s(xdst + (VC + N) * PB, xsrc + (VC + N) * PB, PB, bar);
      }
    }
    __syncwarp();
    const unsigned char* bsrc =
        reinterpret_cast<const unsigned char*>(Bv + (int64_t)b * g.bstride + VC * LXY);
    for (int z = tid; z < N; z += 32)
      bulk_g2s(reinterpret_cast<unsigned char*>(bs) + z * LXY * sizeof(T) + L::ROW_LO,
               bsrc + z * LXY * sizeof(T) + L::ROW_LO, L::B_PLANE, bar);
  }
  // block constants while the copies run
  const T* cf = a.cf + (int64_t)b * 8;
  const T c0 = cf[0], c1 = cf[1], c2 = cf[2], c3 = cf[3], c4 = cf[4], c5 = cf[5], c6 = cf[6];
  const T om = a.omega;
  unsigned dmask = 0;
  if (a.bc.type) {
#pragma unroll
    for (int fc = 0; fc < 6; fc++)
      if (a.bc.type[b * 6 + fc] == 1) dmask |= 1u << fc;
  }
  const int w = tid >> 5, lane = tid & 31;
  int i, j;
  if (N == 16) {
    constexpr int D = L::D;
    i = lane & 15;
    j = (w % D) + 2 * D * (w / D) + D * (lane >> 4);
  } else {
    i = tid % N;
    j = tid / N;
  }
  // pull form: this thread's cell of each face, loads issued before the wait
  T gv0 = 0, gv1 = 0, gv2 = 0, gv3 = 0, gv4 = 0, gv5 = 0;
  int gfed = 0;
  const int pp = tid % N, pq = tid / N;
  if (PULL && a.pull_now) {
#define BCMG_PULL_FACE(F)                                                   \
    {                                                                       \
      const FaceIn fi = fin[F];                                             \
      if (fi.kind >= 0) {                                                   \
        int ga, gc, gx, gy, gz;                                             \
        pull_map<N, F>(pp, pq, ga, gc, gx, gy, gz);                         \
        gv##F = pull_cell<T, N, F>(fi, ga, gc, X0, g);                      \
        gfed |= 1 << F;                                                     \
      }                                                                     \
    }
    BCMG_PULL_FACE(0) BCMG_PULL_FACE(1) BCMG_PULL_FACE(2)
    BCMG_PULL_FACE(3) BCMG_PULL_FACE(4) BCMG_PULL_FACE(5)
#undef BCMG_PULL_FACE
  }
  __syncthreads();  // the barrier is initialised before anyone polls it
  const bool ok = mbar_wait(bar, 0, a.err);
  if (!__syncthreads_and(ok)) {
    if (tid == 0) mbar_wait(bar, 0, nullptr);  // drain the copies, bounded
    __syncthreads();
    return;
  }
  if (PULL && a.pull_now) {
    // x0's first ghost layer from the neighbours' interiors (the ghost update
    // that followed the previous sweep) and its Dirichlet ghosts
#define BCMG_PUT_FACE(F)                                                    \
    if (gfed & (1 << F)) {                                                  \
      int ga, gc, gx, gy, gz;                                               \
      pull_map<N, F>(pp, pq, ga, gc, gx, gy, gz);                           \
      xs[BL::at(gx, gy, gz)] = gv##F;                                       \
    }
    BCMG_PUT_FACE(0) BCMG_PUT_FACE(1) BCMG_PUT_FACE(2)
    BCMG_PUT_FACE(3) BCMG_PUT_FACE(4) BCMG_PUT_FACE(5)
#undef BCMG_PUT_FACE
    if (dmask) tile_dirichlet<T, N, VC, BL>(xs, dmask, a.bc.value + b * 6, a.bc.bcx, tid, NT);
    __syncthreads();
  }

  const T* xc_p = xs + BL::at(i, j, 0);
  T* bp = bs + (VC + j) * LX + VC + i;
  T* gp = X1 + (int64_t)b * g.bstride + BL::at(i, j, 0);
  SqAcc<T> acc;
  T xm = xc_p[-LXY], xc = xc_p[0];
#pragma unroll
  for (int k = 0; k < N; k++) {
    const T* q = xc_p + k * LXY;
    const T xp = q[LXY];
    T r = bp[k * LXY];  // b
    r = xsub(r, xmul(c1, q[-1]));
    r = xsub(r, xmul(c2, q[1]));
    r = xsub(r, xmul(c3, q[-LX]));
    r = xsub(r, xmul(c4, q[LX]));
    r = xsub(r, xmul(c5, xm));
    r = xsub(r, xmul(c6, xp));
    if (RES) acc.add(xsub(r, xmul(c0, xc)));
    const T xt = xdiv(r, c0);
    const T x1 = xsub(xc, xmul(om, xsub(xc, xt)));
    bp[k * LXY] = x1;
    gp[k * LXY] = x1;
    xm = xc;
    xc = xp;
  }
  if (RES) {
    // deterministic block sum of the squared residuals of x0
    acc.warp_reduce();
    if (lane == 0) red[w] = acc.value();
  }
  __syncthreads();
  if (RES && tid == 0) {
    double v = 0.0;
    for (int q = 0; q < NW; q++) v += red[q];
    a.partial[b] = v;
  }
  T* fb = X1 + (int64_t)b * g.bstride;
  if (PULL) {
    // The ghost cells of planes [0,N) (rows y outside, cells x outside) from
    // x0's tile: the brick's sectors in those planes are written whole by
    // this CTA alone.  Ghosts of fed faces hold no meaning between launches
    // (the next launch pulls them again; a ghost update closes the run);
    // ghosts no update writes keep their values.
    constexpr int W = 2 * VC, PER = W * LX + N * W;
    for (int e = tid; e < N * PER; e += NT) {
      const int z = e / PER, r = e - z * PER;
      int x, y;
      if (r < W * LX) {
        x = r % LX - VC;
        y = shell_coord<N, VC>(r / LX);
      } else {
        const int q = r - W * LX;
        x = shell_coord<N, VC>(q % W);
        y = q / W;
      }
      const int idx = BL::at(x, y, z);
      fb[idx] = xs[idx];
    }
    return;
  }
  // Cells of x1's brick no other CTA writes: edges and corners, and the ghost
  // layers of faces no neighbour feeds (Dirichlet ghosts where the boundary
  // prescribes them, sor1/Solver.cpp:232-294 and bcx.f90's second layer; x0's
  // values elsewhere).  Writing every such cell keeps each 32-byte sector of
  // the brick whole in L2, so no partial sector costs a DRAM read-fill.
  {
    constexpr int W = 2 * VC;
    constexpr int NA = W * W * LX;  // z and y outside: whole rows
    constexpr int NE = W * N * W;   // z outside, y inside, x outside
    constexpr int NC = N * W * W;   // z inside, y and x outside
    for (int e = tid; e < NA + NE + NC; e += NT) {
      int x, y, z;
      if (e < NA) {
        x = e % LX - VC;
        y = shell_coord<N, VC>((e / LX) % W);
        z = shell_coord<N, VC>(e / (LX * W));
      } else if (e < NA + NE) {
        const int q = e - NA;
        x = shell_coord<N, VC>(q % W);
        y = (q / W) % N;
        z = shell_coord<N, VC>(q / (W * N));
      } else {
        const int q = e - NA - NE;
        x = shell_coord<N, VC>(q % W);
        y = shell_coord<N, VC>((q / W) % W);
        z = q / (W * W);
      }
      const int idx = BL::at(x, y, z);
      fb[idx] = xs[idx];
    }
  }
  const unsigned own = a.push.fed ? (~(unsigned)a.push.fed[b] & 0x3fu) : dmask;
  if (own) {
    const double* dval = a.bc.value + b * 6;
    for (int fc = 0; fc < 6; fc++) {
      if (!((own >> fc) & 1)) continue;
      const bool dir = (dmask >> fc) & 1;
      double v = dir ? dval[fc] : 0.0;
      if (a.bc.bcx) v = (double)(T)v;
      const double v2 = xmul(2.0, v);
      const int ax = fc >> 1;
      const bool minus = (fc & 1) == 0;
      const bool second = a.bc.bcx && VC >= 2;
      for (int e = tid; e < VC * N * N; e += NT) {
        const int p = e % N, q = (e / N) % N, u = e / (N * N);
        const int l = minus ? -1 - u : N + u, l0 = minus ? 0 : N - 1;
        int gi, ii;
        if (ax == 0) { gi = BL::at(l, p, q); ii = BL::at(l0, p, q); }
        else if (ax == 1) { gi = BL::at(p, l, q); ii = BL::at(p, l0, q); }
        else { gi = BL::at(p, q, l); ii = BL::at(p, q, l0); }
        T val = xs[gi];
        if (dir && u == 0) val = to_t<T>(xsub(v2, (double)x1s[ii]));
        else if (dir && u == 1 && second) val = (T)v;
        fb[gi] = val;
      }
    }
  }
  const int p0 = a.push.ptr[b], p1 = a.push.ptr[b + 1];
  for (int q = p0 + w; q < p1; q += NW) {
    const VcTask t = a.push.tasks[q];
    push_dispatch<T, N, VC, BL>(t, X1 + (int64_t)t.dst * g.bstride, g, x1s, lane);
  }
}

template <typename T, int N, int VC>
static cudaError_t jacobi_tile_launch(const T* x0, T* x1, const T* b, const Geom& g,
                                      const JacArgs<T>& a, bool pull, cudaStream_t st) {
  using L = JacLayout<T, N, VC>;
  if (L::SMEM > kSorMaxSmem) return cudaErrorInvalidValue;
  const int ki = (a.partial ? 1 : 0) + (pull ? 2 : 0);
  auto kern = ki == 0   ? jacobi_tile_kernel<T, N, VC, false, false>
              : ki == 1 ? jacobi_tile_kernel<T, N, VC, true, false>
              : ki == 2 ? jacobi_tile_kernel<T, N, VC, false, true>
                        : jacobi_tile_kernel<T, N, VC, true, true>;
  // set once per process (it is not a stream operation, and runs before any
  // CUDA-graph capture of these launches)
  static bool attr_set[4] = {false, false, false, false};
  if (!attr_set[ki]) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)L::SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    attr_set[ki] = true;
  }
  kern<<<g.nb, L::NT, L::SMEM, st>>>(x0, x1, b, g, a);
  return cudaGetLastError();
}

// Shapes the fused kernel covers: cubic 8^3 or 16^3 blocks, vc 1 or 2, tile
// within shared memory.
template <typename T>
static bool jacobi_tile_ok(const Geom& g) {
  if (g.nx != g.ny || g.ny != g.nz || (g.vc != 1 && g.vc != 2)) return false;
  if (g.nx != 8 && g.nx != 16) return false;
  const size_t n = g.nx, lx = n + 2 * g.vc;
  return 16 + (lx * lx * lx + n * lx * lx) * sizeof(T) <= kSorMaxSmem;
}

template <typename T>
cudaError_t launch_jacobi_fused_impl(const T* x0, T* x1, const T* b, const Geom& g, const T* cf,
                                     T omega, BlockBc bc, PushTable push, const FaceIn* in,
                                     int ghost_mode, double* partial, int* err, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  if (!jacobi_tile_ok<T>(g)) return cudaErrorInvalidValue;
  const bool pl = ghost_mode != kGhostPush;
  JacArgs<T> a{cf, omega, bc, push, in, ghost_mode == kGhostPull ? 1 : 0, partial, err};
  if (g.nx == 16)
    return g.vc == 1 ? jacobi_tile_launch<T, 16, 1>(x0, x1, b, g, a, pl, st)
                     : jacobi_tile_launch<T, 16, 2>(x0, x1, b, g, a, pl, st);
  return g.vc == 1 ? jacobi_tile_launch<T, 8, 1>(x0, x1, b, g, a, pl, st)
                   : jacobi_tile_launch<T, 8, 2>(x0, x1, b, g, a, pl, st);
}

}  // namespace bcmg
