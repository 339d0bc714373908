// jacobi_impl.cuh -- the fused Jacobi sweep: jacobi_smoother
// (SolverTest/blas.f90:452-502) followed by the ghost update and Dirichlet
// ghosts of the new iterate (Jacobi_Smoother's LSSwap + ImposeBoundaryCondition,
// ILS3D.h:108-123) in one launch, optionally with calc_r2 of the input iterate
// (blas.f90:650-698) accumulated on the way.
//
// Pull ghost form: one CTA per block (jacobi_tile_kernel) or the pipelined
// kernel of pipe.cuh.  Push ghost form: one CTA per block, one thread per
// (i,j) column; 32^3 blocks: jacobi_cubic_push_kernel, no staging.
// The first warp starts bulk copies (the TMA engine's non-tensor form) at
// once: the whole x0 brick (one copy) and the interior rows of each interior
// plane of b (one per plane), completing on one mbarrier.  Each thread then
// walks its column in k with x0(k-1), x0(k), x0(k+1) in registers (five shared
// loads per cell), computes x1 in the reference's `real` operation order,
// stores it to HBM and over the b value it consumed; the CTA then writes the
// cells of x1's brick no neighbour writes (Dirichlet ghosts, edges, unfed
// faces) and every ghost value x1's interior feeds in the neighbours' bricks
// of the output field, reading x1 from shared memory.
#pragma once
#include "cells.cuh"
#include "pipe.cuh"
#include "stage.cuh"
#include "stream.cuh"

namespace bcmg {

template <typename T>
struct JacArgs {
  int pull_now;      // pull form: fill x0's ghosts from its neighbours first
  const T* cf;       // [nb*8] {Ap, Aw, Ae, As, An, Ab, At, 1/Ap} rounded to T
  T omega;
  BlockBc bc;        // Dirichlet faces and values of the output iterate
  PushTable push;     // ghost entries by source block
  double* partial;   // [nb] sum of squared residuals of x0 (or null)
  int* err;          // device error word (bounded-wait timeouts)
  int zero_x0;       // 32^3 push form: x0 is zero everywhere and is not read
  JacPre<T> pre;     // 32^3 streamed zero-start pass: b made in the same pass
};

// Index of the out-of-range coordinate u in [0, 2VC): -VC..-1, then N..N+VC-1.
template <int N, int VC>
__device__ __forceinline__ int shell_coord(int u) { return u < VC ? u - VC : N + u - VC; }

template <typename T, int N, int VC, bool RES, bool PULL>
__global__ void __launch_bounds__(N * N, (BrickStage<T, N, VC, true>::MIN_BLOCKS))
    jacobi_tile_kernel(const T* __restrict__ X0, T* __restrict__ X1, const T* __restrict__ Bv,
                       Geom g, JacArgs<T> a) {
  using L = BrickStage<T, N, VC, true>;
  using BL = typename L::BL;
  constexpr int NT = L::NT, NW = NT / 32, LX = BL::LX, LXY = BL::LXY, NN = N * N;
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ double red[NW];
  __shared__ VcTask outs[PULL ? kMaxOutEntries : 1];
  __shared__ float dv2f[8];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw);
  T* xs = reinterpret_cast<T*>(smraw + L::X_OFF);
  T* bs = reinterpret_cast<T*>(smraw + L::B_OFF);
  T* x1s = bs - VC * LXY;  // x1 (planes [0,N)) indexed by BL::at
  const int b = blockIdx.x, tid = threadIdx.x;
  if (!PULL) {
    if (tid < 32) {
      if (tid == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
      }
      __syncwarp();
      L::issue(smraw, bar, X0, Bv, b, g.bstride, true, true, true, tid);
    }
  } else if (tid < 32) {
    // planes [0,N) and b's rows at once; the ghost planes -1 / N once the
    // descriptor says no neighbour fills them; the arrival closes the phase
    constexpr unsigned PB = L::PB;
    unsigned char* xdst = smraw + L::X_OFF;
    const unsigned char* xsrc = reinterpret_cast<const unsigned char*>(X0 + (int64_t)b * g.bstride);
    if (tid == 0) {
      mbar_init(bar, 1);
      mbar_fence_init();
      mbar_add_tx(bar, N * PB + N * L::B_PLANE);
      bulk_g2s(xdst + VC * PB, xsrc + VC * PB, N * PB, bar);
    }
    __syncwarp();
    const unsigned char* bsrc =
        reinterpret_cast<const unsigned char*>(Bv + (int64_t)b * g.bstride) + VC * PB;
    for (int z = tid; z < N; z += 32)
      bulk_g2s(reinterpret_cast<unsigned char*>(bs) + z * PB + L::ROW_LO,
               bsrc + z * PB + L::ROW_LO, L::B_PLANE, bar);
  }
  const BlockInfo inf = PULL ? a.push.info[b] : BlockInfo{};
  const unsigned flags = (unsigned)inf.flags;
  if (PULL && tid == 0) {
    constexpr unsigned PB = L::PB;
    unsigned char* xdst = smraw + L::X_OFF;
    const unsigned char* xsrc = reinterpret_cast<const unsigned char*>(X0 + (int64_t)b * g.bstride);
    const bool lo = !a.pull_now || !(flags & (BI_FED << 4));
    const bool hi = !a.pull_now || !(flags & (BI_FED << 5));
    mbar_add_tx(bar, (lo + hi) * PB);
    if (lo) bulk_g2s(xdst + (VC - 1) * PB, xsrc + (VC - 1) * PB, PB, bar);
    if (hi) bulk_g2s(xdst + (VC + N) * PB, xsrc + (VC + N) * PB, PB, bar);
    mbar_arrive(bar);
  }
  // block constants while the copies run
  const T* cf = a.cf + (int64_t)b * 8;
  const T c0 = cf[0], c1 = cf[1], c2 = cf[2], c3 = cf[3], c4 = cf[4], c5 = cf[5], c6 = cf[6];
  const T rc0 = cf[7];  // RN(1/Ap), or 0
  const T om = a.omega;
  unsigned dmask = 0;
  if (PULL) {
    dmask = (flags >> BI_DIR_SHIFT) & 0x3fu;
  } else if (a.bc.type) {
#pragma unroll
    for (int fc = 0; fc < 6; fc++)
      if (a.bc.type[b * 6 + fc] == 1) dmask |= 1u << fc;
  }
  const int w = tid >> 5, lane = tid & 31;
  int i, j;
  L::column(tid, i, j);
  // pull form: this thread's cell of every fed face, loads issued before the
  // wait -- same-level faces from the neighbour (X faces: its x-face layer),
  // faces on a coarser block interpolated here from its interior, faces on
  // finer blocks from the side buffer -- and the F2C entries this block feeds
  T g0 = 0, g1 = 0, g2 = 0, g3 = 0, g4 = 0, g5 = 0;
  const int gpp = tid % N, gq = tid / N;
  // vc = 2: same-level X ghosts from the x-face layers the source CTAs write
  // (measured faster there; at vc = 1 the row-end loads from the brick win)
  constexpr bool XF = VC == 2;
  int nout = 0;
  if (PULL) {
    nout = (flags >> BI_OUT_SHIFT) & 0x7f;
    if (tid < nout) outs[tid] = a.push.out_tasks[inf.out_begin + tid];
    if (dmask && tid >= 32 && tid < 38) dv2f[tid - 32] = a.bc.v2f[(int64_t)b * 8 + tid - 32];
  }
  if (PULL && a.pull_now) {
    const T* side = static_cast<const T*>(a.push.side_in);
    const T* xfin = static_cast<const T*>(a.push.xf_in);
#define BCMG_JAC_LOAD(F, V)                                                  \
    if (flags & (BI_FED << F)) {                                             \
      const int64_t src = inf.csrc[F];                                       \
      if (XF && (F >> 1) == 0 && (flags & (BI_COPY << F))) {                 \
        V = __ldcg(xfin + (src * 2 + (F == 0 ? 1 : 0)) * NN + gq * N + gpp); \
      } else if (flags & (1u << bi_c2f_bit(F))) {                            \
        V = c2f_pull<T, N, VC, F>(X0 + (src >> 2) * g.bstride, (int)(src & 3), gpp, gq); \
      } else if (flags & (BI_COPY << F)) {                                   \
        int ga, gc, gx, gy, gz;                                              \
        pull_map<N, F>(gpp, gq, ga, gc, gx, gy, gz);                         \
        face_xyz<(F >> 1)>((F & 1) == 0 ? N - 1 : 0, ga, gc, gx, gy, gz);    \
        V = __ldcg(X0 + (int64_t)inf.csrc[F] * g.bstride + g.at(gx, gy, gz)); \
      } else {                                                               \
        V = __ldcg(side + (int64_t)inf.csrc[F] * NN + gq * N + gpp);         \
      }                                                                      \
    }
    BCMG_JAC_LOAD(0, g0) BCMG_JAC_LOAD(1, g1) BCMG_JAC_LOAD(2, g2)
    BCMG_JAC_LOAD(3, g3) BCMG_JAC_LOAD(4, g4) BCMG_JAC_LOAD(5, g5)
#undef BCMG_JAC_LOAD
  }
  __syncthreads();  // the barrier is initialised before anyone polls it
  const bool ok = mbar_wait(bar, 0, a.err);
  if (!__syncthreads_and(ok)) {
    if (tid == 0) mbar_wait(bar, 0, nullptr);  // drain the copies, bounded
    __syncthreads();
    return;
  }
  if (PULL && a.pull_now) {
#define BCMG_JAC_PUT(F, V)                                                   \
    if (flags & (BI_FED << F)) {                                             \
      int ga, gc, gx, gy, gz;                                                \
      pull_map<N, F>(gpp, gq, ga, gc, gx, gy, gz);                           \
      xs[BL::at(gx, gy, gz)] = V;                                            \
    }
    BCMG_JAC_PUT(0, g0) BCMG_JAC_PUT(1, g1) BCMG_JAC_PUT(2, g2)
    BCMG_JAC_PUT(3, g3) BCMG_JAC_PUT(4, g4) BCMG_JAC_PUT(5, g5)
#undef BCMG_JAC_PUT
    if (dmask)
      tile_dirichlet<T, N, VC, BL>(xs, dmask, a.bc.value + b * 6, a.bc.bcx, tid, NT, dv2f);
    __syncthreads();
  }

  const T* xc_p = xs + BL::at(i, j, 0);
  T* bp = bs + (VC + j) * LX + VC + i;
  T* gp = X1 + (int64_t)b * g.bstride + BL::at(i, j, 0);
  SqAcc<T> acc;
  T xm = xc_p[-LXY], xc = xc_p[0];
  static_assert(N % 4 == 0, "cells in groups of four");
#pragma unroll
  for (int k0 = 0; k0 < N; k0 += 4) {
    // four cells: every load before the first store into b's area, so the
    // loads overlap
    T xw[4], xe[4], xs_[4], xn[4], xu[4], bv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const T* q = xc_p + (k0 + u) * LXY;
      xw[u] = q[-1];
      xe[u] = q[1];
      xs_[u] = q[-LX];
      xn[u] = q[LX];
      xu[u] = q[LXY];
      bv[u] = bp[(k0 + u) * LXY];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int k = k0 + u;
      const T xp = xu[u];
      T r = bv[u];  // b
      r = xsub(r, xmul(c1, xw[u]));
      r = xsub(r, xmul(c2, xe[u]));
      r = xsub(r, xmul(c3, xs_[u]));
      r = xsub(r, xmul(c4, xn[u]));
      r = xsub(r, xmul(c5, xm));
      r = xsub(r, xmul(c6, xp));
      if (RES) acc.add(xsub(r, xmul(c0, xc)));
      const T xt = sweep_div(r, c0, rc0);
      const T x1 = xsub(xc, xmul(om, xsub(xc, xt)));
      bp[k * LXY] = x1;
      gp[k * LXY] = x1;
      xm = xc;
      xc = xp;
    }
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
    // x1's x-face layers, for the same-level X neighbours of the next launch
    if (XF) {
      T* xo = static_cast<T*>(a.push.xf_out) + (int64_t)b * 2 * NN + tid;
      if (flags & (BI_COPY << 0)) xo[0] = x1s[BL::at(0, gpp, gq)];
      if (flags & (BI_COPY << 1)) xo[NN] = x1s[BL::at(N - 1, gpp, gq)];
    }
    // F2C ghosts this block feeds, into the side buffer of x1.
    T* side = static_cast<T*>(a.push.side_out);
    for (int q = 0; q < nout; q++) {
      const VcTask t = outs[q];
      side_push<T, N, VC, BL, NT>(t, side + (int64_t)t.slot * NN, g, x1s, tid);
    }
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

// The part of a push-form fused Jacobi launch that follows the sweep, with
// the block's new interior already in its brick of X1 (visible to the whole
// CTA): the cells of that brick no other CTA writes (edges, faces no
// neighbour feeds: Dirichlet ghosts or x0's values; zeros when x0 is zero),
// then every ghost value the interior feeds in the neighbours' bricks, read
// back from the brick.  NT threads, one warp per face-table entry, UB cells
// in flight per lane; !COPIES: the same-level entries were written during
// the sweep and are skipped here.
template <typename T, int N, int VC, int NT, int UB = 8, bool COPIES = true>
__device__ __forceinline__ void jacobi_push_tail(const T* __restrict__ X0, T* __restrict__ X1,
                                                 const Geom& g, const JacArgs<T>& a, int b,
                                                 int tid, bool zero, int skip_x = 0) {
  using BL = BrickTile<T, N, VC>;
  constexpr int NW = NT / 32, LX = BL::LX;
  const int w = tid >> 5, lane = tid & 31;
  const int64_t base = (int64_t)b * g.bstride;
  const T* xs = X0 + base;
  T* fb = X1 + base;
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
      fb[idx] = zero ? T(0) : xs[idx];
    }
  }
  unsigned dmask = 0;
  if (a.bc.type) {
#pragma unroll
    for (int fc = 0; fc < 6; fc++)
      if (a.bc.type[b * 6 + fc] == 1) dmask |= 1u << fc;
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
        T val = zero ? T(0) : xs[gi];
        if (dir && u == 0) val = to_t<T>(xsub(v2, (double)fb[ii]));
        else if (dir && u == 1 && second) val = (T)v;
        fb[gi] = val;
      }
    }
  }
  const int p0 = a.push.ptr[b], p1 = a.push.ptr[b + 1];
  if (COPIES) {
    for (int q = p0 + w; q < p1; q += NW) {
      const VcTask t = a.push.tasks[q];
      push_dispatch<T, N, VC, BL, UB>(t, X1 + (int64_t)t.dst * g.bstride, g, fb, lane);
    }
  } else {
    // the same-level entries were written during the sweep, and so were the
    // first skip_x level-change entries of x faces; the level-change entries
    // left (about two per block) take the whole CTA each
    int nx = 0;
    for (int q = p0; q < p1; q++) {
      const VcTask t = a.push.tasks[q];
      if (t.kind == VC_COPY) continue;
      if ((t.face >> 1) == 0 && nx++ < skip_x) continue;
      push_dispatch_cta<T, N, VC, BL, NT, UB>(t, X1 + (int64_t)t.dst * g.bstride, g, fb, tid);
    }
  }
}

// Push-form fused Jacobi on 32^3 blocks (too large to stage in shared
// memory): the cubic sweep's column walk (CPT columns per thread side by
// side, x0 and b read through L1), then -- with the block's x1 in its own
// brick -- the cells of x1's brick no other CTA writes (edges, faces no
// neighbour feeds: Dirichlet ghosts or x0's values) and every ghost value x1's
// interior feeds in the neighbours' bricks, read back from that brick.
template <typename T, int N, int VC, int CPT, bool RES>
__global__ void __launch_bounds__(N * N / CPT, sizeof(T) == 4 ? (CPT >= 4 ? 4 : 2) : 1)
    jacobi_cubic_push_kernel(const T* __restrict__ X0, T* __restrict__ X1,
                             const T* __restrict__ Bv, Geom g, JacArgs<T> a) {
  using BL = BrickTile<T, N, VC>;
  constexpr int NT = N * N / CPT, NW = NT / 32, LX = BL::LX, LXY = BL::LXY;
  __shared__ double red[NW];
  const int b = blockIdx.x, tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const T* cf = a.cf + (int64_t)b * 8;
  const T c0 = cf[0], c1 = cf[1], c2 = cf[2], c3 = cf[3], c4 = cf[4], c5 = cf[5], c6 = cf[6];
  const T rc0 = cf[7];
  const T om = a.omega;
  const int64_t base = (int64_t)b * g.bstride;
  // x0 == 0 (the first pass of a preconditioner from a zero start): the same
  // arithmetic on zeros, with x0 neither read nor cleared beforehand
  const bool zero = a.zero_x0 != 0;
  int off[CPT];
  T xm[CPT], xc[CPT];
#pragma unroll
  for (int c = 0; c < CPT; c++) {
    const int ij = tid + c * NT;
    off[c] = BL::at(ij % N, ij / N, 0);
    xm[c] = zero ? T(0) : X0[base + off[c] - LXY];
    xc[c] = zero ? T(0) : X0[base + off[c]];
  }
  SqAcc<T> acc;
#pragma unroll 2
  for (int k = 0; k < N; k++) {
    T xw[CPT], xe[CPT], xs_[CPT], xn[CPT], up[CPT], bv[CPT];
#pragma unroll
    for (int c = 0; c < CPT; c++) {
      const T* q = X0 + base + off[c] + k * LXY;
      if (zero) {
        xw[c] = xe[c] = xs_[c] = xn[c] = up[c] = T(0);
      } else {
        xw[c] = q[-1];
        xe[c] = q[1];
        xs_[c] = q[-LX];
        xn[c] = q[LX];
        up[c] = q[LXY];
      }
      bv[c] = Bv[base + off[c] + k * LXY];
    }
#pragma unroll
    for (int c = 0; c < CPT; c++) {
      T r = bv[c];
      r = xsub(r, xmul(c1, xw[c]));
      r = xsub(r, xmul(c2, xe[c]));
      r = xsub(r, xmul(c3, xs_[c]));
      r = xsub(r, xmul(c4, xn[c]));
      r = xsub(r, xmul(c5, xm[c]));
      r = xsub(r, xmul(c6, up[c]));
      if (RES) acc.add(xsub(r, xmul(c0, xc[c])));
      const T xt = sweep_div(r, c0, rc0);
      X1[base + off[c] + k * LXY] = xsub(xc[c], xmul(om, xsub(xc[c], xt)));
      xm[c] = xc[c];
      xc[c] = up[c];
    }
  }
  if (RES) {
    acc.warp_reduce();
    if (lane == 0) red[w] = acc.value();
  }
  __syncthreads();  // the block's x1 interior is in its brick, seen by the whole CTA
  if (RES && tid == 0) {
    double v = 0.0;
    for (int q = 0; q < NW; q++) v += red[q];
    a.partial[b] = v;
  }
  jacobi_push_tail<T, N, VC, NT>(X0, X1, g, a, b, tid, zero);
}

// Push-form fused Jacobi on 32^3 blocks with x0 and b streamed through
// shared memory one z-plane at a time (stream.cuh): 256 threads, each four
// cells (i, j), (i, j+8), (i, j+16), (i, j+24) of every plane, a warp per
// row, so every shared-memory access of a warp is one row segment.  The
// arithmetic is the column walk's (jacobi_smoother's term order); the
// planes of x1 go to HBM as rows.  A value in the first VC layers of a face
// whose neighbour is on the same level goes, as computed, to that
// neighbour's ghost cell as well (the same-level entries of the push table,
// copies); in FP32 at vc = 1 so do the C2F and F2C entries of x faces, from
// the block's outermost x1 columns staged in shared memory; jacobi_push_tail
// then does the rest (edges, unfed faces, the other level-change entries).  ZERO: x0 == 0, only b is streamed.  PRE (with ZERO): b made
// in the same pass from the BiCGSTAB vectors streamed instead (JacPre, the
// operations of kr_p / kr_s) and written back.
template <int PRE>
__host__ __device__ constexpr int jac_pre_fields() { return PRE == kPreP ? 3 : PRE == kPreS ? 2 : 1; }

template <typename T, int N, int VC, int S, bool RES, bool ZERO, int NT_ = 256, int PRE = 0>
struct JacStream {
  static_assert(PRE == 0 || ZERO, "the right-hand side is made in the zero-start pass");
  using R = PlaneRing<T, N, VC, S, !ZERO, jac_pre_fields<PRE>()>;
  static constexpr int NT = NT_;
  static constexpr size_t SMEM = R::SMEM;
  // at most 6 CTAs (40 registers): at 8 the push tail spills
  static constexpr int MINB = stream_minb<SMEM + 64, (NT_ == 256 ? 6 : 2048 / NT_)>();
};

template <typename T, int N, int VC, int S, bool RES, bool ZERO, int NT_ = 256, int PRE = 0>
__global__ void __launch_bounds__(NT_, (JacStream<T, N, VC, S, RES, ZERO, NT_, PRE>::MINB))
    jacobi_stream_push_kernel(const T* __restrict__ X0, T* __restrict__ X1,
                              const T* Bv, Geom g, JacArgs<T> a) {
  using JS = JacStream<T, N, VC, S, RES, ZERO, NT_, PRE>;
  using R = typename JS::R;
  using BL = typename R::BL;
  constexpr int NT = JS::NT, NW = NT / 32, CPT = N * N / NT, LX = R::LX, LXY = R::LXY;
  static_assert(N * N % NT == 0 && NT % N == 0, "whole rows per warp");
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ double red[NW];
  __shared__ int same[6];  // same-level neighbour across each face of this block, or -1
  // FP32, vc = 1: the x faces' level-change entries (C2F to finer
  // neighbours, F2C to a coarser one) are made during the walk, from the
  // block's two outermost x1 columns on each x side kept in shared memory
  // for the last three planes (xface[side][plane % 3][j][column]); the tail
  // makes the rest.  Up to kXle such entries (2:1 balance gives at most 8:
  // four finer neighbours on each x face).
  constexpr bool XW = sizeof(T) == 4 && VC == 1;
  constexpr int kXle = 12;
  __shared__ float xface[XW ? 2 * 3 * N * 2 : 1];
  __shared__ VcTask xle[XW ? kXle : 1];
  __shared__ int nxle;
  const int b = blockIdx.x, tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const int64_t base = (int64_t)b * g.bstride;
  // the update's scalars; a finished segment's blocks change nothing (their
  // x1 is never read: no face joins two segments)
  T s_beta = T(0), s_ng = T(0), s_na = T(0);
  if (PRE != 0) {
    const KSeg& sg = a.pre.segs.seg[kseg_of(a.pre.segs, b)];
    if (sg.status != kRunning) return;
    s_beta = (T)sg.beta;
    s_ng = (T)(-sg.gamma);
    s_na = (T)(-sg.alpha);
  }
  R ring(smraw);
  constexpr int NB = jac_pre_fields<PRE>();
  const T* C[NB];
  if (PRE == kPreP) { C[0] = a.pre.r; C[1] = Bv; C[NB - 1] = a.pre.q; }
  else if (PRE == kPreS) { C[0] = a.pre.r; C[NB - 1] = a.pre.q; }
  else if (PRE == kPreCopy) { C[0] = a.pre.r; }
  else { C[0] = Bv; }
  if (tid == 0) ring.start(X0, C, base);
  if (w == NW - 1) {
    if (lane < 6) same[lane] = -1;
    __syncwarp();
    const int p0 = a.push.ptr[b], p1 = a.push.ptr[b + 1];
    int nx = 0;  // x-face level-change entries so far, in table order
    for (int q0 = p0; q0 < p1; q0 += 32) {
      const int q = q0 + lane;
      VcTask t{};
      if (q < p1) t = a.push.tasks[q];
      if (q < p1 && t.kind == VC_COPY) same[t.face ^ 1] = t.dst;  // t.face: the destination's face
      const bool xl = XW && q < p1 && t.kind != VC_COPY && (t.face >> 1) == 0;
      const unsigned m = __ballot_sync(0xffffffffu, xl);
      const int k = nx + __popc(m & ((1u << lane) - 1u));
      if (xl && k < kXle) xle[k] = t;
      nx += __popc(m);
    }
    if (lane == 0) nxle = nx < kXle ? nx : kXle;
  }
  const T* cf = a.cf + (int64_t)b * 8;
  const T c0 = cf[0], c1 = cf[1], c2 = cf[2], c3 = cf[3], c4 = cf[4], c5 = cf[5], c6 = cf[6];
  const T rc0 = cf[7];
  const T om = a.omega;
  int o[CPT];
#pragma unroll
  for (int c = 0; c < CPT; c++) {
    const int e = tid + c * NT;
    o[c] = R::at(e % N, e / N);
  }
  SqAcc<T> acc;
  __syncthreads();  // the ring's barriers are initialised, same[] is set
  // Same-level ghost targets of this thread's cells.  All its cells share
  // i = tid % N (x faces: a neighbour brick and ghost column, or none); its
  // first cell is the lowest j (-y face), its last the highest (+y face); z
  // faces by plane.
  constexpr int JSTEP = NT / N;  // j step between a thread's cells
  static_assert(JSTEP >= VC, "the y-face cells are a thread's first and last");
  const int i0 = tid % N, j0 = tid / N;
  T* xdst = nullptr;
  int xg = 0;
  if (!XW && i0 < VC && same[0] >= 0) {
    xdst = X1 + (int64_t)same[0] * g.bstride;
    xg = N + i0;
  } else if (!XW && i0 >= N - VC && same[1] >= 0) {
    xdst = X1 + (int64_t)same[1] * g.bstride;
    xg = i0 - N;
  }
  const int ylo = j0 < VC ? same[2] : -1;
  const int yhi = j0 + (CPT - 1) * JSTEP >= N - VC ? same[3] : -1;
  const int zlo = same[4], zhi = same[5];
  const int nxl = XW ? nxle : 0;
  // this thread's x1 values of the outermost x columns go to xface (FP32,
  // vc = 1: the same-level x pushes are made from there too, a plane late,
  // one thread per row)
  const int xcol = !XW || (nxl == 0 && same[0] < 0 && same[1] < 0) ? -1 : i0 < 2 ? i0 : i0 >= N - 2 ? 2 + i0 - (N - 2) : -1;
  // Before output plane m (and once more after the walk, m = N): the x-face
  // level-change ghosts whose sources are complete by plane m - 1 -- C2F
  // ghosts interpolated from coarse planes K = m-2 and m-1 (fine z rows
  // 2K+1, 2K+2; the clamped ends add rows 0 and 2N-1), F2C ghosts averaged
  // from fine planes m-2 and m-1 (m even).  Operations and order as
  // push_entry's.
  auto xlev = [&](int m) {
    // same-level x faces: plane m-1's outermost columns into the neighbours'
    // ghost columns
    if (XW && m >= 1 && tid < 2 * N) {
      const int sd = tid / N, jj = tid % N, nbr = same[sd];
      if (nbr >= 0)
        reinterpret_cast<float*>(X1)[(int64_t)nbr * g.bstride + BL::at(sd ? -1 : N, jj, m - 1)] =
            xface[(sd * 3 + (m - 1) % 3) * 2 * N + jj * 2 + sd];
    }
    if (!XW || m < 2) return;
    for (int e = tid; e < nxl * 3 * N; e += NT) {
      const VcTask t = xle[e / (3 * N)];
      const int it = e % (3 * N);
      const bool minus = (t.face & 1) == 0;
      const int side = minus ? 1 : 0;  // the source's x columns N-2, N-1 or 0, 1
      const int o0 = t.subface & 1, o1 = (t.subface >> 1) & 1;
      const int dn = minus ? -1 : N;
      float* dst = reinterpret_cast<float*>(X1) + (int64_t)t.dst * g.bstride;
      if (t.kind == VC_C2F) {
        const int K = m - 2;
        const int f0 = K == 0 ? 0 : 2 * K + 1, nr = (K == 0 || K == N - 2) ? 3 : 2;
        const int row = it / N, av = it % N;
        if (row >= nr) continue;
        const int fz = f0 + row, cz = fz - N * o1;
        if (cz < 0 || cz >= N) continue;
        const int fy = av + N * o0, fn = minus ? 2 * N - 1 : 0;
        const int I = lin_I(fn, N), J = lin_I(fy, N);
        const float* pK = xface + (side * 3 + K % 3) * 2 * N;
        const float* pK1 = xface + (side * 3 + (K + 1) % 3) * 2 * N;
        dst[g.at(dn, av, cz)] = C2F<float>::value(pK + J * 2, 2, (int)(pK1 - pK), lin_r(fn, I),
                                                   lin_r(fy, J), lin_r(fz, K));
      } else if (t.kind == VC_F2C) {
        if ((m & 1) || it >= N / 2) continue;
        const int cz = (m - 2) / 2, av = it;
        const float* p = xface + (side * 3 + (2 * cz) % 3) * 2 * N + 2 * av * 2;
        const float* p1 = xface + (side * 3 + (2 * cz + 1) % 3) * 2 * N + 2 * av * 2;
        dst[g.at(dn, av + (N / 2) * o0, cz + (N / 2) * o1)] = f2c_value<float>(p, 2, (int)(p1 - p));
      }
    }
  };
  const bool ok = plane_walk(ring, X0, C, base, a.err, tid, [&](int m) {
    xlev(m);
    const T* xm = ring.xp(m);
    const T* xc = ring.xp(m + 1);
    const T* xu = ring.xp(m + 2);
    const T* bp = ring.cp(ZERO ? m : m + 1, 0);
    T* out = X1 + base + (int64_t)(VC + m) * LXY;
    T* bout = const_cast<T*>(Bv) + base + (int64_t)(VC + m) * LXY;
    const int zd = m < VC ? zlo : (m >= N - VC ? zhi : -1);
    const int zg = m < VC ? N + m : m - N;
#pragma unroll
    for (int c = 0; c < CPT; c++) {
      const int q = o[c];
      T xw, xe, xs_, xn, xmv, up, xcv;
      if (ZERO) {
        xw = xe = xs_ = xn = xmv = up = xcv = T(0);
      } else {
        xw = xc[q - 1];
        xe = xc[q + 1];
        xs_ = xc[q - LX];
        xn = xc[q + LX];
        xmv = xm[q];
        up = xu[q];
        xcv = xc[q];
      }
      T r;
      if (PRE == kPreP) {  // kr_p: p = r + beta (p - gamma q)
        r = xadd(bp[q], xmul(s_beta, xadd(ring.cp(m, 1)[q], xmul(s_ng, ring.cp(m, NB - 1)[q]))));
        bout[q] = r;
      } else if (PRE == kPreS) {  // kr_s: s = r - alpha q
        r = xadd(xmul(s_na, ring.cp(m, NB - 1)[q]), bp[q]);
        bout[q] = r;
      } else if (PRE == kPreCopy) {  // the first iteration: p = r
        r = bp[q];
        bout[q] = r;
      } else {
        r = bp[q];
      }
      r = xsub(r, xmul(c1, xw));
      r = xsub(r, xmul(c2, xe));
      r = xsub(r, xmul(c3, xs_));
      r = xsub(r, xmul(c4, xn));
      r = xsub(r, xmul(c5, xmv));
      r = xsub(r, xmul(c6, up));
      if (RES) acc.add(xsub(r, xmul(c0, xcv)));
      const T xt = sweep_div(r, c0, rc0);
      const T v = xsub(xcv, xmul(om, xsub(xcv, xt)));
      out[q] = v;
      // same-level copies: this cell feeds the ghost layer of every face it
      // lies within VC cells of
      const int j = j0 + c * JSTEP;
      if (XW && xcol >= 0)
        xface[((xcol >> 1) * 3 + m % 3) * 2 * N + j * 2 + (xcol & 1)] = (float)v;
      if (xdst) xdst[BL::at(xg, j, m)] = v;
      if (c == 0 && ylo >= 0) X1[(int64_t)ylo * g.bstride + BL::at(i0, N + j, m)] = v;
      if (c == CPT - 1 && yhi >= 0) X1[(int64_t)yhi * g.bstride + BL::at(i0, j - N, m)] = v;
      if (zd >= 0) X1[(int64_t)zd * g.bstride + BL::at(i0, j, zg)] = v;
    }
  });
  if (!ok) return;  // a copy never arrived: the error word says so
  xlev(N);  // the walk's last barrier made planes N-2 and N-1 visible
  if (RES) {
    acc.warp_reduce();
    if (lane == 0) red[w] = acc.value();
    __syncthreads();
    if (tid == 0) {
      double v = 0.0;
      for (int q = 0; q < NW; q++) v += red[q];
      a.partial[b] = v;
    }
  }
  // the walk's last barrier made the block's x1 interior visible to the CTA
  jacobi_push_tail<T, N, VC, NT, 4, false>(X0, X1, g, a, b, tid, ZERO, nxl);
}

template <typename T, int N, int VC, int S, bool RES, bool ZERO, int PRE = 0>
static cudaError_t jacobi_stream_launch_one(const T* x0, T* x1, const T* b, const Geom& g,
                                            const JacArgs<T>& a, cudaStream_t st) {
  using JS = JacStream<T, N, VC, S, RES, ZERO, 256, PRE>;
  auto kern = jacobi_stream_push_kernel<T, N, VC, S, RES, ZERO, 256, PRE>;
  // set once per process (not a stream operation; runs before any CUDA-graph
  // capture of these launches)
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)JS::SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  kern<<<g.nb, JS::NT, JS::SMEM, st>>>(x0, x1, b, g, a);
  return cudaGetLastError();
}

// Ring depths of the streamed Jacobi (74 KB of shared memory, 3 CTAs per
// SM): with x0 8 slots in FP32, 4 in FP64; b alone 16 and 8.  Measured on
// 2920 blocks of 32^3 with a same-level push table (FP32): with x0 264 us
// at 8 slots against 298 at 4 (6 CTAs per SM) and 329 at 10; b alone 215 us
// at 16 against 243 at 6-8 and 272 at 4.
template <typename T, int N, int VC>
static cudaError_t jacobi_stream_launch(const T* x0, T* x1, const T* b, const Geom& g,
                                        const JacArgs<T>& a, cudaStream_t st) {
  constexpr int SX = sizeof(T) == 4 ? 8 : 4, SZ = sizeof(T) == 4 ? 16 : 8;
  // with the vector update fused: 3 / 2 / 1 streamed fields a plane (74 KB)
  constexpr int SP = sizeof(T) == 4 ? 5 : 2, SS = sizeof(T) == 4 ? 8 : 4;
  const bool res = a.partial != nullptr, zero = a.zero_x0 != 0;
  if (a.pre.kind != kPreNone) {
    if (!zero || res) return cudaErrorInvalidValue;
    if (a.pre.kind == kPreP) return jacobi_stream_launch_one<T, N, VC, SP, false, true, kPreP>(x0, x1, b, g, a, st);
    if (a.pre.kind == kPreS) return jacobi_stream_launch_one<T, N, VC, SS, false, true, kPreS>(x0, x1, b, g, a, st);
    return jacobi_stream_launch_one<T, N, VC, SZ, false, true, kPreCopy>(x0, x1, b, g, a, st);
  }
  if (zero)
    return res ? jacobi_stream_launch_one<T, N, VC, SZ, true, true>(x0, x1, b, g, a, st)
               : jacobi_stream_launch_one<T, N, VC, SZ, false, true>(x0, x1, b, g, a, st);
  return res ? jacobi_stream_launch_one<T, N, VC, SX, true, false>(x0, x1, b, g, a, st)
             : jacobi_stream_launch_one<T, N, VC, SX, false, false>(x0, x1, b, g, a, st);
}

template <typename T, int N, int VC>
static cudaError_t jacobi_cubic_push_launch(const T* x0, T* x1, const T* b, const Geom& g,
                                            const JacArgs<T>& a, cudaStream_t st) {
  constexpr int CPT = 2, NT = N * N / CPT;
  if (a.partial)
    jacobi_cubic_push_kernel<T, N, VC, CPT, true><<<g.nb, NT, 0, st>>>(x0, x1, b, g, a);
  else
    jacobi_cubic_push_kernel<T, N, VC, CPT, false><<<g.nb, NT, 0, st>>>(x0, x1, b, g, a);
  return cudaGetLastError();
}

template <typename T, int N, int VC>
static cudaError_t jacobi_tile_launch(const T* x0, T* x1, const T* b, const Geom& g,
                                      const JacArgs<T>& a, bool pull, cudaStream_t st) {
  using L = BrickStage<T, N, VC, true>;
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

template <typename T, int N, int VC>
static cudaError_t jacobi_pipe_launch(const T* x0, T* x1, const T* b, const Geom& g,
                                      const PipeArgs<T>& p, cudaStream_t st) {
  // launches after a run's first follow the run's previous launch
  const bool pdl = p.pull_now != 0;
  return p.partial ? pipe_launch<T, N, VC, kOpJacobi, true>(x0, x1, b, g, p, st, pdl)
                   : pipe_launch<T, N, VC, kOpJacobi, false>(x0, x1, b, g, p, st, pdl);
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
                                     T omega, BlockBc bc, PushTable push, int ghost_mode,
                                     int shape, double* partial, int* err, const JacPre<T>* pre,
                                     cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  if (ghost_mode == kGhostPushZero && !(g.nx == 32 && g.ny == 32 && g.nz == 32))
    return cudaErrorInvalidValue;
  if (g.nx == 32 && g.ny == 32 && g.nz == 32 && (g.vc == 1 || g.vc == 2)) {
    // 32^3: push form only
    if (ghost_mode != kGhostPush && ghost_mode != kGhostPushZero) return cudaErrorInvalidValue;
    JacArgs<T> a{0, cf, omega, bc, push, partial, err, ghost_mode == kGhostPushZero ? 1 : 0,
                 pre ? *pre : JacPre<T>{kPreNone, nullptr, nullptr, KSegs{}}};
    const bool streamed = plane_stream_enabled() && stream_aligned<T>(g, x0, b) &&
                          (!pre || (stream_aligned<T>(g, pre->r, pre->q ? pre->q : pre->r)));
    if (a.pre.kind != kPreNone && !streamed) return cudaErrorNotSupported;
    if (streamed)
      return g.vc == 1 ? jacobi_stream_launch<T, 32, 1>(x0, x1, b, g, a, st)
                       : jacobi_stream_launch<T, 32, 2>(x0, x1, b, g, a, st);
    return g.vc == 1 ? jacobi_cubic_push_launch<T, 32, 1>(x0, x1, b, g, a, st)
                     : jacobi_cubic_push_launch<T, 32, 2>(x0, x1, b, g, a, st);
  }
  if (!jacobi_tile_ok<T>(g)) return cudaErrorInvalidValue;
  if (ghost_mode != kGhostPush && shape == kJacobiPipe) {
    if (!pipe_shape_ok((int)sizeof(T), g.nx, g.vc, true)) return cudaErrorInvalidValue;
    PipeArgs<T> p{cf, omega, (T)0, 0, bc, push.info, push.out_tasks,
                  static_cast<const T*>(push.side_in), static_cast<T*>(push.side_out),
                  static_cast<const T*>(push.xf_in), static_cast<T*>(push.xf_out),
                  ghost_mode == kGhostPull ? 1 : 0, partial, err};
    if (g.nx == 16)
      return g.vc == 1 ? jacobi_pipe_launch<T, 16, 1>(x0, x1, b, g, p, st)
                       : jacobi_pipe_launch<T, 16, 2>(x0, x1, b, g, p, st);
    return g.vc == 1 ? jacobi_pipe_launch<T, 8, 1>(x0, x1, b, g, p, st)
                     : jacobi_pipe_launch<T, 8, 2>(x0, x1, b, g, p, st);
  }
  const bool pl = ghost_mode != kGhostPush;
  JacArgs<T> a{ghost_mode == kGhostPull ? 1 : 0, cf, omega, bc, push, partial, err};
  if (g.nx == 16)
    return g.vc == 1 ? jacobi_tile_launch<T, 16, 1>(x0, x1, b, g, a, pl, st)
                     : jacobi_tile_launch<T, 16, 2>(x0, x1, b, g, a, pl, st);
  return g.vc == 1 ? jacobi_tile_launch<T, 8, 1>(x0, x1, b, g, a, pl, st)
                   : jacobi_tile_launch<T, 8, 2>(x0, x1, b, g, a, pl, st);
}

}  // namespace bcmg
