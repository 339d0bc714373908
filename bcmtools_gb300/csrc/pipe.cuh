// pipe.cuh -- fused sweeps in the pull ghost form, one CTA per block or
// persistent and double-buffered (Jacobi: SolverTest/blas.f90:452-502 with
// ILS3D.h:108-123's ghost update; red-black SOR: sor1/Solver.cpp:132-153,
// sor2/Solver.cpp:136-160).
//
// A CTA of N*N threads walks blocks b, b + grid, ... (one block when the grid
// covers them all).  A block's stage arrives by bulk copies (the TMA engine's
// non-tensor form) on the stage's mbarrier: its planes, its second field
// (Jacobi's b; sor2's source, packed N^3 per block for SOR runs), its
// coefficients and Dirichlet values.  Each thread loads its cell of every
// pulled ghost face into a register before the wait: from the neighbour's
// brick rows for same-level Y and Z faces, from the neighbour's x-face layer
// for same-level X faces (each CTA writes its block's columns x = 0 and
// x = N-1 contiguously after its sweep, so no X ghost costs a 32-byte sector
// of its own), interpolated from the coarse interior for faces on a coarser
// block, from the side buffer for faces on finer blocks.  With
// two stages the copies of block n+1 are issued before block n's wait and its
// ghost loads right after, so their latency hides behind block n's sweep.
// Output planes leave as bulk stores.  So HBM sees whole rows in and out.
//
// Ghosts: a launch with pull_now fills the first ghost layer of its pulled
// faces and its Dirichlet ghosts from its own interior -- the ghost update
// that followed the previous launch.  A face on a coarser block interpolates
// its C2F ghosts in the reader from the coarse interior in A; F2C averages
// (faces on finer blocks) are computed by their source block's CTA from its
// tile right after its sweep and written to a side buffer (one N*N first
// layer per face), which the reading launch loads like a neighbour's face.  Without pull_now the launch reads A's ghosts as
// they are (the first launch of a run).  It writes to B planes [0,N) only
// (rows [0,N) where those start on a 16-byte boundary): interior, and for
// the ghost cells in them the values A had (or had pulled), so ghosts no
// update writes keep their values; a ghost update closes the run.
#pragma once
#include <algorithm>

#include "bulk.cuh"
#include "cells.cuh"
#include "ghost.cuh"
#include "kernels.h"
#include "tile.cuh"

namespace bcmg {

// kOpSor2P: sor2 with its source packed N^3 per block in sweep order
// (pack_source_kernel), prepared once per SOR run
enum : int { kOpJacobi = 0, kOpSor1 = 1, kOpSor2 = 2, kOpSor2P = 3 };

template <typename T>
struct PipeArgs {
  const T* coef;      // per block: Jacobi {Ap..At, 1/Ap} (8), SOR {c0, cx, cy, cz} (4)
  T omega, om1;       // SOR: omega, 1 - omega; Jacobi: omega
  int n_inner;        // SOR inner passes
  BlockBc bc;         // Dirichlet values [nb*6] (and bcx form)
  const BlockInfo* info;  // [nb] block descriptors
  const VcTask* out_tasks;  // F2C entries by source block
  const T* side_in;       // first-layer F2C ghosts of A, by slot
  T* side_out;            // ... of B, written here
  const T* xf_in;         // x-face layers of A's blocks (PushTable::xf_in)
  T* xf_out;              // ... of B's, written here
  int pull_now;
  double* partial;    // Jacobi: [nb] sum of squared residuals of the input (or null)
  int* err;           // device error word (bounded-wait timeouts)
};

// The (i, j) column thread tid of an N*N-thread CTA sweeps.  N = 16: rows j
// and j+D share a warp, D*LX = 16 (mod 32) keeping float accesses of the two
// half-warps on disjoint banks.
template <typename T, int N, int LX>
__device__ __forceinline__ void sweep_column(int tid, int& i, int& j) {
  if (N == 16) {
    constexpr int D = sizeof(T) == 4 ? ((LX * 8) % 32 == 16 ? 8 : (LX * 4) % 32 == 16 ? 4
                                        : (LX * 2) % 32 == 16 ? 2 : 1) : 1;
    const int w = tid >> 5, lane = tid & 31;
    i = lane & 15;
    j = (w % D) + 2 * D * (w / D) + D * (lane >> 4);
  } else {
    i = tid % N;
    j = tid / N;
  }
}

// The packed source of SOR runs: per block N planes of N*N values, value
// (i, j, k) at k*N*N + t with t the thread that sweeps column (i, j), so a
// plane's values are read by consecutive threads (no bank conflict).  One
// CTA of N*N threads per block.
template <typename T, int N, int VC>
__global__ void __launch_bounds__(N * N) pack_source_kernel(T* __restrict__ dst,
                                                            const T* __restrict__ src, Geom g) {
  constexpr int LX = N + 2 * VC;
  int i, j;
  sweep_column<T, N, LX>(threadIdx.x, i, j);
  const T* sb = src + (int64_t)blockIdx.x * g.bstride + (VC + j) * LX + VC + i;
  T* db = dst + (int64_t)blockIdx.x * (N * N * N) + threadIdx.x;
  for (int k = 0; k < N; k++) db[k * N * N] = sb[(VC + k) * LX * LX];
}

// Stage layout.  Tile: Tile<T,N,VC> (rows and planes [-1,N], full row pitch).
// Second field: per interior plane either its rows [0,N) (COMPACT, when they
// start on a 16-byte boundary), the whole brick plane, or (packed source) the
// N*N interior cells in sweep order.  Meta: coefficients, Dirichlet values, descriptor
// flags, outgoing F2C entries.
template <typename T, int N, int VC, int OP>
struct PipeStage {
  using TL = Tile<T, N, VC>;
  static constexpr int NT = N * N;
  static constexpr int LX = TL::LX, TP = TL::LXY;   // tile row and plane pitch
  static constexpr int BLXY = LX * LX;              // brick plane pitch
  static constexpr bool HAS_S = OP != kOpSor1;
  static constexpr bool SPACK = OP == kOpSor2P;
  static constexpr bool COMPACT = (VC * LX * sizeof(T)) % 16 == 0;
  // vc = 2: the tile's rows [0,N) of planes [0,N) come in one copy per plane,
  // rows -1 / N only where no pulled ghost replaces them
  static constexpr bool YSPLIT = VC == 2 && COMPACT;
  static constexpr int SR = SPACK ? N : LX;                     // second-field row pitch
  static constexpr int SP = SPACK ? N * N : COMPACT ? N * LX : BLXY;  // ... plane pitch
  static constexpr int SROW0 = SPACK || COMPACT ? 0 : VC;       // its row of y = 0
  static constexpr int SX0 = SPACK ? 0 : VC;                    // its column of x = 0
  // rows of each plane [0,N) the launch writes: [0,N) when they start on a
  // 16-byte boundary, else (vc = 1, float) the whole plane [-1,N]
  static constexpr int OUT_Y0 = COMPACT ? 0 : -1;
  static constexpr int OUT_LEN = (COMPACT ? N : N + 2) * LX;  // elements per plane
  static_assert((OUT_LEN * sizeof(T)) % 16 == 0, "output planes leave as 16-byte multiples");
  static constexpr int NCOEF = OP == kOpJacobi ? 8 : 4;
  static constexpr unsigned TILE_B = (TL::SIZE * sizeof(T) + 127) / 128 * 128;
  static constexpr unsigned S_B = HAS_S ? (N * SP * sizeof(T) + 127) / 128 * 128 : 0;
  static constexpr unsigned S_OFF = TILE_B;
  static constexpr unsigned META_OFF = S_OFF + S_B;
  static constexpr unsigned COEF_B = NCOEF * sizeof(T);
  static constexpr unsigned DVAL_OFF = META_OFF + 64;  // 6 doubles
  static constexpr unsigned FLAGS_OFF = DVAL_OFF + 48;
  static constexpr unsigned V2F_OFF = META_OFF + 128;     // 8 floats (BlockBc::v2f)
  static constexpr unsigned TASKS_OFF = META_OFF + 160;  // outgoing F2C entries
  static constexpr unsigned STAGE =
      (TASKS_OFF + kMaxOutEntries * sizeof(VcTask) + 127) / 128 * 128;

  static_assert(COEF_B <= 64, "coefficients fit the meta area");
  static_assert((TP * sizeof(T)) % 16 == 0 && (BLXY * sizeof(T)) % 16 == 0 &&
                    (LX * sizeof(T) * (VC - 1)) % 16 == 0 && (SP * sizeof(T)) % 16 == 0,
                "plane copies need 16-byte offsets");
  static __device__ __forceinline__ int s_at(int i, int j, int k) {
    return k * SP + (SROW0 + j) * SR + SX0 + i;
  }
  // the second-field area as a tile layout (Jacobi's x1 image)
  struct Img {
    static constexpr int LX = PipeStage::LX, LXY = SP, O = SROW0 * PipeStage::LX + VC;
    static __device__ __forceinline__ int at(int i, int j, int k) { return O + i + LX * j + LXY * k; }
  };
};

// F2C ghosts entry t feeds (first layer), from this block's tile (layout TL)
// into the side-buffer slot of (t.dst, t.face); NT workers (worker `tid`)
// split the cells.  (C2F ghosts are interpolated by their readers.)
template <typename T, int N, int VC, class TL, int NT>
__device__ __forceinline__ void side_push(const VcTask& t, T* slot, const Geom& g, const T* sf,
                                          int tid) {
  switch (t.face >> 1) {
    case 0: push_entry<T, N, VC, VC_F2C, 0, TL, true, true, NT>(t, slot, g, sf, tid); break;
    case 1: push_entry<T, N, VC, VC_F2C, 1, TL, true, true, NT>(t, slot, g, sf, tid); break;
    default: push_entry<T, N, VC, VC_F2C, 2, TL, true, true, NT>(t, slot, g, sf, tid); break;
  }
}

// Column walk of one Jacobi sweep (the reference's `real` operation order);
// x1 replaces b in the second-field area.  RES accumulates the squared
// residuals of x0.
template <typename T, int N, int VC, bool RES>
__device__ __forceinline__ void pipe_jacobi(const T* tile, T* sv, const T* cf, T om, int i, int j,
                                            SqAcc<T>& acc) {
  using PS = PipeStage<T, N, VC, kOpJacobi>;
  constexpr int LX = PS::LX, TP = PS::TP;
  const T c0 = cf[0], c1 = cf[1], c2 = cf[2], c3 = cf[3], c4 = cf[4], c5 = cf[5], c6 = cf[6];
  const T rc0 = cf[7];  // RN(1/Ap), or 0
  const T* xc_p = tile + PS::TL::at(i, j, 0);
  T* bp = sv + PS::s_at(i, j, 0);
  T xm = xc_p[-TP], xc = xc_p[0];
  static_assert(N % 4 == 0, "cells in groups of four");
#pragma unroll
  for (int k0 = 0; k0 < N; k0 += 4) {
    // four cells: every load before the first store into b's area, so the
    // loads overlap
    T xw[4], xe[4], xs_[4], xn[4], xu[4], bv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const T* q = xc_p + (k0 + u) * TP;
      xw[u] = q[-1];
      xe[u] = q[1];
      xs_[u] = q[-LX];
      xn[u] = q[LX];
      xu[u] = q[TP];
      bv[u] = bp[(k0 + u) * PS::SP];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
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
      bp[(k0 + u) * PS::SP] = xsub(xc, xmul(om, xsub(xc, xt)));
      xm = xc;
      xc = xp;
    }
  }
}

// CTAs per SM the registers are planned for.  STAGES = 2: persistent, two
// CTAs of 256 threads per SM for 16^3 blocks (at most 128 registers).
// STAGES = 1: one CTA per block (grid = blocks), no prefetch across blocks;
// five per SM for 16^3 float SOR blocks without a padded source (at most 48
// registers; the packed-source stage of 42 KB admits five), else four.
template <typename T, int N, int OP, int STAGES>
constexpr int pipe_min_blocks() {
  return STAGES == 2 ? (N == 16 ? 2 : 4)
         : N != 16   ? 8
         : (sizeof(T) == 4 && (OP == kOpSor1 || OP == kOpSor2P)) ? 5 : 4;
}

template <typename T, int N, int VC, int OP, bool RES, int STAGES>
__global__ void __launch_bounds__(N * N, (pipe_min_blocks<T, N, OP, STAGES>()))
    sweep_pipe_kernel(const T* __restrict__ A, T* __restrict__ Bf, const T* __restrict__ S,
                      Geom g, PipeArgs<T> a) {
  using PS = PipeStage<T, N, VC, OP>;
  using TL = typename PS::TL;
  constexpr int NT = PS::NT, NW = NT / 32, LX = PS::LX, TP = PS::TP, BLXY = PS::BLXY;
  constexpr int NN = N * N;
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ uint64_t bar[2];
  __shared__ double red[NW];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int grid = gridDim.x;
  const bool pull = a.pull_now != 0;
  const int gp = tid % N, gq = tid / N;  // this thread's cell of every face
  // the first block's descriptor, loaded first (the longest chain of loads
  // starts from it)
  BlockInfo nxt = a.info[blockIdx.x < g.nb ? blockIdx.x : 0];
  // the next launch of the run may start its CTAs as slots free up: they
  // issue their constant copies and then wait for this grid to complete
  griddep_launch_dependents();
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();

  // Warp 0: bulk copies of block blk into stage st, in three parts on one
  // mbarrier phase.  Part C (coefficients, second field) is data no launch
  // of the run writes: a dependent launch issues it before waiting for its
  // predecessor.  Part A (the tile's rows [0,N) of planes [0,N) -- the whole
  // planes for vc = 1) needs no descriptor and starts before it arrives;
  // part B (rows and planes of ghosts no pulled face replaces, Dirichlet
  // values, outgoing entries) follows it, and its arrival closes the phase.
  constexpr unsigned PBY = TP * sizeof(T);
  constexpr unsigned RBY = LX * sizeof(T);                  // one row
  constexpr unsigned ABY = PS::YSPLIT ? N * RBY : PBY;      // part A bytes per plane
  constexpr unsigned SBY = !PS::HAS_S ? 0
                           : PS::SPACK ? N * NN * sizeof(T)
                                       : N * (PS::COMPACT ? N * LX : BLXY) * sizeof(T);
  // Part C: what no launch of the run writes (coefficients, second field);
  // a dependent launch issues it before waiting for its predecessor.
  auto copies_c = [&](int blk, int st) {
    if (w != 0) return;
    // the stage's last output stores (two blocks back) have read it
    if (STAGES == 2) bulk_wait_read();
    __syncwarp();
    unsigned char* base = smraw + st * PS::STAGE;
    if (lane == 0) {
      mbar_add_tx(&bar[st], SBY + PS::COEF_B);
      bulk_g2s(base + PS::META_OFF, a.coef + (int64_t)blk * PS::NCOEF, PS::COEF_B, &bar[st]);
    }
    if (PS::HAS_S) {
      unsigned char* sd = base + PS::S_OFF;
      if (PS::SPACK) {
        if (lane == 2) bulk_g2s(sd, S + (int64_t)blk * (N * NN), SBY, &bar[st]);
      } else if (PS::COMPACT) {
        const T* sb = S + (int64_t)blk * g.bstride;
        constexpr unsigned RB = N * LX * sizeof(T);
        for (int k = lane; k < N; k += 32)
          bulk_g2s(sd + k * RB, sb + (VC + k) * BLXY + VC * LX, RB, &bar[st]);
      } else if (lane == 2) {
        bulk_g2s(sd, S + (int64_t)blk * g.bstride + VC * BLXY, SBY, &bar[st]);
      }
    }
  };
  auto copies_a = [&](int blk, int st) {
    if (w != 0) return;
    unsigned char* base = smraw + st * PS::STAGE;
    const T* xb = A + (int64_t)blk * g.bstride;
    if (lane == 0) mbar_add_tx(&bar[st], N * ABY);
    __syncwarp();
    if (VC == 1) {
      // tile planes = brick planes: one copy for planes [0,N)
      if (lane == 1) bulk_g2s(base + PBY, xb + VC * BLXY, N * PBY, &bar[st]);
    } else {
      constexpr int R0 = PS::YSPLIT ? 1 : 0;  // first tile row copied
      for (int k = lane; k < N; k += 32)
        bulk_g2s(base + (k + 1) * PBY + R0 * RBY, xb + (VC + k) * BLXY + (VC - 1 + R0) * LX, ABY,
                 &bar[st]);
    }
  };
  auto copies_b = [&](int blk, int st, const BlockInfo& inf) {
    if (w != 0) return;
    const unsigned flags = (unsigned)inf.flags;
    unsigned char* base = smraw + st * PS::STAGE;
    // ghost planes -1 / N and (vc = 2) ghost rows -1 / N unless pulled
    const bool lo = !pull || !(flags & (BI_FED << 4)), hi = !pull || !(flags & (BI_FED << 5));
    const bool ylo = PS::YSPLIT && (!pull || !(flags & (BI_FED << 2)));
    const bool yhi = PS::YSPLIT && (!pull || !(flags & (BI_FED << 3)));
    const bool dir = (flags & (0x3fu << BI_DIR_SHIFT)) != 0;
    const unsigned nout = (flags >> BI_OUT_SHIFT) & 0x7fu;
    const unsigned nbytes = (lo + hi) * PBY + (ylo + yhi) * N * RBY + (dir ? 80u : 0u) +
                            nout * (unsigned)sizeof(VcTask);
    const T* xb = A + (int64_t)blk * g.bstride;
    if (lane == 0) {
      *reinterpret_cast<int*>(base + PS::FLAGS_OFF) = (int)flags;
      mbar_add_tx(&bar[st], nbytes);
      if (dir) {
        bulk_g2s(base + PS::DVAL_OFF, a.bc.value + (int64_t)blk * 6, 48, &bar[st]);
        bulk_g2s(base + PS::V2F_OFF, a.bc.v2f + (int64_t)blk * 8, 32, &bar[st]);
      }
      if (nout)
        bulk_g2s(base + PS::TASKS_OFF, a.out_tasks + inf.out_begin, nout * sizeof(VcTask), &bar[st]);
    }
    __syncwarp();
    if (PS::YSPLIT && (ylo || yhi)) {
      for (int q = lane; q < 2 * N; q += 32) {
        const bool up = q >= N;
        const int k = up ? q - N : q;
        if (up ? yhi : ylo)
          bulk_g2s(base + (k + 1) * PBY + (up ? (N + 1) * RBY : 0u),
                   xb + (VC + k) * BLXY + (up ? VC + N : VC - 1) * LX, RBY, &bar[st]);
      }
    }
    const int glo = VC == 1 ? 0 : (VC - 1) * LX;  // the ghost plane's rows [-1, N]
    if (lane == 2 && lo) bulk_g2s(base, xb + (VC - 1) * BLXY + glo, PBY, &bar[st]);
    if (lane == 3 && hi) bulk_g2s(base + (N + 1) * PBY, xb + (VC + N) * BLXY + glo, PBY, &bar[st]);
    __syncwarp();
    if (lane == 0) mbar_arrive(&bar[st]);  // every copy of the phase has been issued
  };

  // Every thread: its cell of each pulled face of block blk, into registers
  // -- same level: from the neighbour's x-face layer (X faces) or brick in A
  // (Y, Z faces: rows); from a coarser block: interpolated here from its
  // interior in A; from finer blocks: the face's side-buffer slot (F2C
  // averages their CTAs wrote).
  T g0 = 0, g1 = 0, g2 = 0, g3 = 0, g4 = 0, g5 = 0;
  auto gather = [&](const BlockInfo& inf) {
    const unsigned flags = (unsigned)inf.flags;
#define BCMG_PIPE_LOAD(F, V)                                                   \
    if (flags & (BI_FED << F)) {                                               \
      const int64_t src = inf.csrc[F];                                         \
      if ((F >> 1) == 0 && (flags & (BI_COPY << F))) {                         \
        /* X- ghost: the neighbour's column x = N-1 (layer 1), X+: x = 0 */    \
        V = __ldcg(a.xf_in + (src * 2 + (F == 0 ? 1 : 0)) * NN + gq * N + gp); \
      } else if (flags & (1u << bi_c2f_bit(F))) {                              \
        V = c2f_pull<T, N, VC, F>(A + (src >> 2) * g.bstride, (int)(src & 3), gp, gq); \
      } else if (flags & (BI_COPY << F)) {                                     \
        int ga, gc, gx, gy, gz;                                                \
        pull_map<N, F>(gp, gq, ga, gc, gx, gy, gz);                            \
        constexpr int AX = F >> 1;                                             \
        face_xyz<AX>((F & 1) == 0 ? N - 1 : 0, ga, gc, gx, gy, gz);            \
        V = __ldcg(A + src * g.bstride + (VC + gx) + LX * (VC + gy) + BLXY * (VC + gz)); \
      } else {                                                                 \
        V = __ldcg(a.side_in + src * NN + gq * N + gp);                        \
      }                                                                        \
    }
    BCMG_PIPE_LOAD(0, g0) BCMG_PIPE_LOAD(1, g1) BCMG_PIPE_LOAD(2, g2)
    BCMG_PIPE_LOAD(3, g3) BCMG_PIPE_LOAD(4, g4) BCMG_PIPE_LOAD(5, g5)
#undef BCMG_PIPE_LOAD
  };

  int b = blockIdx.x;
  if (b >= g.nb) return;
  copies_c(b, 0);
  // A, the side buffers and the x-face layers come from the previous launch
  // (a no-op unless this launch depends on it programmatically)
  griddep_wait();
  copies_a(b, 0);
  copies_b(b, 0, nxt);
  if (pull) gather(nxt);
  if (STAGES == 2 && b + grid < g.nb) nxt = a.info[b + grid];

  for (int n = 0; b < g.nb; n++, b += grid) {
    const int st = n & 1;
    const int bn = b + grid;
    // ---- 1. block bn's copies into the other stage --------------------------
    if (STAGES == 2 && bn < g.nb) {
      copies_c(bn, st ^ 1);
      copies_a(bn, st ^ 1);
      copies_b(bn, st ^ 1, nxt);
    }
    unsigned char* base = smraw + st * PS::STAGE;
    T* tile = reinterpret_cast<T*>(base);
    T* sv = reinterpret_cast<T*>(base + PS::S_OFF);
    const T* cf = reinterpret_cast<const T*>(base + PS::META_OFF);
    const double* dval = reinterpret_cast<const double*>(base + PS::DVAL_OFF);
    const float* dv2f = reinterpret_cast<const float*>(base + PS::V2F_OFF);
    // ---- 2. block b's copies ------------------------------------------------
    const bool ok = mbar_wait(&bar[st], (n >> 1) & 1, a.err);
    if (!__syncthreads_and(ok)) {
      // drain what is in flight (both stages), bounded, and leave together
      if (tid == 0) {
        mbar_wait(&bar[st], (n >> 1) & 1, nullptr);
        if (STAGES == 2 && bn < g.nb) mbar_wait(&bar[st ^ 1], ((n + 1) >> 1) & 1, nullptr);
      }
      if (w == 0) bulk_wait_read();
      __syncthreads();
      return;
    }
    const unsigned flags = (unsigned)*reinterpret_cast<const int*>(base + PS::FLAGS_OFF);
    const unsigned dmask = (flags >> BI_DIR_SHIFT) & 0x3fu;
    // ---- 3. ghosts of block b, from the registers ------------------------------
    if (pull) {
#define BCMG_PIPE_PUT(F, V)                                                   \
      if (flags & (BI_FED << F)) {                                            \
        int ga, gc, gx, gy, gz;                                               \
        pull_map<N, F>(gp, gq, ga, gc, gx, gy, gz);                           \
        tile[TL::at(gx, gy, gz)] = V;                                         \
      }
      BCMG_PIPE_PUT(0, g0) BCMG_PIPE_PUT(1, g1) BCMG_PIPE_PUT(2, g2)
      BCMG_PIPE_PUT(3, g3) BCMG_PIPE_PUT(4, g4) BCMG_PIPE_PUT(5, g5)
#undef BCMG_PIPE_PUT
      if (dmask) tile_dirichlet<T, N, VC, TL>(tile, dmask, dval, a.bc.bcx, tid, NT, dv2f);
      __syncthreads();
      // block bn's ghost loads: in flight during block b's sweep
      if (STAGES == 2 && bn < g.nb) gather(nxt);
    }
    if (STAGES == 2 && bn + grid < g.nb) nxt = a.info[bn + grid];
    // ---- 4. sweep ---------------------------------------------------------
    int i, j;
    sweep_column<T, N, LX>(tid, i, j);
    const T* img;     // plane k of the output image starts at img + k * ipitch
    int ipitch;
    if constexpr (OP == kOpJacobi) {
      SqAcc<T> acc;
      pipe_jacobi<T, N, VC, RES>(tile, sv, cf, a.omega, i, j, acc);
      if (RES) {
        acc.warp_reduce();
        if (lane == 0) red[w] = acc.value();
      }
      __syncthreads();
      if (RES && tid == 0) {
        double v = 0.0;
        for (int q = 0; q < NW; q++) v += red[q];
        a.partial[b] = v;
      }
      // the ghost cells of the output rows, from x0's tile: the planes leave
      // with the values A had (or had pulled) there
      if (PS::COMPACT) {
        constexpr int W = 2 * VC, PER = N * W;
        for (int e = tid; e < N * PER; e += NT) {
          const int k = e / PER, r = e - k * PER, jj = r / W, u = r - jj * W;
          const int x = u < VC ? u - VC : N + u - VC;
          sv[PS::s_at(x, jj, k)] = tile[TL::at(x, jj, k)];
        }
      } else {
        constexpr int PER = 2 * LX + 2 * N;  // rows y = -1, N; cells x = -1, N
        for (int e = tid; e < N * PER; e += NT) {
          const int k = e / PER, r = e - k * PER;
          int x, y;
          if (r < 2 * LX) { x = r % LX - 1; y = r < LX ? -1 : N; }
          else { const int r2 = r - 2 * LX; x = (r2 & 1) ? N : -1; y = r2 >> 1; }
          sv[k * PS::SP + (1 + y) * LX + 1 + x] = tile[TL::at(x, y, k)];
        }
      }
      __syncthreads();
      img = sv;
      ipitch = PS::SP;
    } else {
      SorCell<T, OP> cell;
      cell.c0 = cf[0]; cell.cx = cf[1]; cell.cy = cf[2]; cell.cz = cf[3];
      cell.om = a.omega; cell.om1 = a.om1;
      T* col = tile + TL::at(i, j, 0);
      const T* scol = PS::SPACK ? sv + tid : sv + PS::s_at(i, j, 0);
      for (int it = 0; it < a.n_inner; it++) {
#pragma unroll
        for (int c = 0; c < 2; c++) {
          const int k0 = (c + i + j) & 1;  // cells with (i + j + k) % 2 == c
          static_assert((N / 2) % 4 == 0, "colour cells in groups of four");
          for (int h = 0; h < N / 2; h += 4) {
            // four cells of the colour: every load before the first store
            // (their neighbours have the other colour, which this half-pass
            // does not write), so the loads overlap
            T sw[4], sn[4], sb[4], pc[4], sr[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const int k = k0 + 2 * (h + u);
              const T* p = col + k * TP;
              sw[u] = xadd(p[-1], p[1]);
              sn[u] = xadd(p[-LX], p[LX]);
              sb[u] = xadd(p[-TP], p[TP]);
              pc[u] = p[0];
              sr[u] = PS::HAS_S ? scol[k * PS::SP] : (T)0;
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
              col[(k0 + 2 * (h + u)) * TP] = cell(pc[u], sw[u], sn[u], sb[u], sr[u]);
          }
          __syncthreads();
        }
        if (dmask) {
          tile_dirichlet<T, N, VC, TL>(tile, dmask, dval, a.bc.bcx, tid, NT, dv2f);
          __syncthreads();
        }
      }
      img = tile + TP + (PS::OUT_Y0 + 1) * LX;
      ipitch = TP;
    }
    // ---- x-face layers of B's block b, for its same-level X neighbours -----
    {
      T* xo = a.xf_out + (int64_t)b * 2 * NN + tid;
      const T* xi = img + (gp - PS::OUT_Y0) * LX + gq * ipitch + VC;  // cell (0, gp, gq)
      if (flags & (BI_COPY << 0)) xo[0] = xi[0];
      if (flags & (BI_COPY << 1)) xo[NN] = xi[N - 1];
    }
    // ---- F2C ghosts this block feeds, into B's side buffer -----------------
    {
      const int nout = (flags >> BI_OUT_SHIFT) & 0x7f;
      const VcTask* ot = reinterpret_cast<const VcTask*>(base + PS::TASKS_OFF);
      // four groups of NT/4 threads take alternate entries, a few cells of
      // each per thread (independent cells: their loads and arithmetic
      // overlap)
      constexpr int GS = NT / 4;
      const int grp = tid / GS, gl = tid % GS;
      for (int q = grp; q < nout; q += 4) {
        const VcTask t = ot[q];
        T* slot = a.side_out + (int64_t)t.slot * NN;
        if constexpr (OP == kOpJacobi)
          side_push<T, N, VC, typename PS::Img, GS>(t, slot, g, sv, gl);
        else
          side_push<T, N, VC, TL, GS>(t, slot, g, tile, gl);
      }
    }
    // ---- 5. the output rows of planes [0,N) -> B, one bulk store per plane --
    fence_proxy_async_smem();  // the stage's writes, before the bulk engine reads
    __syncthreads();
    if (w == 0) {
      T* ob = Bf + (int64_t)b * g.bstride + (VC + PS::OUT_Y0) * LX + VC * BLXY;
      for (int k = lane; k < N; k += 32)
        bulk_s2g(ob + k * BLXY, img + k * ipitch, PS::OUT_LEN * sizeof(T));
      bulk_commit();
      if (STAGES == 1) bulk_wait_read();  // shared memory outlives the stores' reads
    }
  }
  if (STAGES == 2 && w == 0) bulk_wait_read();
}

// pdl: the launch may begin while the previous kernel in the stream (the
// previous launch of the run) finishes (programmatic dependent launch).
template <typename T, int N, int VC, int OP, bool RES, int STAGES = 2>
cudaError_t pipe_launch(const T* A, T* B, const T* S, const Geom& g, const PipeArgs<T>& a,
                        cudaStream_t st, bool pdl = false) {
  using PS = PipeStage<T, N, VC, OP>;
  constexpr size_t SMEM = STAGES * (size_t)PS::STAGE;
  if (SMEM > kPipeMaxSmem) return cudaErrorInvalidValue;
  auto kern = sweep_pipe_kernel<T, N, VC, OP, RES, STAGES>;
  // attributes and residency: once per process (not stream operations; the
  // first launch of every caller runs before any CUDA-graph capture)
  static int per_sm = 0, sms = 0;
  if (per_sm == 0) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PS::NT, SMEM);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
  }
  const int grid = STAGES == 1 ? g.nb : std::max(1, std::min(g.nb, sms * per_sm));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(PS::NT);
  cfg.dynamicSmemBytes = SMEM;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, A, B, S, g, a);
}

}  // namespace bcmg
