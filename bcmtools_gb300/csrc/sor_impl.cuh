// sor_impl.cuh -- red-black SOR sweeps (sor1/Solver.cpp:132-153,
// sor2/Solver.cpp:136-160), one CTA per block.
//
// Two variants:
//   in place  the block (interior + first ghost layer) is staged in shared
//             memory, swept n_inner times with its Dirichlet ghosts refreshed
//             between passes (setBoundaryConditionInBlock), and written back;
//             the ghost update then runs as a separate gather launch.
//   fused     ping-pong: the block is read from buffer A and its new interior
//             written to buffer B, and the CTA also writes, straight from
//             shared memory, every ghost value its interior feeds -- the
//             same-level, F2C and C2F ghosts of its neighbours in B and its own
//             Dirichlet ghosts.  B then holds the next iterate with all ghosts
//             updated: one launch per outer iteration, and no ghost source is
//             re-read from HBM.
// Both colours read the ghosts as they were when the pass began (the reference
// refreshes ghosts only between outer iterations), so results do not depend on
// the order of blocks.
//
// Arithmetic: FP64 fields follow the reference's double expression exactly.
// FP32 fields sweep in FP32 with FMA (coefficients rounded to float); the
// result agrees with the double-evaluated expression to ~1e-7 relative.
#pragma once
#include "ghost.cuh"
#include "kernels.h"
#include "tile.cuh"
#include "bulk.cuh"
#include "cells.cuh"
#include "pipe.cuh"
#include "stage.cuh"

#include <algorithm>

namespace bcmg {

constexpr int kBcDirichlet = 1;

struct SorArgs {
  const double* coef;   // [nb*4]
  const float* coef32;  // [nb*4] the same, rounded to float
  double omega;
  float omega32, om1_32;
  int n_inner;
  BlockBc bc;
  PushTable push;
  int* err;  // device error word (bounded-wait timeouts)
  int pull_now;  // pull form: fill A's ghosts from its neighbours first
  bool s_packed;  // pull form, sor2: the source is packed N^3 per block
};

// Pull-form launcher for one block edge N (8 or 16; instantiated per dtype
// and N in the tile translation units).
template <typename T, int N>
cudaError_t launch_sor_pull(const T* A, T* B, const T* s, const Geom& g, const SorArgs& a,
                            int stages, cudaStream_t st);

// Tile-kernel launcher for one block edge N (instantiated per dtype and N in
// its own translation unit).
template <typename T, int N>
cudaError_t launch_sor_tile(const T* A, T* B, const T* s, const Geom& g, const SorArgs& a,
                            bool push, int variant, cudaStream_t st);

// SMEM: stage (n+2)^3 in shared memory; otherwise sweep in place in global
// memory (bricks too large for shared memory).  PUSH requires SMEM.
template <typename T, int FORM, bool SMEM, bool PUSH>
__global__ void __launch_bounds__(512) sor_kernel(const T* A, T* Bf,
                                                  const T* __restrict__ s, Geom g, SorArgs a) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int b = blockIdx.x;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const T* ab = A + (int64_t)b * g.bstride;  // A == Bf when sweeping in place
  T* fb = Bf + (int64_t)b * g.bstride;
  const T* __restrict__ sbk = (FORM == 2) ? s + (int64_t)b * g.bstride : nullptr;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int lx = nx + 2, ly = ny + 2, lz = nz + 2;
  T* base;
  int sy, sz, o;
  if (SMEM) {
    base = reinterpret_cast<T*>(smraw);
    sy = lx; sz = lx * ly; o = 1 + lx + lx * ly;
    for (int row = warp; row < ly * lz; row += nw) {
      const int jj = row % ly, kk = row / ly;
      if ((jj == 0 || jj == ly - 1) && (kk == 0 || kk == lz - 1)) continue;  // edges unused
      const T* src = ab + g.at(-1, jj - 1, kk - 1);
      T* d = base + row * lx;
      for (int i = lane; i < lx; i += 32) d[i] = src[i];
    }
    __syncthreads();
  } else {
    base = fb; sy = g.sy; sz = g.sz; o = g.off0;
  }
  SorCell<T, FORM> cell;
  cell.init(a, b);

  bool dir[6];
  double dv[6];
  bool anyd = false;
  for (int fc = 0; fc < 6; fc++) {
    dir[fc] = a.bc.type && a.bc.type[b * 6 + fc] == kBcDirichlet;
    double v = dir[fc] ? a.bc.value[b * 6 + fc] : 0.0;
    if (a.bc.bcx) v = (double)(T)v;
    dv[fc] = v;
    anyd |= dir[fc];
  }

  // Fixed per-thread (i2, j, k0) when a whole number of k-slices fits the CTA.
  const int hx = nx / 2, slice = hx * ny;
  const bool regular = (nt % slice) == 0;
  const int kstep = regular ? nt / slice : 0;
  const int ti2 = tid % hx, tj = (tid / hx) % ny, tk0 = tid / slice;

  for (int it = 0; it < a.n_inner; it++) {
    for (int c = 0; c < 2; c++) {
      if (regular) {
        for (int k = tk0; k < nz; k += kstep) {
          const int i = 2 * ti2 + ((c + tj + k) & 1);
          const int p = o + i + sy * tj + sz * k;
          const T sw = xadd(base[p - 1], base[p + 1]);
          const T ss = xadd(base[p - sy], base[p + sy]);
          const T sbt = xadd(base[p - sz], base[p + sz]);
          const T src = (FORM == 2) ? sbk[g.at(i, tj, k)] : (T)0;
          base[p] = cell(base[p], sw, ss, sbt, src);
        }
      } else {
        for (int t = tid; t < slice * nz; t += nt) {
          const int k = t / slice, r = t - k * slice, j = r / hx;
          const int i = 2 * (r - j * hx) + ((c + j + k) & 1);
          const int p = o + i + sy * j + sz * k;
          const T sw = xadd(base[p - 1], base[p + 1]);
          const T ss = xadd(base[p - sy], base[p + sy]);
          const T sbt = xadd(base[p - sz], base[p + sz]);
          const T src = (FORM == 2) ? sbk[g.at(i, j, k)] : (T)0;
          base[p] = cell(base[p], sw, ss, sbt, src);
        }
      }
      __syncthreads();
    }
    if (anyd) {
      // setBoundaryConditionInBlock: first ghost layer g = 2v - f.
      for (int fc = 0; fc < 6; fc++) {
        if (!dir[fc]) continue;
        const int ax = fc >> 1, minus = (fc & 1) == 0;
        const int n0 = ax == 0 ? ny : nx, n1 = ax == 2 ? ny : nz;
        const int nn = ax == 0 ? nx : ax == 1 ? ny : nz;
        const double v2 = xmul(2.0, dv[fc]);
        for (int e = tid; e < n0 * n1; e += nt) {
          int bq, q;
          divmod(e, n0, bq, q);
          int gi[3], ii[3];
          if (ax == 0) { gi[1] = ii[1] = q; gi[2] = ii[2] = bq; }
          else if (ax == 1) { gi[0] = ii[0] = q; gi[2] = ii[2] = bq; }
          else { gi[0] = ii[0] = q; gi[1] = ii[1] = bq; }
          gi[ax] = minus ? -1 : nn;
          ii[ax] = minus ? 0 : nn - 1;
          const T fin = base[o + ii[0] + sy * ii[1] + sz * ii[2]];
          base[o + gi[0] + sy * gi[1] + sz * gi[2]] = to_t<T>(xsub(v2, (double)fin));
        }
      }
      __syncthreads();
    }
  }

  if (SMEM) {
    // interior rows
    for (int row = warp; row < ny * nz; row += nw) {
      const int j = row % ny, k = row / ny;
      const T* sr = base + o + sy * j + sz * k;
      T* d = fb + g.at(0, j, k);
      for (int i = lane; i < nx; i += 32) d[i] = sr[i];
    }
    // Dirichlet ghost faces (first layer)
    if (anyd && a.n_inner > 0) {
      for (int fc = 0; fc < 6; fc++) {
        if (!dir[fc]) continue;
        const int ax = fc >> 1, minus = (fc & 1) == 0;
        const int n0 = ax == 0 ? ny : nx, n1 = ax == 2 ? ny : nz;
        const int nn = ax == 0 ? nx : ax == 1 ? ny : nz;
        for (int e = tid; e < n0 * n1; e += nt) {
          int bq, q;
          divmod(e, n0, bq, q);
          int gi[3];
          if (ax == 0) { gi[1] = q; gi[2] = bq; }
          else if (ax == 1) { gi[0] = q; gi[2] = bq; }
          else { gi[0] = q; gi[1] = bq; }
          gi[ax] = minus ? -1 : nn;
          fb[g.at(gi[0], gi[1], gi[2])] = base[o + gi[0] + sy * gi[1] + sz * gi[2]];
        }
      }
    }
  }
  if (anyd && a.bc.bcx && g.vc >= 2 && a.n_inner > 0) {
    // bcx.f90: second ghost layer = v.
    for (int fc = 0; fc < 6; fc++) {
      if (!dir[fc]) continue;
      const int ax = fc >> 1, minus = (fc & 1) == 0;
      const int n0 = ax == 0 ? ny : nx, n1 = ax == 2 ? ny : nz;
      const int nn = ax == 0 ? nx : ax == 1 ? ny : nz;
      for (int e = tid; e < n0 * n1; e += nt) {
        int bq, q;
        divmod(e, n0, bq, q);
        int gi[3];
        if (ax == 0) { gi[1] = q; gi[2] = bq; }
        else if (ax == 1) { gi[0] = q; gi[2] = bq; }
        else { gi[0] = q; gi[1] = bq; }
        gi[ax] = minus ? -2 : nn + 1;
        fb[g.at(gi[0], gi[1], gi[2])] = (T)dv[fc];
      }
    }
  }
  if (PUSH) {
    // Ghost values this block's interior feeds, straight from shared memory.
    const Acc<T> src{base, sy, sz, o};
    const int p0 = a.push.ptr[b], p1 = a.push.ptr[b + 1];
    for (int q = p0 + warp; q < p1; q += nw) {
      const VcTask t = a.push.tasks[q];
      task_apply<T>(t, Bf + (int64_t)t.dst * g.bstride, g, src, 0.0, lane, 32);
    }
  }
}

// ---- tile kernels for cubic blocks N = 8, 16, 32 and ghost width VC = 1, 2 --
// Compile-time tile strides, Dirichlet faces as a bit mask, ghost pushes
// specialised per (kind, axis); NT threads per CTA.

// n_inner red-black passes over the tile (+ block Dirichlet between passes);
// src(i,j,k) gives the source term (FORM 2).
template <typename T, int N, int VC, int FORM, int NT, class SrcFn>
__device__ __forceinline__ void sweep_tile(T* sf, const SrcFn& src, const SorCell<T, FORM>& cell,
                                           unsigned dmask, const double* dval, const SorArgs& a,
                                           int tid) {
  using TL = Tile<T, N, VC>;
  constexpr int N3 = N * N * N, H = N / 2;
  for (int it = 0; it < a.n_inner; it++) {
#pragma unroll
    for (int c = 0; c < 2; c++) {
#pragma unroll 4
      for (int t = tid; t < N3 / 2; t += NT) {
        const int i2 = t % H, r = t / H, j = r % N, k = r / N;
        const int i = 2 * i2 + ((c + j + k) & 1);
        const int p = TL::at(i, j, k);
        const T sw = xadd(sf[p - 1], sf[p + 1]);
        const T sn = xadd(sf[p - TL::LX], sf[p + TL::LX]);
        const T sbt = xadd(sf[p - TL::LXY], sf[p + TL::LXY]);
        sf[p] = cell(sf[p], sw, sn, sbt, FORM == 2 ? src(i, j, k) : (T)0);
      }
      __syncthreads();
    }
    if (dmask) {
      tile_dirichlet<T, N, VC>(sf, dmask, dval, a.bc.bcx, tid, NT);
      __syncthreads();
    }
  }
}

// Interior and Dirichlet ghosts of block b into its brick fb; with PUSH, every
// ghost value this block feeds, into the neighbours' bricks of Bf.
template <typename T, int N, int VC, bool PUSH, int NT>
__device__ __forceinline__ void emit_block(const T* sf, T* fb, T* Bf, const Geom& g,
                                           unsigned dmask, const double* dval,
                                           const SorArgs& a, int b, int tid) {
  store_interior<T, N, VC>(sf, fb, g, tid, NT);
  if (dmask && a.n_inner > 0) store_dirichlet<T, N, VC>(sf, fb, g, dmask, dval, a.bc.bcx, tid, NT);
  if (PUSH) {
    const int lane = tid & 31, warp = tid >> 5;
    const int p0 = a.push.ptr[b], p1 = a.push.ptr[b + 1];
    for (int q = p0 + warp; q < p1; q += NT / 32) {
      const VcTask t = a.push.tasks[q];
      push_dispatch<T, N, VC>(t, Bf + (int64_t)t.dst * g.bstride, g, sf, lane);
    }
  }
}

__device__ __forceinline__ unsigned dirichlet_mask(const SorArgs& a, int b) {
  unsigned m = 0;
  if (a.bc.type) {
#pragma unroll
    for (int fc = 0; fc < 6; fc++)
      if (a.bc.type[b * 6 + fc] == kBcDirichlet) m |= 1u << fc;
  }
  return m;
}

// One CTA per block: staging with vector loads, then sweep and emit.
template <typename T, int N, int VC, int FORM, bool SS, bool PUSH, int NT>
__global__ void __launch_bounds__(NT) sor_tile_kernel(const T* A, T* Bf, const T* __restrict__ S,
                                                      Geom g, SorArgs a) {
  using TL = Tile<T, N, VC>;
  constexpr int SOFF = (TL::SIZE * (int)sizeof(T) + 15) / 16 * 16 / (int)sizeof(T);
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sf = reinterpret_cast<T*>(smraw);
  T* ss = sf + SOFF;  // source rows j,k in [0,N), full pitch LX
  const int b = blockIdx.x, tid = threadIdx.x;
  const T* ab = A + (int64_t)b * g.bstride;  // A == Bf when sweeping in place
  T* fb = Bf + (int64_t)b * g.bstride;
  const T* sb = (FORM == 2) ? S + (int64_t)b * g.bstride : nullptr;
  stage_rows<T, TL::LX, TL::VEC_BYTES>(sf, ab, TL::LX, TL::LX * TL::LX, VC - 1, N + 2, VC - 1,
                                       N + 2, tid, NT);
  if (FORM == 2 && SS)
    stage_rows<T, TL::LX, TL::VEC_BYTES>(ss, sb, TL::LX, TL::LX * TL::LX, VC, N, VC, N, tid, NT);
  const unsigned dmask = dirichlet_mask(a, b);
  const double* dval = a.bc.value + b * 6;
  SorCell<T, FORM> cell;
  cell.init(a, b);
  __syncthreads();
  auto src = [&](int i, int j, int k) -> T {
    return SS ? ss[VC + i + TL::LX * (j + N * k)] : sb[g.at(i, j, k)];
  };
  sweep_tile<T, N, VC, FORM, NT>(sf, src, cell, dmask, dval, a, tid);
  emit_block<T, N, VC, PUSH, NT>(sf, fb, Bf, g, dmask, dval, a, b, tid);
}

template <typename T, int N>
cudaError_t launch_sor_pull(const T* A, T* B, const T* s, const Geom& g, const SorArgs& a,
                            int stages, cudaStream_t st) {
  PipeArgs<T> p{};
  if constexpr (sizeof(T) == 4) {
    p.coef = a.coef32;
    p.omega = a.omega32;
    p.om1 = a.om1_32;
  } else {
    p.coef = a.coef;
    p.omega = a.omega;
    p.om1 = 1.0 - a.omega;
  }
  p.n_inner = a.n_inner;
  p.bc = a.bc;
  p.info = a.push.info;
  p.out_tasks = a.push.out_tasks;
  p.side_in = static_cast<const T*>(a.push.side_in);
  p.side_out = static_cast<T*>(a.push.side_out);
  p.xf_in = static_cast<const T*>(a.push.xf_in);
  p.xf_out = static_cast<T*>(a.push.xf_out);
  p.pull_now = a.pull_now;
  p.partial = nullptr;
  p.err = a.err;
  const bool pk = a.s_packed;
  // every launch but a run's first follows the run's previous launch
  const bool pdl = a.pull_now != 0;
  if (stages == 1) {
    if (g.vc == 1)
      return !s ? pipe_launch<T, N, 1, kOpSor1, false, 1>(A, B, s, g, p, st, pdl)
             : pk ? pipe_launch<T, N, 1, kOpSor2P, false, 1>(A, B, s, g, p, st, pdl)
                  : pipe_launch<T, N, 1, kOpSor2, false, 1>(A, B, s, g, p, st, pdl);
    return !s ? pipe_launch<T, N, 2, kOpSor1, false, 1>(A, B, s, g, p, st, pdl)
           : pk ? pipe_launch<T, N, 2, kOpSor2P, false, 1>(A, B, s, g, p, st, pdl)
                : pipe_launch<T, N, 2, kOpSor2, false, 1>(A, B, s, g, p, st, pdl);
  }
  if (g.vc == 1)
    return !s ? pipe_launch<T, N, 1, kOpSor1, false>(A, B, s, g, p, st, pdl)
           : pk ? pipe_launch<T, N, 1, kOpSor2P, false>(A, B, s, g, p, st, pdl)
                : pipe_launch<T, N, 1, kOpSor2, false>(A, B, s, g, p, st, pdl);
  return !s ? pipe_launch<T, N, 2, kOpSor1, false>(A, B, s, g, p, st, pdl)
         : pk ? pipe_launch<T, N, 2, kOpSor2P, false>(A, B, s, g, p, st, pdl)
              : pipe_launch<T, N, 2, kOpSor2, false>(A, B, s, g, p, st, pdl);
}

template <typename T>
cudaError_t launch_pack_source(T* dst, const T* src, const Geom& g, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  if (g.nx != g.ny || g.ny != g.nz || (g.nx != 8 && g.nx != 16) || (g.vc != 1 && g.vc != 2))
    return cudaErrorInvalidValue;
  const int nt = g.nx * g.nx;
  if (g.nx == 16) {
    if (g.vc == 1) pack_source_kernel<T, 16, 1><<<g.nb, nt, 0, st>>>(dst, src, g);
    else pack_source_kernel<T, 16, 2><<<g.nb, nt, 0, st>>>(dst, src, g);
  } else {
    if (g.vc == 1) pack_source_kernel<T, 8, 1><<<g.nb, nt, 0, st>>>(dst, src, g);
    else pack_source_kernel<T, 8, 2><<<g.nb, nt, 0, st>>>(dst, src, g);
  }
  return cudaGetLastError();
}

// Bulk-copy layout of one pipeline stage: the field tile and the source tile.
template <typename T, int N, int VC>
struct PipeLayout {
  using TL = Tile<T, N, VC>;
  static constexpr int LX = TL::LX;
  static constexpr int F_BYTES = TL::SIZE * (int)sizeof(T);
  // source: VC = 1 keeps whole planes (rows 16-B aligned only as a plane),
  // VC = 2 the interior rows of each interior plane
  static constexpr int S_ELEMS = VC == 1 ? LX * LX * N : LX * N * N;
  static constexpr int S_BYTES = S_ELEMS * (int)sizeof(T);
  static constexpr int S_OFF = (F_BYTES + 127) / 128 * 128;
  static constexpr int STAGE = (S_OFF + S_BYTES + 127) / 128 * 128;
  static __device__ __forceinline__ int s_at(int i, int j, int k) {
    return VC == 1 ? (i + 1) + LX * (j + 1) + LX * LX * k : (i + VC) + LX * j + LX * N * k;
  }
};

// Persistent, double-buffered: while a CTA sweeps one block, the bulk-copy
// engine fills the other stage with the next block's field and source tiles.
template <typename T, int N, int VC, int FORM>
__global__ void __launch_bounds__(256) sor_pipe_kernel(const T* A, T* Bf, const T* __restrict__ S,
                                                       Geom g, SorArgs a) {
  using PL = PipeLayout<T, N, VC>;
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ uint64_t bar[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();

  // Warp 0 fills stage st with block blk.
  auto issue = [&](int blk, int st) {
    unsigned char* base = smraw + st * PL::STAGE;
    const T* fsrc = A + (int64_t)blk * g.bstride;
    const T* ssrc = FORM == 2 ? S + (int64_t)blk * g.bstride : nullptr;
    const unsigned tx = PL::F_BYTES + (FORM == 2 ? PL::S_BYTES : 0);
    if (lane == 0) mbar_expect_tx(&bar[st], tx);
    __syncwarp();
    if (VC == 1) {
      if (lane == 0) bulk_g2s(base, fsrc, PL::F_BYTES, &bar[st]);
      if (FORM == 2 && lane == 1)
        bulk_g2s(base + PL::S_OFF, ssrc + PL::LX * PL::LX, PL::S_BYTES, &bar[st]);
    } else {
      constexpr int FB = (N + 2) * PL::LX * (int)sizeof(T);
      for (int q = lane; q < N + 2; q += 32)
        bulk_g2s(base + q * FB, fsrc + (q + VC - 1) * PL::LX * PL::LX + (VC - 1) * PL::LX, FB,
                 &bar[st]);
      if (FORM == 2) {
        constexpr int SB = N * PL::LX * (int)sizeof(T);
        for (int q = lane; q < N; q += 32)
          bulk_g2s(base + PL::S_OFF + q * SB, ssrc + (q + VC) * PL::LX * PL::LX + VC * PL::LX, SB,
                   &bar[st]);
      }
    }
  };

  int it = 0;
  if (warp == 0 && (int)blockIdx.x < g.nb) issue(blockIdx.x, 0);
  for (int b = blockIdx.x; b < g.nb; b += gridDim.x, it++) {
    const int st = it & 1;
    const int bn = b + gridDim.x;
    if (warp == 0 && bn < g.nb) issue(bn, st ^ 1);
    const bool ok = mbar_wait(&bar[st], (it >> 1) & 1, a.err);
    if (!__syncthreads_and(ok)) {  // uniform decision: every thread leaves together
      if (bn < g.nb) mbar_wait(&bar[st ^ 1], ((it + 1) >> 1) & 1, nullptr);  // drain, bounded
      return;
    }
    T* sf = reinterpret_cast<T*>(smraw + st * PL::STAGE);
    const T* ss = reinterpret_cast<const T*>(smraw + st * PL::STAGE + PL::S_OFF);
    const unsigned dmask = dirichlet_mask(a, b);
    const double* dval = a.bc.value + b * 6;
    SorCell<T, FORM> cell;
    cell.init(a, b);
    auto src = [&](int i, int j, int k) -> T { return ss[PL::s_at(i, j, k)]; };
    sweep_tile<T, N, VC, FORM, 256>(sf, src, cell, dmask, dval, a, tid);
    emit_block<T, N, VC, true, 256>(sf, Bf + (int64_t)b * g.bstride, Bf, g, dmask, dval, a, b, tid);
    fence_proxy_async_smem();  // this stage is refilled by the bulk engine next
    __syncthreads();
  }
}

template <typename T, int N, int VC>
static bool pipe_ok() {
  return 2 * (size_t)PipeLayout<T, N, VC>::STAGE <= kSorMaxSmem;
}

template <typename T, int N, int VC, int FORM>
static cudaError_t pipe_launch(const T* A, T* B, const T* s, const Geom& g, const SorArgs& a,
                               cudaStream_t st) {
  using PL = PipeLayout<T, N, VC>;
  const size_t smem = 2 * (size_t)PL::STAGE;
  auto kern = sor_pipe_kernel<T, N, VC, FORM>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem);
  const int grid = std::max(1, std::min(g.nb, sms * std::max(per_sm, 1)));
  kern<<<grid, 256, smem, st>>>(A, B, s, g, a);
  return cudaGetLastError();
}

template <typename T, int N, int VC, int FORM, bool SS, bool PUSH, int NT>
static cudaError_t tile_launch(const T* A, T* B, const T* s, const Geom& g, const SorArgs& a,
                               cudaStream_t st) {
  using TL = Tile<T, N, VC>;
  const size_t f_bytes = (size_t)(TL::SIZE * sizeof(T) + 15) / 16 * 16;
  const size_t smem = f_bytes + (SS && FORM == 2 ? (size_t)TL::LX * N * N * sizeof(T) : 0);
  if (smem > kSorMaxSmem) return cudaErrorInvalidValue;
  auto kern = sor_tile_kernel<T, N, VC, FORM, SS, PUSH, NT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<g.nb, NT, smem, st>>>(A, B, s, g, a);
  return cudaGetLastError();
}

// Variant dispatch for one (N, VC, FORM).  In-place sweeps (no push) always
// use the staged-source 256-thread tile.
template <typename T, int N, int VC, int FORM>
static cudaError_t tile_variant(const T* A, T* B, const T* s, const Geom& g, const SorArgs& a,
                                bool push, int v, cudaStream_t st) {
  using TL = Tile<T, N, VC>;
  const bool ss_fits = (size_t)(TL::SIZE + TL::LX * N * N) * sizeof(T) + 16 <= kSorMaxSmem;
  if (!push) {
    if (ss_fits) return tile_launch<T, N, VC, FORM, true, false, 256>(A, B, s, g, a, st);
    return tile_launch<T, N, VC, FORM, false, false, 256>(A, B, s, g, a, st);
  }
  if (v == SV_PIPE_256 && pipe_ok<T, N, VC>()) return pipe_launch<T, N, VC, FORM>(A, B, s, g, a, st);
  const bool big = N * N * N / 2 >= 512;  // 512 threads only when every thread has cells
  if (v == SV_TILE_GS_256 || !ss_fits) return tile_launch<T, N, VC, FORM, false, true, 256>(A, B, s, g, a, st);
  if (big && v == SV_TILE_SS_512) return tile_launch<T, N, VC, FORM, true, true, 512>(A, B, s, g, a, st);
  if (big && v == SV_TILE_GS_512) return tile_launch<T, N, VC, FORM, false, true, 512>(A, B, s, g, a, st);
  return tile_launch<T, N, VC, FORM, true, true, 256>(A, B, s, g, a, st);
}

template <typename T, int N>
cudaError_t launch_sor_tile(const T* A, T* B, const T* s, const Geom& g, const SorArgs& a,
                            bool push, int variant, cudaStream_t st) {
  const bool form2 = s != nullptr;
  if (g.vc == 1)
    return form2 ? tile_variant<T, N, 1, 2>(A, B, s, g, a, push, variant, st)
                 : tile_variant<T, N, 1, 1>(A, B, s, g, a, push, variant, st);
  return form2 ? tile_variant<T, N, 2, 2>(A, B, s, g, a, push, variant, st)
               : tile_variant<T, N, 2, 1>(A, B, s, g, a, push, variant, st);
}

// Whether a tile kernel covers this geometry.
template <typename T>
static bool tile_ok(const Geom& g) {
  if (g.nx != g.ny || g.ny != g.nz || (g.vc != 1 && g.vc != 2)) return false;
  if (g.nx != 8 && g.nx != 16 && g.nx != 32) return false;
  const size_t f = (size_t)(g.nx + 2 * g.vc) * (g.nx + 2) * (g.nx + 2) * sizeof(T);
  return f <= kSorMaxSmem;
}

static int sor_threads(const Geom& g) {
  const int slice = (g.nx / 2) * g.ny;
  if (slice <= 256) return 256;
  return slice <= 512 ? 512 : 256;
}

// Generic shapes: the SMEM / in-place sor_kernel.
template <typename T, int FORM>
static cudaError_t generic_dispatch(const T* A, T* B, const T* s, const Geom& g, const SorArgs& a,
                                    bool push, cudaStream_t st) {
  const size_t tile = (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2) * sizeof(T);
  const int threads = sor_threads(g);
  if (tile <= kSorMaxSmem) {
    if (push) {
      auto k = sor_kernel<T, FORM, true, true>;
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile);
      if (e != cudaSuccess) return e;
      k<<<g.nb, threads, tile, st>>>(A, B, s, g, a);
    } else {
      auto k = sor_kernel<T, FORM, true, false>;
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile);
      if (e != cudaSuccess) return e;
      k<<<g.nb, threads, tile, st>>>(A, B, s, g, a);
    }
  } else {
    if (push) return cudaErrorInvalidValue;
    sor_kernel<T, FORM, false, false><<<g.nb, threads, 0, st>>>(A, B, s, g, a);
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_sor_impl(const T* A, T* B, const T* s, const Geom& g, const double* coef,
                            double omega, int form, int n_inner, BlockBc bc, PushTable push,
                            bool fused, int* err, int variant, int pull_now, cudaStream_t st,
                            bool s_packed = false) {
  if (g.nb == 0) return cudaSuccess;
  SorArgs a{coef, reinterpret_cast<const float*>(coef + 4 * (int64_t)g.nb), omega,
            (float)omega, (float)(1.0 - omega), n_inner, bc, push, err, pull_now,
            s_packed && form == 2};
  if (a.s_packed && !(fused && (variant == SV_PULL || variant == SV_PULL_TILE)))
    return cudaErrorInvalidValue;  // only the pull-form kernels read a packed source
  if (fused && (variant == SV_PULL || variant == SV_PULL_TILE)) {
    if (!sor_pull_ok((int)sizeof(T), g.nx, g.vc, form) || g.nx != g.ny || g.ny != g.nz)
      return cudaErrorInvalidValue;
    const T* sp = form == 2 ? s : nullptr;
    const int stages = variant == SV_PULL ? 2 : 1;
    return g.nx == 16 ? launch_sor_pull<T, 16>(A, B, sp, g, a, stages, st)
                      : launch_sor_pull<T, 8>(A, B, sp, g, a, stages, st);
  }
  if (variant == SV_PULL || variant == SV_PULL_TILE) variant = SV_AUTO;
  if (tile_ok<T>(g)) {
    const T* sp = form == 2 ? s : nullptr;
    if (g.nx == 16) return launch_sor_tile<T, 16>(A, B, sp, g, a, fused, variant, st);
    if (g.nx == 8) return launch_sor_tile<T, 8>(A, B, sp, g, a, fused, variant, st);
    return launch_sor_tile<T, 32>(A, B, sp, g, a, fused, variant, st);
  }
  if (form == 1) return generic_dispatch<T, 1>(A, B, s, g, a, fused, st);
  return generic_dispatch<T, 2>(A, B, s, g, a, fused, st);
}

}  // namespace bcmg
