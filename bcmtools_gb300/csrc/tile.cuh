// tile.cuh -- shared-memory tile of one block and the ghost values its
// interior feeds, specialised on the block edge N and the ghost width VC so
// that all tile arithmetic is compile-time.
//
// The tile keeps whole brick rows in x (x in [-VC, N+VC)) for rows y, z in
// [-1, N]: the interior plus the first ghost layer that a 7-point sweep
// reads.  Whole rows make every staged row start at a multiple of the row
// pitch, so the copy from HBM runs in 16-byte vectors when the pitch allows.
#pragma once
#include "ghost.cuh"
#include "kernels.h"

namespace bcmg {

template <typename T, int N, int VC>
struct Tile {
  static constexpr int LX = N + 2 * VC;  // = brick row pitch
  static constexpr int LY = N + 2;
  static constexpr int LZ = N + 2;
  static constexpr int LXY = LX * LY;
  static constexpr int SIZE = LXY * LZ;
  static constexpr int O = VC + LX + LXY;  // tile index of (0,0,0)
  // vector width of a row copy: widest of 16 B whose lane count divides LX
  static constexpr int VEC_BYTES = (LX * sizeof(T)) % 16 == 0 ? 16
                                   : (LX * sizeof(T)) % 8 == 0 ? 8 : (int)sizeof(T);
  static constexpr int VEC = VEC_BYTES / sizeof(T);
  static __device__ __forceinline__ int at(int i, int j, int k) { return O + i + LX * j + LXY * k; }
};

// Shared-memory copy of a whole brick in the brick's own layout
// (Scalar3D's Index3DS: x fastest, row pitch N+2VC, plane pitch (N+2VC)^2).
template <typename T, int N, int VC>
struct BrickTile {
  static constexpr int LX = N + 2 * VC;
  static constexpr int LXY = LX * LX;
  static constexpr int SIZE = LXY * LX;
  static constexpr int O = VC * (1 + LX + LXY);  // index of (0,0,0)
  static __device__ __forceinline__ int at(int i, int j, int k) { return O + i + LX * j + LXY * k; }
};

template <int BYTES>
struct VecOf;
template <>
struct VecOf<16> { using type = float4; };
template <>
struct VecOf<8> { using type = float2; };
template <>
struct VecOf<4> { using type = float; };

// Copies rows y, z in [y0, y0+ny) x [z0, z0+nz) (padded brick indices) of a
// brick into a row-major shared array of the same row pitch, in vectors.
template <typename T, int LX, int VB>
__device__ __forceinline__ void stage_rows(T* __restrict__ dst, const T* __restrict__ brick,
                                           int sy, int sz, int y0, int ny, int z0, int nz,
                                           int tid, int nt) {
  using V = typename VecOf<VB>::type;
  constexpr int NV = LX * (int)sizeof(T) / VB;  // vectors per row
  const int total = NV * ny * nz;
  for (int e = tid; e < total; e += nt) {
    const int v = e % NV, row = e / NV;
    const int y = row % ny, z = row / ny;
    const V* src = reinterpret_cast<const V*>(brick + (y0 + y) * sy + (z0 + z) * sz);
    V* d = reinterpret_cast<V*>(dst + row * LX);
    d[v] = src[v];
  }
}

// Coordinates (normal, t0, t1) on face axis AX to (x, y, z); the in-plane
// order follows the reference's subface numbering: X faces (y,z), Y faces
// (z,x), Z faces (x,y) (Scalar3DUpdater.h:527-584).
template <int AX>
__device__ __forceinline__ void face_xyz(int nrm, int t0, int t1, int& x, int& y, int& z) {
  if (AX == 0) { x = nrm; y = t0; z = t1; }
  else if (AX == 1) { y = nrm; z = t0; x = t1; }
  else { z = nrm; x = t0; y = t1; }
}

// Writes the ghost cells of entry t (destination brick `dst` in global
// memory) from the source block's tile `sf` (layout TL: the interior of the
// source block is all it reads -- a tile in shared memory, or with BrickTile
// the source brick itself); the lanes of one warp split the cells, walking x
// fastest where x lies in the face.  FIRST: the first ghost layer only.
// SIDE: `dst` is the face's N*N slot of a side buffer instead, cell (p, q) at
// q*N + p with (p, q) = (y, z), (x, z), (x, y) for X, Y, Z faces.  STRIDE
// workers split the cells (a warp, or with lane = thread a whole CTA).
template <typename T, int N, int VC, int KIND, int AX, class TL = Tile<T, N, VC>,
          bool FIRST = false, bool SIDE = false, int STRIDE = 32, int UB = 8>
__device__ __forceinline__ void push_entry(const VcTask& t, T* __restrict__ dst, const Geom& g,
                                           const T* __restrict__ sf, int lane) {
  constexpr int TN = KIND == VC_F2C ? N / 2 : N;
  constexpr int NL = FIRST ? 1 : VC;  // ghost layers written
  constexpr int CNT = NL * TN * TN;
  // cells per worker and per batch (at most UB): every read of a batch is
  // issued before its first write (ghost cells are never sources), so the
  // reads overlap
  constexpr int PER = (CNT + STRIDE - 1) / STRIDE;
  constexpr int U = PER < UB ? PER : UB;
  const bool minus = (t.face & 1) == 0;
  const int o0 = t.subface & 1, o1 = (t.subface >> 1) & 1;
  for (int e0 = lane; e0 < CNT; e0 += U * STRIDE) {
    T vals[U];
    int at[U];
#pragma unroll
    for (int q = 0; q < U; q++) {
      const int e = e0 + q * STRIDE;
      at[q] = -1;
      if (e >= CNT) continue;
      int u, a, c;  // normal index in [0,VC), first and second in-plane index
      if (AX == 2) {
        a = e % TN; c = (e / TN) % TN; u = e / (TN * TN);
      } else if (AX == 0) {
        a = e % TN; u = (e / TN) % NL; c = e / (TN * NL);
      } else {
        c = e % TN; u = (e / TN) % NL; a = e / (TN * NL);
      }
      if (FIRST) u = minus ? VC - 1 : 0;
      const int dn = minus ? u - VC : N + u;
      int x, y, z;
      T v;
      if (KIND == VC_COPY) {
        face_xyz<AX>(dn, a, c, x, y, z);
        int sx, sy_, sz_;
        face_xyz<AX>(minus ? N - VC + u : u, a, c, sx, sy_, sz_);
        v = sf[TL::at(sx, sy_, sz_)];
      } else if (KIND == VC_F2C) {
        face_xyz<AX>(dn, a + (N / 2) * o0, c + (N / 2) * o1, x, y, z);
        int fx, fy, fz;
        face_xyz<AX>(2 * (minus ? N / 2 - VC + u : u), 2 * a, 2 * c, fx, fy, fz);
        v = f2c_value<T>(sf + TL::at(fx, fy, fz), TL::LX, TL::LXY);
      } else {
        face_xyz<AX>(dn, a, c, x, y, z);
        int fx, fy, fz;  // fine indices in the coarse block's fine index space
        face_xyz<AX>(minus ? 2 * N - VC + u : u, a + N * o0, c + N * o1, fx, fy, fz);
        const int I = lin_I(fx, N), J = lin_I(fy, N), K = lin_I(fz, N);
        v = (T)C2F<T>::value(sf + TL::at(I, J, K), TL::LX, TL::LXY, lin_r(fx, I), lin_r(fy, J),
                             lin_r(fz, K));
      }
      vals[q] = v;
      at[q] = SIDE ? (AX == 2 ? y : z) * N + (AX == 0 ? y : x) : g.at(x, y, z);
    }
#pragma unroll
    for (int q = 0; q < U; q++)
      if (at[q] >= 0) dst[at[q]] = vals[q];
  }
}

// push_dispatch with the cells of one entry split over a whole CTA of NT
// threads (lane = the thread index): a block's few level-change entries then
// take all its warps instead of one each.
template <typename T, int N, int VC, class TL, int NT, int UB = 4>
__device__ __forceinline__ void push_dispatch_cta(const VcTask& t, T* dst, const Geom& g,
                                                  const T* sf, int tid) {
  const int key = t.kind * 3 + (t.face >> 1);
  switch (key) {
    case VC_COPY * 3 + 0: push_entry<T, N, VC, VC_COPY, 0, TL, false, false, NT, UB>(t, dst, g, sf, tid); break;
    case VC_COPY * 3 + 1: push_entry<T, N, VC, VC_COPY, 1, TL, false, false, NT, UB>(t, dst, g, sf, tid); break;
    case VC_COPY * 3 + 2: push_entry<T, N, VC, VC_COPY, 2, TL, false, false, NT, UB>(t, dst, g, sf, tid); break;
    case VC_F2C * 3 + 0: push_entry<T, N, VC, VC_F2C, 0, TL, false, false, NT, UB>(t, dst, g, sf, tid); break;
    case VC_F2C * 3 + 1: push_entry<T, N, VC, VC_F2C, 1, TL, false, false, NT, UB>(t, dst, g, sf, tid); break;
    case VC_F2C * 3 + 2: push_entry<T, N, VC, VC_F2C, 2, TL, false, false, NT, UB>(t, dst, g, sf, tid); break;
    case VC_C2F * 3 + 0: push_entry<T, N, VC, VC_C2F, 0, TL, false, false, NT, UB>(t, dst, g, sf, tid); break;
    case VC_C2F * 3 + 1: push_entry<T, N, VC, VC_C2F, 1, TL, false, false, NT, UB>(t, dst, g, sf, tid); break;
    case VC_C2F * 3 + 2: push_entry<T, N, VC, VC_C2F, 2, TL, false, false, NT, UB>(t, dst, g, sf, tid); break;
    default: break;
  }
}

// C2F entry of a double field in two stages (blocks of up to 16^3 cells).
// The reference's expression (C2F<double>::value) starts with the x-step
// pairs a(J', K') = (1 - r) c(I, J', K') + r c(I + 1, J', K'); the four a
// values a ghost reads are shared with its neighbouring ghosts.  Stage 1
// evaluates each pair the entry's ghosts read once, into the warp's scratch
// (X * Y * Z doubles: X fine x positions, Y coarse y rows, Z coarse z rows);
// stage 2 finishes every ghost from four of them with the y- and z-steps.
// Each value sees the same operations in the same order as C2F<double>::value.
constexpr int kC2fScratch = 320;  // doubles per warp: 16 * 2 * 10 at N = 16
template <int N, int VC, int AX, class TL>
__device__ __forceinline__ void c2f_entry_sep(const VcTask& t, double* __restrict__ dst,
                                              const Geom& g, const double* __restrict__ sf,
                                              int lane, double* __restrict__ scr) {
  static_assert(N <= 16, "scratch sized for 16^3 blocks");
  const bool minus = (t.face & 1) == 0;
  const int P0 = N * (t.subface & 1), P1 = N * ((t.subface >> 1) & 1);
  // fine bases of the varying axes, in x, y, z
  int fb[3];
  face_xyz<AX>(0, P0, P1, fb[0], fb[1], fb[2]);
  for (int u = 0; u < VC; u++) {
    const int fn = minus ? 2 * N - VC + u : u;  // fine index along the face normal
    int lo[3], cnt[3];
    for (int a = 0; a < 3; a++) {
      if (a == AX) {
        lo[a] = lin_I(fn, N);
        cnt[a] = a == 0 ? 1 : 2;
      } else {
        lo[a] = lin_I(fb[a], N);
        cnt[a] = a == 0 ? N : lin_I(fb[a] + N - 1, N) + 2 - lo[a];
      }
    }
    const int X = cnt[0], Y = cnt[1], Z = cnt[2];
    // stage 1: x-steps.  x position xi: fine x = fn (x faces) or fb[0] + xi.
    for (int e = lane; e < X * Y * Z; e += 32) {
      const int xi = e % X, yi = (e / X) % Y, zi = e / (X * Y);
      const int fx = AX == 0 ? fn : fb[0] + xi;
      const int I = lin_I(fx, N);
      const double r = (double)lin_r(fx, I), r1 = 1.0 - r;
      const double* c = sf + TL::at(I, lo[1] + yi, lo[2] + zi);
      scr[e] = xadd(xmul(r1, c[0]), xmul(r, c[1]));
    }
    __syncwarp();
    // stage 2: y- and z-steps of every ghost of this layer
    for (int e = lane; e < N * N; e += 32) {
      int x, y, z, fx, fy, fz;
      // x fastest where x lies in the face (Y faces: (z, x); Z faces: (x, y))
      const int a = AX == 1 ? e / N : e % N, cc = AX == 1 ? e % N : e / N;
      face_xyz<AX>(minus ? u - VC : N + u, a, cc, x, y, z);
      face_xyz<AX>(fn, a + P0, cc + P1, fx, fy, fz);
      const int J = lin_I(fy, N), K = lin_I(fz, N);
      const double s = (double)lin_r(fy, J), s1 = 1.0 - s;
      const double tt = (double)lin_r(fz, K), t1 = 1.0 - tt;
      const int xi = AX == 0 ? 0 : fx - fb[0];
      const double* A = scr + xi + X * ((J - lo[1]) + Y * (K - lo[2]));
      const double a00 = A[0], a10 = A[X], a01 = A[X * Y], a11 = A[X + X * Y];
      dst[g.at(x, y, z)] = xadd(xmul(t1, xadd(xmul(s1, a00), xmul(s, a10))),
                                xmul(tt, xadd(xmul(s1, a01), xmul(s, a11))));
    }
    __syncwarp();  // the next layer overwrites the scratch
  }
}

template <int N, int VC, class TL>
__device__ __forceinline__ void c2f_sep_dispatch(const VcTask& t, double* dst, const Geom& g,
                                                 const double* sf, int lane, double* scr) {
  switch (t.face >> 1) {
    case 0: c2f_entry_sep<N, VC, 0, TL>(t, dst, g, sf, lane, scr); break;
    case 1: c2f_entry_sep<N, VC, 1, TL>(t, dst, g, sf, lane, scr); break;
    default: c2f_entry_sep<N, VC, 2, TL>(t, dst, g, sf, lane, scr); break;
  }
}

template <typename T, int N, int VC, class TL = Tile<T, N, VC>, int UB = 8>
__device__ __forceinline__ void push_dispatch(const VcTask& t, T* dst, const Geom& g,
                                              const T* sf, int lane) {
  const int key = t.kind * 3 + (t.face >> 1);
  switch (key) {
    case VC_COPY * 3 + 0: push_entry<T, N, VC, VC_COPY, 0, TL, false, false, 32, UB>(t, dst, g, sf, lane); break;
    case VC_COPY * 3 + 1: push_entry<T, N, VC, VC_COPY, 1, TL, false, false, 32, UB>(t, dst, g, sf, lane); break;
    case VC_COPY * 3 + 2: push_entry<T, N, VC, VC_COPY, 2, TL, false, false, 32, UB>(t, dst, g, sf, lane); break;
    case VC_F2C * 3 + 0: push_entry<T, N, VC, VC_F2C, 0, TL, false, false, 32, UB>(t, dst, g, sf, lane); break;
    case VC_F2C * 3 + 1: push_entry<T, N, VC, VC_F2C, 1, TL, false, false, 32, UB>(t, dst, g, sf, lane); break;
    case VC_F2C * 3 + 2: push_entry<T, N, VC, VC_F2C, 2, TL, false, false, 32, UB>(t, dst, g, sf, lane); break;
    case VC_C2F * 3 + 0: push_entry<T, N, VC, VC_C2F, 0, TL, false, false, 32, UB>(t, dst, g, sf, lane); break;
    case VC_C2F * 3 + 1: push_entry<T, N, VC, VC_C2F, 1, TL, false, false, 32, UB>(t, dst, g, sf, lane); break;
    case VC_C2F * 3 + 2: push_entry<T, N, VC, VC_C2F, 2, TL, false, false, 32, UB>(t, dst, g, sf, lane); break;
    default: break;
  }
}

// Dirichlet first ghost layer of the faces in `mask` inside the tile:
// g = 2v - f(adjacent interior) in double (sor1/Solver.cpp:232-294).
// v2f (optional, float tiles): 2v per face as an exact float, or NaN (then
// the double expression is evaluated).  When 2v is a float, the reference's
// double difference rounded to float equals the float subtraction: double
// rounding from 53 to 24 bits is innocuous for one addition of float operands
// (53 >= 2*24 + 2; S. A. Figueroa, "When is double rounding innocuous?",
// SIGNUM Newsl. 30(3), 1995).
template <typename T, int N, int VC, class TL = Tile<T, N, VC>>
__device__ __forceinline__ void tile_dirichlet(T* sf, unsigned mask, const double* val, bool bcx,
                                               int tid, int nt, const float* v2f = nullptr) {
  for (int fc = 0; fc < 6; fc++) {
    if (!((mask >> fc) & 1)) continue;
    const int ax = fc >> 1;
    const bool minus = (fc & 1) == 0;
    const float w2 = (sizeof(T) == 4 && v2f) ? v2f[fc] : __int_as_float(0x7fc00000);
    const bool fast = w2 == w2;
    double v2 = 0.0;
    if (!fast) {
      double v = val[fc];
      if (bcx) v = (double)(T)v;
      v2 = xmul(2.0, v);
    }
    for (int e = tid; e < N * N; e += nt) {
      const int p = e % N, q = e / N;
      int gi, ii;
      if (ax == 0) { gi = TL::at(minus ? -1 : N, p, q); ii = TL::at(minus ? 0 : N - 1, p, q); }
      else if (ax == 1) { gi = TL::at(p, minus ? -1 : N, q); ii = TL::at(p, minus ? 0 : N - 1, q); }
      else { gi = TL::at(p, q, minus ? -1 : N); ii = TL::at(p, q, minus ? 0 : N - 1); }
      if (sizeof(T) == 4 && fast) sf[gi] = (T)__fsub_rn(w2, (float)sf[ii]);
      else sf[gi] = to_t<T>(xsub(v2, (double)sf[ii]));
    }
  }
}

// Copies the Dirichlet ghost layers of `mask` from the tile to the brick
// (and, for the bcx.f90 form with vc >= 2, sets the second layer to v).
template <typename T, int N, int VC>
__device__ __forceinline__ void store_dirichlet(const T* sf, T* __restrict__ fb, const Geom& g,
                                                unsigned mask, const double* val, bool bcx,
                                                int tid, int nt) {
  using TL = Tile<T, N, VC>;
  for (int fc = 0; fc < 6; fc++) {
    if (!((mask >> fc) & 1)) continue;
    const int ax = fc >> 1;
    const bool minus = (fc & 1) == 0;
    const bool second = bcx && VC >= 2;
    const T v = (T)val[fc];
    for (int e = tid; e < N * N; e += nt) {
      const int p = e % N, q = e / N;
      const int l1 = minus ? -1 : N, l2 = minus ? -2 : N + 1;
      if (ax == 0) {
        fb[g.at(l1, p, q)] = sf[TL::at(l1, p, q)];
        if (second) fb[g.at(l2, p, q)] = v;
      } else if (ax == 1) {
        fb[g.at(p, l1, q)] = sf[TL::at(p, l1, q)];
        if (second) fb[g.at(p, l2, q)] = v;
      } else {
        fb[g.at(p, q, l1)] = sf[TL::at(p, q, l1)];
        if (second) fb[g.at(p, q, l2)] = v;
      }
    }
  }
}

// Interior rows from the tile to the brick, in vectors of VC elements when
// the row start (offset VC in the brick row) allows it.
template <typename T, int N, int VC>
__device__ __forceinline__ void store_interior(const T* __restrict__ sf, T* __restrict__ fb,
                                               const Geom& g, int tid, int nt) {
  using TL = Tile<T, N, VC>;
  constexpr int SB = (VC * sizeof(T)) % 16 == 0 ? 16 : (VC * sizeof(T)) % 8 == 0 ? 8 : (int)sizeof(T);
  constexpr int SV = SB / sizeof(T);
  using V = typename VecOf<SB>::type;
  if constexpr (SV == 1) {
    for (int e = tid; e < N * N * N; e += nt) {
      const int i = e % N, r = e / N, j = r % N, k = r / N;
      fb[g.at(i, j, k)] = sf[TL::at(i, j, k)];
    }
  } else {
    constexpr int NV = N / SV;
    for (int e = tid; e < NV * N * N; e += nt) {
      const int v = e % NV, r = e / NV, j = r % N, k = r / N;
      reinterpret_cast<V*>(fb + g.at(0, j, k))[v] =
          reinterpret_cast<const V*>(sf + TL::at(0, j, k))[v];
    }
  }
}

// Thread-to-cell map of the pull form for face F: thread t of an N*N-thread
// CTA takes in-plane cell (p, q) = (t % N, t / N) in (x, y), (x, z) or (y, z)
// order, returned as subface-order indices (a, c) and the ghost cell.
template <int N, int F>
__device__ __forceinline__ void pull_map(int p, int q, int& a, int& c, int& x, int& y, int& z) {
  constexpr int AX = F >> 1;
  constexpr bool MINUS = (F & 1) == 0;
  if (AX == 1) { a = q; c = p; }  // Y faces: (z, x)
  else { a = p; c = q; }          // X faces (y, z), Z faces (x, y)
  face_xyz<AX>(MINUS ? -1 : N, a, c, x, y, z);
}

// This thread's cell (p, q) of the first ghost layer of face F fed by a
// coarser block (C2F): the interpolation of the coarse block's interior in its
// brick `cb` (Scalar3DUpdater.h:221-266), `sub` this block's subface on the
// coarse face -- the value the coarse block's push_entry writes for it.
template <typename T, int N, int VC, int F>
__device__ __forceinline__ T c2f_pull(const T* __restrict__ cb, int sub, int p, int q) {
  using BL = BrickTile<T, N, VC>;
  constexpr int AX = F >> 1;
  int a, c, x, y, z;
  pull_map<N, F>(p, q, a, c, x, y, z);
  int fx, fy, fz;  // fine indices in the coarse block's fine index space
  face_xyz<AX>((F & 1) == 0 ? 2 * N - 1 : 0, a + N * (sub & 1), c + N * ((sub >> 1) & 1), fx,
               fy, fz);
  const int I = lin_I(fx, N), J = lin_I(fy, N), K = lin_I(fz, N);
  return (T)C2F<T>::value(cb + BL::at(I, J, K), BL::LX, BL::LXY, lin_r(fx, I), lin_r(fy, J),
                          lin_r(fz, K));
}

}  // namespace bcmg
