// stream.cuh -- z-plane streaming of one cubic brick through shared memory,
// for the one-CTA-per-block stencil kernels of blocks too large to stage
// whole (32^3).
//
// A brick's planes are contiguous (x fastest, plane pitch (N+2VC)^2), so one
// bulk copy (the TMA engine's non-tensor form) moves one plane.  A ring of S
// slots holds "units": with a halo field X, unit u is X's plane VC-1+u (the
// N interior planes and the two first-layer ghost planes, N+2 units) and,
// for u in [1, N], the interior rows of the same plane of up to NB cell-only
// fields (a right-hand side, a dot-product partner); without X, unit u is
// the cell-only fields' plane VC+u (N units).  Each unit completes on its
// slot's mbarrier.  Output plane m (brick plane VC+m) reads units m..m+2
// (with X; unit m without), so after it the slot of unit m is free for unit
// m+S.  S-3 units (S-1 with no X) are in flight while a plane is computed,
// and several CTAs per SM keep the copy engine busy, so HBM sees whole
// planes and the threads never wait on a load of their own.
//
// Waits are bounded (bulk.cuh): on a timeout the kernel records the error
// code, waits (bounded) for the copies it issued and returns.
#pragma once
#include <cstdint>
#include <cstdlib>

#include "bulk.cuh"
#include "tile.cuh"

namespace bcmg {

// Host: the streamed kernels are the default for the shapes they cover;
// BCMG_PLANE_STREAM=0 selects the column-walk kernels instead (comparison
// runs).
inline bool plane_stream_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("BCMG_PLANE_STREAM");
    return !(v && v[0] == '0');
  }();
  return on;
}

// Host: the bulk copies need 16-byte aligned planes: cubic bricks of the
// standard pitch, a brick stride of whole 16-byte units, aligned fields.
template <typename T>
inline bool stream_aligned(const Geom& g, const void* p0, const void* p1) {
  const int lx = g.nx + 2 * g.vc;
  return g.nx == g.ny && g.ny == g.nz && g.sy == lx && g.sz == lx * lx &&
         ((size_t)g.bstride * sizeof(T)) % 16 == 0 && (reinterpret_cast<uintptr_t>(p0) % 16) == 0 &&
         (reinterpret_cast<uintptr_t>(p1) % 16) == 0;
}

// CTAs per SM a streamed kernel is compiled for: as many as its shared
// memory admits (228 KB per SM, 1 KB reserved per CTA), at most CAP.
template <size_t SMEM, int CAP>
__host__ __device__ constexpr int stream_minb() {
  return (int)(233472 / (SMEM + 1024)) < CAP ? (int)(233472 / (SMEM + 1024)) : CAP;
}

template <typename T, int N, int VC, int S, bool HX, int NB>
struct PlaneRing {
  using BL = BrickTile<T, N, VC>;
  static constexpr int LX = BL::LX, LXY = BL::LXY;
  static constexpr unsigned PB = LXY * sizeof(T);  // bytes of one brick plane
  // interior rows [VC, VC+N) of a plane, widened to 16-byte bounds (kept at
  // the same offsets in shared memory as in the brick)
  static constexpr unsigned ROW_LO = VC * LX * sizeof(T) / 16 * 16;
  static constexpr unsigned ROW_HI = ((VC + N) * LX * sizeof(T) + 15) / 16 * 16;
  static constexpr unsigned RB = ROW_HI - ROW_LO;
  static constexpr int NU = HX ? N + 2 : N;  // units per block
  static constexpr unsigned SLOT = (HX ? PB : 0) + NB * PB;
  static constexpr unsigned BAR_BYTES = 128;
  static constexpr size_t SMEM = BAR_BYTES + (size_t)S * SLOT;
  static_assert(S >= 2 && S <= 16, "ring depth");
  static_assert(PB % 16 == 0 && ROW_LO % 16 == 0 && RB % 16 == 0 && ROW_HI <= PB,
                "bulk copies need 16-byte sizes and offsets");
  static_assert(!HX || NB <= 2, "at most two cell-only fields");

  // Offset of cell (i, j) of a plane (interior coordinates).
  static __device__ __forceinline__ int at(int i, int j) { return (j + VC) * LX + VC + i; }

  uint64_t* bar;
  unsigned char* slots;

  __device__ __forceinline__ PlaneRing(unsigned char* smraw)
      : bar(reinterpret_cast<uint64_t*>(smraw)), slots(smraw + BAR_BYTES) {}

  // Plane of X held by unit u; plane of cell-only field f held by unit u.
  __device__ __forceinline__ const T* xp(int u) const {
    return reinterpret_cast<const T*>(slots + (u % S) * SLOT);
  }
  __device__ __forceinline__ const T* cp(int u, int f) const {
    return reinterpret_cast<const T*>(slots + (u % S) * SLOT + (HX ? PB : 0) + f * PB);
  }

  // Thread 0: the barriers, then the first S units of block b.
  __device__ __forceinline__ void start(const T* X, const T* const* C, int64_t base) {
    for (int s = 0; s < S; s++) mbar_init(&bar[s], 1);
    mbar_fence_init();
    for (int u = 0; u < S && u < NU; u++) issue(u, X, C, base);
  }

  // Thread 0: unit u of the block whose brick starts at element `base`.
  __device__ __forceinline__ void issue(int u, const T* X, const T* const* C, int64_t base) {
    unsigned char* dst = slots + (u % S) * SLOT;
    const int z = HX ? VC - 1 + u : VC + u;  // brick plane
    const bool cells = !HX || (u >= 1 && u <= N);
    const unsigned bytes = (HX ? PB : 0) + (cells ? NB * RB : 0);
    mbar_expect_tx(&bar[u % S], bytes);
    if (HX) bulk_g2s(dst, X + base + (int64_t)z * LXY, PB, &bar[u % S]);
    if (cells) {
#pragma unroll
      for (int f = 0; f < NB; f++)
        bulk_g2s(dst + (HX ? PB : 0) + f * PB + ROW_LO,
                 reinterpret_cast<const unsigned char*>(C[f] + base + (int64_t)z * LXY) + ROW_LO,
                 RB, &bar[u % S]);
    }
  }

  __device__ __forceinline__ bool wait(int u, int* err) {
    return mbar_wait_quiet(&bar[u % S], (unsigned)(u / S) & 1u, err);
  }

  // Thread 0 after a failed wait: waits (bounded, silently) for the last
  // unit issued into each slot, so that no copy lands after the CTA has left.
  __device__ __forceinline__ void drain(int issued) {
    for (int s = 0; s < S; s++) {
      const int u = issued - 1 - ((issued - 1 - s) % S + S) % S;  // last unit of slot s
      if (u >= 0) mbar_wait_quiet(&bar[s], (unsigned)(u / S) & 1u, nullptr);
    }
  }
};

// The walk of one block: for each output plane m, thread 0 waits for the
// unit it adds (the others do not spin: they wait at the CTA barrier), the
// barrier also tells that every thread is done with unit m-1, so thread 0
// issues unit m-1+S into its slot, then every thread runs body(m) (its
// cells of plane m).  One CTA barrier per plane, and one at the end (the
// walk's global writes are then visible to the whole CTA).  Returns false
// (after draining) when a wait timed out: the caller's results are void
// (the error word says so).  Every thread returns the same value.
template <typename T, int N, int VC, int S, bool HX, int NB, class Body>
__device__ __forceinline__ bool plane_walk(PlaneRing<T, N, VC, S, HX, NB>& ring, const T* X,
                                           const T* const* C, int64_t base, int* err, int tid,
                                           Body&& body) {
  using R = PlaneRing<T, N, VC, S, HX, NB>;
  // unit m+2 (HX) is waited for at plane m and issued at plane m+3-S: S >= 4
  static_assert(S >= (HX ? 4 : 2), "ring too shallow for the walk");
  int issued = S < R::NU ? S : R::NU;
  bool ok = true;
  for (int m = 0; m < N; m++) {
    if (tid == 0) {
      if (HX && m == 0) ok = ring.wait(0, err) && ring.wait(1, err);
      ok = ok && ring.wait(HX ? m + 2 : m, err);
    }
    if (!__syncthreads_and(ok)) {
      if (tid == 0) ring.drain(issued);
      __syncthreads();
      return false;
    }
    if (tid == 0 && m > 0 && m - 1 + S < R::NU) {
      ring.issue(m - 1 + S, X, C, base);
      issued = m + S;
    }
    body(m);
  }
  __syncthreads();
  return true;
}

}  // namespace bcmg
