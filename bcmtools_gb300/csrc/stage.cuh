// stage.cuh -- staging of one block for the one-CTA-per-block fused Jacobi
// sweep: the shared-memory layout and the bulk copies that fill it.
#pragma once
#include "bulk.cuh"
#include "ghost.cuh"
#include "kernels.h"
#include "tile.cuh"

namespace bcmg {

// Shared-memory layout: mbarrier, the block's brick (BrickTile layout), and
// with SRC the interior planes [VC, VC+N) of a second field (Jacobi's b,
// sor2's source), each plane at the brick's plane pitch.  N*N threads.
template <typename T, int N, int VC, bool SRC>
struct BrickStage {
  using BL = BrickTile<T, N, VC>;
  static constexpr int NT = N * N;
  static constexpr unsigned PB = BL::LXY * sizeof(T);  // plane bytes
  static constexpr unsigned X_BYTES = BL::SIZE * sizeof(T);
  static constexpr unsigned B_BYTES = SRC ? N * PB : 0;
  static constexpr unsigned X_OFF = 16;
  static constexpr unsigned B_OFF = X_OFF + X_BYTES;
  static constexpr size_t SMEM = B_OFF + B_BYTES;
  static_assert(X_BYTES % 16 == 0 && PB % 16 == 0, "bulk copies need 16-byte sizes and offsets");
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
  // second field: rows [VC, VC+N) of each interior plane, widened to 16-byte
  // bounds (same offsets in shared memory as in the brick)
  static constexpr unsigned ROW_LO = VC * BL::LX * sizeof(T) / 16 * 16;
  static constexpr unsigned ROW_HI = ((VC + N) * BL::LX * sizeof(T) + 15) / 16 * 16;
  static constexpr unsigned B_PLANE = ROW_HI - ROW_LO;
  static_assert(ROW_HI <= PB, "row range within a plane");

  // This thread's (i, j) column of the sweeps.
  static __device__ __forceinline__ void column(int tid, int& i, int& j) {
    if (N == 16) {
      const int w = tid >> 5, lane = tid & 31;
      i = lane & 15;
      j = (w % D) + 2 * D * (w / D) + D * (lane >> 4);
    } else {
      i = tid % N;
      j = tid / N;
    }
  }

  // Called by warp 0 after thread 0 initialised `bar`: starts the copies of
  // block b.  full: the whole brick; otherwise planes [0,N) and the ghost
  // planes -1 / N only when `lo` / `hi`.  The second field's rows follow.
  static __device__ __forceinline__ void issue(unsigned char* smraw, uint64_t* bar, const T* X,
                                               const T* S, int64_t b, int64_t bstride, bool full,
                                               bool lo, bool hi, int lane) {
    const unsigned char* xsrc = reinterpret_cast<const unsigned char*>(X + b * bstride);
    unsigned char* xdst = smraw + X_OFF;
    if (lane == 0) {
      const unsigned xb = full ? X_BYTES : (N + (lo ? 1 : 0) + (hi ? 1 : 0)) * PB;
      mbar_expect_tx(bar, xb + (SRC ? N * B_PLANE : 0));
      if (full) {
        bulk_g2s(xdst, xsrc, X_BYTES, bar);
      } else {
        bulk_g2s(xdst + VC * PB, xsrc + VC * PB, N * PB, bar);
        if (lo) bulk_g2s(xdst + (VC - 1) * PB, xsrc + (VC - 1) * PB, PB, bar);
        if (hi) bulk_g2s(xdst + (VC + N) * PB, xsrc + (VC + N) * PB, PB, bar);
      }
    }
    if (SRC) {
      __syncwarp();
      const unsigned char* ssrc = reinterpret_cast<const unsigned char*>(S + b * bstride) + VC * PB;
      unsigned char* sdst = smraw + B_OFF;
      for (int z = lane; z < N; z += 32)
        bulk_g2s(sdst + z * PB + ROW_LO, ssrc + z * PB + ROW_LO, B_PLANE, bar);
    }
  }
};

}  // namespace bcmg
