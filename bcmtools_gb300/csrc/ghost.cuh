// ghost.cuh -- device-side ghost (virtual cell) values of one face-table
// entry, shared by the gather kernel (sources read from global memory) and
// the fused sweep kernels (sources read from the sweeping CTA's shared
// memory).
//
// Reference math (Scalar3DUpdater.h):
//   same-level copy   copyFromNeighbor           :321-347
//   F2C average       interpolateF2C             :190-198, loops :519-612
//   C2F interpolation interpolateC2F, linearInterpolate :221-266, loops :615-708
//   Dirichlet ghost   sor1/Solver.cpp:232-294, SolverTest/bcx.f90:18-76
//   Neumann ghost     SolverTest/bcx.f90:198-376
//
// Precision: FP64 fields evaluate C2F exactly in the reference's operation
// order in double.  FP32 fields evaluate the same expression in compensated
// float-float arithmetic (GB300 runs FP64 at a small fraction of its FP32
// rate), which agrees with the reference's double evaluation rounded to
// float to within one ulp, and bit for bit except where the value lies
// within ~2^-44 of a rounding boundary.  F2C and copies are bit-exact in both.
#pragma once
#include "common.cuh"

namespace bcmg {

template <typename T>
__device__ __forceinline__ T to_t(double v);
template <>
__device__ __forceinline__ float to_t<float>(double v) { return __double2float_rn(v); }
template <>
__device__ __forceinline__ double to_t<double>(double v) { return v; }

// Reads cell (i,j,k) of one brick-like array (global brick or shared tile).
template <typename T>
struct Acc {
  const T* p;
  int sy, sz, off;
  __device__ __forceinline__ const T* at(int i, int j, int k) const {
    return p + off + i + sy * j + sz * k;
  }
};

// ---- compensated float-float arithmetic (error-free transforms) ----------
struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ff ff_add(ff x, ff y) {
  const ff s = two_sum(x.hi, y.hi);
  return two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
// Dekker's Fast2Sum: the same pair as two_sum when exponent(a) >= exponent(b)
// (or a = 0).
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
// x * f for a normalised x (|x.lo| <= ulp(x.hi) / 2): the correction
// x.lo*f + err(x.hi*f) stays below 2 ulp(x.hi*f), so Fast2Sum renormalises.
__device__ __forceinline__ ff ff_mul(ff x, float f) {
  const ff p = two_prod(x.hi, f);
  return fast_two_sum(p.hi, __fmaf_rn(x.lo, f, p.lo));
}
// hi part of ff_add(x, y): the final two_sum's sum alone.
__device__ __forceinline__ float ff_add_hi(ff x, ff y) {
  const ff s = two_sum(x.hi, y.hi);
  return __fadd_rn(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

// linearInterpolate: I = min(max(i/2 - 1 + i%2, 0), n-2), r = -0.25 + 0.5 i - I.
__device__ __forceinline__ int lin_I(int i, int n) { return max(0, min(i / 2 - 1 + (i & 1), n - 2)); }
__device__ __forceinline__ float lin_r(int i, int I) {
  return __fsub_rn(__fmaf_rn(0.5f, (float)i, -0.25f), (float)I);  // exact: quarters
}

template <typename T>
struct C2F;

template <>
struct C2F<double> {
  // The reference's expression, in double, products and sums in its order.
  static __device__ __forceinline__ double value(const double* c, int sy, int sz, float rf,
                                                 float sf, float tf) {
    const double r = rf, s = sf, t = tf, r1 = 1.0 - r, s1 = 1.0 - s, t1 = 1.0 - t;
    const double a00 = xadd(xmul(r1, c[0]), xmul(r, c[1]));
    const double a10 = xadd(xmul(r1, c[sy]), xmul(r, c[sy + 1]));
    const double a01 = xadd(xmul(r1, c[sz]), xmul(r, c[sz + 1]));
    const double a11 = xadd(xmul(r1, c[sy + sz]), xmul(r, c[sy + sz + 1]));
    return xadd(xmul(t1, xadd(xmul(s1, a00), xmul(s, a10))),
                xmul(t, xadd(xmul(s1, a01), xmul(s, a11))));
  }
};

template <>
struct C2F<float> {
  // Same expression; (1-r)*c is exact in float-float, r*c is the float
  // product of the reference's float build, the rest compensated.
  static __device__ __forceinline__ float value(const float* c, int sy, int sz, float r,
                                                float s, float t) {
    const float r1 = 1.0f - r, s1 = 1.0f - s, t1 = 1.0f - t;  // exact
    const ff a00 = x_step(two_prod(r1, c[0]), __fmul_rn(r, c[1]));
    const ff a10 = x_step(two_prod(r1, c[sy]), __fmul_rn(r, c[sy + 1]));
    const ff a01 = x_step(two_prod(r1, c[sz]), __fmul_rn(r, c[sz + 1]));
    const ff a11 = x_step(two_prod(r1, c[sy + sz]), __fmul_rn(r, c[sy + sz + 1]));
    const ff u0 = ff_add(ff_mul(a00, s1), ff_mul(a10, s));
    const ff u1 = ff_add(ff_mul(a01, s1), ff_mul(a11, s));
    return ff_add_hi(ff_mul(u0, t1), ff_mul(u1, t));
  }
  // (1-r)*c (exact pair p) + fl(r*c') (float q), normalised
  static __device__ __forceinline__ ff x_step(ff p, float q) {
    const ff s = two_sum(p.hi, q);
    return two_sum(s.hi, __fadd_rn(s.lo, p.lo));
  }
};

// F2C: eight-cell sum in T left to right, times 0.125 (exact scaling).
template <typename T>
__device__ __forceinline__ T f2c_value(const T* p, int sy, int sz) {
  T sum = p[0];
  sum = xadd(sum, p[1]);
  sum = xadd(sum, p[sy]);
  sum = xadd(sum, p[sy + 1]);
  sum = xadd(sum, p[sz]);
  sum = xadd(sum, p[sz + 1]);
  sum = xadd(sum, p[sy + sz]);
  sum = xadd(sum, p[sy + sz + 1]);
  return xmul(sum, (T)0.125);
}

// Divide by a small box extent: shifts for powers of two.
__device__ __forceinline__ void divmod(int e, int d, int& q, int& r) {
  if ((d & (d - 1)) == 0) {
    const int s = __ffs(d) - 1;
    q = e >> s;
    r = e & (d - 1);
  } else {
    q = e / d;
    r = e - q * d;
  }
}

// Ghost box of one entry, from the destination block's point of view:
// ghost cell (d + x) of dst, x in [0,b), takes its value from source
// coordinates derived from (x + o) of the source block.
struct Box {
  int b[3];  // extents
  int d[3];  // first ghost cell in dst
  int o[3];  // copy: source offset; F2C: fine-index base (halved); C2F: fine index base
};

__device__ __forceinline__ Box task_box(const VcTask& t, const Geom& g) {
  const int n[3] = {g.nx, g.ny, g.nz};
  const int vc = g.vc, ax = t.face >> 1, minus = (t.face & 1) == 0;
  // in-plane axes in subface order: X (y,z), Y (z,x), Z (x,y) (Scalar3DUpdater.h:527-584)
  const int a0 = ax == 0 ? 1 : (ax == 1 ? 2 : 0);
  const int a1 = ax == 0 ? 2 : (ax == 1 ? 0 : 1);
  const int o0 = t.subface & 1, o1 = (t.subface >> 1) & 1;
  Box B;
  for (int a = 0; a < 3; a++) { B.b[a] = n[a]; B.d[a] = 0; B.o[a] = 0; }
  if (t.kind == VC_COPY) {
    B.b[ax] = vc;
    B.d[ax] = minus ? -vc : n[ax];
    B.o[ax] = minus ? n[ax] - vc : 0;
  } else if (t.kind == VC_F2C) {
    B.b[a0] = n[a0] / 2; B.b[a1] = n[a1] / 2; B.b[ax] = vc;
    B.d[a0] = (n[a0] / 2) * o0; B.d[a1] = (n[a1] / 2) * o1;
    B.d[ax] = minus ? -vc : n[ax];
    B.o[ax] = minus ? n[ax] / 2 - vc : 0;
  } else if (t.kind == VC_C2F) {
    B.b[ax] = vc;
    B.d[ax] = minus ? -vc : n[ax];
    B.o[a0] = n[a0] * o0; B.o[a1] = n[a1] * o1;
    B.o[ax] = minus ? 2 * n[ax] - vc : 0;
  } else {  // Dirichlet: first ghost layer, reading the adjacent interior layer
    B.b[ax] = 1;
    B.d[ax] = minus ? -1 : n[ax];
    B.o[ax] = minus ? 0 : n[ax] - 1;
  }
  return B;
}

// Writes the ghost cells of entry t into `dst` (the destination brick in
// global memory), reading sources through `src`.  Cells are split over
// `nl` workers starting at `lane`, in batches of four per worker whose reads
// (interior cells only) are all issued before the batch's writes (ghost
// cells only), so the reads overlap.  TOBUF (neighbour entries only): the
// values go to dst[e] instead, e the cell's position in the ghost box with x
// fastest -- the reference's communication-buffer order.
template <typename T, bool TOBUF = false>
__device__ __forceinline__ void task_apply(const VcTask& t, T* __restrict__ dst, const Geom& g,
                                           const Acc<T>& src, double bcv, int lane, int nl) {
  constexpr int U = 4;
  const Box B = task_box(t, g);
  const int cnt = B.b[0] * B.b[1] * B.b[2];
  const int bxy = B.b[0] * B.b[1];
  for (int e0 = lane; e0 < cnt; e0 += U * nl) {
    T vals[U], second[U];
    int at[U], at2[U];
#pragma unroll
    for (int q = 0; q < U; q++) {
      const int e = e0 + q * nl;
      at[q] = -1;
      at2[q] = -1;
      if (e >= cnt) continue;
      int k, r, j, i;
      divmod(e, bxy, k, r);
      divmod(r, B.b[0], j, i);
      at[q] = TOBUF ? e : g.at(B.d[0] + i, B.d[1] + j, B.d[2] + k);
      if (t.kind == VC_COPY) {
        vals[q] = *src.at(B.o[0] + i, B.o[1] + j, B.o[2] + k);
      } else if (t.kind == VC_F2C) {
        vals[q] = f2c_value<T>(src.at(2 * (B.o[0] + i), 2 * (B.o[1] + j), 2 * (B.o[2] + k)),
                               src.sy, src.sz);
      } else if (t.kind == VC_C2F) {
        const int fi = B.o[0] + i, fj = B.o[1] + j, fk = B.o[2] + k;
        const int I = lin_I(fi, g.nx), J = lin_I(fj, g.ny), K = lin_I(fk, g.nz);
        vals[q] = (T)C2F<T>::value(src.at(I, J, K), src.sy, src.sz, lin_r(fi, I), lin_r(fj, J),
                                   lin_r(fk, K));
      } else if (t.flags & kTaskNeumann) {
        // SolverTest/bcx.f90:198-376: interior -/+ xc in T, the second layer
        // interior -/+ xc*2 in double (xc `real`)
        const T fin = *src.at(B.o[0] + i, B.o[1] + j, B.o[2] + k);
        const T xc = (T)bcv;
        const int ax = t.face >> 1, minus = (t.face & 1) == 0;
        vals[q] = minus ? xsub(fin, xc) : xadd(fin, xc);
        if (g.vc >= 2) {
          int c[3] = {B.d[0] + i, B.d[1] + j, B.d[2] + k};
          c[ax] += minus ? -1 : 1;
          at2[q] = g.at(c[0], c[1], c[2]);
          const double x2 = xmul((double)xc, 2.0);
          second[q] = to_t<T>(minus ? xsub((double)fin, x2) : xadd((double)fin, x2));
        }
      } else {
        const T fin = *src.at(B.o[0] + i, B.o[1] + j, B.o[2] + k);
        double v = bcv;
        if (t.flags & 1) v = (double)(T)v;
        vals[q] = to_t<T>(xsub(xmul(2.0, v), (double)fin));
        if ((t.flags & 1) && g.vc >= 2) {
          const int ax = t.face >> 1, minus = (t.face & 1) == 0;
          int c[3] = {B.d[0] + i, B.d[1] + j, B.d[2] + k};
          c[ax] += minus ? -1 : 1;
          at2[q] = g.at(c[0], c[1], c[2]);
          second[q] = (T)v;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < U; q++) {
      if (at[q] >= 0) dst[at[q]] = vals[q];
      if (at2[q] >= 0) dst[at2[q]] = second[q];
    }
  }
}

}  // namespace bcmg
