// krylov.cu -- the device-resident BiCGSTAB iteration kernels (krylov.cuh).
//
// One CTA per block.  Cubic 8/16/32-cell blocks take N*N threads, one
// (i, j) column each, the k walk unrolled so that a thread has several
// planes' loads in flight; other block shapes loop over the columns.
// Inner products: FP64 multiply-add per element along the column, then the
// CTA's fixed-order tree (kr_block_sum); partial sums per block go to
// partial[slot * nb + b] and kr_scalar reduces them per segment.
#include <cfloat>

#include "bcmg.h"
#include "kernels.h"
#include "krylov.cuh"
#include "stream.cuh"

namespace bcmg {

// ---------------------------------------------------------------------------
// The columns of one thread: tid, tid + blockDim.x, ... one after another,
// each walked along k (four planes unrolled when the block edge is known at
// compile time, N > 0); thread counts and register budgets in krylov.cuh.
#define KR_COLUMNS(N, g, BODY)                                                          \
  {                                                                                     \
    const int64_t base_ = (int64_t)blockIdx.x * (g).bstride;                            \
    const int nx_ = N ? N : (g).nx, nc_ = N ? N * N : (g).nx * (g).ny;                  \
    const int nz_ = N ? N : (g).nz;                                                     \
    for (int ij_ = threadIdx.x; ij_ < nc_; ij_ += blockDim.x) {                         \
      const int64_t oc_ = base_ + (g).at(ij_ % nx_, ij_ / nx_, 0);                      \
      _Pragma("unroll 4") for (int k_ = 0; k_ < nz_; k_++) {                            \
        const int64_t o = oc_ + (int64_t)k_ * (g).sz;                                   \
        BODY                                                                            \
      }                                                                                 \
    }                                                                                   \
  }

// p = r + beta (p - gamma q): ILS3D's AXPY(p, q_, -gamma) then XPAY(p, r,
// beta) (ILS3D.h:727-736, blas.f90:242-308), both roundings kept.
template <typename T, int N>
__global__ void __launch_bounds__(kr_nt<N>(), (kr_minb<T, N, false>())) kr_p_kernel(T* __restrict__ p,
                                                          const T* __restrict__ r,
                                                          const T* __restrict__ q, Geom g,
                                                          KSegs S) {
  const KSeg& sg = S.seg[kseg_of(S, blockIdx.x)];
  if (sg.status != kRunning) return;
  const T beta = (T)sg.beta, ng = (T)(-sg.gamma);
  KR_COLUMNS(N, g, { p[o] = xadd(r[o], xmul(beta, xadd(p[o], xmul(ng, q[o])))); })
}

// s = r - alpha q: AXPYZ(s, q_, r, -alpha) (ILS3D.h:747, blas.f90:310-343).
template <typename T, int N>
__global__ void __launch_bounds__(kr_nt<N>(), (kr_minb<T, N, false>())) kr_s_kernel(T* __restrict__ s,
                                                          const T* __restrict__ r,
                                                          const T* __restrict__ q, Geom g,
                                                          KSegs S) {
  const KSeg& sg = S.seg[kseg_of(S, blockIdx.x)];
  if (sg.status != kRunning) return;
  const T na = (T)(-sg.alpha);
  KR_COLUMNS(N, g, { s[o] = xadd(xmul(na, q[o]), r[o]); })
}

// out = A x (calc_ax, blas.f90:556-600, the reference's term order) with
// partial[b] = sum out.y0 and, for NDOT == 2, partial[nb + b] = sum out.out.
// CC: per-block constant coefficients cf8[b*8 + 0..6] rounded to T; else
// the seven coefficient fields of op.
template <typename T, int N, bool CC, int NDOT>
__global__ void __launch_bounds__(kr_nt<N>(), (kr_minb<T, N, true>())) kr_ax_kernel(
    T* __restrict__ out, const T* __restrict__ x, const T* __restrict__ cf8, Op<T> op,
    const T* __restrict__ y0, Geom g, KSegs S, double* __restrict__ partial) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  if (S.seg[kseg_of(S, b)].status != kRunning) return;
  T c[7];
  if (CC) {
#pragma unroll
    for (int q = 0; q < 7; q++) c[q] = cf8[(int64_t)b * 8 + q];
  }
  const int sy = g.sy, sz = g.sz;
  DotAcc<T> a0, a1;
  KR_COLUMNS(N, g, {
    if (!CC) {
      _Pragma("unroll") for (int q = 0; q < 7; q++) c[q] = op.A[q][o];
    }
    T a = xmul(c[1], x[o - 1]);
    a = xadd(a, xmul(c[2], x[o + 1]));
    a = xadd(a, xmul(c[3], x[o - sy]));
    a = xadd(a, xmul(c[4], x[o + sy]));
    a = xadd(a, xmul(c[5], x[o - sz]));
    a = xadd(a, xmul(c[6], x[o + sz]));
    a = xadd(a, xmul(c[0], x[o]));
    out[o] = a;
    a0.add(a, y0[o]);
    if (NDOT == 2) a1.add(a, a);
  })
  const double v0 = kr_block_sum(a0.value(), red);
  const double v1 = NDOT == 2 ? kr_block_sum(a1.value(), red) : 0.0;
  if (threadIdx.x == 0) {
    partial[b] = v0;
    if (NDOT == 2) partial[g.nb + b] = v1;
  }
}

// kr_ax for cubic 16^3 / 32^3 blocks with per-block constant coefficients:
// x and y0 streamed through shared memory one z-plane at a time
// (stream.cuh), 256 threads, each N*N/256 cells (i, j), (i, j + 256/N), ...
// of every plane, a warp per row segment.  Same arithmetic and the same
// products summed as kr_ax_kernel (each thread's cells in plane order).
template <typename T, int N, int VC, int S, int NT_ = 256>
struct AxStream {
  using R = PlaneRing<T, N, VC, S, true, 1>;
  static constexpr int NT = NT_;
  static constexpr size_t SMEM = R::SMEM;
  static constexpr int MINB = stream_minb<SMEM + 256, (NT_ == 256 ? 6 : 2048 / NT_)>();
};

template <typename T, int N, int VC, int NDOT, int S, int NT_ = 256>
__global__ void __launch_bounds__(NT_, (AxStream<T, N, VC, S, NT_>::MINB)) kr_ax_stream_kernel(
    T* __restrict__ out, const T* __restrict__ x, const T* __restrict__ cf8,
    const T* __restrict__ y0, Geom g, KSegs S_, double* __restrict__ partial, int* err) {
  using AS = AxStream<T, N, VC, S, NT_>;
  using R = typename AS::R;
  constexpr int NT = AS::NT, CPT = N * N / NT, LX = R::LX, LXY = R::LXY;
  static_assert(N * N % NT == 0, "whole planes per CTA");
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ double red[32];
  const int b = blockIdx.x, tid = threadIdx.x;
  if (S_.seg[kseg_of(S_, b)].status != kRunning) return;
  const int64_t base = (int64_t)b * g.bstride;
  R ring(smraw);
  const T* C[1] = {y0};
  if (tid == 0) ring.start(x, C, base);
  T c[7];
#pragma unroll
  for (int q = 0; q < 7; q++) c[q] = cf8[(int64_t)b * 8 + q];
  int o[CPT];
#pragma unroll
  for (int k = 0; k < CPT; k++) {
    const int e = tid + k * NT;
    o[k] = R::at(e % N, e / N);
  }
  DotAcc<T> a0, a1;
  __syncthreads();  // the ring's barriers are initialised
  const bool ok = plane_walk(ring, x, C, base, err, tid, [&](int m) {
    const T* xm = ring.xp(m);
    const T* xc = ring.xp(m + 1);
    const T* xu = ring.xp(m + 2);
    const T* yp = ring.cp(m + 1, 0);
    T* op = out + base + (int64_t)(VC + m) * LXY;
#pragma unroll
    for (int k = 0; k < CPT; k++) {
      const int q = o[k];
      T a = xmul(c[1], xc[q - 1]);
      a = xadd(a, xmul(c[2], xc[q + 1]));
      a = xadd(a, xmul(c[3], xc[q - LX]));
      a = xadd(a, xmul(c[4], xc[q + LX]));
      a = xadd(a, xmul(c[5], xm[q]));
      a = xadd(a, xmul(c[6], xu[q]));
      a = xadd(a, xmul(c[0], xc[q]));
      op[q] = a;
      a0.add(a, yp[q]);
      if (NDOT == 2) a1.add(a, a);
    }
  });
  // a copy that never arrived (the error word says so) makes the sums NaN,
  // so the segment's scalars break down instead of going on
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const double v0 = kr_block_sum(ok ? a0.value() : nan, red);
  const double v1 = NDOT == 2 ? kr_block_sum(ok ? a1.value() : nan, red) : 0.0;
  if (tid == 0) {
    partial[b] = v0;
    if (NDOT == 2) partial[g.nb + b] = v1;
  }
}

template <typename T, int N, int VC, int NDOT, int S>
static cudaError_t kr_ax_stream_one(T* out, const T* x, const T* cf8, const T* y0, const Geom& g,
                                    KSegs S_, double* partial, int* err, cudaStream_t st) {
  using AS = AxStream<T, N, VC, S>;
  auto kern = kr_ax_stream_kernel<T, N, VC, NDOT, S>;
  // set once per process (not a stream operation; runs before any CUDA-graph
  // capture of these launches)
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)AS::SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  kern<<<g.nb, AS::NT, AS::SMEM, st>>>(out, x, cf8, y0, g, S_, partial, err);
  return cudaGetLastError();
}

// Ring depths: 32^3 4 slots (FP32: 6 CTAs per SM, FP64: 3); 16^3 8 (FP32)
// and 6 (FP64).  Measured on 2920 blocks of 32^3 (FP32, two inner
// products): 294 us at 4 slots, 322 at 5-6, 397 at 8 (fewer CTAs per SM),
// 394 for the column walk.
template <typename T, int N, int VC>
static cudaError_t kr_ax_stream(T* out, const T* x, const T* cf8, const T* y0, int ndot,
                                const Geom& g, KSegs S_, double* partial, int* err,
                                cudaStream_t st) {
  constexpr int SS = N == 32 ? 4 : (sizeof(T) == 4 ? 8 : 6);
  return ndot == 2 ? kr_ax_stream_one<T, N, VC, 2, SS>(out, x, cf8, y0, g, S_, partial, err, st)
                   : kr_ax_stream_one<T, N, VC, 1, SS>(out, x, cf8, y0, g, S_, partial, err, st);
}

// kr_xr for cubic 16^3 / 32^3 blocks: the six fields it reads streamed
// through shared memory one z-plane at a time (interior rows only,
// stream.cuh), x and r written from registers.  Same arithmetic and inner
// products as kr_xr_kernel.
template <typename T, int N, int VC, int S>
struct XrStream {
  using R = PlaneRing<T, N, VC, S, false, 6>;
  static constexpr int NT = 256;
  static constexpr size_t SMEM = R::SMEM;
  static constexpr int MINB = stream_minb<SMEM + 256, 6>();
};

template <typename T, int N, int VC, int S>
__global__ void __launch_bounds__(256, (XrStream<T, N, VC, S>::MINB)) kr_xr_stream_kernel(
    T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p_, const T* __restrict__ s_,
    const T* __restrict__ s, const T* __restrict__ t, const T* __restrict__ r0, Geom g,
    KSegs S_, double* __restrict__ partial, int* err) {
  using XS = XrStream<T, N, VC, S>;
  using R = typename XS::R;
  constexpr int NT = XS::NT, CPT = N * N / NT, LXY = R::LXY;
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ double red[32];
  const int b = blockIdx.x, tid = threadIdx.x;
  const KSeg& sg = S_.seg[kseg_of(S_, b)];
  if (sg.status != kRunning) return;
  const T al = (T)sg.alpha, gm = (T)sg.gamma, ngm = (T)(-sg.gamma);
  const int64_t base = (int64_t)b * g.bstride;
  R ring(smraw);
  const T* C[6] = {x, p_, s_, s, t, r0};
  if (tid == 0) ring.start(nullptr, C, base);
  int o[CPT];
#pragma unroll
  for (int k = 0; k < CPT; k++) {
    const int e = tid + k * NT;
    o[k] = R::at(e % N, e / N);
  }
  DotAcc<T> a0, a1;
  __syncthreads();  // the ring's barriers are initialised
  const bool ok = plane_walk(ring, (const T*)nullptr, C, base, err, tid, [&](int m) {
    const T* xv = ring.cp(m, 0);
    const T* pv = ring.cp(m, 1);
    const T* sv_ = ring.cp(m, 2);
    const T* sv = ring.cp(m, 3);
    const T* tv = ring.cp(m, 4);
    const T* r0v = ring.cp(m, 5);
    const int64_t pl = base + (int64_t)(VC + m) * LXY;
#pragma unroll
    for (int k = 0; k < CPT; k++) {
      const int q = o[k];
      x[pl + q] = xadd(xadd(xmul(al, pv[q]), xmul(gm, sv_[q])), xv[q]);
      const T rv = xadd(xmul(ngm, tv[q]), sv[q]);
      r[pl + q] = rv;
      a0.add(rv, rv);
      a1.add(rv, r0v[q]);
    }
  });
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const double v0 = kr_block_sum(ok ? a0.value() : nan, red);
  const double v1 = kr_block_sum(ok ? a1.value() : nan, red);
  if (tid == 0) {
    partial[b] = v0;
    partial[g.nb + b] = v1;
  }
}

template <typename T, int N, int VC, int S>
static cudaError_t kr_xr_stream(T* x, T* r, const T* p_, const T* s_, const T* s, const T* t,
                                const T* r0, const Geom& g, KSegs S_, double* partial, int* err,
                                cudaStream_t st) {
  using XS = XrStream<T, N, VC, S>;
  auto kern = kr_xr_stream_kernel<T, N, VC, S>;
  // set once per process (not a stream operation; runs before any CUDA-graph
  // capture of these launches)
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)XS::SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  kern<<<g.nb, XS::NT, XS::SMEM, st>>>(x, r, p_, s_, s, t, r0, g, S_, partial, err);
  return cudaGetLastError();
}

// x = alpha p^ + gamma s^ + x (AXPBYPZ, ILS3D.h:783, blas.f90:345-377) and
// r = s - gamma t (AXPYZ, ILS3D.h:786), with partial[b] = r.r and
// partial[nb + b] = r.r0 (the next iteration's rho).
template <typename T, int N>
__global__ void __launch_bounds__(kr_nt<N>(), (kr_minb<T, N, true>())) kr_xr_kernel(
    T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p_, const T* __restrict__ s_,
    const T* __restrict__ s, const T* __restrict__ t, const T* __restrict__ r0, Geom g, KSegs S,
    double* __restrict__ partial) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  const KSeg& sg = S.seg[kseg_of(S, b)];
  if (sg.status != kRunning) return;
  const T al = (T)sg.alpha, gm = (T)sg.gamma, ngm = (T)(-sg.gamma);
  DotAcc<T> a0, a1;
  KR_COLUMNS(N, g, {
    x[o] = xadd(xadd(xmul(al, p_[o]), xmul(gm, s_[o])), x[o]);
    const T rv = xadd(xmul(ngm, t[o]), s[o]);
    r[o] = rv;
    a0.add(rv, rv);
    a1.add(rv, r0[o]);
  })
  const double v0 = kr_block_sum(a0.value(), red);
  const double v1 = kr_block_sum(a1.value(), red);
  if (threadIdx.x == 0) {
    partial[b] = v0;
    partial[g.nb + b] = v1;
  }
}

// partial[b] = x.y, partial[nb + b] = u.v (the set-up's b.b and r.r0, the
// mixed-precision driver's norms).
template <typename T, int N>
__global__ void __launch_bounds__(kr_nt<N>(), (kr_minb<T, N, true>())) kr_dot2_kernel(
    const T* __restrict__ x, const T* __restrict__ y, const T* __restrict__ u,
    const T* __restrict__ v, Geom g, double* __restrict__ partial) {
  __shared__ double red[32];
  DotAcc<T> a0, a1;
  KR_COLUMNS(N, g, {
    a0.add(x[o], y[o]);
    a1.add(u[o], v[o]);
  })
  const double v0 = kr_block_sum(a0.value(), red);
  const double v1 = kr_block_sum(a1.value(), red);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = v0;
    partial[g.nb + blockIdx.x] = v1;
  }
}

// keep-best: the whole brick of x into xbest where this iteration improved
// the segment's smallest residual.
template <typename T>
__global__ void __launch_bounds__(256) kr_best_kernel(T* __restrict__ xbest,
                                                      const T* __restrict__ x, Geom g,
                                                      KSegs S) {
  const int b = blockIdx.x;
  if (!S.seg[kseg_of(S, b)].improved) return;
  const int64_t base = (int64_t)b * g.bstride;
  for (int64_t e = threadIdx.x; e < g.bstride; e += blockDim.x) xbest[base + e] = x[base + e];
}

// Whole bricks of src into dst for the blocks of segments with flag[s] != 0.
template <typename T>
__global__ void __launch_bounds__(256) kr_seg_copy_kernel(T* __restrict__ dst,
                                                          const T* __restrict__ src, Geom g,
                                                          const int* __restrict__ seg_of,
                                                          const unsigned char* __restrict__ flag) {
  const int b = blockIdx.x;
  if (!flag[seg_of ? seg_of[b] : 0]) return;
  const int64_t base = (int64_t)b * g.bstride;
  for (int64_t e = threadIdx.x; e < g.bstride; e += blockDim.x) dst[base + e] = src[base + e];
}

// The mixed-precision driver's correction problem, per segment s with
// flag[s]: r32 = (float)(r64) * (float)scale[s] on the interior (the FP64
// residual rounded to FP32, then scaled to a unit norm in FP32).
template <int N>
__global__ void __launch_bounds__(kr_nt<N>(), (kr_minb<float, N, false>())) kr_seg_to32_kernel(
    float* __restrict__ r32, const double* __restrict__ r64, Geom g32, Geom g64,
    const int* __restrict__ seg_of, const unsigned char* __restrict__ flag,
    const double* __restrict__ scale) {
  const int b = blockIdx.x, sg = seg_of ? seg_of[b] : 0;
  if (!flag[sg]) return;
  const float f = (float)scale[sg];
  const int64_t shift = (int64_t)b * (g64.bstride - g32.bstride) + (g64.off0 - g32.off0);
  // g32 and g64 share block shape and vc: one cell's offsets differ by the
  // bricks' strides only
  KR_COLUMNS(N, g32, { r32[o] = xmul((float)r64[o + shift], f); })
}

// x64 += (double)((float)scale[s] * d32) on the interior, per segment with
// flag[s] (the correction scaled back in FP32, accumulated in FP64).
template <int N>
__global__ void __launch_bounds__(kr_nt<N>(), (kr_minb<double, N, false>())) kr_seg_acc_kernel(
    double* __restrict__ x64, const float* __restrict__ d32, Geom g32, Geom g64,
    const int* __restrict__ seg_of, const unsigned char* __restrict__ flag,
    const double* __restrict__ scale) {
  const int b = blockIdx.x, sg = seg_of ? seg_of[b] : 0;
  if (!flag[sg]) return;
  const float f = (float)scale[sg];
  const int64_t shift = (int64_t)b * (g64.bstride - g32.bstride) + (g64.off0 - g32.off0);
  KR_COLUMNS(N, g32, { x64[o + shift] = __dadd_rn(x64[o + shift], (double)xmul(f, d32[o])); })
}

// ---------------------------------------------------------------------------
// Per segment: reduce its blocks' partial sums (fixed order), then one stage
// of the scalar recurrence of ILS3D.h:663-844 in FP64.
__global__ void __launch_bounds__(256) kr_scalar_kernel(const double* __restrict__ partial, int nb,
                                                        KSegs S, int stage, int max_iter,
                                                        double eps2, int keep_best) {
  __shared__ double red[32];
  const int sgi = blockIdx.x;
  KSeg& sg = S.seg[sgi];
  if (stage != KS_INIT && sg.status != kRunning) return;
  const int f0 = S.seg_first ? S.seg_first[sgi] : 0;
  const int f1 = S.seg_first ? S.seg_first[sgi + 1] : nb;
  double v0 = 0.0, v1 = 0.0;
  for (int q = f0 + threadIdx.x; q < f1; q += blockDim.x) {
    v0 = __dadd_rn(v0, partial[q]);
    v1 = __dadd_rn(v1, partial[nb + q]);
  }
  v0 = kr_block_sum(v0, red);
  v1 = kr_block_sum(v1, red);
  if (threadIdx.x != 0) return;
  const double fmin = (double)FLT_MIN;
  if (stage == KS_INIT) {
    // v0 = b.b, v1 = r.r0 (ILS3D.h:690-716)
    if (S.seg_max_iter) max_iter = S.seg_max_iter[sgi];
    if (S.seg_eps2) eps2 = S.seg_eps2[sgi];
    sg.bb = v0;
    sg.rr0 = 1.0;
    sg.alpha = 0.0;
    sg.gamma = 1.0;
    sg.beta = 0.0;
    sg.res = 0.0;
    sg.best_rr = 1e300;
    sg.eps2 = eps2;
    sg.count = 1;
    sg.max_iter = max_iter;
    sg.improved = 0;
    sg.first = 1;
    sg.best_saved = 0;
    sg.keep_best = keep_best;
    sg.status = kRunning;
    if (S.seg_active && !S.seg_active[sgi]) {  // not part of this solve
      sg.count = 0;
      sg.status = kSkipped;
    } else if (fabs(v0) < fmin) {  // b = 0: nothing to solve
      sg.count = 0;
      sg.status = BCMG_SUCCESS;
    } else if (max_iter < 1) {
      sg.count = 0;
      sg.status = BCMG_NOT_CONVERGED;
    } else {
      sg.rr1 = v1;
      if (fabs(v1) < fmin) {
        sg.res = v1;
        sg.count = 0;
        sg.status = BCMG_BREAKDOWN;
      }
    }
  } else if (stage == KS_ALPHA) {
    // v0 = q.r0 (ILS3D.h:744-746)
    sg.improved = 0;
    const double a = sg.rr1 / v0;
    if (!isfinite(a)) sg.status = isnan(v0) ? BCMG_DIVERGED : BCMG_BREAKDOWN;
    else sg.alpha = a;
  } else if (stage == KS_GAMMA) {
    // v0 = t.s, v1 = t.t (ILS3D.h:771-781)
    if (v1 == 0.0) sg.status = BCMG_BREAKDOWN;
    else if (isnan(v1) || isnan(v0)) sg.status = BCMG_DIVERGED;
    else sg.gamma = v0 / v1;
  } else {
    // v0 = r.r, v1 = the next iteration's r.r0 (ILS3D.h:789-843)
    const double rr = v0;
    const double res = (fabs(sg.bb) > fmin) ? fabs(rr) / fabs(sg.bb) : fabs(rr);
    sg.res = res;
    if (res <= sg.eps2) {
      sg.status = BCMG_SUCCESS;
    } else if (isnan(res) || isinf(res)) {
      sg.status = BCMG_DIVERGED;
    } else {
      if (sg.keep_best && rr < sg.best_rr) {
        sg.best_rr = rr;
        sg.improved = 1;
        sg.best_saved = 1;
      }
      if (sg.count >= sg.max_iter) {
        sg.status = BCMG_NOT_CONVERGED;
      } else {
        sg.rr0 = sg.rr1;
        sg.rr1 = v1;
        sg.count += 1;
        sg.first = 0;
        if (fabs(v1) < fmin) {
          sg.res = v1;
          sg.count = 0;
          sg.status = BCMG_BREAKDOWN;
        } else {
          sg.beta = sg.rr1 / sg.rr0 * sg.alpha / sg.gamma;
        }
      }
    }
  }
}

// Per segment: out[2s] and out[2s+1], the sums of its blocks' two partial
// sums (fixed order).
__global__ void __launch_bounds__(256) kr_segsum_kernel(const double* __restrict__ partial, int nb,
                                                        KSegs S, double* __restrict__ out) {
  __shared__ double red[32];
  const int sgi = blockIdx.x;
  const int f0 = S.seg_first ? S.seg_first[sgi] : 0;
  const int f1 = S.seg_first ? S.seg_first[sgi + 1] : nb;
  double v0 = 0.0, v1 = 0.0;
  for (int q = f0 + threadIdx.x; q < f1; q += blockDim.x) {
    v0 = __dadd_rn(v0, partial[q]);
    v1 = __dadd_rn(v1, partial[nb + q]);
  }
  v0 = kr_block_sum(v0, red);
  v1 = kr_block_sum(v1, red);
  if (threadIdx.x == 0) {
    out[2 * sgi] = v0;
    out[2 * sgi + 1] = v1;
  }
}

// ---------------------------------------------------------------------------
template <int N>
static int kr_threads(const Geom&) {
  return kr_nt<N>();
}

static int kr_shape(const Geom& g) {
  if (g.nx == g.ny && g.ny == g.nz && (g.nx == 8 || g.nx == 16 || g.nx == 32)) return g.nx;
  return 0;
}

#define KR_DISPATCH(CALL)                  \
  switch (kr_shape(g)) {                   \
    case 8: CALL(8); break;                \
    case 16: CALL(16); break;              \
    case 32: CALL(32); break;              \
    default: CALL(0); break;               \
  }

template <typename T>
cudaError_t launch_kr_p(T* p, const T* r, const T* q, const Geom& g, KSegs S, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
#define C_(N) kr_p_kernel<T, N><<<g.nb, kr_threads<N>(g), 0, st>>>(p, r, q, g, S)
  KR_DISPATCH(C_)
#undef C_
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_kr_s(T* s, const T* r, const T* q, const Geom& g, KSegs S, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
#define C_(N) kr_s_kernel<T, N><<<g.nb, kr_threads<N>(g), 0, st>>>(s, r, q, g, S)
  KR_DISPATCH(C_)
#undef C_
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_kr_ax(T* out, const T* x, Op<T> op, const T* y0, int ndot, const Geom& g,
                         KSegs S, double* partial, int* err, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  const bool cc = op.cc && op.cf8;
  if (cc && plane_stream_enabled() && (g.vc == 1 || g.vc == 2) &&
      (g.nx == 16 || g.nx == 32) && stream_aligned<T>(g, x, y0) &&
      (reinterpret_cast<uintptr_t>(out) % 16) == 0) {
    if (g.nx == 32)
      return g.vc == 1 ? kr_ax_stream<T, 32, 1>(out, x, op.cf8, y0, ndot, g, S, partial, err, st)
                       : kr_ax_stream<T, 32, 2>(out, x, op.cf8, y0, ndot, g, S, partial, err, st);
    return g.vc == 1 ? kr_ax_stream<T, 16, 1>(out, x, op.cf8, y0, ndot, g, S, partial, err, st)
                     : kr_ax_stream<T, 16, 2>(out, x, op.cf8, y0, ndot, g, S, partial, err, st);
  }
#define C_(N)                                                                                     \
  if (cc && ndot == 2)                                                                            \
    kr_ax_kernel<T, N, true, 2><<<g.nb, kr_threads<N>(g), 0, st>>>(out, x, op.cf8, op, y0, g, S,  \
                                                                   partial);                      \
  else if (cc)                                                                                    \
    kr_ax_kernel<T, N, true, 1><<<g.nb, kr_threads<N>(g), 0, st>>>(out, x, op.cf8, op, y0, g, S,  \
                                                                   partial);                      \
  else if (ndot == 2)                                                                             \
    kr_ax_kernel<T, N, false, 2><<<g.nb, kr_threads<N>(g), 0, st>>>(out, x, op.cf8, op, y0, g, S, \
                                                                    partial);                     \
  else                                                                                            \
    kr_ax_kernel<T, N, false, 1><<<g.nb, kr_threads<N>(g), 0, st>>>(out, x, op.cf8, op, y0, g, S, \
                                                                    partial)
  KR_DISPATCH(C_)
#undef C_
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_kr_xr(T* x, T* r, const T* p_, const T* s_, const T* s, const T* t,
                         const T* r0, const Geom& g, KSegs S, double* partial, int* err,
                         cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  // 32^3 FP32: six planes a slot, 2 slots (4 CTAs per SM)
  if (sizeof(T) == 4 && g.nx == 32 && (g.vc == 1 || g.vc == 2) && plane_stream_enabled() &&
      stream_aligned<T>(g, x, r) && stream_aligned<T>(g, p_, s_) && stream_aligned<T>(g, s, t) &&
      stream_aligned<T>(g, r0, r0))
    return g.vc == 1 ? kr_xr_stream<T, 32, 1, 2>(x, r, p_, s_, s, t, r0, g, S, partial, err, st)
                     : kr_xr_stream<T, 32, 2, 2>(x, r, p_, s_, s, t, r0, g, S, partial, err, st);
#define C_(N) \
  kr_xr_kernel<T, N><<<g.nb, kr_threads<N>(g), 0, st>>>(x, r, p_, s_, s, t, r0, g, S, partial)
  KR_DISPATCH(C_)
#undef C_
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_kr_dot2(const T* x, const T* y, const T* u, const T* v, const Geom& g,
                           double* partial, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
#define C_(N) kr_dot2_kernel<T, N><<<g.nb, kr_threads<N>(g), 0, st>>>(x, y, u, v, g, partial)
  KR_DISPATCH(C_)
#undef C_
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_kr_best(T* xbest, const T* x, const Geom& g, KSegs S, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  kr_best_kernel<T><<<g.nb, 256, 0, st>>>(xbest, x, g, S);
  return cudaGetLastError();
}

cudaError_t launch_kr_scalar(const double* partial, int nb, KSegs S, int stage, int max_iter,
                             double eps2, int keep_best, cudaStream_t st) {
  kr_scalar_kernel<<<S.nseg, 256, 0, st>>>(partial, nb, S, stage, max_iter, eps2, keep_best);
  return cudaGetLastError();
}

cudaError_t launch_kr_segsum(const double* partial, int nb, KSegs S, double* out,
                             cudaStream_t st) {
  kr_segsum_kernel<<<S.nseg, 256, 0, st>>>(partial, nb, S, out);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_kr_seg_copy(T* dst, const T* src, const Geom& g, const int* seg_of,
                               const unsigned char* flag, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  kr_seg_copy_kernel<T><<<g.nb, 256, 0, st>>>(dst, src, g, seg_of, flag);
  return cudaGetLastError();
}

cudaError_t launch_kr_seg_to32(float* r32, const double* r64, const Geom& g32, const Geom& g64,
                               const int* seg_of, const unsigned char* flag, const double* scale,
                               cudaStream_t st) {
  if (g32.nb == 0) return cudaSuccess;
  const Geom& g = g32;
#define C_(N) \
  kr_seg_to32_kernel<N><<<g.nb, kr_threads<N>(g), 0, st>>>(r32, r64, g32, g64, seg_of, flag, scale)
  KR_DISPATCH(C_)
#undef C_
  return cudaGetLastError();
}

cudaError_t launch_kr_seg_acc(double* x64, const float* d32, const Geom& g32, const Geom& g64,
                              const int* seg_of, const unsigned char* flag, const double* scale,
                              cudaStream_t st) {
  if (g32.nb == 0) return cudaSuccess;
  const Geom& g = g32;
#define C_(N) \
  kr_seg_acc_kernel<N><<<g.nb, kr_threads<N>(g), 0, st>>>(x64, d32, g32, g64, seg_of, flag, scale)
  KR_DISPATCH(C_)
#undef C_
  return cudaGetLastError();
}

#define INST(T)                                                                                    \
  template cudaError_t launch_kr_p<T>(T*, const T*, const T*, const Geom&, KSegs, cudaStream_t);  \
  template cudaError_t launch_kr_s<T>(T*, const T*, const T*, const Geom&, KSegs, cudaStream_t);  \
  template cudaError_t launch_kr_ax<T>(T*, const T*, Op<T>, const T*, int, const Geom&, KSegs,    \
                                       double*, int*, cudaStream_t);                              \
  template cudaError_t launch_kr_xr<T>(T*, T*, const T*, const T*, const T*, const T*, const T*,  \
                                       const Geom&, KSegs, double*, int*, cudaStream_t);          \
  template cudaError_t launch_kr_dot2<T>(const T*, const T*, const T*, const T*, const Geom&,     \
                                         double*, cudaStream_t);                                  \
  template cudaError_t launch_kr_best<T>(T*, const T*, const Geom&, KSegs, cudaStream_t);        \
  template cudaError_t launch_kr_seg_copy<T>(T*, const T*, const Geom&, const int*,               \
                                             const unsigned char*, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace bcmg
