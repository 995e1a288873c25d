// Native FP64 recomputation of one element tile, for the double-float kernels.
//
// The double-float arithmetic carries about 47 significand bits in the FP32
// exponent range.  Its operator inputs are split by d2df_op, which turns a
// nonzero value outside the window [2^-70, 2^90) into NaN, and an
// intermediate that overflows the FP32 range becomes Inf or NaN as well.  A
// tile whose double-float results hold such a value is recomputed here in
// native FP64 from the FP64 inputs, with the phases and shared-memory line
// exchanges of k_apply2, and stored over its double-float results before the
// cross-tile completion; every other tile keeps its double-float results.  So
// the double-float operator never returns a result outside its accuracy for a
// finite input: such tiles cost the FP64 rate instead.  (A result that is NaN
// in FP64 too, from a NaN or Inf input, stays NaN, as the reference's Float64
// arithmetic gives it.)  Included by sem_apply_kernels.cuh after
// tile_dss_store.
#pragma once

#include "sem_arith.cuh"

namespace sem {

// coefficient of a double-float set as the double it came from (h + l of two
// floats is exact in double)
__device__ __forceinline__ double df_exact(df v) { return __dadd_rn((double)v.h, (double)v.l); }

// y = D x in FP64 for a centro-antisymmetric D in even-odd form with
// double-float coefficients
template <int N>
__device__ __forceinline__ void eo_apply_f64(const EOCoef<N, df>& D, const double (&x)[N], double (&y)[N]) {
  constexpr int M = N / 2;
  double e[M], o[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    e[k] = __dadd_rn(x[k], x[N - 1 - k]);
    o[k] = __dsub_rn(x[k], x[N - 1 - k]);
  }
#pragma unroll
  for (int i = 0; i < M; ++i) {
    double s = __dmul_rn(df_exact(D.A[i][0]), o[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) s = __fma_rn(df_exact(D.A[i][k]), o[k], s);
    double t = __dmul_rn(df_exact(D.Cc[i][0]), e[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) t = __fma_rn(df_exact(D.Cc[i][k]), e[k], t);
    if (N & 1) t = __fma_rn(df_exact(D.cm[i]), x[M], t);
    y[i] = __dadd_rn(s, t);
    y[N - 1 - i] = __dsub_rn(s, t);
  }
  if (N & 1) {
    double s = __dmul_rn(df_exact(D.mr[0]), o[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) s = __fma_rn(df_exact(D.mr[k]), o[k], s);
    y[M] = s;
  }
}

// Recompute one element tile in FP64 and store it over the double-float
// results: the operator nu .* D'GD u (+ k B u) of the tile whose first element
// is (ex0, ey0), QQ' inside the tile and the mask (tile_dss_store), and, when
// dpart is not NULL, the tile's part of u . (A u) in slot `slot`.  S0 and S1
// are the kernel's two tile-sized line buffers (8-byte entries).  The caller
// has finished its own stores, so it holds almost no live state across this
// call (a non-inlined call in the middle of the kernel would make the hot path
// spill); every thread of the block calls it (it holds barriers).
template <int N, int TX, int TY>
__device__ __noinline__ void tile_f64_redo(const double* __restrict__ u, double* out, long long NX, int Ex, int Ey,
                                           int ex0, int ey0, unsigned mode, const double* __restrict__ G11,
                                           const double* __restrict__ G12, const double* __restrict__ G22,
                                           const double* __restrict__ B, const double* __restrict__ nu,
                                           double nu_s, double k_s, const EOCoef<N, df>* Dr,
                                           const EOCoef<N, df>* Drt, const EOCoef<N, df>* Ds,
                                           const EOCoef<N, df>* Dst, double* S0, double* S1, df* dpart,
                                           long long slot) {
  constexpr int SP = N | 1;
  constexpr int ES = N * SP;
  const int t = threadIdx.x;
  const int elem = t / N;
  const int lane = t - elem * N;
  const int ex = ex0 + elem % TX;
  const int ey = ey0 + elem / TX;
  const bool valid = ex < Ex && ey < Ey;
  const long long base = (long long)ex * N + lane + (long long)ey * N * NX;
  double* s1 = S1 + elem * ES;
  double uu[N], r[N];
  __syncthreads();  // the caller's stores may still read the line buffers
#pragma unroll
  for (int j = 0; j < N; ++j) uu[j] = valid ? u[base + (long long)j * NX] : 0.0;
  if (mode & M_STIFF) {
    double us[N];
#pragma unroll
    for (int j = 0; j < N; ++j) s1[j * SP + lane] = uu[j];
    eo_apply_f64<N>(*Ds, uu, us);
    __syncthreads();
    {
      double col[N], ur[N];
#pragma unroll
      for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
      eo_apply_f64<N>(*Dr, col, ur);
#pragma unroll
      for (int i = 0; i < N; ++i) s1[lane * SP + i] = ur[i];
    }
    __syncthreads();
    double os[N];
    {
      double ws[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const long long gi = base + (long long)j * NX;
        const double g11 = valid ? G11[gi] : 0.0, g12 = valid ? G12[gi] : 0.0, g22 = valid ? G22[gi] : 0.0;
        const double ur = s1[j * SP + lane];
        double wr = __fma_rn(g11, ur, __dmul_rn(g12, us[j]));
        ws[j] = __fma_rn(g12, ur, __dmul_rn(g22, us[j]));
        if (mode & M_NUG) {
          const double nv = valid ? nu[gi] : 0.0;
          wr = __dmul_rn(nv, wr);
          ws[j] = __dmul_rn(nv, ws[j]);
        }
        s1[j * SP + lane] = wr;
      }
      eo_apply_f64<N>(*Dst, ws, os);
    }
    __syncthreads();
    {
      double col[N], o[N];
#pragma unroll
      for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
      eo_apply_f64<N>(*Drt, col, o);
#pragma unroll
      for (int i = 0; i < N; ++i) s1[lane * SP + i] = o[i];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const double v = __dadd_rn(s1[j * SP + lane], os[j]);
      const double c = (mode & M_NU) ? (valid ? nu[base + (long long)j * NX] : 0.0) : nu_s;
      r[j] = __dmul_rn(c, v);
    }
  } else {
#pragma unroll
    for (int j = 0; j < N; ++j) r[j] = 0.0;
  }
  if (mode & M_MASS) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const double b = valid ? B[base + (long long)j * NX] : 0.0;
      r[j] = __fma_rn(__dmul_rn(k_s, b), uu[j], r[j]);
    }
  }
  if (dpart) {
    df acc = {0.0f, 0.0f};
#pragma unroll
    for (int j = 0; j < N; ++j) acc = df_add_u(acc, dot_term(uu[j], r[j]));
    const df tot = block_sum_df(df_norm(acc));
    if (threadIdx.x == 0) dpart[slot] = tot;
  }
  __syncthreads();  // every thread has read the line buffers
  tile_dss_store<PF64, N, TX, TY>(r, S1, S0, elem, lane, ex, ey, valid, base, Ex, Ey, NX, mode, out);
}

}  // namespace sem
