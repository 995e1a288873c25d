// Arithmetic policies of the fused operator kernels.
//
//  PF64 : FP64 storage, native FP64 arithmetic.
//  PF32 : FP32 storage and arithmetic (inner solve of the mixed-precision CG).
//  PDF  : FP64 storage, double-float arithmetic on the FP32 pipe.  GB300 runs
//         FP64 at about 1/64 of its FP32 rate, so a value is carried as an
//         unevaluated sum h + l of two floats (about 47 significant bits after
//         the input split below) and every product / sum is made error-free
//         with the TwoProd (fma) and TwoSum transformations of Dekker and
//         Knuth.  Accumulators stay unnormalised inside a dot product and are
//         renormalised once (fin).
#pragma once

#include <cuda_runtime.h>

#include "sem_internal.cuh"

namespace sem {

// ---------------------------------------------------------------------------
// error-free transformations (contraction-proof intrinsics)
// ---------------------------------------------------------------------------
__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

__device__ __forceinline__ df df_norm(df a) { return fast_two_sum(a.h, a.l); }

__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.h, b.h);
  float e = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
  return fast_two_sum(s.h, e);
}

// unnormalised sum (no final renormalisation; l may reach a few ulp(h))
__device__ __forceinline__ df df_add_u(df a, df b) {
  df s = two_sum(a.h, b.h);
  return {s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l))};
}

__device__ __forceinline__ df df_neg(df a) { return {-a.h, -a.l}; }

__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

// unnormalised product (h = rounded product of the high parts)
__device__ __forceinline__ df df_mul_u(df a, df b) {
  float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return {p, e};
}

// unnormalised c + a*b: the high parts are summed with TwoSum, all error terms
// are collected in l
__device__ __forceinline__ df df_fma_u(df a, df b, df c) {
  float p = __fmul_rn(a.h, b.h);
  float pe = __fmaf_rn(a.h, b.h, -p);
  pe = __fmaf_rn(a.h, b.l, pe);
  pe = __fmaf_rn(a.l, b.h, pe);
  df s = two_sum(p, c.h);
  return {s.h, __fadd_rn(s.l, __fadd_rn(pe, c.l))};
}

// GB300 runs every FP64 instruction, conversions included, at 1/64 of the FP32
// rate, so the conversions below use integer operations only (plus one FP32
// subtraction and, on the way out, one FP64 addition).
//
// double -> (h, l): h keeps the leading 24 significand bits (truncated), l the
// next 23; |x| in [2^-103, 2^128).  Outside that range: smaller magnitudes keep
// h only (normal floats) or flush to a signed zero (below 2^-126, far below any
// field value of this code's workloads), larger ones and Inf map to a signed
// Inf and NaN stays NaN.
__device__ __forceinline__ df d2df(double x) {
  const unsigned lo = (unsigned)__double2loint(x);
  const unsigned hi = (unsigned)__double2hiint(x);
  const unsigned ed = (hi >> 20) & 0x7ffu;
  const unsigned sg = hi & 0x80000000u;
  const unsigned hb = (__funnelshift_l(lo, hi, 3) + 0x40000000u) | sg;  // valid for ed in [897, 1150]
  const unsigned pb = (hb & 0xff800000u) - 0x0B800000u;
  const unsigned fb = pb | ((lo >> 6) & 0x007fffffu);
  float h = __uint_as_float(hb);
  float l = __fsub_rn(__uint_as_float(fb), __uint_as_float(pb));
  if (ed - 920u >= 231u) {  // rare: out of the split range (selects, no FP64 instruction)
    const bool nan = ed == 0x7ffu && (((hi & 0xfffffu) | lo) != 0u);
    const unsigned big = sg | 0x7f800000u | (nan ? 0x00400000u : 0u);
    h = __uint_as_float(ed > 1150u ? big : (ed >= 897u ? hb : sg));
    l = 0.0f;
  }
  return {h, l};
}

// Range guard of the double-float format.  Pairs keep about 47 bits for
// magnitudes from 2^-101 up to the FP32 range; the FP32 subnormals below give
// an absolute resolution of 2^-149.  Loads split with d2df_op, which turns a
// magnitude at or above 2^90 (and Inf) into NaN, so that intermediates never
// overflow silently, and a nonzero magnitude below 2^-126 (which the split
// would flush to zero) into NaN as well: a marker value would not survive the
// arithmetic (products of the smallest subnormals underflow to zero, and the
// derivative of a constant row is zero).  A NaN or Inf result flags the
// call, and so does a row whose stiffness sum (before nu) or result is tiny
// throughout, below 2^-90 and not zero: it is small because of its scale.
// The host side re-runs a flagged call in native FP64.
constexpr unsigned kDfExpHi = 1023u + 90u;   // first biased exponent that is poisoned
constexpr unsigned kDfExpLo = 1023u - 126u;  // nonzero values below this biased exponent are poisoned
constexpr float kRowTiny = 0x1p-90f;
__device__ __forceinline__ df d2df_op(double x) {
  const unsigned hi = (unsigned)__double2hiint(x);
  const unsigned mag = hi & 0x7fffffffu;
  df v = d2df(x);
  if (mag >= (kDfExpHi << 20) || (mag < (kDfExpLo << 20) && (mag | (unsigned)__double2loint(x)) != 0u))
    v = {__uint_as_float(0x7fc00000u), 0.0f};
  return v;
}

// a row of pairs whose largest magnitude lies in (0, 2^-90)
template <int N>
__device__ __forceinline__ bool df_row_tiny(const df (&v)[N]) {
  float m = 0.0f;
#pragma unroll
  for (int j = 0; j < N; ++j) m = fmaxf(m, fabsf(v[j].h));
  return m != 0.0f && m < kRowTiny;
}

// Geometry and mass-term guard: a point whose metric terms G11 and G22 both
// lie below 2^-40 in magnitude (a degenerate or absurdly scaled mesh: in 2D
// the metric terms are scale-free), or a nonzero k B product below 2^-100,
// would leave the pair format's accurate range inside the contraction.  The
// pre-split geometry turns such points into NaN pairs; the kernels that split
// on load test the same conditions.
constexpr float kGeoTiny = 0x1p-40f;
constexpr float kKbTiny = 0x1p-100f;
__host__ __device__ __forceinline__ bool geo_tiny(double g11, double g22) {
  const double m = fmax(fabs(g11), fabs(g22));
  return m != 0.0 && m < (double)kGeoTiny;
}
__device__ __forceinline__ bool geo_tiny(df g11, df g22) {  // FP32 pipe only
  const float m = fmaxf(fabsf(g11.h), fabsf(g22.h));
  return m != 0.0f && m < kGeoTiny;
}
__device__ __forceinline__ bool df_tiny_nz(df a, float t) {
  const float h = fabsf(a.h);
  return h != 0.0f && h < t;
}

// a double-float value whose high part is Inf or NaN
__device__ __forceinline__ bool df_bad(df a) { return (__float_as_uint(a.h) & 0x7f800000u) == 0x7f800000u; }

// host: whether a nonzero scalar coefficient lies in the double-float window
inline bool df_window_ok(double v) {
  if (v == 0.0) return true;
  const double a = v < 0 ? -v : v;
  return a >= 0x1p-70 && a < 0x1p90;
}

// exact float -> double by bit manipulation (subnormal floats flush to zero)
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned ef = (b >> 23) & 0xffu;
  const unsigned sg = b & 0x80000000u;
  unsigned hi = sg | ((ef + 896u) << 20) | ((b & 0x007fffffu) >> 3);
  unsigned lo = b << 29;
  if (ef == 0u) {
    hi = sg;
    lo = 0u;
  } else if (ef == 0xffu) {
    hi = sg | 0x7ff00000u | ((b & 0x007fffffu) ? 0x00080000u : 0u);
    lo = 0u;
  }
  return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ double df2d(df a) { return __dadd_rn(f2d_bits(a.h), f2d_bits(a.l)); }

// M .* v for M = 0 (src/mask.jl:14): a signed zero, NaN for Inf/NaN inputs,
// without an FP64 multiply
__device__ __forceinline__ double masked_zero(double v) {
  const long long b = __double_as_longlong(v);
  const bool special = ((b >> 52) & 0x7ff) == 0x7ff;
  return special ? __longlong_as_double(0x7ff8000000000000LL)
                 : __longlong_as_double(b & (long long)0x8000000000000000ULL);
}
__device__ __forceinline__ float masked_zero(float v) {
  const unsigned b = __float_as_uint(v);
  return ((b >> 23) & 0xffu) == 0xffu ? __uint_as_float(0x7fc00000u) : __uint_as_float(b & 0x80000000u);
}

// correctly rounded sums of stored values (never contracted into an FMA)
// Programmatic dependent launch (PTX griddepcontrol, sm_90 and later): a
// kernel calls pdl_trigger() to let the next kernel of its stream, when that
// one is launched with programmatic stream serialization, be scheduled before
// it has finished; that next kernel calls pdl_wait() before it reads anything
// the first one writes (it returns once the first grid has completed and its
// memory operations are visible).  Both are no-ops without such a launch.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ double io_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float io_add(float a, float b) { return __fadd_rn(a, b); }

// CG direction p = h + beta p_old with h = dinv .* r (Jacobi) or r, formed in
// double-float and rounded once for FP64 vectors, in FP32 for FP32 vectors
// (src/pcg.jl:40-45)
__device__ __forceinline__ double cg_direction(double r, double d, double beta, double p, bool jac) {
  const df rd = d2df(r);
  const df h = jac ? df_mul_u(rd, d2df(d)) : rd;
  return df2d(df_fma_u(d2df(beta), d2df(p), h));
}
__device__ __forceinline__ float cg_direction(float r, float d, float beta, float p, bool jac) {
  return __fmaf_rn(beta, p, jac ? r * d : r);
}

// block-wide double-float sum in a fixed order (warp trees, then the warps in
// order); the result is valid in thread 0.  Every thread of the block calls it.
// one term of the CG denominator p . A p, formed in double-float
__device__ __forceinline__ df dot_term(df a, df b) { return df_mul_u(a, b); }
__device__ __forceinline__ df dot_term(double a, double b) { return df_mul_u(d2df(a), d2df(b)); }
__device__ __forceinline__ df dot_term(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df block_sum_df(df x) {
  __shared__ df warp_sums[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  for (int o = 16; o > 0; o >>= 1) {
    const df y = {__shfl_down_sync(full, x.h, o), __shfl_down_sync(full, x.l, o)};
    x = df_add(x, y);
  }
  __syncthreads();  // warp_sums may still be read by a previous call
  if (lane == 0) warp_sums[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    x = warp_sums[0];
    for (int i = 1; i < nw; ++i) x = df_add(x, warp_sums[i]);
  }
  return x;
}

// block-wide FP64 sum in a fixed order (warp trees, then the warps in order);
// valid in thread 0; every thread of the block calls it
__device__ __forceinline__ double block_sum_d(double x) {
  __shared__ double warp_sums_d[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) x = __dadd_rn(x, __shfl_down_sync(0xffffffffu, x, o));
  __syncthreads();
  if (lane == 0) warp_sums_d[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    x = warp_sums_d[0];
    for (int i = 1; i < nw; ++i) x = __dadd_rn(x, warp_sums_d[i]);
  }
  return x;
}

// Each CTA's part of p . A p over its unassembled local products: native FP64
// for the FP64 policy (stored as a double in the 8-byte part slot), double-float
// otherwise.  Every thread of the block calls it.
template <class P, int N, class U, class R>
__device__ __forceinline__ void store_dot_part(const U& u, const R& res, df* dpart, long long slot) {
  if constexpr (P::kPrecision == SEM_F64) {
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < N; ++j) acc = __fma_rn((double)u(j), (double)res(j), acc);
    const double tot = block_sum_d(acc);
    if (threadIdx.x == 0) reinterpret_cast<double*>(dpart)[slot] = tot;
  } else {
    df acc = {0.0f, 0.0f};
#pragma unroll
    for (int j = 0; j < N; ++j) acc = df_add_u(acc, dot_term(u(j), res(j)));
    const df tot = block_sum_df(df_norm(acc));
    if (threadIdx.x == 0) dpart[slot] = tot;
  }
}

// ---------------------------------------------------------------------------
// policies
// ---------------------------------------------------------------------------
struct PF64 {
  typedef double io;
  typedef double v;
  static constexpr int kPrecision = SEM_F64;
  static __device__ __forceinline__ v ld(const io* p) { return __ldg(p); }
  static __device__ __forceinline__ v cvt(io x) { return x; }
  static __device__ __forceinline__ io st(v a) { return a; }
  static __device__ __forceinline__ v zero() { return 0.0; }
  static __device__ __forceinline__ v add(v a, v b) { return a + b; }
  static __device__ __forceinline__ v sub(v a, v b) { return a - b; }
  static __device__ __forceinline__ v add_u(v a, v b) { return a + b; }
  static __device__ __forceinline__ v sub_u(v a, v b) { return a - b; }
  static __device__ __forceinline__ v mul(v a, v b) { return a * b; }
  static __device__ __forceinline__ v fma(v a, v b, v c) { return __fma_rn(a, b, c); }
  static __device__ __forceinline__ v fin(v a) { return a; }
  static __host__ v from_double(double d) { return d; }
};

struct PF32 {
  typedef float io;
  typedef float v;
  static constexpr int kPrecision = SEM_F32;
  static __device__ __forceinline__ v ld(const io* p) { return __ldg(p); }
  static __device__ __forceinline__ v cvt(io x) { return x; }
  static __device__ __forceinline__ io st(v a) { return a; }
  static __device__ __forceinline__ v zero() { return 0.0f; }
  static __device__ __forceinline__ v add(v a, v b) { return a + b; }
  static __device__ __forceinline__ v sub(v a, v b) { return a - b; }
  static __device__ __forceinline__ v add_u(v a, v b) { return a + b; }
  static __device__ __forceinline__ v sub_u(v a, v b) { return a - b; }
  static __device__ __forceinline__ v mul(v a, v b) { return a * b; }
  static __device__ __forceinline__ v fma(v a, v b, v c) { return __fmaf_rn(a, b, c); }
  static __device__ __forceinline__ v fin(v a) { return a; }
  static __host__ v from_double(double d) { return (float)d; }
};

struct PDF {
  typedef double io;
  typedef df v;
  static constexpr int kPrecision = SEM_F64_DF;
  static __device__ __forceinline__ v ld(const io* p) { return d2df_op(__ldg(p)); }
  static __device__ __forceinline__ v cvt(io x) { return d2df_op(x); }
  static __device__ __forceinline__ io st(v a) { return df2d(a); }
  static __device__ __forceinline__ v zero() { return {0.0f, 0.0f}; }
  static __device__ __forceinline__ v add(v a, v b) { return df_add(a, b); }
  static __device__ __forceinline__ v sub(v a, v b) { return df_sub(a, b); }
  static __device__ __forceinline__ v add_u(v a, v b) { return df_add_u(a, b); }
  static __device__ __forceinline__ v sub_u(v a, v b) { return df_add_u(a, df_neg(b)); }
  static __device__ __forceinline__ v mul(v a, v b) { return df_mul_u(a, b); }
  static __device__ __forceinline__ v fma(v a, v b, v c) { return df_fma_u(a, b, c); }
  static __device__ __forceinline__ v fin(v a) { return df_norm(a); }
  static __host__ v from_double(double d) {
    float h = (float)d;
    float l = (float)(d - (double)h);
    return {h, l};
  }
};

}  // namespace sem
