// Preconditioned CG (src/pcg.jl:16-60) on the device, the Jacobi diagonal and
// the adjoint gradient kernel.
//
// One CG iteration is a fixed sequence of launches that all read a device
// "done" flag first, so the host can enqueue many iterations ahead and only
// read the flag back every `check_every` iterations; the iteration count and
// the returned x are exactly those of the sequential loop.
//
//   pdir   : h = dinv .* r, p = h + beta p                      (r, dinv, p -> p)
//   apply  : Ap = mask(QQ'(hlmz(p)))                            (fused kernel + fixup)
//   dot    : partial sums of p .* Ap .* mult
//   alpha  : alpha = t / pAp, k += 1                            (one block)
//   update : x += alpha p, r -= alpha Ap, partial t' = r.h.mult, max|r|
//   beta   : beta = t'/t, done = !(max|r| > tol) || k == maxiter
//
// Reductions are two-stage with a fixed grid, so results are deterministic.
// mult = 1/(copies) is computed from the local index (1, 1/2 or 1/4).
// Mixed precision (SEM_MIXED): FP64 defect correction x += A32^{-1} r with
// r = b - A x recomputed in FP64 after every inner FP32 CG solve.
// SEM_MIXED_RR: one FP32 CG with residual replacement, r32 <- (float)(b - A x)
// in FP64 whenever r32 has fallen by inner_tol, keeping the search direction.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "sem_arith.cuh"
#include "sem_internal.cuh"

namespace sem {

namespace {

constexpr int kRB = 1216;  // reduction grid, 8 blocks per SM (fixed: deterministic sums)
constexpr int kRT = 256;

struct Scalars {
  double t, t_prev, pAp, alpha, beta, rmax, tol;
  int k, maxiter, done, converged, nan;
};

__device__ __forceinline__ double mult_at(unsigned r, unsigned c, const Grid& g) {
  if (g.topo & M_MULT1) return 1.0;
  const int cc = copies_at(g, r, c);
  return cc == 1 ? 1.0 : (cc == 2 ? 0.5 : 0.25);
}

__device__ __forceinline__ double nanmax(double a, double b) {
  return (b > a || b != b) ? b : a;
}

template <int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV], const bool (&is_max)[NV],
                                             double* out) {
  __shared__ double sh[NV][kRT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_down_sync(0xffffffffu, x, o);
      x = is_max[q] ? nanmax(x, y) : x + y;
    }
    if (lane == 0) sh[q][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double x = sh[q][0];
      for (int i = 1; i < kRT / 32; ++i) x = is_max[q] ? nanmax(x, sh[q][i]) : x + sh[q][i];
      out[blockIdx.x * NV + q] = x;
    }
  }
}

template <int NV>
__device__ __forceinline__ void final_reduce(const double* part, int nparts,
                                             const bool (&is_max)[NV], double (&res)[NV]) {
  // single block, fixed order
  double v[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = is_max[q] ? 0.0 : 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x)
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = is_max[q] ? nanmax(v[q], part[i * NV + q]) : v[q] + part[i * NV + q];
  __shared__ double sh[NV][kRT];
#pragma unroll
  for (int q = 0; q < NV; ++q) sh[q][threadIdx.x] = v[q];
  __syncthreads();
  for (int s = kRT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
#pragma unroll
      for (int q = 0; q < NV; ++q)
        sh[q][threadIdx.x] = is_max[q] ? nanmax(sh[q][threadIdx.x], sh[q][threadIdx.x + s])
                                       : sh[q][threadIdx.x] + sh[q][threadIdx.x + s];
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < NV; ++q) res[q] = sh[q][0];
}

// Per-thread accumulators of the vector kernels.  GB300 runs FP64 at 1/64 of
// the FP32 rate, so for FP64 vectors the products and sums of the dots are
// formed in double-float on the FP32 pipe and max|r| is an integer maximum of
// the magnitude bits (NaN patterns order above Inf, so a NaN propagates); only
// the x and r updates stay native FP64 FMAs.  FP32 vectors accumulate in FP32
// (the inner solve of the mixed-precision CG).
template <class T>
struct Acc;

template <>
struct Acc<double> {
  df s = {0.0f, 0.0f};
  unsigned long long mx = 0ull;
  // s += a * b * m with m an exact power of two
  __device__ __forceinline__ void prod(double a, double b, double m) {
    df p = df_mul_u(d2df(a), d2df(b));
    const float mf = (float)m;
    p.h *= mf;
    p.l *= mf;
    s = df_add_u(s, p);
  }
  // s += a * (a * d) * m  (the Jacobi-weighted residual dot r.h.mult)
  __device__ __forceinline__ void rhr(double a, double d, double m) {
    const df ad = d2df(a);
    df h = df_mul_u(ad, d2df(d));
    const float mf = (float)m;
    h.h *= mf;
    h.l *= mf;
    s = df_fma_u(ad, h, s);
  }
  __device__ __forceinline__ void amax(double a) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
    mx = b > mx ? b : mx;
  }
  __device__ __forceinline__ double sum() const { return df2d(df_norm(s)); }
  __device__ __forceinline__ double max() const { return __longlong_as_double((long long)mx); }
};

// Native FP64 accumulation for the SEM_F64 solves: the dots span the whole
// double range (the double-float accumulators above are bound to the FP32
// exponent range), at the FP64 rate.
struct AccN {
  double s = 0.0;
  unsigned long long mx = 0ull;
  __device__ __forceinline__ void prod(double a, double b, double m) { s = __fma_rn(__dmul_rn(a, m), b, s); }
  __device__ __forceinline__ void rhr(double a, double d, double m) {
    s = __fma_rn(a, __dmul_rn(__dmul_rn(a, d), m), s);
  }
  __device__ __forceinline__ void amax(double a) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
    mx = b > mx ? b : mx;
  }
  __device__ __forceinline__ double sum() const { return s; }
  __device__ __forceinline__ double max() const { return __longlong_as_double((long long)mx); }
};

template <class T, bool NAT>
struct AccOf {
  typedef Acc<T> type;
};
template <>
struct AccOf<double, true> {
  typedef AccN type;
};

template <>
struct Acc<float> {
  float s = 0.0f;
  unsigned mx = 0u;
  __device__ __forceinline__ void prod(float a, float b, double m) { s = __fmaf_rn(a * (float)m, b, s); }
  __device__ __forceinline__ void rhr(float a, float d, double m) { s = __fmaf_rn(a, a * d * (float)m, s); }
  __device__ __forceinline__ void amax(float a) {
    const unsigned b = __float_as_uint(a) & 0x7fffffffu;
    mx = b > mx ? b : mx;
  }
  __device__ __forceinline__ double sum() const { return (double)s; }
  __device__ __forceinline__ double max() const { return (double)__uint_as_float(mx); }
};

// p = h + beta p_old with h = r .* dinv
// x = 0, r = b (converted), p = 0; partials of t = r.h.mult and max|r|
// (p == NULL: p is kept, the residual replacement of SEM_MIXED_RR)
template <class T, class TB, bool NAT = false>
__global__ void k_init(const TB* __restrict__ b, T* __restrict__ x, T* __restrict__ r,
                       T* __restrict__ p, const T* __restrict__ dinv, double* part, Grid g) {
  typename AccOf<T, NAT>::type acc;
  for_each_point(g, [&](unsigned rr, unsigned cc, long long i) {
    const T ri = (T)b[i];
    x[i] = (T)0;
    if (p) p[i] = (T)0;
    r[i] = ri;
    if (dinv)
      acc.rhr(ri, dinv[i], mult_at(rr, cc, g));
    else
      acc.prod(ri, ri, mult_at(rr, cc, g));
    acc.amax(ri);
  });
  double v[2] = {acc.sum(), acc.max()};
  const bool mx[2] = {false, true};
  block_reduce<2>(v, mx, part);
}

__global__ void k_scal_init(const double* part, int np, Scalars* sc, double tol, int maxiter) {
  double res[2];
  const bool mx[2] = {false, true};
  final_reduce<2>(part, np, mx, res);
  if (threadIdx.x == 0) {
    sc->t = res[0];
    sc->t_prev = 1.0;
    sc->beta = 0.0;
    sc->alpha = 0.0;
    sc->rmax = res[1];
    sc->tol = tol;
    sc->k = 0;
    sc->maxiter = maxiter;
    sc->nan = res[1] != res[1];
    sc->converged = !(res[1] > tol) && !sc->nan;
    sc->done = !(res[1] > tol) || maxiter == 0;
  }
}

// after a residual replacement: t from the replaced residual, beta with the
// previous t (the recurrence continues), a new tolerance and iteration limit;
// k stays
__global__ void k_scal_replace(const double* part, int np, Scalars* sc, double tol, int maxiter) {
  double res[2];
  const bool mx[2] = {false, true};
  final_reduce<2>(part, np, mx, res);
  if (threadIdx.x == 0) {
    sc->t = res[0];
    sc->beta = sc->k > 0 ? res[0] / sc->t_prev : 0.0;
    sc->rmax = res[1];
    sc->tol = tol;
    sc->maxiter = maxiter;
    sc->nan = res[1] != res[1];
    sc->converged = !(res[1] > tol) && !sc->nan;
    sc->done = !(res[1] > tol) || sc->k >= sc->maxiter || sc->nan;
  }
}

template <class T, bool NAT = false>
__global__ void k_pdir(const T* __restrict__ r, const T* __restrict__ dinv, T* __restrict__ p,
                       const Scalars* sc, long long L) {
  pdl_trigger();
  pdl_wait();  // launched as a programmatic dependent inside the CG chunks
  if (sc->done) return;
  const T beta = (T)sc->beta;
  const bool jac = dinv != nullptr;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L;
       i += (long long)gridDim.x * blockDim.x) {
    if constexpr (NAT)  // native FP64 (the whole double range)
      p[i] = __fma_rn((double)beta, (double)p[i], jac ? __dmul_rn((double)r[i], (double)dinv[i]) : (double)r[i]);
    else
      p[i] = cg_direction(r[i], jac ? dinv[i] : (T)1, beta, p[i], jac);
  }
}

template <class T, bool NAT = false>
__global__ void k_dot_pap(const T* __restrict__ p, const T* __restrict__ Ap, double* part,
                          const Scalars* sc, Grid g) {
  pdl_trigger();
  pdl_wait();  // launched as a programmatic dependent inside the CG chunks
  if (sc->done) return;
  typename AccOf<T, NAT>::type acc;
  for_each_point(g, [&](unsigned rr, unsigned cc, long long i) {
    acc.prod(p[i], Ap[i], mult_at(rr, cc, g));
  });
  double v[1] = {acc.sum()};
  const bool mx[1] = {false};
  block_reduce<1>(v, mx, part);
}

__global__ void k_scal_alpha(const double* part, int np, Scalars* sc) {
  pdl_trigger();
  pdl_wait();  // launched as a programmatic dependent inside the CG chunks
  if (sc->done) return;
  double res[1];
  const bool mx[1] = {false};
  final_reduce<1>(part, np, mx, res);
  if (threadIdx.x == 0) {
    sc->pAp = res[0];
    sc->alpha = sc->t / res[0];
    sc->k += 1;
  }
}

// alpha = t / (p . A p) from the per-CTA parts of the operator launch before
// the update kernel (FP64 parts for native FP64 solves, double-float parts
// otherwise), formed by every block of the update kernel in one fixed order
// (thread-strided partial sums over kRT threads, then the block tree), so that
// all blocks hold the same value without a one-block kernel between the
// launches; block 0 records p . A p, alpha and the iteration count
template <bool NATP>
__device__ __forceinline__ double alpha_from_parts(const void* parts, long long np, Scalars* sc) {
  __shared__ double s_alpha;
  double pap;
  if constexpr (NATP) {
    double res[1];
    const bool mx[1] = {false};
    final_reduce<1>(static_cast<const double*>(parts), (int)np, mx, res);
    pap = res[0];
  } else {
    const df* part = static_cast<const df*>(parts);
    df x = {0.0f, 0.0f};
    for (long long i = threadIdx.x; i < np; i += blockDim.x) x = df_add(x, part[i]);
    x = block_sum_df(x);
    pap = df2d(x);  // valid in thread 0
  }
  if (threadIdx.x == 0) {
    const double a = sc->t / pap;
    s_alpha = a;
    if (blockIdx.x == 0) {
      sc->pAp = pap;
      sc->alpha = a;
      sc->k += 1;
    }
  }
  __syncthreads();
  return s_alpha;
}

// x += alpha p, r -= alpha A p and the per-block parts of r.h.mult and
// max|r|.  FOLD: alpha is formed here from the operator's p . A p parts
// (apart, anp), which must not alias part
template <class T, bool NAT = false, bool FOLD = false>
__global__ void k_update(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                         const T* __restrict__ Ap, const T* __restrict__ dinv, double* part,
                         Scalars* sc, Grid g, const void* apart, long long anp) {
  pdl_trigger();
  pdl_wait();  // launched as a programmatic dependent inside the CG chunks
  if (sc->done) return;
  double alpha_d;
  if constexpr (FOLD)
    alpha_d = alpha_from_parts<NAT>(apart, anp, sc);
  else
    alpha_d = sc->alpha;
  const T alpha = (T)alpha_d;
  typename AccOf<T, NAT>::type acc;
  for_each_point(g, [&](unsigned rr, unsigned cc, long long i) {
    x[i] = x[i] + alpha * p[i];
    const T ri = r[i] - alpha * Ap[i];
    r[i] = ri;
    if (dinv)
      acc.rhr(ri, dinv[i], mult_at(rr, cc, g));
    else
      acc.prod(ri, ri, mult_at(rr, cc, g));
    acc.amax(ri);
  });
  double v[2] = {acc.sum(), acc.max()};
  const bool mx[2] = {false, true};
  block_reduce<2>(v, mx, part);
}

__global__ void k_scal_beta(const double* part, int np, Scalars* sc) {
  pdl_trigger();
  pdl_wait();  // launched as a programmatic dependent inside the CG chunks
  if (sc->done) return;
  double res[2];
  const bool mx[2] = {false, true};
  final_reduce<2>(part, np, mx, res);
  if (threadIdx.x == 0) {
    sc->t_prev = sc->t;
    sc->t = res[0];
    sc->beta = res[0] / sc->t_prev;
    sc->rmax = res[1];
    const bool nan = (res[1] != res[1]) || (sc->alpha != sc->alpha);
    sc->nan = nan;
    sc->converged = !(res[1] > sc->tol) && !nan;
    sc->done = !(res[1] > sc->tol) || sc->k >= sc->maxiter || nan;
  }
}

// ---------------------------------------------------------------------------
// Jacobi diagonal (local part): nu*(sum_k Dr[k,i]^2 G11(k,j) + sum_l Ds[l,j]^2
// G22(i,l) + 2 Dr[i,i] Ds[j,j] G12(i,j)) + k B(i,j), with nu pointwise folded
// into G when a field is given
// ---------------------------------------------------------------------------
struct DiagArgs {
  double Dr[kMaxN * kMaxN];
  double Ds[kMaxN * kMaxN];
  double nu, k;
};

__global__ void k_diag_local(const __grid_constant__ DiagArgs a, const double* __restrict__ G11,
                             const double* __restrict__ G12, const double* __restrict__ G22,
                             const double* __restrict__ B, const double* __restrict__ nuf,
                             double* __restrict__ d, Grid g) {
  const long long L = g.NX * g.NY;
  const int n = g.n;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < L;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long c = idx / g.NX;
    const long long r = idx - c * g.NX;
    const long long ex = r / n, ey = c / n;
    const int i = (int)(r - ex * n), j = (int)(c - ey * n);
    double s = 0.0;
    for (int k = 0; k < n; ++k) {
      const long long pr = ex * n + k + c * g.NX;
      const long long ps = r + (ey * n + k) * g.NX;
      const double dr = a.Dr[k + i * n], ds = a.Ds[k + j * n];
      const double wr = nuf ? nuf[pr] : 1.0, ws = nuf ? nuf[ps] : 1.0;
      s += dr * dr * G11[pr] * wr + ds * ds * G22[ps] * ws;
    }
    const double w0 = nuf ? nuf[idx] : 1.0;
    s += 2.0 * a.Dr[i + i * n] * a.Ds[j + j * n] * G12[idx] * w0;
    d[idx] = a.nu * s + a.k * B[idx];
  }
}

// dinv = keep ? 1/d : 1 (masked entries of the diagonal are set to 1)
template <class T>
__global__ void k_diag_inv(const double* __restrict__ d, T* __restrict__ dinv, Grid g) {
  for_each_point(g, [&](unsigned r, unsigned c, long long idx) {
    const bool keep = !((g.rinfo[r] | g.cinfo[c]) & L_ZERO);
    dinv[idx] = keep ? (T)(1.0 / d[idx]) : (T)1;
  });
}

__global__ void k_diag_mask(double* __restrict__ d, Grid g) {
  for_each_point(g, [&](unsigned r, unsigned c, long long idx) {
    if ((g.rinfo[r] | g.cinfo[c]) & L_ZERO) d[idx] = 1.0;
  });
}

// r = b - Ax, max|r| partials (outer FP64 residual of the mixed solver)
__global__ void k_residual(const double* __restrict__ b, const double* __restrict__ Ax,
                           double* __restrict__ r, double* part, long long L) {
  double rm = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = b[i] - Ax[i];
    r[i] = v;
    rm = nanmax(rm, fabs(v));
  }
  double v[1] = {rm};
  const bool mx[1] = {true};
  block_reduce<1>(v, mx, part);
}

__global__ void k_scal_max(const double* part, int np, double* out) {
  double res[1];
  const bool mx[1] = {true};
  final_reduce<1>(part, np, mx, res);
  if (threadIdx.x == 0) *out = res[0];
}

__global__ void k_axpy_f2d(double* __restrict__ x, const float* __restrict__ d, long long L) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L;
       i += (long long)gridDim.x * blockDim.x)
    x[i] += (double)d[i];
}

__global__ void k_add_d(double* __restrict__ x, const double* __restrict__ d, long long L) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = x[i] + d[i];
}

__global__ void k_zero(double* __restrict__ x, long long L) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = 0.0;
}

// ---------------------------------------------------------------------------
// adjoint gradient: g = -(G11 lr ur + G12 (lr us + ls ur) + G22 ls us)
// ---------------------------------------------------------------------------
__global__ void k_adjoint_grad(const __grid_constant__ DiagArgs a, const double* __restrict__ lam,
                               const double* __restrict__ u, const double* __restrict__ G11,
                               const double* __restrict__ G12, const double* __restrict__ G22,
                               double* __restrict__ grad, Grid g) {
  const long long L = g.NX * g.NY;
  const int n = g.n;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < L;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long c = idx / g.NX;
    const long long r = idx - c * g.NX;
    const long long ex = r / n, ey = c / n;
    const int i = (int)(r - ex * n), j = (int)(c - ey * n);
    double lr = 0, ls = 0, ur = 0, us = 0;
    for (int k = 0; k < n; ++k) {
      const long long pr = ex * n + k + c * g.NX;
      const long long ps = r + (ey * n + k) * g.NX;
      const double dr = a.Dr[i + k * n], ds = a.Ds[j + k * n];
      lr = fma(dr, lam[pr], lr);
      ur = fma(dr, u[pr], ur);
      ls = fma(ds, lam[ps], ls);
      us = fma(ds, u[ps], us);
    }
    grad[idx] = -(G11[idx] * lr * ur + G12[idx] * (lr * us + ls * ur) + G22[idx] * ls * us);
  }
}

unsigned nblocks(long long L) {
  long long b = (L + kRT - 1) / kRT;
  if (b > kRB) b = kRB;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// workspace layout (bytes, 256-aligned pieces)
struct WS {
  double *r, *p, *Ap, *dinv, *d, *x64tmp;  // FP64 vectors
  float *r32, *p32, *Ap32, *x32, *dinv32;   // FP32 vectors (mixed)
  double* part;
  df* dpart;             // per-CTA parts of p.Ap of CG-fused operator launches
  long long dpart_n;
  SmallProb* small;      // problem record of the single-launch small-mesh solver
  Scalars* sc;
  double* dmax;
  Scalars* sc_h;  // pinned host mirror
};

int get_ws(sem_mesh* m, bool mixed, WS& w) {
  const long long L = m->g.NX * m->g.NY;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t v64 = al(sizeof(double) * L), v32 = al(sizeof(float) * L);
  const long long np = cg_apply_parts(m->g);
  const size_t need = 6 * v64 + 5 * v32 + al(sizeof(double) * kRB * 4) + al(sizeof(df) * np) +
                      al(sizeof(SmallProb)) + al(sizeof(Scalars)) + al(sizeof(double));
  if (m->ws_bytes < need) {
    if (m->ws) cudaFree(m->ws);
    m->ws = nullptr;
    m->ws_bytes = 0;
    SEM_CUDA(cudaMalloc(&m->ws, need));
    m->ws_bytes = need;
  }
  (void)mixed;
  char* p = static_cast<char*>(m->ws);
  w.r = (double*)p; p += v64;
  w.p = (double*)p; p += v64;
  w.Ap = (double*)p; p += v64;
  w.dinv = (double*)p; p += v64;
  w.d = (double*)p; p += v64;
  w.x64tmp = (double*)p; p += v64;
  w.r32 = (float*)p; p += v32;
  w.p32 = (float*)p; p += v32;
  w.Ap32 = (float*)p; p += v32;
  w.x32 = (float*)p; p += v32;
  w.dinv32 = (float*)p; p += v32;
  w.part = (double*)p; p += al(sizeof(double) * kRB * 4);
  w.dpart = (df*)p; p += al(sizeof(df) * np);
  w.dpart_n = np;
  w.small = (SmallProb*)p; p += al(sizeof(SmallProb));
  w.sc = (Scalars*)p; p += al(sizeof(Scalars));
  w.dmax = (double*)p;
  static thread_local Scalars* host = nullptr;
  if (!host) SEM_CUDA(cudaMallocHost(&host, sizeof(Scalars) + sizeof(double)));
  w.sc_h = host;
  return SEM_OK;
}

// the operator a solve works on: grid, coefficient set and geometry, from a
// mesh handle or from caller-owned arrays
struct OpCtx {
  Grid g;
  const OperatorSet* ops;
  bool has_bc;
  const double *G11, *G12, *G22, *B;
  const float *G11f, *G12f, *G22f, *Bf;
  const void* Gdf;     // double-float split geometry (or NULL)
  unsigned* ctr;       // interface arrival counters (or NULL)
  const int* variant;  // per precision
};

OpCtx ctx_of(const sem_mesh* m) {
  OpCtx cx;
  cx.g = m->g;
  cx.ops = m->ops;
  cx.has_bc = m->has_bc;
  cx.G11 = m->G11;
  cx.G12 = m->G12;
  cx.G22 = m->G22;
  cx.B = m->B;
  cx.G11f = m->G11_f;
  cx.G12f = m->G12_f;
  cx.G22f = m->G22_f;
  cx.Bf = m->B_f;
  cx.Gdf = m->Gdf;
  cx.ctr = m->fix_ctr;
  cx.variant = m->variant;
  return cx;
}

int diag_build(const OpCtx& cx, const double* nu_field, double nu, double k, double* d,
               double* tmp, cudaStream_t s) {
  DiagArgs a;
  std::memset(&a, 0, sizeof(a));
  const int n = cx.g.n;
  std::memcpy(a.Dr, cx.ops->Dr, sizeof(double) * n * n);
  std::memcpy(a.Ds, cx.ops->Ds, sizeof(double) * n * n);
  a.nu = nu_field ? 1.0 : nu;
  a.k = k;
  const long long L = cx.g.NX * cx.g.NY;
  k_diag_local<<<nblocks(L) * 4, kRT, 0, s>>>(a, cx.G11, cx.G12, cx.G22, cx.B, nu_field, tmp, cx.g);
  SEM_CUDA(cudaGetLastError());
  SEM_CHECK(launch_gather_scatter(cx.g, tmp, d, cx.g.topo, s));
  return SEM_OK;
}

// one chunk of CG iterations (src/pcg.jl:36-55) followed by the copy of the
// device scalars to the host; every kernel returns at once when the device
// "done" flag is set, so iterations past convergence cost only launch slots
template <class T>
int enqueue_chunk(const OpCtx& cx, const Grid& gv, const WS& w, T* x, T* r, T* p, T* Ap,
                  const T* dinv, const ApplyCall& c, int check_every, cudaStream_t s) {
  const long long L = cx.g.NX * cx.g.NY;
  const unsigned nb = nblocks(L);
  const bool fused = c.cg_p != nullptr;  // direction and p.Ap inside the operator launch
  // every launch of a chunk is a programmatic dependent of the one before it:
  // it is scheduled while its predecessor finishes and waits for it
  // (griddepcontrol.wait) before it touches memory
  ApplyCall cp = c;
  cp.pdl = 1;
  const long long np = cg_apply_parts(cx.g);
  // the native FP64 operator writes FP64 parts of p.Ap and the solve's dots are
  // native FP64 (the whole double range); the other arithmetics use
  // double-float parts and dots
  const bool nat = sizeof(T) == 8 && c.precision == SEM_F64;
  // with the p.Ap parts in their own buffer (dpart), the update kernel forms
  // alpha itself: one launch fewer per iteration
  const bool fold = fused || cp.cg_dpart;
  for (int it = 0; it < check_every; ++it) {
    if (fused) {
      SEM_CHECK(launch_apply(cx.g, cx.ops, cp, s));
    } else if (cp.cg_dpart) {  // direction pass, then the operator with the p.Ap parts
      if (nat)
        SEM_CHECK(launch_pdl(k_pdir<T, true>, nb, kRT, s, (const T*)r, dinv, p, (const Scalars*)w.sc, L));
      else
        SEM_CHECK(launch_pdl(k_pdir<T>, nb, kRT, s, (const T*)r, dinv, p, (const Scalars*)w.sc, L));
      SEM_CHECK(launch_apply(cx.g, cx.ops, cp, s));
    } else {
      if (nat)
        SEM_CHECK(launch_pdl(k_pdir<T, true>, nb, kRT, s, (const T*)r, dinv, p, (const Scalars*)w.sc, L));
      else
        SEM_CHECK(launch_pdl(k_pdir<T>, nb, kRT, s, (const T*)r, dinv, p, (const Scalars*)w.sc, L));
      SEM_CHECK(launch_apply(cx.g, cx.ops, cp, s));
      if (nat)
        SEM_CHECK(launch_pdl(k_dot_pap<T, true>, nb, kRT, s, (const T*)p, (const T*)Ap, w.part,
                             (const Scalars*)w.sc, gv));
      else
        SEM_CHECK(launch_pdl(k_dot_pap<T>, nb, kRT, s, (const T*)p, (const T*)Ap, w.part,
                             (const Scalars*)w.sc, gv));
      SEM_CHECK(launch_pdl(k_scal_alpha, 1, kRT, s, (const double*)w.part, (int)nb, w.sc));
    }
    const void* ap = w.dpart;
    if (fold && nat)
      SEM_CHECK(launch_pdl(k_update<T, true, true>, nb, kRT, s, x, r, (const T*)p, (const T*)Ap, dinv, w.part,
                           w.sc, gv, ap, np));
    else if (fold)
      SEM_CHECK(launch_pdl(k_update<T, false, true>, nb, kRT, s, x, r, (const T*)p, (const T*)Ap, dinv, w.part,
                           w.sc, gv, ap, np));
    else if (nat)
      SEM_CHECK(launch_pdl(k_update<T, true>, nb, kRT, s, x, r, (const T*)p, (const T*)Ap, dinv, w.part,
                           w.sc, gv, (const void*)nullptr, 0LL));
    else
      SEM_CHECK(launch_pdl(k_update<T>, nb, kRT, s, x, r, (const T*)p, (const T*)Ap, dinv, w.part,
                           w.sc, gv, (const void*)nullptr, 0LL));
    SEM_CHECK(launch_pdl(k_scal_beta, 1, kRT, s, (const double*)w.part, (int)nb, w.sc));
  }
  SEM_CUDA(cudaGetLastError());
  SEM_CUDA(cudaMemcpyAsync(w.sc_h, w.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  return SEM_OK;
}

// ---- CUDA graphs of the iteration chunks
// A mesh handle keeps one instantiated graph per vector type (FP64/DF and the
// FP32 inner solve), keyed by every argument the captured launches bake in.
// A solve with the same key replays it; a different key re-captures and
// updates the executable graph in place (cudaGraphExecUpdate), or
// re-instantiates it when the topology changed.
struct GraphKey {
  const void* ptr[10];
  ApplyCall c;
  Grid g, gv;
  const OperatorSet* ops;
  int check_every;
  int tsize;
};
struct GraphEntry {
  bool valid;
  GraphKey key;
  cudaGraphExec_t exec;
};
struct GraphCache {
  cudaStream_t cap;  // private capture stream
  GraphEntry e[2];
};

template <class T>
int chunk_graph(sem_mesh* m, const OpCtx& cx, const Grid& gv, const WS& w, T* x, T* r, T* p, T* Ap,
                const T* dinv, const ApplyCall& c, int check_every, cudaGraphExec_t* out) {
  GraphKey key;
  std::memset(&key, 0, sizeof(key));  // padding bytes take part in the comparison
  const void* ptrs[10] = {x, r, p, Ap, dinv, w.sc, w.part, w.sc_h, cx.g.rinfo, cx.g.cinfo};
  std::memcpy(key.ptr, ptrs, sizeof(ptrs));
  key.c = c;
  key.g = cx.g;
  key.gv = gv;
  key.ops = cx.ops;
  key.check_every = check_every;
  key.tsize = (int)sizeof(T);
  GraphCache* gc = static_cast<GraphCache*>(m->graphs);
  if (!gc) {
    gc = new GraphCache;
    std::memset(gc, 0, sizeof(*gc));
    const cudaError_t e = cudaStreamCreateWithFlags(&gc->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete gc;
      return cuda_error(e, "cudaStreamCreate(capture)");
    }
    m->graphs = gc;
  }
  GraphEntry& ent = gc->e[sizeof(T) == 4 ? 1 : 0];
  if (ent.valid && std::memcmp(&ent.key, &key, sizeof(key)) == 0) {
    *out = ent.exec;
    return SEM_OK;
  }
  SEM_CUDA(cudaStreamBeginCapture(gc->cap, cudaStreamCaptureModeThreadLocal));
  const int st = enqueue_chunk<T>(cx, gv, w, x, r, p, Ap, dinv, c, check_every, gc->cap);
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(gc->cap, &graph);
  if (st != SEM_OK || ce != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return st != SEM_OK ? st : cuda_error(ce, "cudaStreamEndCapture");
  }
  bool ok = false;
  if (ent.valid) {
    cudaGraphExecUpdateResultInfo info;
    ok = cudaGraphExecUpdate(ent.exec, graph, &info) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      cudaGraphExecDestroy(ent.exec);
      ent.valid = false;
    }
  }
  if (!ok) {
    const cudaError_t ie = cudaGraphInstantiate(&ent.exec, graph, 0);
    if (ie != cudaSuccess) {
      cudaGraphDestroy(graph);
      return cuda_error(ie, "cudaGraphInstantiate");
    }
  }
  cudaGraphDestroy(graph);
  ent.valid = true;
  ent.key = key;
  *out = ent.exec;
  return SEM_OK;
}

// run CG iterations until done; T = double (F64/DF operator) or float (F32).
// With a mesh handle (m non-NULL) and kernel timing off, each chunk is one
// graph launch; otherwise the chunk's kernels are launched one by one.
template <class T>
int run_cg(sem_mesh* m, const OpCtx& cx, const Grid& gv, const WS& w, T* x, T* r, T* p, T* Ap,
           const T* dinv, int op_precision, const double* nu_field, double nu, double k,
           int check_every, Scalars* out, cudaStream_t s) {
  ApplyCall c;
  std::memset(&c, 0, sizeof(c));
  c.u = p;
  c.out = Ap;
  if (op_precision == SEM_F32) {
    c.G11 = cx.G11f;
    c.G12 = cx.G12f;
    c.G22 = cx.G22f;
    c.B = cx.Bf;
  } else {
    c.G11 = cx.G11;
    c.G12 = cx.G12;
    c.G22 = cx.G22;
    c.B = cx.B;
  }
  c.nu = nullptr;
  c.nu_s = nu_field ? 1.0 : nu;
  c.k_s = k;
  c.mode = cx.g.topo | M_STIFF | M_MASS | M_GS | (cx.has_bc ? M_MASK : 0u);
  if (nu_field) {
    if (op_precision == SEM_F32)
      return set_error(SEM_ERR_UNSUPPORTED, "a nu field is not served by the FP32 inner solve");
    c.nu = nu_field;
    c.mode |= M_NUG;
  }
  if (k == 0.0) c.mode &= ~M_MASS;
  c.precision = op_precision;
  c.variant = cx.variant[op_precision];
  c.Gdf = cx.Gdf;
  c.ctr = cx.ctr;
  c.skip = &w.sc->done;
  if (m) SEM_CHECK(use_kB(m, c, s));
  // CG-fused operator launches with the kernels that provide them (variants 2
  // and 5; double-float arithmetic also needs the pre-split geometry).  Their
  // unassembled p.Ap equals the mult-weighted dot only: unweighted dots
  // (mult = ones) keep the separate passes.
  const bool geo_ok = op_precision != SEM_F64_DF || c.Gdf;
  const bool parts_ok = w.dpart && cg_apply_parts(cx.g) <= w.dpart_n && !(gv.topo & M_MULT1);
  if ((c.variant == 2 || c.variant == 5) && geo_ok && parts_ok) {
    c.cg_r = r;
    c.cg_dinv = dinv;
    c.cg_p = p;
    c.cg_beta = &w.sc->beta;
    c.cg_dpart = w.dpart;
  } else if ((c.variant <= 1 || (c.variant != 4 && !geo_ok)) && parts_ok) {
    // the k_apply variants write the parts of p.Ap (no separate dot pass)
    c.cg_dpart = w.dpart;
  }
  cudaGraphExec_t exec = nullptr;
  if (m && !timing_enabled())
    SEM_CHECK(chunk_graph<T>(m, cx, gv, w, x, r, p, Ap, dinv, c, check_every, &exec));
  for (;;) {
    if (exec)
      SEM_CUDA(cudaGraphLaunch(exec, s));
    else
      SEM_CHECK(enqueue_chunk<T>(cx, gv, w, x, r, p, Ap, dinv, c, check_every, s));
    SEM_CUDA(cudaStreamSynchronize(s));
    if (w.sc_h->done) break;
  }
  *out = *w.sc_h;
  return SEM_OK;
}

// nu .* G11, nu .* G12, nu .* G22 rounded to FP32 (three blocks of L): the
// metric of the G-folded variable-coefficient operator for an FP32 inner solve
__global__ void k_nu_geom_f32(const double* __restrict__ nu, const double* __restrict__ G11,
                              const double* __restrict__ G12, const double* __restrict__ G22,
                              float* __restrict__ o, long long L) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = nu[i];
    o[i] = (float)(v * G11[i]);
    o[L + i] = (float)(v * G12[i]);
    o[2 * L + i] = (float)(v * G22[i]);
  }
}

// scratch of the FP32 metric nu .* G, freed in stream order
struct NuGeomF32 {
  cudaStream_t s;
  float* g = nullptr;
  explicit NuGeomF32(cudaStream_t st) : s(st) {}
  int build(const double* nu, const OpCtx& cx, long long L) {
    SEM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&g), sizeof(float) * 3 * (size_t)L, s));
    k_nu_geom_f32<<<nblocks(L) * 4, kRT, 0, s>>>(nu, cx.G11, cx.G12, cx.G22, g, L);
    SEM_CUDA(cudaGetLastError());
    return SEM_OK;
  }
  ~NuGeomF32() {
    if (g) cudaFreeAsync(g, s);
  }
};

// inverse Jacobi diagonal of the solve's operator into w.dinv (and w.dinv32
// for the mixed precisions)
int jacobi_build(const OpCtx& cx, const WS& w, const sem_pcg_opts* o, cudaStream_t s) {
  const unsigned nb = nblocks(cx.g.NX * cx.g.NY);
  SEM_CHECK(diag_build(cx, o->nu_field, o->nu, o->k, w.x64tmp, w.d, s));
  k_diag_inv<double><<<nb * 4, kRT, 0, s>>>(w.x64tmp, w.dinv, cx.g);
  if (o->precision == SEM_MIXED || o->precision == SEM_MIXED_RR)
    k_diag_inv<float><<<nb * 4, kRT, 0, s>>>(w.x64tmp, w.dinv32, cx.g);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

// whether the single-launch small-mesh solver serves this problem
bool small_eligible(const sem_mesh* m, const Grid& g, const sem_pcg_opts* o) {
  const int prec = o->precision;
  return m && g.NX * g.NY <= SEM_SMALL_MAX_LOCAL && g.n <= 11 && !o->nu_field &&
         df_window_ok(o->nu) && df_window_ok(o->k) &&
         (prec == SEM_F64_DF || prec == SEM_MIXED || prec == SEM_MIXED_RR);
}

// the record of one small-mesh solve (the geometry copies it reads are made
// on first use)
int small_record(const OpCtx& cx, const WS& w, sem_mesh* m, const sem_pcg_opts* o, const double* b,
                 double* x, int maxiter, SmallProb& sp, cudaStream_t s) {
  const int prec = o->precision;
  SEM_CHECK(ensure_df_geometry(m, s));
  if (prec != SEM_F64_DF) SEM_CHECK(ensure_f32_geometry(m, s));
  std::memset(&sp, 0, sizeof(sp));
  sp.n = cx.g.n;
  sp.Ex = cx.g.Ex;
  sp.Ey = cx.g.Ey;
  sp.NX = cx.g.NX;
  sp.NY = cx.g.NY;
  sp.rinfo = cx.g.rinfo;
  sp.cinfo = cx.g.cinfo;
  sp.has_bc = cx.has_bc;
  sp.jacobi = o->precond == SEM_PRECOND_JACOBI ? 1 : 0;
  sp.mult_ones = o->mult_ones ? 1 : 0;
  sp.nu = o->nu;
  sp.k = o->k;
  sp.tol = o->tol;
  sp.maxiter = maxiter;
  sp.precision = prec;
  const bool rr = prec == SEM_MIXED_RR;
  sp.inner_tol = o->inner_tol > 0 ? o->inner_tol : (rr ? 0.3 : 1e-4);
  sp.max_outer = o->max_outer > 0 ? o->max_outer : (rr ? 100 : 6);
  sp.b = b;
  sp.x = x;
  sp.r = w.r;
  sp.p = w.p;
  sp.raw = w.x64tmp;
  sp.dinv = w.dinv;
  sp.r32 = w.r32;
  sp.p32 = w.p32;
  sp.raw32 = w.Ap32;
  sp.x32 = w.x32;
  sp.dinv32 = w.dinv32;
  sp.Gdf = m->Gdf;
  sp.Gf = m->G11_f;
  return SEM_OK;
}

int default_maxiter(const Grid& g, const sem_pcg_opts* o) {
  const long long L = g.NX * g.NY;
  return o->maxiter > 0 ? o->maxiter : (int)(L > 2147483647LL ? 2147483647LL : L);
}

// argument checks shared by the solver entry points
int pcg_check(const sem_pcg_opts* o, const double* b, double* x) {
  if (!o || !b || !x) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (b == x) return set_error(SEM_ERR_BAD_ARG, "x must not alias b");
  if (o->precond != SEM_PRECOND_NONE && o->precond != SEM_PRECOND_JACOBI)
    return set_error(SEM_ERR_BAD_ARG, "unknown preconditioner %d", o->precond);
  const int prec = o->precision;
  if (prec != SEM_F64 && prec != SEM_F64_DF && prec != SEM_MIXED && prec != SEM_MIXED_RR)
    return set_error(SEM_ERR_BAD_ARG, "precision must be SEM_F64, SEM_F64_DF, SEM_MIXED or SEM_MIXED_RR");
  return SEM_OK;
}

// the FP64 operator of the solve (the mesh's FP64 arithmetic) applied to x
// into w.Ap, for residuals r = b - A x
ApplyCall residual_call(const OpCtx& cx, const sem_mesh* m, const sem_pcg_opts* o, const double* x,
                        const WS& w) {
  ApplyCall c;
  std::memset(&c, 0, sizeof(c));
  c.u = x;
  c.out = w.Ap;
  c.G11 = cx.G11;
  c.G12 = cx.G12;
  c.G22 = cx.G22;
  c.B = cx.B;
  c.nu_s = o->nu_field ? 1.0 : o->nu;
  c.k_s = o->k;
  c.mode = cx.g.topo | M_STIFF | M_GS | (o->k != 0.0 ? M_MASS : 0u) | (cx.has_bc ? M_MASK : 0u);
  if (o->nu_field) {
    c.nu = o->nu_field;
    c.mode |= M_NUG;
  }
  c.precision = m->precision;
  c.variant = cx.variant[m->precision];
  c.Gdf = cx.Gdf;
  c.ctr = cx.ctr;
  return c;
}

// Finishes a mixed-precision solve whose FP32 recurrences stopped gaining on
// the FP64 residual: the FP64 CG solves A d = r (r = b - A x in w.r) from
// d = 0 to the solve's tolerance, then x += d.  At most `budget` iterations.
int fp64_finish(sem_mesh* m, const OpCtx& cx, const Grid& gv, const WS& w, const sem_pcg_opts* o, double* x,
                int budget, bool jac, int check_every, Scalars* fr, cudaStream_t s) {
  const long long L = cx.g.NX * cx.g.NY;
  const unsigned nb = nblocks(L);
  double* d = w.x64tmp;
  double* rd = w.d;
  if (m->precision == SEM_F64)
    k_init<double, double, true><<<nb, kRT, 0, s>>>(w.r, d, rd, w.p, jac ? w.dinv : nullptr, w.part, gv);
  else
    k_init<double, double><<<nb, kRT, 0, s>>>(w.r, d, rd, w.p, jac ? w.dinv : nullptr, w.part, gv);
  k_scal_init<<<1, kRT, 0, s>>>(w.part, (int)nb, w.sc, o->tol, budget);
  SEM_CUDA(cudaGetLastError());
  SEM_CUDA(cudaMemcpyAsync(w.sc_h, w.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  SEM_CUDA(cudaStreamSynchronize(s));
  *fr = *w.sc_h;
  if (!fr->done)
    SEM_CHECK(run_cg<double>(m, cx, gv, w, d, rd, w.p, w.Ap, jac ? w.dinv : nullptr, m->precision,
                             o->nu_field, o->nu, o->k, check_every, fr, s));
  k_add_d<<<nb, kRT, 0, s>>>(x, d, L);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

// pcg (src/pcg.jl:16-60) on an operator context with workspace w; the mixed
// path needs the mesh handle m (FP32 geometry copies)
int pcg_core(const OpCtx& cx0, const WS& w, sem_mesh* m, const sem_pcg_opts* o, const double* b,
             double* x, sem_solve_info* info, cudaStream_t s) {
  const int prec = o->precision;
  OpCtx cx = cx0;
  const long long L = cx.g.NX * cx.g.NY;
  const int maxiter = default_maxiter(cx.g, o);
  int check_every = o->check_every > 0 ? o->check_every : (L < 200000 ? 64 : 16);
  const unsigned nb = nblocks(L);
  const bool jac = o->precond == SEM_PRECOND_JACOBI;
  Grid gv = cx.g;
  if (o->mult_ones) gv.topo |= M_MULT1;
  if (jac) SEM_CHECK(jacobi_build(cx, w, o, s));
  Scalars res;
  std::memset(&res, 0, sizeof(res));
  int outer = 0;
  double res0 = 0.0;
  const bool small_ok = w.small && small_eligible(m, cx.g, o);
  if (o->path == SEM_PATH_SMALL && !small_ok)
    return set_error(SEM_ERR_UNSUPPORTED,
                     "the small-mesh path serves meshes of at most %d local DOF, n <= 11, scalar nu, "
                     "SEM_F64_DF, SEM_MIXED or SEM_MIXED_RR", SEM_SMALL_MAX_LOCAL);
  if (small_ok && o->path != SEM_PATH_CHUNKED) {
    // the whole solve in one cluster launch
    SmallProb sp;
    SEM_CHECK(small_record(cx, w, m, o, b, x, maxiter, sp, s));
    SEM_CUDA(cudaMemcpyAsync(w.small, &sp, sizeof(sp), cudaMemcpyHostToDevice, s));
    // SEM_MIXED in a small cluster whose CTAs hold the FP32 working set in
    // shared memory, one strip of element rows each, when it fits (the
    // restarted form whose FP32 iterations the single-cluster kernel cannot
    // make cheaper than FP64 ones)
    const size_t tiny = tiny_smem_bytes(cx.g.n, cx.g.Ex, cx.g.Ey, o->k != 0.0, jac);
    if (prec == SEM_MIXED && tiny <= max_smem_optin())
      SEM_CHECK(launch_tiny_pcg(w.small, sp, *cx.ops, tiny, s));
    else
      SEM_CHECK(launch_small_pcg(w.small, *cx.ops, cx.g.n, s));
    SEM_CUDA(cudaMemcpyAsync(&sp, w.small, sizeof(sp), cudaMemcpyDeviceToHost, s));
    SEM_CUDA(cudaStreamSynchronize(s));
    res.k = sp.iters;
    res.rmax = sp.res_inf;
    res.nan = sp.nan;
    res.converged = sp.converged;
    outer = sp.outer;
    res0 = sp.res0_inf;
    if ((prec == SEM_MIXED || prec == SEM_MIXED_RR) && !res.converged && !res.nan && res.k < maxiter) {
      // the single-launch mixed solve ran out of sweeps or replacements: the
      // FP64 CG finishes from the current x, on the whole GPU
      const ApplyCall c = residual_call(cx, m, o, x, w);
      SEM_CHECK(launch_apply(cx.g, cx.ops, c, s));
      k_residual<<<nb, kRT, 0, s>>>(b, w.Ap, w.r, w.part, L);
      SEM_CUDA(cudaGetLastError());
      Scalars fr;
      SEM_CHECK(fp64_finish(m, cx, gv, w, o, x, maxiter - res.k, jac, check_every, &fr, s));
      res.k += fr.k;
      res.rmax = fr.rmax;
      res.nan = fr.nan;
      res.converged = fr.converged;
      ++outer;
    }
  } else if (prec != SEM_MIXED && prec != SEM_MIXED_RR) {
    if (prec == SEM_F64)
      k_init<double, double, true><<<nb, kRT, 0, s>>>(b, x, w.r, w.p, jac ? w.dinv : nullptr, w.part, gv);
    else
      k_init<double, double><<<nb, kRT, 0, s>>>(b, x, w.r, w.p, jac ? w.dinv : nullptr, w.part, gv);
    k_scal_init<<<1, kRT, 0, s>>>(w.part, (int)nb, w.sc, o->tol, maxiter);
    SEM_CUDA(cudaGetLastError());
    SEM_CUDA(cudaMemcpyAsync(w.sc_h, w.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
    SEM_CUDA(cudaStreamSynchronize(s));
    res0 = w.sc_h->rmax;
    res = *w.sc_h;
    if (!w.sc_h->done)
      SEM_CHECK(run_cg<double>(m, cx, gv, w, x, w.r, w.p, w.Ap, jac ? w.dinv : nullptr, prec, o->nu_field,
                               o->nu, o->k, check_every, &res, s));
  } else {
    if (!m) return set_error(SEM_ERR_UNSUPPORTED, "mixed precision needs a mesh handle");
    SEM_CHECK(ensure_f32_geometry(m, s));
    cx = ctx_of(m);
    // the FP32 inner operator; with a nu field its metric is nu .* G in FP32
    // (the G-folded operator with the coefficient already applied)
    OpCtx cxf = cx;
    NuGeomF32 nug(s);
    if (o->nu_field) {
      SEM_CHECK(nug.build(o->nu_field, cx, L));
      cxf.G11f = nug.g;
      cxf.G12f = nug.g + L;
      cxf.G22f = nug.g + 2 * L;
    }
    const double nu_in = o->nu_field ? 1.0 : o->nu;
    const bool rr = prec == SEM_MIXED_RR;
    // SEM_MIXED_RR replaces the FP32 residual after every 0.3-fold drop: rarer
    // replacements let the FP32 recurrence drift (cfg2: 0.3 -> 7,504 iterations,
    // 0.1 -> 10,365, 0.03 -> 29,513; the FP64 CG takes 6,974)
    const double inner_tol = o->inner_tol > 0 ? o->inner_tol : (rr ? 0.3 : 1e-4);
    const int max_outer = o->max_outer > 0 ? o->max_outer : (rr ? 100 : 6);
    // x = 0, r = b
    k_zero<<<nb, kRT, 0, s>>>(x, L);
    k_residual<<<nb, kRT, 0, s>>>(b, x, w.r, w.part, L);  // r = b - 0
    k_scal_max<<<1, kRT, 0, s>>>(w.part, (int)nb, w.dmax);
    SEM_CUDA(cudaMemcpyAsync(&w.sc_h[1], w.dmax, sizeof(double), cudaMemcpyDeviceToHost, s));
    SEM_CUDA(cudaStreamSynchronize(s));
    double rmax = *reinterpret_cast<double*>(&w.sc_h[1]);
    res0 = rmax;
    int total_it = 0;
    const ApplyCall c = residual_call(cx, m, o, x, w);
    bool nan = rmax != rmax;
    if (rr && !(rmax <= o->tol) && !nan) {
      // one FP32 CG; its residual is replaced by the FP64 b - A x whenever it
      // has fallen by inner_tol since the last replacement
      k_init<float, double><<<nb, kRT, 0, s>>>(w.r, w.x32, w.r32, w.p32, jac ? w.dinv32 : nullptr, w.part, gv);
      k_scal_init<<<1, kRT, 0, s>>>(w.part, (int)nb, w.sc, inner_tol * rmax, maxiter);
      SEM_CUDA(cudaGetLastError());
      // a segment (the FP32 iterations between replacements) that runs 4 times
      // longer than the longest before it (at least 500 iterations) has hit
      // the FP32 floor: the FP64 CG finishes the solve
      int seg_start = 0, longest = 0, seg_limit = maxiter;
      bool stalled = false;
      for (;;) {
        Scalars ir;
        SEM_CHECK(run_cg<float>(m, cxf, gv, w, w.x32, w.r32, w.p32, w.Ap32, jac ? w.dinv32 : nullptr, SEM_F32,
                                nullptr, nu_in, o->k, check_every, &ir, s));
        total_it = ir.k;
        stalled = !ir.converged && !ir.nan && ir.k >= seg_limit && seg_limit < maxiter;
        if (ir.k - seg_start > longest) longest = ir.k - seg_start;
        seg_start = ir.k;
        k_axpy_f2d<<<nb, kRT, 0, s>>>(x, w.x32, L);
        SEM_CHECK(launch_apply(cx.g, cx.ops, c, s));
        k_residual<<<nb, kRT, 0, s>>>(b, w.Ap, w.r, w.part, L);
        k_scal_max<<<1, kRT, 0, s>>>(w.part, (int)nb, w.dmax);
        SEM_CUDA(cudaGetLastError());
        SEM_CUDA(cudaMemcpyAsync(&w.sc_h[1], w.dmax, sizeof(double), cudaMemcpyDeviceToHost, s));
        SEM_CUDA(cudaStreamSynchronize(s));
        rmax = *reinterpret_cast<double*>(&w.sc_h[1]);
        nan = rmax != rmax || ir.nan;
        ++outer;
        if (rmax <= o->tol || nan || ir.k >= maxiter || outer >= max_outer || stalled) break;
        // replace: r32 = r (FP64 residual), x32 = 0, p32 kept
        const long long lim = (long long)ir.k + (longest > 125 ? 4LL * longest : 500LL);
        seg_limit = lim < maxiter ? (int)lim : maxiter;
        k_init<float, double><<<nb, kRT, 0, s>>>(w.r, w.x32, w.r32, nullptr, jac ? w.dinv32 : nullptr, w.part, gv);
        k_scal_replace<<<1, kRT, 0, s>>>(w.part, (int)nb, w.sc, inner_tol * rmax, seg_limit);
        SEM_CUDA(cudaGetLastError());
      }
    }
    while (!rr && !(rmax <= o->tol) && !nan && outer < max_outer) {
      ++outer;
      // inner FP32 CG on A d = r to inner_tol * |r|_inf
      k_init<float, double><<<nb, kRT, 0, s>>>(w.r, w.x32, w.r32, w.p32, jac ? w.dinv32 : nullptr, w.part, gv);
      k_scal_init<<<1, kRT, 0, s>>>(w.part, (int)nb, w.sc, inner_tol * rmax, maxiter);
      SEM_CUDA(cudaGetLastError());
      Scalars ir;
      SEM_CHECK(run_cg<float>(m, cxf, gv, w, w.x32, w.r32, w.p32, w.Ap32, jac ? w.dinv32 : nullptr, SEM_F32,
                              nullptr, nu_in, o->k, check_every, &ir, s));
      total_it += ir.k;
      k_axpy_f2d<<<nb, kRT, 0, s>>>(x, w.x32, L);
      SEM_CHECK(launch_apply(cx.g, cx.ops, c, s));
      k_residual<<<nb, kRT, 0, s>>>(b, w.Ap, w.r, w.part, L);
      k_scal_max<<<1, kRT, 0, s>>>(w.part, (int)nb, w.dmax);
      SEM_CUDA(cudaGetLastError());
      SEM_CUDA(cudaMemcpyAsync(&w.sc_h[1], w.dmax, sizeof(double), cudaMemcpyDeviceToHost, s));
      SEM_CUDA(cudaStreamSynchronize(s));
      rmax = *reinterpret_cast<double*>(&w.sc_h[1]);
      nan = rmax != rmax;
    }
    bool fin_conv = rmax <= o->tol;
    if (!fin_conv && !nan && total_it < maxiter) {
      // the FP32 solves stopped gaining on the FP64 residual (stalled
      // segment, or the sweep / replacement budget ran out)
      Scalars fr;
      SEM_CHECK(fp64_finish(m, cx, gv, w, o, x, maxiter - total_it, jac, check_every, &fr, s));
      total_it += fr.k;
      rmax = fr.rmax;
      nan = nan || fr.nan;
      fin_conv = fr.converged != 0;
      ++outer;
    }
    res.k = total_it;
    res.rmax = rmax;
    res.nan = nan;
    res.converged = fin_conv;
  }
  if (info) {
    info->iters = res.k;
    info->outer = outer;
    info->res_inf = res.rmax;
    info->res0_inf = res0;
    info->converged = res.converged;
  }
  if (res.nan) return set_error(SEM_ERR_NAN, "NaN/Inf in the residual after %d iterations", res.k);
  if (!res.converged)
    return set_error(SEM_ERR_NOT_CONVERGED, "warning: res: %.17g after %d iterations", res.rmax, res.k);
  return SEM_OK;
}


// pcg_core with the range guard of the pair and FP32 arithmetics: a solve
// whose scalar coefficients lie outside the double-float window runs in native
// FP64 from the start, and a double-float or mixed solve that ends in NaN or
// Inf although b is finite (a value the pair or FP32 format cannot carry), or
// whose b lies below 2^-60 in magnitude, is solved again in native FP64
// (operator, vectors and dots), on the chunked path.  A NaN or Inf in b
// itself is reported as before.
int pcg_guarded(const OpCtx& cx, const WS& w, sem_mesh* m, const sem_pcg_opts* o, const double* b, double* x,
                sem_solve_info* info, cudaStream_t s) {
  sem_pcg_opts o64 = *o;
  o64.precision = SEM_F64;
  o64.path = SEM_PATH_CHUNKED;
  if (o->precision != SEM_F64 && !(df_window_ok(o->nu) && df_window_ok(o->k)))
    return pcg_core(cx, w, m, &o64, b, x, info, s);
  sem_solve_info mine;
  std::memset(&mine, 0, sizeof(mine));
  const int st = pcg_core(cx, w, m, o, b, x, &mine, s);
  const double r0 = mine.res0_inf;
  // a right-hand side below 2^-60 takes the solve's vectors below the pair
  // format's accurate range (2^-101) by the usual 1e-12 reduction
  const bool tiny_b = r0 > 0.0 && r0 < 0x1p-60;
  if (o->precision != SEM_F64 &&
      ((st == SEM_ERR_NAN && r0 == r0 && r0 <= 1.7976931348623157e308) || tiny_b)) {
    const int st64 = pcg_core(cx, w, m, &o64, b, x, info, s);
    if (info) info->outer += mine.outer;
    return st64;
  }
  if (info) *info = mine;
  return st;
}

}  // namespace

void free_graph_cache(sem_mesh* m) {
  GraphCache* gc = static_cast<GraphCache*>(m->graphs);
  if (!gc) return;
  for (GraphEntry& e : gc->e)
    if (e.valid) cudaGraphExecDestroy(e.exec);
  if (gc->cap) cudaStreamDestroy(gc->cap);
  delete gc;
  m->graphs = nullptr;
}


// Jacobi inverse diagonal of a mesh's mask(QQ'(hlmz(., nu, k))) into dinv
// (tmp: one scratch field); used by the batched solver's set-up
int batch_diag(sem_mesh* m, double nu, double k, double* dinv, double* tmp, cudaStream_t s) {
  const OpCtx cx = ctx_of(m);
  SEM_CHECK(diag_build(cx, nullptr, nu, k, dinv, tmp, s));
  k_diag_inv<double><<<nblocks(m->g.NX * m->g.NY) * 4, kRT, 0, s>>>(dinv, dinv, m->g);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

bool small_path_taken(const sem_mesh* m, const sem_pcg_opts* o) {
  return o->path != SEM_PATH_CHUNKED && small_eligible(m, m->g, o);
}

int small_prepare(sem_mesh* m, const sem_pcg_opts* o, const double* b, double* x, SmallProb* rec,
                  cudaStream_t s) {
  SEM_CHECK(pcg_check(o, b, x));
  if (!small_path_taken(m, o)) return set_error(SEM_ERR_BAD_ARG, "problem is not served by the small path");
  WS w;
  SEM_CHECK(get_ws(m, o->precision == SEM_MIXED || o->precision == SEM_MIXED_RR, w));
  const OpCtx cx = ctx_of(m);
  if (o->precond == SEM_PRECOND_JACOBI) SEM_CHECK(jacobi_build(cx, w, o, s));
  return small_record(cx, w, m, o, b, x, default_maxiter(cx.g, o), *rec, s);
}

}  // namespace sem

using namespace sem;

extern "C" {

int sem_jacobi_diag(sem_mesh_t* m, const double* nu_field, double nu, double k, double* diag,
                    sem_stream_t stream) {
  if (!m || !diag) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  WS w;
  SEM_CHECK(get_ws(m, false, w));
  SEM_CHECK(diag_build(ctx_of(m), nu_field, nu, k, diag, w.d, s));
  if (m->has_bc) {
    k_diag_mask<<<nblocks(m->g.NX * m->g.NY) * 4, kRT, 0, s>>>(diag, m->g);
    SEM_CUDA(cudaGetLastError());
  }
  return SEM_OK;
}

int sem_adjoint_grad(sem_mesh_t* m, const double* lam, const double* u, double* grad,
                     unsigned flags, sem_stream_t stream) {
  if (!m || !lam || !u || !grad) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (grad == lam || grad == u) return set_error(SEM_ERR_BAD_ARG, "grad must not alias an input");
  cudaStream_t s = (cudaStream_t)stream;
  DiagArgs a;
  std::memset(&a, 0, sizeof(a));
  const int n = m->g.n;
  std::memcpy(a.Dr, m->Dr_h, sizeof(double) * n * n);
  std::memcpy(a.Ds, m->Ds_h, sizeof(double) * n * n);
  const long long L = m->g.NX * m->g.NY;
  double* dst = grad;
  WS w;
  if (flags & SEM_GS) {
    SEM_CHECK(get_ws(m, false, w));
    dst = w.d;
  }
  k_adjoint_grad<<<nblocks(L) * 4, kRT, 0, s>>>(a, lam, u, m->G11, m->G12, m->G22, dst, m->g);
  SEM_CUDA(cudaGetLastError());
  if (flags & SEM_GS) SEM_CHECK(launch_gather_scatter(m->g, dst, grad, m->g.topo, s));
  return SEM_OK;
}

int sem_pcg(sem_mesh_t* m, const sem_pcg_opts* o, const double* b, double* x,
            sem_solve_info* info, sem_stream_t stream) {
  if (!m) return set_error(SEM_ERR_BAD_ARG, "NULL mesh");
  SEM_CHECK(pcg_check(o, b, x));
  WS w;
  SEM_CHECK(get_ws(m, o->precision == SEM_MIXED || o->precision == SEM_MIXED_RR, w));
  return pcg_guarded(ctx_of(m), w, m, o, b, x, info, (cudaStream_t)stream);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free solve.
//
// Some callers cannot call cudaMalloc while they run: code inside an
// allocation-free region of a host application (a real-time loop, a memory
// manager that owns every device byte, a plug-in that may not grow the
// process's device footprint).  sem_pcg_noalloc serves them: the caller
// passes the geometry, b and x, and every scratch vector of the solve lives in
// the file-scope device array below.  Its size is fixed at build time.  With
// CUDA's default lazy module loading the array and the kernels are loaded on
// a device by the first call there, and stay until the process exits, so the
// first call (a warm-up of the same order and precision) belongs before any
// allocation-free region and before any stream capture.  The solve runs the
// direct operator kernel (variant 0, no pre-split geometry, which would need
// more scratch), so it is slower than a tuned sem_pcg on a mesh handle.
// ---------------------------------------------------------------------------
namespace sem {
namespace {

constexpr long long kNoAllocMaxLocal = SEM_NOALLOC_MAX_LOCAL;
constexpr size_t kNoAllocVec = (size_t)kNoAllocMaxLocal * sizeof(double);     // 256-multiple
constexpr size_t kNoAllocInfo = (((size_t)kNoAllocMaxLocal + 1) + 255) & ~(size_t)255;
constexpr size_t kNoAllocPart = ((sizeof(double) * kRB * 4) + 255) & ~(size_t)255;
// per-tile parts of p.Ap: at most one tile per element, n >= 2 points a side
constexpr long long kNoAllocTiles = kNoAllocMaxLocal / 4;
constexpr size_t kNoAllocDpart = (((size_t)kNoAllocTiles * sizeof(df)) + 255) & ~(size_t)255;
constexpr size_t kNoAllocBytes = 6 * kNoAllocVec + kNoAllocInfo + kNoAllocPart + kNoAllocDpart + 256 + 256;

}  // namespace
}  // namespace sem

static __device__ __align__(256) unsigned char g_noalloc_scratch[sem::kNoAllocBytes];

namespace sem {
namespace {

// device address of the scratch array for the current device.  The array's
// host-side name is not a device address; the lookup runs on every call, so a
// device whose context was reset and recreated gets the address of its new
// module image, never a stale one.
int noalloc_scratch(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
  *out = p;
  return SEM_OK;
}

__global__ void k_line_info(unsigned char* rinfo, unsigned char* cinfo, Grid g, int has_bc) {
  const unsigned t = g.topo;
  const long long tot = g.NX + g.NY;
  for (long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x; l < tot;
       l += (long long)gridDim.x * blockDim.x) {
    if (l < g.NX)
      rinfo[l] = line_info(l, g.n, g.Ex, (t & M_PERX) != 0, has_bc && (t & M_DXMIN), has_bc && (t & M_DXMAX));
    else
      cinfo[l - g.NX] = line_info(l - g.NX, g.n, g.Ey, (t & M_PERY) != 0, has_bc && (t & M_DYMIN),
                                  has_bc && (t & M_DYMAX));
  }
}

}  // namespace
}  // namespace sem

extern "C" int sem_pcg_noalloc(int nr, int Ex, int Ey, int periodic_x, int periodic_y,
                               const char* bc, const double* Dr, const double* Ds,
                               const double* G11, const double* G12, const double* G22,
                               const double* B, const sem_pcg_opts* o, const double* b, double* x,
                               sem_solve_info* info, sem_stream_t stream) {
  using namespace sem;
  SEM_CHECK(pcg_check(o, b, x));
  if (nr < 2 || Ex < 1 || Ey < 1) return set_error(SEM_ERR_BAD_ARG, "bad sizes nr=%d Ex=%d Ey=%d", nr, Ex, Ey);
  if (!Dr || !Ds || !G11 || !G12 || !G22 || !B) return set_error(SEM_ERR_BAD_ARG, "NULL geometry");
  if (bc && !(bc[0] && bc[1] && bc[2] && bc[3]))
    return set_error(SEM_ERR_BAD_ARG, "bc must be 4 chars of 'D'/'N'");
  if (bc)
    for (int i = 0; i < 4; ++i)
      if (bc[i] != 'D' && bc[i] != 'N') return set_error(SEM_ERR_BAD_ARG, "bc must be 4 chars of 'D'/'N'");
  if (o->precision == SEM_MIXED || o->precision == SEM_MIXED_RR)
    return set_error(SEM_ERR_UNSUPPORTED, "the allocation-free solve serves SEM_F64 and SEM_F64_DF");
  const long long NX = (long long)nr * Ex, NY = (long long)nr * Ey;
  if (NX * NY > kNoAllocMaxLocal)
    return set_error(SEM_ERR_BAD_ARG,
                     "the allocation-free solve holds at most %lld local DOF in its fixed scratch "
                     "array; this mesh has %lld (use sem_pcg)",
                     kNoAllocMaxLocal, NX * NY);
  OperatorSet ops;
  SEM_CHECK(init_operator_set(Dr, Ds, nr, &ops));
  void* base = nullptr;
  SEM_CHECK(noalloc_scratch(&base));
  cudaStream_t s = (cudaStream_t)stream;
  char* p = static_cast<char*>(base);
  WS w;
  std::memset(&w, 0, sizeof(w));
  w.r = (double*)p; p += kNoAllocVec;
  w.p = (double*)p; p += kNoAllocVec;
  w.Ap = (double*)p; p += kNoAllocVec;
  w.dinv = (double*)p; p += kNoAllocVec;
  w.d = (double*)p; p += kNoAllocVec;
  w.x64tmp = (double*)p; p += kNoAllocVec;
  unsigned char* info_tab = (unsigned char*)p; p += kNoAllocInfo;
  w.part = (double*)p; p += kNoAllocPart;
  w.dpart = (df*)p; p += kNoAllocDpart;
  w.dpart_n = kNoAllocTiles;
  w.sc = (Scalars*)p; p += 256;
  w.dmax = (double*)p;
  Scalars host_sc[2];
  w.sc_h = host_sc;  // pageable host copy: read back with a plain copy, no pinned allocation
  Grid g;
  std::memset(&g, 0, sizeof(g));
  g.n = nr;
  g.Ex = Ex;
  g.Ey = Ey;
  g.NX = NX;
  g.NY = NY;
  g.topo = (periodic_x ? M_PERX : 0u) | (periodic_y ? M_PERY : 0u);
  if (bc) {
    if (bc[0] == 'D') g.topo |= M_DXMIN;
    if (bc[1] == 'D') g.topo |= M_DXMAX;
    if (bc[2] == 'D') g.topo |= M_DYMIN;
    if (bc[3] == 'D') g.topo |= M_DYMAX;
  }
  g.rinfo = info_tab;
  g.cinfo = info_tab + NX;
  k_line_info<<<nblocks(NX + NY), kRT, 0, s>>>(info_tab, info_tab + NX, g, bc ? 1 : 0);
  SEM_CUDA(cudaGetLastError());
  static const int kDirect[4] = {0, 0, 0, 0};
  OpCtx cx;
  std::memset(&cx, 0, sizeof(cx));
  cx.g = g;
  cx.ops = &ops;
  cx.has_bc = bc != nullptr;
  cx.G11 = G11;
  cx.G12 = G12;
  cx.G22 = G22;
  cx.B = B;
  cx.variant = kDirect;
  return pcg_guarded(cx, w, nullptr, o, b, x, info, s);
}
