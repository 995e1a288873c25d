// Batched PCG: many independent mask(QQ'(hlmz)) systems of different sizes
// solved by persistent launches of thread-block clusters, one launch per
// polynomial order (each with the register budget of its order), all running
// concurrently.
//
// Each cluster (C CTAs of kBT threads; C chosen per launch) takes problems from a device
// work queue (problems sorted by estimated work, largest first) and runs the
// whole CG loop of src/pcg.jl:16-60 for one problem before taking the next.
// Inside a problem the cluster's CTAs share the element tiles (tile t goes to
// CTA t mod C) and every pointwise vector operation runs on the points
// of the CTA's own tiles, so one iteration needs three cluster barriers:
//
//   apply   own tiles: p = dinv.*r + beta p fused into the element operator,
//           Ap written (summed inside the tile), p.Ap.mult of finished points
//   barrier
//   fixup   cross-tile interface points of the problem, split over the cluster,
//           plus their p.Ap.mult;  cluster sum (DSMEM, fixed rank order) -> alpha
//   update  own points: x += alpha p, r -= alpha Ap, r.h.mult, max|r|;
//           cluster sum -> beta, convergence (identical in every CTA)
//
// SEM_MIXED runs FP64 defect correction around an FP32 inner CG inside the
// same launch.  Cluster barriers are hardware barriers; every decision that
// steers control flow is computed identically by all CTAs of a cluster.
#pragma once

#include <cooperative_groups.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "sem_apply2.cuh"

namespace cg = cooperative_groups;

namespace sem {

constexpr int kBT = 256;             // threads per CTA
constexpr int kBatchMaxN = 11;       // GLL points per direction served by the batch kernel

// CTAs of this CTA's cluster (the launch's cluster size: 2, 4, 8 or 16)
__device__ __forceinline__ int bcsize() {
  unsigned v;
  asm("mov.u32 %0, %%cluster_nctarank;" : "=r"(v));
  return (int)v;
}

__device__ __forceinline__ long long bclock_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return (long long)t;
}


template <int N>
struct BTile {  // element tile of the batch kernel: TX*TY*N <= kBT
  static constexpr int TX = N <= 2 ? 8 : (N <= 6 ? 8 : (N == 7 ? 6 : (N == 8 ? 8 : (N == 9 ? 7 : 5))));
  static constexpr int TY = N <= 2 ? 16 : (N == 3 ? 10 : (N == 4 ? 8 : (N == 5 ? 6 : (N == 6 ? 5 :
                            (N == 7 ? 6 : (N == 8 ? 4 : (N == 9 ? 4 : (N == 10 ? 5 : 4))))))));
  static constexpr int SP = N | 1;
  static constexpr int ES = N * SP;
  // element slots of one line buffer: every thread of the CTA owns one (the
  // threads beyond the tile write into slots no tile thread reads)
  static constexpr int SLOTS = (kBT + N - 1) / N;
  static_assert(TX * TY * N <= kBT, "tile exceeds the CTA");
};

struct BProb {
  int n, Ex, Ey;
  long long NX, NY;
  unsigned topo;  // M_PERX | M_PERY | M_D* | M_MASK
  double nu, k, tol;
  int maxiter;
  const df* Gdf;  // G11, G12, G22, B split into double-float pairs (4 blocks of NX*NY)
  const float *G11f, *G12f, *G22f, *Bf;
  const double* b;
  double* x;
  double *r, *p, *Ap, *dinv;
  float *r32, *p32, *Ap32, *x32, *dinv32;
  // results
  int iters, outer, converged, nan;
  double res_inf, res0_inf;
  // timeline: device clock (ns) when the cluster took the problem and when it
  // finished it, and the cluster (its index in the launch)
  long long t_start, t_end;
  int cluster;
};

// launch description shared by the per-order kernels
struct BatchCommon {
  BProb* probs;
  int count;
  int* queue;
  int precision;
  int jacobi;
  double inner_tol;
  int max_outer;
  int clusters;      // <= 0: as many as fit
  int cluster_size;  // CTAs per cluster: 2, 4, 8 or 16
  int ctas_per_sm;   // register budget of the kernel: 1 or 2 resident CTAs per SM
};

template <int N>
struct BatchArgs {
  BProb* probs;  // this order's problems, largest estimated work first
  int count;
  int* queue;
  int precision;  // SEM_F64_DF or SEM_MIXED
  int jacobi;
  double inner_tol;
  int max_outer;
  EOCoef<N, df> cdf[4];    // Dr, Dr', Ds, Ds' in double-float
  EOCoef<N, float> cf[4];  // the same in FP32 (inner solve)
};

// ---- per-thread accumulators: double-float sums (FP32 pipe) and the maximum
// of |value| as the bit pattern of a non-negative double (NaN sorts last)
template <class T>
struct BAcc;
template <>
struct BAcc<double> {
  df s = {0.0f, 0.0f};
  unsigned long long mx = 0ull;
  __device__ __forceinline__ void prod_v(df a, double b, float m) {
    df p = df_mul_u(a, d2df(b));
    p.h *= m;
    p.l *= m;
    s = df_add_u(s, p);
  }
  __device__ __forceinline__ void prod(double a, double b, float m) { prod_v(d2df(a), b, m); }
  __device__ __forceinline__ void rhr(double a, double d, float m) {
    const df ad = d2df(a);
    df h = df_mul_u(ad, d2df(d));
    h.h *= m;
    h.l *= m;
    s = df_fma_u(ad, h, s);
  }
  __device__ __forceinline__ void amax(double a) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(a) & 0x7fffffffffffffffull;
    mx = b > mx ? b : mx;
  }
  __device__ __forceinline__ df sum() const { return df_norm(s); }
  __device__ __forceinline__ unsigned long long max_bits() const { return mx; }
};
template <>
struct BAcc<float> {
  float s = 0.0f;
  unsigned mx = 0u;
  __device__ __forceinline__ void prod_v(float a, float b, float m) { s = __fmaf_rn(a * m, b, s); }
  __device__ __forceinline__ void prod(float a, float b, float m) { prod_v(a, b, m); }
  __device__ __forceinline__ void rhr(float a, float d, float m) { s = __fmaf_rn(a, a * d * m, s); }
  __device__ __forceinline__ void amax(float a) {
    const unsigned b = __float_as_uint(a) & 0x7fffffffu;
    mx = b > mx ? b : mx;
  }
  __device__ __forceinline__ df sum() const { return {s, 0.0f}; }
  __device__ __forceinline__ unsigned long long max_bits() const {
    return (unsigned long long)__double_as_longlong((double)__uint_as_float(mx));
  }
};

__device__ __forceinline__ double bpdir(double r, double d, double beta, double p, bool jac) {
  const df rd = d2df(r);
  const df h = jac ? df_mul_u(rd, d2df(d)) : rd;
  return df2d(df_fma_u(d2df(beta), d2df(p), h));
}
__device__ __forceinline__ float bpdir(float r, float d, float beta, float p, bool jac) {
  return __fmaf_rn(beta, p, jac ? r * d : r);
}

__device__ __forceinline__ double bits_to_double(unsigned long long b) {
  return __longlong_as_double((long long)b);
}

// copies of the node behind local row r of element e (1 or 2)
__device__ __forceinline__ int bcopies(int e, int i, int n, int E, bool per) {
  return ((i == 0 && (e > 0 || per)) || (i == n - 1 && (e < E - 1 || per))) ? 2 : 1;
}
__device__ __forceinline__ float bmult(int cc) { return cc == 1 ? 1.0f : (cc == 2 ? 0.5f : 0.25f); }

// shared state of the cluster reductions
struct BRed {
  df ws[2][kBT / 32];
  unsigned long long wm[2][kBT / 32];
  df slot_s[3][2];
  unsigned long long slot_m[3][2];
  df res_s[2];
  unsigned long long res_m[2];
};

// Cluster-wide sums (NS double-float values) and maxima (NM bit patterns) in a
// fixed order: warp trees, then the warps of a CTA in order, then the CTAs in
// rank order, so every CTA gets the same, deterministic result.  All the
// arithmetic runs on the FP32 pipe.  Calls rotate over three slots (rc counts
// the calls, identically in every thread of the cluster): a slot is written
// again only after two more cluster barriers, when no CTA still reads it.
template <int NS, int NM>
__device__ __forceinline__ void cluster_reduce(cg::cluster_group& cl, BRed& sh, int& rc, df (&s)[NS],
                                               unsigned long long (&m)[NM]) {
  const int slot = rc % 3;
  ++rc;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NS; ++q) {
    df x = s[q];
    for (int o = 16; o > 0; o >>= 1) {
      const df y = {__shfl_down_sync(0xffffffffu, x.h, o), __shfl_down_sync(0xffffffffu, x.l, o)};
      x = df_add(x, y);
    }
    if (lane == 0) sh.ws[q][w] = x;
  }
#pragma unroll
  for (int q = 0; q < NM; ++q) {
    unsigned long long x = m[q];
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long y = __shfl_down_sync(0xffffffffu, x, o);
      x = y > x ? y : x;
    }
    if (lane == 0) sh.wm[q][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NS; ++q) {
      df x = sh.ws[q][0];
      for (int i = 1; i < kBT / 32; ++i) x = df_add(x, sh.ws[q][i]);
      sh.slot_s[slot][q] = x;
    }
#pragma unroll
    for (int q = 0; q < NM; ++q) {
      unsigned long long x = sh.wm[q][0];
      for (int i = 1; i < kBT / 32; ++i) x = sh.wm[q][i] > x ? sh.wm[q][i] : x;
      sh.slot_m[slot][q] = x;
    }
  }
  cl.sync();
  // warp 0 combines the ranks' parts in rank order and shares the result
  // through shared memory (identical in every CTA)
  if (threadIdx.x == 0) {
    const int csz = bcsize();
#pragma unroll
    for (int q = 0; q < NS; ++q) {
      df x = *cl.map_shared_rank(&sh.slot_s[slot][q], 0);
      for (int rk = 1; rk < csz; ++rk) x = df_add(x, *cl.map_shared_rank(&sh.slot_s[slot][q], rk));
      sh.res_s[q] = x;
    }
#pragma unroll
    for (int q = 0; q < NM; ++q) {
      unsigned long long x = *cl.map_shared_rank(&sh.slot_m[slot][q], 0);
      for (int rk = 1; rk < csz; ++rk) {
        const unsigned long long y = *cl.map_shared_rank(&sh.slot_m[slot][q], rk);
        x = y > x ? y : x;
      }
      sh.res_m[q] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NS; ++q) s[q] = sh.res_s[q];
#pragma unroll
  for (int q = 0; q < NM; ++q) m[q] = sh.res_m[q];
}

// One element tile of the operator mask(QQ'(nu lapl(u) + k B u)) in the
// phases of k_apply2 (and with its arithmetic, so a tile's Ap equals the
// single-problem operator's), optionally with the CG direction update fused
// in front: u = p = dinv.*r + beta p_old.  Writes Ap (cross-tile points
// unsummed) and adds u.Ap.mult of the finished points to acc.  Every thread
// of the CTA calls it; S0, S1 and X0 have one element slot per thread.
template <class P, int N, int TX, int TY>
__device__ __noinline__ void btile(const BProb& pr, const EOCoef<N, typename P::v>* D, int bx, int by,
                      const typename P::io* u_src, const typename P::io* r, const typename P::io* dinv,
                      typename P::io beta, typename P::io* p, bool pdir, typename P::io* Ap,
                      const typename GeoT<P>::type* Geo, long long L, typename P::v* S0,
                      typename P::v* S1, typename P::io* X0, BAcc<typename P::io>& acc) {
  typedef typename P::v V;
  typedef typename P::io IO;
  typedef typename GeoT<P>::type GT;
  constexpr int SP = N | 1, ES = N * SP;
  const int t = threadIdx.x;
  const int elem = t / N;
  const int lane = t - elem * N;
  const bool inside = elem < TX * TY;
  const int exl = elem % TX, eyl = elem / TX;
  const int ex = bx * TX + exl, ey = by * TY + eyl;
  const bool valid = inside && ex < pr.Ex && ey < pr.Ey;
  const long long NX = pr.NX;
  const long long base = (long long)ex * N + lane + (long long)ey * N * NX;
  V* s0 = S0 + elem * ES;
  V* s1 = S1 + elem * ES;
  const GT* G11 = Geo;
  const GT* G12 = Geo + L;
  const GT* G22 = Geo + 2 * L;
  const GT* B = Geo + 3 * L;
  const bool jac = dinv != nullptr;

  // ---- A: row `lane` of u (the CG direction, formed here in pdir mode)
  V us[N];
  {
    V u[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
      IO v = 0;
      if (valid) {
        const long long gi = base + (long long)j * NX;
        if (pdir) {
          v = bpdir(r[gi], jac ? dinv[gi] : (IO)1, beta, p[gi], jac);
          p[gi] = v;
        } else {
          v = u_src[gi];
        }
      }
      u[j] = P::cvt(v);
      s0[j * SP + lane] = u[j];
      s1[j * SP + lane] = u[j];
    }
    eo_apply<P, N>(D[2], u, us);
  }
  __syncthreads();
  // ---- B: column `lane` in place; x-direction derivative
  {
    V col[N], ur[N];
#pragma unroll
    for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
    eo_apply<P, N>(D[0], col, ur);
#pragma unroll
    for (int i = 0; i < N; ++i) s1[lane * SP + i] = ur[i];
  }
  __syncthreads();
  // ---- C: row `lane` in place; metric terms, transposed y-derivative
  V os[N];
  {
    V ws[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const long long gi = base + (long long)j * NX;
      const V g11 = valid ? GeoT<P>::ld(G11 + gi) : P::zero();
      const V g12 = valid ? GeoT<P>::ld(G12 + gi) : P::zero();
      const V g22 = valid ? GeoT<P>::ld(G22 + gi) : P::zero();
      const V ur = s1[j * SP + lane];
      s1[j * SP + lane] = P::fma(g11, ur, P::mul(g12, us[j]));
      ws[j] = P::fma(g12, ur, P::mul(g22, us[j]));
    }
    eo_apply<P, N>(D[3], ws, os);
  }
  __syncthreads();
  // ---- D: column `lane` in place; transposed x-derivative
  {
    V col[N], o[N];
#pragma unroll
    for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
    eo_apply<P, N>(D[1], col, o);
#pragma unroll
    for (int i = 0; i < N; ++i) s1[lane * SP + i] = o[i];
  }
  __syncthreads();
  // ---- E: assemble nu (or + os) + k B u
  V res[N];
  const V nu = P::cvt((IO)pr.nu);
  const V kk = P::cvt((IO)pr.k);
#pragma unroll
  for (int j = 0; j < N; ++j) res[j] = P::fin(P::mul(nu, P::add(s1[j * SP + lane], os[j])));
  if (pr.k != 0.0) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const V b = valid ? GeoT<P>::ld(B + base + (long long)j * NX) : P::zero();
      res[j] = P::fin(P::fma(P::mul(kk, b), s0[j * SP + lane], res[j]));
    }
  }
  // ---- in-tile QQ', mask, store; u.Ap.mult of the finished points
  const bool perx = (pr.topo & M_PERX) != 0, pery = (pr.topo & M_PERY) != 0;
  const int cx = bcopies(ex, lane, N, pr.Ex, perx);
  tile_dss_store<P, N, TX, TY>(res, reinterpret_cast<IO*>(S1), X0, elem, lane, ex, ey, valid, base,
                               pr.Ex, pr.Ey, NX, pr.topo | M_GS, Ap, [&](int j, IO val) {
                                 acc.prod_v(s0[j * SP + lane], val, bmult(cx * bcopies(ey, j, N, pr.Ey, pery)));
                               });
  __syncthreads();  // the next tile overwrites the line buffers
}

// cross-tile QQ' completion (the interface rows of k_dss_fixup), work split
// over the whole cluster; adds p.Ap.mult of every copy it finishes
template <class IO, int TX, int TY>
__device__ __noinline__ void bfixup(const BProb& pr, int n, IO* __restrict__ Ap, const IO* __restrict__ p,
                       int rank, BAcc<IO>& acc) {
  FixArgs f;
  f.n = n;
  f.Ex = pr.Ex;
  f.Ey = pr.Ey;
  f.TX = TX;
  f.TY = TY;
  f.NX = pr.NX;
  f.NY = pr.NY;
  f.mode = pr.topo | M_GS;
  f.skip = nullptr;
  f.key_lo = 0;
  f.key_hi = 1LL << 62;
  f.gate = nullptr;
  f.gate_tag = 0;
  const bool perx = (pr.topo & M_PERX) != 0, pery = (pr.topo & M_PERY) != 0;
  f.nxi = (pr.Ex - 1) / TX + (perx ? 1 : 0);
  f.nyi = (pr.Ey - 1) / TY + (pery ? 1 : 0);
  const long long nI = fix_rows(f);
  const long long first = (long long)rank * kBT + threadIdx.x;
  const unsigned un = (unsigned)n;
  for (long long q = 0; q < nI; ++q)
    fix_interface(Ap, f, q, first, (long long)bcsize() * kBT, [&](long long r, long long c, IO v) {
      const int ex = (int)((unsigned)r / un), ey = (int)((unsigned)c / un);
      const int cc = bcopies(ex, (int)r - ex * n, n, pr.Ex, perx) * bcopies(ey, (int)c - ey * n, n, pr.Ey, pery);
      acc.prod(p[r + c * pr.NX], v, bmult(cc));
    });
}

// run `f(row, col, idx, mult)` over the points of this CTA's tiles
template <int N, int TX, int TY, class F>
__device__ __forceinline__ void own_points(const BProb& pr, int rank, F&& f) {
  const int ntx = (pr.Ex + TX - 1) / TX, nty = (pr.Ey + TY - 1) / TY;
  const int t = threadIdx.x;
  if (t >= TX * TY * N) return;
  const int elem = t / N, lane = t - elem * N;
  const int exl = elem % TX, eyl = elem / TX;
  const bool perx = (pr.topo & M_PERX) != 0, pery = (pr.topo & M_PERY) != 0;
  for (int tile = rank, csz = bcsize(); tile < ntx * nty; tile += csz) {
    const int by = tile / ntx, bx = tile - by * ntx;
    const int ex = bx * TX + exl, ey = by * TY + eyl;
    if (ex >= pr.Ex || ey >= pr.Ey) continue;
    const long long base = (long long)ex * N + lane + (long long)ey * N * pr.NX;
    const int cx = bcopies(ex, lane, N, pr.Ex, perx);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const int cc = cx * bcopies(ey, j, N, pr.Ey, pery);
      f(base + (long long)j * pr.NX, cc == 1 ? 1.0f : (cc == 2 ? 0.5f : 0.25f));
    }
  }
}

// shared-memory line buffers of one CTA
template <int N>
struct BBuf {
  df* S0;
  df* S1;
  double* X0;
  __device__ BBuf(unsigned char* smem) {
    constexpr size_t E = (size_t)BTile<N>::SLOTS * BTile<N>::ES;
    S0 = reinterpret_cast<df*>(smem);
    S1 = S0 + E;
    X0 = reinterpret_cast<double*>(S1 + E);
  }
  template <class P>
  __device__ typename P::v* s0() const { return reinterpret_cast<typename P::v*>(S0); }
  template <class P>
  __device__ typename P::v* s1() const { return reinterpret_cast<typename P::v*>(S1); }
  template <class P>
  __device__ typename P::io* x0() const { return reinterpret_cast<typename P::io*>(X0); }
};

// CG on A y = rhs (P: PDF for FP64 vectors, PF32 for the FP32 inner solve).
// rhs is read as double (b or the FP64 residual) and converted.
template <class P, int N>
__device__ void bcg(const BatchArgs<N>& a, BProb& pr, cg::cluster_group& cl, int rank,
                    const double* rhs, typename P::io* y, typename P::io* r, typename P::io* p,
                    typename P::io* Ap, const typename P::io* dinv, const typename GeoT<P>::type* Geo,
                    double tol, int maxiter, BRed& red, int& rc, const BBuf<N>& buf, int& iters,
                    double& rmax_out, bool& nan_out) {
  typedef typename P::io IO;
  typedef BTile<N> T;
  const EOCoef<N, typename P::v>* D;
  if constexpr (P::kPrecision == SEM_F32)
    D = a.cf;
  else
    D = a.cdf;
  const bool jac = dinv != nullptr;
  const long long L = pr.NX * pr.NY;
  const int ntx = (pr.Ex + T::TX - 1) / T::TX, nty = (pr.Ey + T::TY - 1) / T::TY;
  // init: y = 0, r = rhs, p = 0; t = r.h.mult, max|r|
  BAcc<IO> acc;
  own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float m) {
    const IO ri = (IO)rhs[i];
    y[i] = (IO)0;
    p[i] = (IO)0;
    r[i] = ri;
    if (jac)
      acc.rhr(ri, dinv[i], m);
    else
      acc.prod(ri, ri, m);
    acc.amax(ri);
  });
  df s1[1] = {acc.sum()};
  unsigned long long m1[1] = {acc.max_bits()};
  cluster_reduce<1, 1>(cl, red, rc, s1, m1);
  double t = df2d(s1[0]), rmax = bits_to_double(m1[0]);
  // the FP64-vector solve starts from x = 0: its first max|r| is max|b|
  if (P::kPrecision == SEM_F64_DF && rank == 0 && threadIdx.x == 0) pr.res0_inf = rmax;
  double tprev = 1.0;
  int k = 0;
  bool nan = rmax != rmax;
  bool done = !(rmax > tol) || maxiter == 0;
  while (!done) {
    const double beta = k == 0 ? 0.0 : t / tprev;
    BAcc<IO> dot;
    for (int tile = rank, csz = bcsize(); tile < ntx * nty; tile += csz) {
      const int by = tile / ntx, bx = tile - by * ntx;
      btile<P, N, T::TX, T::TY>(pr, D, bx, by, nullptr, r, dinv, (IO)beta, p, true, Ap, Geo, L,
                                buf.template s0<P>(), buf.template s1<P>(), buf.template x0<P>(), dot);
    }
    cl.sync();
    bfixup<IO, T::TX, T::TY>(pr, N, Ap, p, rank, dot);
    df s2[1] = {dot.sum()};
    unsigned long long m0[1] = {0ull};
    cluster_reduce<1, 1>(cl, red, rc, s2, m0);
    const double pap = df2d(s2[0]);
    const double alpha = t / pap;
    ++k;
    BAcc<IO> up;
    own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float m) {
      y[i] = y[i] + (IO)alpha * p[i];
      const IO ri = r[i] - (IO)alpha * Ap[i];
      r[i] = ri;
      if (jac)
        up.rhr(ri, dinv[i], m);
      else
        up.prod(ri, ri, m);
      up.amax(ri);
    });
    df s3[1] = {up.sum()};
    unsigned long long m3[1] = {up.max_bits()};
    cluster_reduce<1, 1>(cl, red, rc, s3, m3);
    tprev = t;
    t = df2d(s3[0]);
    rmax = bits_to_double(m3[0]);
    nan = (rmax != rmax) || (alpha != alpha);
    done = !(rmax > tol) || k >= maxiter || nan;
  }
  iters = k;
  rmax_out = rmax;
  nan_out = nan;
}

// Ax (FP64, double-float operator) then r = b - Ax and max|r| over the cluster
template <int N>
__device__ double bresidual(const BatchArgs<N>& a, BProb& pr, cg::cluster_group& cl, int rank,
                            BRed& red, int& rc, const BBuf<N>& buf) {
  typedef BTile<N> T;
  const long long L = pr.NX * pr.NY;
  const int ntx = (pr.Ex + T::TX - 1) / T::TX, nty = (pr.Ey + T::TY - 1) / T::TY;
  BAcc<double> unused;
  for (int tile = rank, csz = bcsize(); tile < ntx * nty; tile += csz) {
    const int by = tile / ntx, bx = tile - by * ntx;
    btile<PDF, N, T::TX, T::TY>(pr, a.cdf, bx, by, pr.x, nullptr, nullptr, 0.0, nullptr, false, pr.Ap,
                                pr.Gdf, L, buf.S0, buf.S1, buf.X0, unused);
  }
  cl.sync();
  bfixup<double, T::TX, T::TY>(pr, N, pr.Ap, pr.x, rank, unused);
  cl.sync();
  BAcc<double> acc;
  own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float) {
    const double v = pr.b[i] - pr.Ap[i];
    pr.r[i] = v;
    acc.amax(v);
  });
  df s0[1] = {{0.0f, 0.0f}};
  unsigned long long m1[1] = {acc.max_bits()};
  cluster_reduce<1, 1>(cl, red, rc, s0, m1);
  return bits_to_double(m1[0]);
}

// SEM_MIXED_RR: one FP32 CG whose residual is replaced by the FP64 b - A x
// (x += x32 first) whenever it has fallen by the factor inner_tol since the
// last replacement; p32 and the beta recurrence continue across replacements
template <int N>
__device__ void brr(const BatchArgs<N>& a, BProb& pr, cg::cluster_group& cl, int rank, BRed& red, int& rc,
                    const BBuf<N>& buf) {
  typedef BTile<N> T;
  const bool jac = a.jacobi != 0;
  const float* dinv32 = jac ? pr.dinv32 : nullptr;
  const long long L = pr.NX * pr.NY;
  const int ntx = (pr.Ex + T::TX - 1) / T::TX, nty = (pr.Ey + T::TY - 1) / T::TY;
  // x = 0, r = b (FP64)
  BAcc<double> a0;
  own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float) {
    pr.x[i] = 0.0;
    pr.r[i] = pr.b[i];
    a0.amax(pr.b[i]);
  });
  df z[1] = {{0.0f, 0.0f}};
  unsigned long long m0[1] = {a0.max_bits()};
  cluster_reduce<1, 1>(cl, red, rc, z, m0);
  double rmax64 = bits_to_double(m0[0]);
  const double res0 = rmax64;
  // r32 = (float) r, x32 = 0 (p32 = 0 the first time); returns t = r32.h.mult
  auto load_r32 = [&](bool zero_p) -> double {
    BAcc<float> acc;
    own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float m) {
      const float ri = (float)pr.r[i];
      pr.r32[i] = ri;
      pr.x32[i] = 0.0f;
      if (zero_p) pr.p32[i] = 0.0f;
      if (jac)
        acc.rhr(ri, dinv32[i], m);
      else
        acc.prod(ri, ri, m);
    });
    df s1[1] = {acc.sum()};
    unsigned long long none[1] = {0ull};
    cluster_reduce<1, 1>(cl, red, rc, s1, none);
    return df2d(s1[0]);
  };
  double t = load_r32(true);
  double tprev = 1.0;
  double thresh = a.inner_tol * rmax64;
  int k = 0, outer = 0;
  bool nan = rmax64 != rmax64;
  bool done = !(rmax64 > pr.tol) || pr.maxiter == 0 || nan;
  while (!done) {
    const float beta = k == 0 ? 0.0f : (float)(t / tprev);
    BAcc<float> dot;
    for (int tile = rank, csz = bcsize(); tile < ntx * nty; tile += csz) {
      const int by = tile / ntx, bx = tile - by * ntx;
      btile<PF32, N, T::TX, T::TY>(pr, a.cf, bx, by, nullptr, pr.r32, dinv32, beta, pr.p32, true, pr.Ap32,
                                   pr.G11f, L, buf.template s0<PF32>(), buf.template s1<PF32>(),
                                   buf.template x0<PF32>(), dot);
    }
    cl.sync();
    bfixup<float, T::TX, T::TY>(pr, N, pr.Ap32, pr.p32, rank, dot);
    df s2[1] = {dot.sum()};
    unsigned long long none[1] = {0ull};
    cluster_reduce<1, 1>(cl, red, rc, s2, none);
    const double alpha = t / df2d(s2[0]);
    const float af = (float)alpha;
    ++k;
    BAcc<float> up;
    own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float m) {
      pr.x32[i] = pr.x32[i] + af * pr.p32[i];
      const float ri = pr.r32[i] - af * pr.Ap32[i];
      pr.r32[i] = ri;
      if (jac)
        up.rhr(ri, dinv32[i], m);
      else
        up.prod(ri, ri, m);
      up.amax(ri);
    });
    df s3[1] = {up.sum()};
    unsigned long long m3[1] = {up.max_bits()};
    cluster_reduce<1, 1>(cl, red, rc, s3, m3);
    tprev = t;
    t = df2d(s3[0]);
    const double rmax32 = bits_to_double(m3[0]);
    const bool nan32 = (rmax32 != rmax32) || (alpha != alpha);
    if (!(rmax32 > thresh) || k >= pr.maxiter || nan32) {
      own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float) { pr.x[i] += (double)pr.x32[i]; });
      cl.sync();
      rmax64 = bresidual<N>(a, pr, cl, rank, red, rc, buf);
      ++outer;
      nan = rmax64 != rmax64 || nan32;
      done = !(rmax64 > pr.tol) || k >= pr.maxiter || nan || outer >= a.max_outer;
      if (!done) {
        t = load_r32(false);
        thresh = a.inner_tol * rmax64;
      }
    }
  }
  if (rank == 0 && threadIdx.x == 0) {
    pr.iters = k;
    pr.outer = outer;
    pr.res_inf = rmax64;
    pr.res0_inf = res0;
    pr.nan = nan;
    pr.converged = !(rmax64 > pr.tol) && !nan;
  }
}

template <int N>
__device__ void bsolve(const BatchArgs<N>& a, BProb& pr, cg::cluster_group& cl, int rank, BRed& red,
                       int& rc, const BBuf<N>& buf) {
  typedef BTile<N> T;
  const bool jac = a.jacobi != 0;
  const int maxiter = pr.maxiter;
  if (maxiter < 0) {  // left to the host's native FP64 solve (scalars outside the pair window)
    if (rank == 0 && threadIdx.x == 0) {
      pr.iters = 0;
      pr.outer = 0;
      pr.res_inf = 0.0;
      pr.res0_inf = 0.0;
      pr.nan = 0;
      pr.converged = 0;
    }
    return;
  }
  if (a.precision == SEM_MIXED_RR) {
    brr<N>(a, pr, cl, rank, red, rc, buf);
    return;
  }
  if (a.precision != SEM_MIXED) {
    int it = 0;
    double rmax = 0.0;
    bool nan = false;
    bcg<PDF, N>(a, pr, cl, rank, pr.b, pr.x, pr.r, pr.p, pr.Ap, jac ? pr.dinv : nullptr, pr.Gdf, pr.tol,
                maxiter, red, rc, buf, it, rmax, nan);
    if (rank == 0 && threadIdx.x == 0) {
      pr.iters = it;
      pr.outer = 0;
      pr.res_inf = rmax;
      pr.nan = nan;
      pr.converged = !(rmax > pr.tol) && !nan;
    }
    return;
  }
  // FP64 defect correction around the FP32 inner CG: x = 0, r = b
  BAcc<double> acc;
  own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float) {
    pr.x[i] = 0.0;
    pr.r[i] = pr.b[i];
    acc.amax(pr.b[i]);
  });
  df s0[1] = {{0.0f, 0.0f}};
  unsigned long long m1[1] = {acc.max_bits()};
  cluster_reduce<1, 1>(cl, red, rc, s0, m1);
  double rmax = bits_to_double(m1[0]);
  const double res0 = rmax;
  int outer = 0, total = 0;
  bool nan = rmax != rmax;
  // the FP32 geometry blocks are contiguous (G11, G12, G22, B)
  const float* Gf = pr.G11f;
  while (!(rmax <= pr.tol) && !nan && outer < a.max_outer) {
    ++outer;
    int it = 0;
    double rin = 0.0;
    bool nin = false;
    bcg<PF32, N>(a, pr, cl, rank, pr.r, pr.x32, pr.r32, pr.p32, pr.Ap32, jac ? pr.dinv32 : nullptr, Gf,
                 a.inner_tol * rmax, maxiter, red, rc, buf, it, rin, nin);
    total += it;
    own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float) { pr.x[i] += (double)pr.x32[i]; });
    cl.sync();
    rmax = bresidual<N>(a, pr, cl, rank, red, rc, buf);
    nan = rmax != rmax;
  }
  if (rank == 0 && threadIdx.x == 0) {
    pr.iters = total;
    pr.outer = outer;
    pr.res_inf = rmax;
    pr.res0_inf = res0;
    pr.nan = nan;
    pr.converged = rmax <= pr.tol;
  }
}

// The persistent kernel: clusters take problems from the group's queue until
// it runs dry.  MB: resident CTAs per SM asked of the register allocator (1:
// up to 255 registers a thread, 2: up to 128); the cluster size is the
// launch's.
template <int N, int MB>
__global__ void __launch_bounds__(kBT, MB) k_batch_pcg(const __grid_constant__ BatchArgs<N> a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BRed red;
  int rc = 0;
  __shared__ int s_pid;
  const BBuf<N> buf(smem);
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) s_pid = atomicAdd(a.queue, 1);
    cl.sync();
    const int pid = *cl.map_shared_rank(&s_pid, 0);
    cl.sync();  // every CTA has read s_pid before rank 0 may overwrite it
    if (pid >= a.count) return;
    BProb& pr = a.probs[pid];
    if (rank == 0 && threadIdx.x == 0) {
      pr.t_start = bclock_ns();
      pr.cluster = (int)(blockIdx.x / (unsigned)bcsize());
    }
    bsolve<N>(a, pr, cl, rank, red, rc, buf);
    cl.sync();  // the problem's results are written before the next one starts
    if (rank == 0 && threadIdx.x == 0) pr.t_end = bclock_ns();
  }
}

template <int N>
static void fill_batch_args(BatchArgs<N>& a, const BatchCommon& c, const OperatorSet& ops) {
  std::memset(&a, 0, sizeof(a));
  a.probs = c.probs;
  a.count = c.count;
  a.queue = c.queue;
  a.precision = c.precision;
  a.jacobi = c.jacobi;
  a.inner_tol = c.inner_tol;
  a.max_outer = c.max_outer;
  constexpr int M = N / 2;
  for (int b = 0; b < 4; ++b) {
    const double* A = ops.eo[b];
    const double* C = A + M * M;
    const double* cm = C + M * M;
    const double* mr = cm + M;
    auto tdf = [](double d) { const float h = (float)d; return df{h, (float)(d - (double)h)}; };
    for (int i = 0; i < M; ++i)
      for (int kk = 0; kk < M; ++kk) {
        a.cdf[b].A[i][kk] = tdf(A[i * M + kk]);
        a.cdf[b].Cc[i][kk] = tdf(C[i * M + kk]);
        a.cf[b].A[i][kk] = (float)A[i * M + kk];
        a.cf[b].Cc[i][kk] = (float)C[i * M + kk];
      }
    for (int i = 0; i < M; ++i) {
      a.cdf[b].cm[i] = tdf(cm[i]);
      a.cdf[b].mr[i] = tdf(mr[i]);
      a.cf[b].cm[i] = (float)cm[i];
      a.cf[b].mr[i] = (float)mr[i];
    }
  }
}

template <int N>
constexpr size_t batch_smem_bytes() {
  return (size_t)BTile<N>::SLOTS * BTile<N>::ES * (2 * sizeof(df) + sizeof(double));
}

// the launch configuration of one group: cluster size and register budget
template <int N, int MB>
static void batch_config(cudaLaunchConfig_t& cfg, cudaLaunchAttribute* at, int csize, int nclusters,
                         cudaStream_t s) {
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)(csize * nclusters));
  cfg.blockDim = dim3(kBT);
  cfg.dynamicSmemBytes = batch_smem_bytes<N>();
  cfg.stream = s;
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
}

template <int N, int MB>
static int prepare_batch_kernel() {
  auto kern = k_batch_pcg<N, MB>;
  SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)batch_smem_bytes<N>()));
  SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  return SEM_OK;
}

// clusters of the given shape that fit the device at once (0: the shape does not launch)
template <int N, int MB>
static int batch_max_clusters_mb(int csize) {
  if ((prepare_batch_kernel<N, MB>()) != SEM_OK) return 0;
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute at[1];
  batch_config<N, MB>(cfg, at, csize, 64, nullptr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_batch_pcg<N, MB>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

// host: launch the persistent kernel of order N over `count` problems
template <int N, int MB>
static int launch_batch_mb(const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  BatchArgs<N> a;
  fill_batch_args<N>(a, c, ops);
  SEM_CHECK((prepare_batch_kernel<N, MB>()));
  int nclusters = c.clusters;
  if (nclusters <= 0) nclusters = batch_max_clusters_mb<N, MB>(c.cluster_size);
  if (nclusters < 1) return set_error(SEM_ERR_UNSUPPORTED, "a cluster of %d CTAs does not fit (n = %d)", c.cluster_size, N);
  if (nclusters > c.count) nclusters = c.count;
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute at[1];
  batch_config<N, MB>(cfg, at, c.cluster_size, nclusters, s);
  SEM_CUDA(cudaLaunchKernelEx(&cfg, k_batch_pcg<N, MB>, a));
  return SEM_OK;
}

// the orders LO..HI at one register budget (one translation unit each)
template <int LO, int HI, int MB>
int launch_batch_range(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  if constexpr (LO > HI) {
    return set_error(SEM_ERR_UNSUPPORTED, "batch order %d not in this unit", n);
  } else {
    if (n == LO) {
      const int cs = c.cluster_size;
      if (cs != 2 && cs != 4 && cs != 8 && cs != 16)
        return set_error(SEM_ERR_BAD_ARG, "batch cluster size %d (2, 4, 8 or 16)", cs);
      return launch_batch_mb<LO, MB>(c, ops, s);
    }
    return launch_batch_range<LO + 1, HI, MB>(n, c, ops, s);
  }
}

template <int LO, int HI, int MB>
int max_clusters_range(int n, int csize) {
  if constexpr (LO > HI) {
    return 0;
  } else {
    if (n == LO) return batch_max_clusters_mb<LO, MB>(csize);
    return max_clusters_range<LO + 1, HI, MB>(n, csize);
  }
}

}  // namespace sem
