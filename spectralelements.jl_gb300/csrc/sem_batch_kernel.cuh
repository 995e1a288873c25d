// Batched PCG: many independent mask(QQ'(hlmz)) systems of different sizes
// solved by persistent launches of thread-block clusters, one launch per
// polynomial order (each with the register budget of its order), all running
// concurrently.
//
// Each cluster (kCluster CTAs of kBT threads) takes problems from a device
// work queue (problems sorted by estimated work, largest first) and runs the
// whole CG loop of src/pcg.jl:16-60 for one problem before taking the next.
// Inside a problem the cluster's CTAs share the element tiles (tile t goes to
// CTA t mod kCluster) and every pointwise vector operation runs on the points
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

#include "sem_apply_kernels.cuh"

namespace cg = cooperative_groups;

namespace sem {

constexpr int kBT = 256;       // threads per CTA
constexpr int kCluster = 8;    // CTAs per cluster (portable size)
constexpr int kBatchMaxN = 11; // GLL points per direction served by the batch kernel

template <int N>
struct BTile {  // element tile of the batch kernel: TX*TY*N <= kBT
  static constexpr int TX = N <= 2 ? 8 : (N <= 6 ? 8 : (N == 7 ? 6 : (N == 8 ? 8 : (N == 9 ? 7 : 5))));
  static constexpr int TY = N <= 2 ? 16 : (N == 3 ? 10 : (N == 4 ? 8 : (N == 5 ? 6 : (N == 6 ? 5 :
                            (N == 7 ? 6 : (N == 8 ? 4 : (N == 9 ? 4 : (N == 10 ? 5 : 4))))))));
  static constexpr int SP = N | 1;
  static constexpr int ES = N * SP;
  static_assert(TX * TY * N <= kBT, "tile exceeds the CTA");
};

struct BProb {
  int n, Ex, Ey;
  long long NX, NY;
  unsigned topo;  // M_PERX | M_PERY | M_D* | M_MASK
  double nu, k, tol;
  int maxiter;
  const double *G11, *G12, *G22, *B;
  const float *G11f, *G12f, *G22f, *Bf;
  const double* b;
  double* x;
  double *r, *p, *Ap, *dinv;
  float *r32, *p32, *Ap32, *x32, *dinv32;
  // results
  int iters, outer, converged, nan;
  double res_inf, res0_inf;
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
  int clusters;  // <= 0: as many as fit
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

// ---- per-thread accumulators (see sem_pcg.cu): double-float sums for FP64
// vectors, FP32 sums for FP32 vectors, integer max of magnitude bits
template <class T>
struct BAcc;
template <>
struct BAcc<double> {
  df s = {0.0f, 0.0f};
  unsigned long long mx = 0ull;
  __device__ __forceinline__ void prod(double a, double b, float m) {
    df p = df_mul_u(d2df(a), d2df(b));
    p.h *= m;
    p.l *= m;
    s = df_add_u(s, p);
  }
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
  __device__ __forceinline__ double sum() const { return df2d(df_norm(s)); }
  __device__ __forceinline__ double max() const { return __longlong_as_double((long long)mx); }
};
template <>
struct BAcc<float> {
  float s = 0.0f;
  unsigned mx = 0u;
  __device__ __forceinline__ void prod(float a, float b, float m) { s = __fmaf_rn(a * m, b, s); }
  __device__ __forceinline__ void rhr(float a, float d, float m) { s = __fmaf_rn(a, a * d * m, s); }
  __device__ __forceinline__ void amax(float a) {
    const unsigned b = __float_as_uint(a) & 0x7fffffffu;
    mx = b > mx ? b : mx;
  }
  __device__ __forceinline__ double sum() const { return (double)s; }
  __device__ __forceinline__ double max() const { return (double)__uint_as_float(mx); }
};

__device__ __forceinline__ double bpdir(double r, double d, double beta, double p, bool jac) {
  const df rd = d2df(r);
  const df h = jac ? df_mul_u(rd, d2df(d)) : rd;
  return df2d(df_fma_u(d2df(beta), d2df(p), h));
}
__device__ __forceinline__ float bpdir(float r, float d, float beta, float p, bool jac) {
  return __fmaf_rn(beta, p, jac ? r * d : r);
}

__device__ __forceinline__ double bnanmax(double a, double b) { return (b > a || b != b) ? b : a; }

// copies of the node behind local row r of element e (1 or 2)
__device__ __forceinline__ int bcopies(int e, int i, int n, int E, bool per) {
  return ((i == 0 && (e > 0 || per)) || (i == n - 1 && (e < E - 1 || per))) ? 2 : 1;
}

// Cluster-wide sum (NV values, is_max selects max) in fixed rank order; every
// CTA gets the same result.  Calls rotate over three slots (rc counts the
// calls, identically in every thread of the cluster): a slot is written again
// only two cluster barriers after its last read, so no CTA overwrites a value
// another CTA may still be reading.
template <int NV>
__device__ __forceinline__ void cluster_reduce(cg::cluster_group& cl, double* slots, int& rc,
                                               double (&v)[NV], const bool (&is_max)[NV]) {
  const int slot = rc % 3;
  ++rc;
  __shared__ double wsum[NV][kBT / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_down_sync(0xffffffffu, x, o);
      x = is_max[q] ? bnanmax(x, y) : x + y;
    }
    if (lane == 0) wsum[q][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double x = wsum[q][0];
      for (int i = 1; i < kBT / 32; ++i) x = is_max[q] ? bnanmax(x, wsum[q][i]) : x + wsum[q][i];
      slots[slot * 4 + q] = x;
    }
  }
  cl.sync();
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double x = 0.0;
    for (int rk = 0; rk < kCluster; ++rk) {
      const double y = cl.map_shared_rank(slots, rk)[slot * 4 + q];
      x = is_max[q] ? bnanmax(x, y) : x + y;
    }
    v[q] = x;
  }
}

// One element tile of the operator mask(QQ'(nu lapl(u) + k B u)), optionally
// with the CG direction update fused in front: u = p = dinv.*r + beta p_old.
// Writes Ap (cross-tile points unsummed) and adds u.Ap.mult of the finished
// points to acc.  All threads of the CTA call it (threads beyond the tile idle).
template <class P, int N, int TX, int TY>
__device__ void btile(const BProb& pr, const EOCoef<N, typename P::v>* D, int bx, int by,
                      const typename P::io* u_src, const typename P::io* r, const typename P::io* dinv,
                      typename P::io beta, typename P::io* p, bool pdir, typename P::io* Ap,
                      const typename P::io* G11, const typename P::io* G12, const typename P::io* G22,
                      const typename P::io* B, typename P::v* S1, typename P::v* S2,
                      BAcc<typename P::io>& acc) {
  typedef typename P::v V;
  typedef typename P::io IO;
  constexpr int SP = N | 1, ES = N * SP;
  const int t = threadIdx.x;
  const bool inside = t < TX * TY * N;
  const int elem = inside ? t / N : 0;
  const int lane = inside ? t - elem * N : 0;
  const int exl = elem % TX, eyl = elem / TX;
  const int ex = bx * TX + exl, ey = by * TY + eyl;
  const bool valid = inside && ex < pr.Ex && ey < pr.Ey;
  const long long NX = pr.NX;
  const long long base = (long long)ex * N + lane + (long long)ey * N * NX;
  V* s1 = S1 + elem * ES;
  V* s2 = S2 + elem * ES;
  const unsigned topo = pr.topo;
  const bool perx = (topo & M_PERX) != 0, pery = (topo & M_PERY) != 0;
  const bool jac = dinv != nullptr;

  V u[N];
  IO uraw[N];
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
    uraw[j] = v;
    u[j] = P::cvt(v);
  }
  V us[N], res[N];
  if (inside)
#pragma unroll
    for (int j = 0; j < N; ++j) s1[j * SP + lane] = u[j];
  eo_apply<P, N>(D[2], u, us);
  __syncthreads();
  if (inside) {
    V col[N], ur[N];
#pragma unroll
    for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
    eo_apply<P, N>(D[0], col, ur);
#pragma unroll
    for (int i = 0; i < N; ++i) s2[lane * SP + i] = ur[i];
  }
  __syncthreads();
  V os[N];
  {
    V ws[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const long long gi = base + (long long)j * NX;
      V g11 = valid ? P::ld(G11 + gi) : P::zero();
      V g12 = valid ? P::ld(G12 + gi) : P::zero();
      V g22 = valid ? P::ld(G22 + gi) : P::zero();
      V ur = s2[j * SP + lane];
      const V wr = P::fma(g11, ur, P::mul(g12, us[j]));
      if (inside) s1[j * SP + lane] = wr;
      ws[j] = P::fma(g12, ur, P::mul(g22, us[j]));
    }
    eo_apply<P, N>(D[3], ws, os);
  }
  __syncthreads();
  if (inside) {
    V col[N], o[N];
#pragma unroll
    for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
    eo_apply<P, N>(D[1], col, o);
#pragma unroll
    for (int i = 0; i < N; ++i) s2[lane * SP + i] = o[i];
  }
  __syncthreads();
  const V nu = P::cvt((IO)pr.nu);
  const V kk = P::cvt((IO)pr.k);
#pragma unroll
  for (int j = 0; j < N; ++j) {
    res[j] = P::fin(P::mul(nu, P::add(s2[j * SP + lane], os[j])));
    if (pr.k != 0.0) {
      V bb = valid ? P::ld(B + base + (long long)j * NX) : P::zero();
      res[j] = P::fin(P::fma(P::fin(P::mul(kk, bb)), u[j], res[j]));
    }
  }
  // in-tile QQ': x pairs then y pairs
  __syncthreads();
  if (inside)
#pragma unroll
    for (int j = 0; j < N; ++j) s1[j * SP + lane] = res[j];
  __syncthreads();
  if (inside && lane == N - 1 && exl + 1 < TX && ex + 1 < pr.Ex) {
    const V* nb = S1 + (elem + 1) * ES;
#pragma unroll
    for (int j = 0; j < N; ++j) res[j] = P::add(res[j], nb[j * SP]);
  }
  if (inside && lane == 0 && exl > 0) {
    const V* nb = S1 + (elem - 1) * ES;
#pragma unroll
    for (int j = 0; j < N; ++j) res[j] = P::add(nb[j * SP + N - 1], res[j]);
  }
  if (inside) {
    s2[lane] = res[0];
    s2[(N - 1) * SP + lane] = res[N - 1];
  }
  __syncthreads();
  if (inside && eyl + 1 < TY && ey + 1 < pr.Ey) res[N - 1] = P::add(res[N - 1], S2[(elem + TX) * ES + lane]);
  if (inside && eyl > 0) res[0] = P::add(S2[(elem - TX) * ES + (N - 1) * SP + lane], res[0]);
  if (valid) {
    const bool xc = xcross_row(ex, lane, N, pr.Ex, TX, perx);
    const long long row = (long long)ex * N + lane;
    const int cx = bcopies(ex, lane, N, pr.Ex, perx);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      bool raw = xc;
      if (j == 0 && eyl == 0 && (ey > 0 || pery)) raw = true;
      if (j == N - 1 && (eyl == TY - 1 || ey == pr.Ey - 1) && (ey < pr.Ey - 1 || pery)) raw = true;
      IO val = P::st(res[j]);
      if (!raw) {
        const long long col = (long long)ey * N + j;
        if ((topo & M_MASK) && !mask_keep(row, col, NX, pr.NY, topo)) val = masked_zero(val);
        const int cc = cx * bcopies(ey, j, N, pr.Ey, pery);
        acc.prod(uraw[j], val, cc == 1 ? 1.0f : (cc == 2 ? 0.5f : 0.25f));
      }
      Ap[base + (long long)j * NX] = val;
    }
  }
  __syncthreads();
}

// cross-tile QQ' completion, work split over the whole cluster; adds
// p.Ap.mult of every copy it finishes
template <class IO, int TX, int TY>
__device__ void bfixup(const BProb& pr, int n, IO* __restrict__ Ap, const IO* __restrict__ p,
                       int rank, BAcc<IO>& acc) {
  const unsigned topo = pr.topo;
  const bool perx = (topo & M_PERX) != 0, pery = (topo & M_PERY) != 0;
  const bool msk = (topo & M_MASK) != 0;
  const long long NX = pr.NX, NY = pr.NY;
  const long long nxi = (pr.Ex - 1) / TX + (perx ? 1 : 0);
  const long long nyi = (pr.Ey - 1) / TY + (pery ? 1 : 0);
  const long long nX = nxi * NY, nY = nyi * NX, nC = nxi * nyi;
  const long long total = nX + nY + nC;
  auto fin = [&](long long r, long long c, IO s, float m) {
    IO v = s;
    if (msk && !mask_keep(r, c, NX, NY, topo)) v = masked_zero(s);
    Ap[r + c * NX] = v;
    acc.prod(p[r + c * NX], v, m);
  };
  for (long long idx = (long long)rank * kBT + threadIdx.x; idx < total; idx += (long long)kCluster * kBT) {
    if (idx < nX) {
      const long long q = idx / NY, c = idx - q * NY;
      const long long ey = c / n;
      const int j = (int)(c - ey * n);
      if (xcross_row((int)ey, j, n, pr.Ey, TY, pery)) continue;
      const long long aa = fix_iface(q, TX, perx);
      const long long rl = aa == 0 ? NX - 1 : aa * n - 1, rr = aa * n;
      const IO s = Ap[rl + c * NX] + Ap[rr + c * NX];
      const float m = 0.5f / (float)bcopies((int)ey, j, n, pr.Ey, pery);
      fin(rl, c, s, m);
      fin(rr, c, s, m);
    } else if (idx < nX + nY) {
      const long long id2 = idx - nX, q = id2 / NX, r = id2 - q * NX;
      const long long ex = r / n;
      const int i = (int)(r - ex * n);
      if (xcross_row((int)ex, i, n, pr.Ex, TX, perx)) continue;
      const long long bb = fix_iface(q, TY, pery);
      const long long cl = bb == 0 ? NY - 1 : bb * n - 1, cr = bb * n;
      const IO s = Ap[r + cl * NX] + Ap[r + cr * NX];
      const float m = 0.5f / (float)bcopies((int)ex, i, n, pr.Ex, perx);
      fin(r, cl, s, m);
      fin(r, cr, s, m);
    } else {
      const long long id3 = idx - nX - nY, q = id3 / nyi, pp = id3 - q * nyi;
      const long long aa = fix_iface(q, TX, perx), bb = fix_iface(pp, TY, pery);
      const long long rl = aa == 0 ? NX - 1 : aa * n - 1, rr = aa * n;
      const long long cl = bb == 0 ? NY - 1 : bb * n - 1, cr = bb * n;
      const IO s = (Ap[rl + cl * NX] + Ap[rr + cl * NX]) + (Ap[rl + cr * NX] + Ap[rr + cr * NX]);
      fin(rl, cl, s, 0.25f);
      fin(rr, cl, s, 0.25f);
      fin(rl, cr, s, 0.25f);
      fin(rr, cr, s, 0.25f);
    }
  }
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
  for (int tile = rank; tile < ntx * nty; tile += kCluster) {
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

// CG on A y = rhs (P: PDF for FP64 vectors, PF32 for the FP32 inner solve).
// rhs is read as double (b or the FP64 residual) and converted.
template <class P, int N>
__device__ void bcg(const BatchArgs<N>& a, BProb& pr, cg::cluster_group& cl, int rank,
                    const double* rhs, typename P::io* y, typename P::io* r, typename P::io* p,
                    typename P::io* Ap, const typename P::io* dinv, const typename P::io* G11,
                    const typename P::io* G12, const typename P::io* G22, const typename P::io* B,
                    double tol, int maxiter, double* slots, int& rc, typename P::v* S1, typename P::v* S2,
                    int& iters, double& rmax_out, bool& nan_out) {
  typedef typename P::io IO;
  typedef BTile<N> T;
  const EOCoef<N, typename P::v>* D;
  if constexpr (P::kPrecision == SEM_F32)
    D = a.cf;
  else
    D = a.cdf;
  const bool jac = dinv != nullptr;
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
  double v2[2] = {acc.sum(), acc.max()};
  const bool mx2[2] = {false, true};
  cluster_reduce<2>(cl, slots, rc, v2, mx2);
  double t = v2[0], rmax = v2[1];
  double tprev = 1.0;
  int k = 0;
  bool nan = rmax != rmax;
  bool done = !(rmax > tol) || maxiter == 0;
  while (!done) {
    const double beta = k == 0 ? 0.0 : t / tprev;
    BAcc<IO> dot;
    for (int tile = rank; tile < ntx * nty; tile += kCluster) {
      const int by = tile / ntx, bx = tile - by * ntx;
      btile<P, N, T::TX, T::TY>(pr, D, bx, by, nullptr, r, dinv, (IO)beta, p, true, Ap, G11, G12,
                                G22, B, S1, S2, dot);
    }
    cl.sync();
    bfixup<IO, T::TX, T::TY>(pr, N, Ap, p, rank, dot);
    double v1[1] = {dot.sum()};
    const bool mx1[1] = {false};
    cluster_reduce<1>(cl, slots, rc, v1, mx1);
    const double alpha = t / v1[0];
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
    double w2[2] = {up.sum(), up.max()};
    cluster_reduce<2>(cl, slots, rc, w2, mx2);
    tprev = t;
    t = w2[0];
    rmax = w2[1];
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
                            double* slots, int& rc, df* S1, df* S2) {
  typedef BTile<N> T;
  const EOCoef<N, df>* D = a.cdf;
  const int ntx = (pr.Ex + T::TX - 1) / T::TX, nty = (pr.Ey + T::TY - 1) / T::TY;
  BAcc<double> unused;
  for (int tile = rank; tile < ntx * nty; tile += kCluster) {
    const int by = tile / ntx, bx = tile - by * ntx;
    btile<PDF, N, T::TX, T::TY>(pr, D, bx, by, pr.x, nullptr, nullptr, 0.0, nullptr, false, pr.Ap,
                                pr.G11, pr.G12, pr.G22, pr.B, S1, S2, unused);
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
  double v1[1] = {acc.max()};
  const bool mx1[1] = {true};
  cluster_reduce<1>(cl, slots, rc, v1, mx1);
  return v1[0];
}

template <int N>
__device__ void bsolve(const BatchArgs<N>& a, BProb& pr, cg::cluster_group& cl, int rank,
                       double* slots, int& rc, unsigned char* smem) {
  typedef BTile<N> T;
  df* S1 = reinterpret_cast<df*>(smem);
  df* S2 = S1 + T::TX * T::TY * T::ES;
  const bool jac = a.jacobi != 0;
  const int maxiter = pr.maxiter;
  if (a.precision != SEM_MIXED) {
    int it = 0;
    double rmax = 0.0;
    bool nan = false;
    bcg<PDF, N>(a, pr, cl, rank, pr.b, pr.x, pr.r, pr.p, pr.Ap, jac ? pr.dinv : nullptr, pr.G11,
                pr.G12, pr.G22, pr.B, pr.tol, maxiter, slots, rc, S1, S2, it, rmax, nan);
    if (rank == 0 && threadIdx.x == 0) {
      pr.iters = it;
      pr.outer = 0;
      pr.res_inf = rmax;
      pr.nan = nan;
      pr.converged = !(rmax > pr.tol) && !nan;
    }
    return;
  }
  float* F1 = reinterpret_cast<float*>(smem);
  float* F2 = F1 + T::TX * T::TY * T::ES;
  // FP64 defect correction around the FP32 inner CG: x = 0, r = b
  BAcc<double> acc;
  own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float) {
    pr.x[i] = 0.0;
    pr.r[i] = pr.b[i];
    acc.amax(pr.b[i]);
  });
  double v1[1] = {acc.max()};
  const bool mx1[1] = {true};
  cluster_reduce<1>(cl, slots, rc, v1, mx1);
  double rmax = v1[0];
  const double res0 = rmax;
  int outer = 0, total = 0;
  bool nan = rmax != rmax;
  while (!(rmax <= pr.tol) && !nan && outer < a.max_outer) {
    ++outer;
    int it = 0;
    double rin = 0.0;
    bool nin = false;
    bcg<PF32, N>(a, pr, cl, rank, pr.r, pr.x32, pr.r32, pr.p32, pr.Ap32, jac ? pr.dinv32 : nullptr,
                 pr.G11f, pr.G12f, pr.G22f, pr.Bf, a.inner_tol * rmax, maxiter, slots, rc, F1, F2, it,
                 rin, nin);
    total += it;
    own_points<N, T::TX, T::TY>(pr, rank, [&](long long i, float) { pr.x[i] += (double)pr.x32[i]; });
    cl.sync();
    rmax = bresidual<N>(a, pr, cl, rank, slots, rc, S1, S2);
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

template <int N>
__global__ void __cluster_dims__(kCluster, 1, 1) __launch_bounds__(kBT, 1)
    k_batch_pcg(const __grid_constant__ BatchArgs<N> a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double slots[3 * 4];
  int rc = 0;
  __shared__ int s_pid;
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) s_pid = atomicAdd(a.queue, 1);
    cl.sync();
    const int pid = *cl.map_shared_rank(&s_pid, 0);
    cl.sync();  // every CTA has read s_pid before rank 0 may overwrite it
    if (pid >= a.count) return;
    bsolve<N>(a, a.probs[pid], cl, rank, slots, rc, smem);
    cl.sync();  // the problem's results are written before the next one starts
  }
}

// host: launch the persistent kernel of order N over `count` problems
template <int N>
int launch_batch_order(const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  BatchArgs<N> a;
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
  typedef BTile<N> T;
  const size_t smem = 2 * (size_t)T::TX * T::TY * T::ES * sizeof(df);
  SEM_CUDA(cudaFuncSetAttribute(k_batch_pcg<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int nclusters = c.clusters;
  if (nclusters <= 0) {
    cudaLaunchConfig_t cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.blockDim = dim3(kBT);
    cfg.gridDim = dim3(kCluster * 64);
    cfg.dynamicSmemBytes = smem;
    SEM_CUDA(cudaOccupancyMaxActiveClusters(&nclusters, k_batch_pcg<N>, &cfg));
  }
  if (nclusters < 1) nclusters = 1;
  if (nclusters > c.count) nclusters = c.count;
  k_batch_pcg<N><<<dim3(kCluster * nclusters), dim3(kBT), smem, s>>>(a);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

}  // namespace sem
