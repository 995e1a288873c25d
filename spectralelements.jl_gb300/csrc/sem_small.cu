// Single-launch PCG for small meshes (the latency path of sem_pcg).
//
// A small solve (cfg1: 8x8 elements, 5,184 local DOF) is bound by latency, not
// by bytes: with one thread per element line a CG iteration costs one long
// per-thread instruction chain plus the launch gaps of its kernels.  Here the
// whole solve of src/pcg.jl:16-60 runs in one thread-block cluster (16 CTAs
// where the device allows it, else 8) and one launch:
//
//   * every CTA owns a contiguous range of elements and applies the operator
//     to them with one thread per point (each output point is one
//     (N-term) dot product per direction, instead of one thread per line),
//     so a tile's instruction chain is about N times shorter;
//   * the unassembled outputs go to a scratch field; after a cluster barrier
//     every point gathers its copies (x pairs first, the order of the other
//     kernels) and masks, so no separate QQ' pass and no fixup exist;
//   * p.Ap is summed over the unassembled local products (as in the CG-fused
//     operator launch), r.dinv.r.mult and max|r| over the owned points, both
//     reduced over the cluster in distributed shared memory in rank order, so
//     every CTA takes the same decisions;
//   * SEM_MIXED runs the FP32 inner CG and the FP64 defect correction of the
//     mixed-precision solver inside the same launch, SEM_MIXED_RR its FP32 CG
//     with FP64 residual replacement.
//
// Reference: pcg (src/pcg.jl:16-60), laplace (src/lapl.jl:70-81), hlmz
// (src/hlmz.jl:12-19), gatherScatter (src/gatherScatter.jl:8-16), mask
// (src/mask.jl:10-18).
#include <cooperative_groups.h>

#include <cstring>

#include "sem_apply2.cuh"

namespace cg = cooperative_groups;

namespace sem {

constexpr int kSmallMaxCluster = 16;
constexpr int kSmallThreads = 512;  // upper bound of a CTA's points per chunk

template <int N>
struct SmallArgs {
  SmallProb* pr;
  df Ddf[2][N][N];    // Dr(i,k), Ds(j,l)
  float Df[2][N][N];
};

struct SmallRed {
  df slot_s[3];
  unsigned long long slot_m[3];
};

// one cluster-wide sum and max, fixed order (block in thread order of the
// warps, then the CTAs in rank order); three rotating slots as in the batched
// solver
__device__ __forceinline__ void small_reduce(cg::cluster_group& cl, SmallRed& red, int& rc, df& s,
                                             unsigned long long& m) {
  __shared__ unsigned long long wmax[32];
  const int slot = rc % 3;
  ++rc;
  const df bs = block_sum_df(s);
  unsigned long long x = m;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, x, o);
    x = y > x ? y : x;
  }
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)((blockDim.x + 31) >> 5); ++i) x = wmax[i] > x ? wmax[i] : x;
    red.slot_s[slot] = bs;
    red.slot_m[slot] = x;
  }
  cl.sync();
  // warp 0 combines the CTAs' parts (lane r reads rank r, fixed shuffle tree:
  // the same order in every CTA) and shares the result through shared memory
  __shared__ df res_s;
  __shared__ unsigned long long res_m;
  if (threadIdx.x < 32) {
    const int nr = (int)cl.num_blocks();
    const int lane = threadIdx.x;
    df t = {0.0f, 0.0f};
    unsigned long long mm = 0ull;
    if (lane < nr) {
      t = *cl.map_shared_rank(&red.slot_s[slot], lane);
      mm = *cl.map_shared_rank(&red.slot_m[slot], lane);
    }
    for (int o = 16; o > 0; o >>= 1) {
      const df y = {__shfl_down_sync(0xffffffffu, t.h, o), __shfl_down_sync(0xffffffffu, t.l, o)};
      t = df_add(t, y);
      const unsigned long long ym = __shfl_down_sync(0xffffffffu, mm, o);
      mm = ym > mm ? ym : mm;
    }
    if (lane == 0) {
      res_s = t;
      res_m = mm;
    }
  }
  __syncthreads();
  s = res_s;
  m = res_m;
}

// elements [e0, e1) of this CTA
__device__ __forceinline__ void small_range(const SmallProb& pr, int rank, int nr, int& e0, int& e1) {
  const long long E = (long long)pr.Ex * pr.Ey;
  e0 = (int)(E * rank / nr);
  e1 = (int)(E * (rank + 1) / nr);
}

// The operator on this CTA's elements, one thread per point, chunks of
// EC = kSmallThreads / N^2 elements: raw = nu (Dr'(G11 ur + G12 us) + ...) + k B u
// unassembled, and acc += u . raw (double-float).  In pdir mode
// u = p = dinv .* r + beta p is formed first (p written back).
template <class P, int N>
__device__ void small_apply(const SmallProb& pr, int e0, int e1, const typename P::v (*Dr)[N],
                            const typename P::v (*Ds)[N], typename P::v* U, typename P::v* W,
                            const typename P::io* src, bool pdir, const typename P::io* r,
                            const typename P::io* dinv, typename P::io beta, typename P::io* p,
                            const typename GeoT<P>::type* Geo, typename P::io* raw, df& acc) {
  typedef typename P::v V;
  typedef typename P::io IO;
  typedef typename GeoT<P>::type GT;
  constexpr int NN = N * N;
  constexpr int EC = kSmallThreads / NN;
  const long long L = pr.NX * pr.NY;
  const GT* G11 = Geo;
  const GT* G12 = Geo + L;
  const GT* G22 = Geo + 2 * L;
  const GT* B = Geo + 3 * L;
  const int t = threadIdx.x;
  const int el = t / NN;
  const int pt = t - el * NN;
  const int j = pt / N;
  const int i = pt - j * N;
  const bool jac = dinv != nullptr;
  const V nu = P::cvt((IO)pr.nu);
  const V kk = P::cvt((IO)pr.k);
  V* u_s = U + el * NN;
  V* wr_s = U + el * NN;  // reuses U after phase B
  V* ws_s = W + el * NN;
  for (int c0 = e0; c0 < e1; c0 += EC) {
    const int e = c0 + el;
    const bool valid = el < EC && e < e1;
    long long gi = 0;
    V u = P::zero();
    if (valid) {
      const int ey = e / pr.Ex, ex = e - ey * pr.Ex;
      gi = ((long long)ex * N + i) + ((long long)ey * N + j) * pr.NX;
      IO v;
      if (pdir) {
        v = cg_direction(r[gi], jac ? dinv[gi] : (IO)1, beta, p[gi], jac);
        p[gi] = v;
      } else {
        v = src[gi];
      }
      u = P::cvt(v);
      u_s[j * N + i] = u;
    }
    __syncthreads();
    V wr = P::zero(), ws = P::zero();
    if (valid) {
      V ur = P::mul(Dr[i][0], u_s[j * N]);
      V us = P::mul(Ds[j][0], u_s[i]);
#pragma unroll
      for (int k = 1; k < N; ++k) {
        ur = P::fma(Dr[i][k], u_s[j * N + k], ur);
        us = P::fma(Ds[j][k], u_s[k * N + i], us);
      }
      ur = P::fin(ur);
      us = P::fin(us);
      const V g11 = GeoT<P>::ld(G11 + gi), g12 = GeoT<P>::ld(G12 + gi), g22 = GeoT<P>::ld(G22 + gi);
      wr = P::fma(g11, ur, P::mul(g12, us));
      ws = P::fma(g12, ur, P::mul(g22, us));
    }
    __syncthreads();
    if (valid) {
      wr_s[j * N + i] = wr;
      ws_s[j * N + i] = ws;
    }
    __syncthreads();
    if (valid) {
      V o_r = P::mul(Dr[0][i], wr_s[j * N]);
      V o_s = P::mul(Ds[0][j], ws_s[i]);
#pragma unroll
      for (int k = 1; k < N; ++k) {
        o_r = P::fma(Dr[k][i], wr_s[j * N + k], o_r);
        o_s = P::fma(Ds[k][j], ws_s[k * N + i], o_s);
      }
      V res = P::fin(P::mul(nu, P::add(P::fin(o_r), P::fin(o_s))));
      if (pr.k != 0.0) res = P::fin(P::fma(P::mul(kk, GeoT<P>::ld(B + gi)), u, res));
      acc = df_add_u(acc, dot_term(u, res));
      raw[gi] = P::st(res);
    }
    __syncthreads();
  }
}

// QQ' and mask at local point (r, c): the sum of its copies, x pairs first
template <class IO>
__device__ __forceinline__ IO small_gather(const SmallProb& pr, const IO* raw, long long r, long long c) {
  const unsigned char br = pr.rinfo[r], bc = pr.cinfo[c];
  if (pr.has_bc && ((br | bc) & L_ZERO)) return (IO)0;  // mask (L_ZERO rows/columns)
  const long long r2 = line_partner(r, br, pr.NX);
  const long long c2 = line_partner(c, bc, pr.NY);
  const IO* col = raw + c * pr.NX;
  if (c2 < 0) return r2 < 0 ? __ldcg(col + r) : io_add(__ldcg(col + r), __ldcg(col + r2));
  const IO* col2 = raw + c2 * pr.NX;
  if (r2 < 0) return io_add(__ldcg(col + r), __ldcg(col2 + r));
  return io_add(io_add(__ldcg(col + r), __ldcg(col + r2)), io_add(__ldcg(col2 + r), __ldcg(col2 + r2)));
}

__device__ __forceinline__ float small_mult(const SmallProb& pr, long long r, long long c) {
  if (pr.mult_ones) return 1.0f;
  const int cc = ((pr.rinfo[r] & L_COPY2) ? 2 : 1) * ((pr.cinfo[c] & L_COPY2) ? 2 : 1);
  return cc == 1 ? 1.0f : (cc == 2 ? 0.5f : 0.25f);
}

// run f(gi, r, c) over this CTA's points (one thread per point of a chunk)
template <int N, class F>
__device__ __forceinline__ void small_points(const SmallProb& pr, int e0, int e1, F&& f) {
  constexpr int NN = N * N;
  constexpr int EC = kSmallThreads / NN;
  const int el = threadIdx.x / NN;
  const int pt = threadIdx.x - el * NN;
  const int j = pt / N, i = pt - j * N;
  if (el >= EC) return;
  for (int e = e0 + el; e < e1; e += EC) {
    const int ey = e / pr.Ex, ex = e - ey * pr.Ex;
    const long long r = (long long)ex * N + i, c = (long long)ey * N + j;
    f(r + c * pr.NX, r, c);
  }
}

__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned long long abs_bits(float v) {
  return (unsigned long long)__double_as_longlong((double)fabsf(v)) | (v != v ? 0x7ff8000000000000ull : 0ull);
}
__device__ __forceinline__ df sq_term(double rr, double d, float m) {
  const df a = d2df(rr);
  df h = df_mul_u(a, d2df(d));
  h.h *= m;
  h.l *= m;
  return df_mul_u(a, h);
}
__device__ __forceinline__ df sq_term(float rr, float d, float m) {
  const float h = rr * d * m;
  const float p = __fmul_rn(rr, h);
  return {p, __fmaf_rn(rr, h, -p)};
}

// CG on A y = rhs (P: PDF for FP64 vectors, PF32 for the FP32 inner solve);
// rhs is read as double and converted
template <class P, int N>
__device__ void small_cg(SmallProb& pr, cg::cluster_group& cl, SmallRed& red, int& rc, int e0, int e1,
                         const typename P::v (*Dr)[N], const typename P::v (*Ds)[N], typename P::v* U,
                         typename P::v* W, const double* rhs, typename P::io* y, typename P::io* r,
                         typename P::io* p, typename P::io* raw, const typename P::io* dinv,
                         const typename GeoT<P>::type* Geo, double tol, int maxiter, int& iters,
                         double& rmax_out, bool& nan_out, double& rmax0) {
  typedef typename P::io IO;
  const bool jac = dinv != nullptr;
  df s = {0.0f, 0.0f};
  unsigned long long mx = 0ull;
  small_points<N>(pr, e0, e1, [&](long long gi, long long rr, long long cc) {
    const IO ri = (IO)rhs[gi];
    y[gi] = (IO)0;
    p[gi] = (IO)0;
    r[gi] = ri;
    s = df_add_u(s, sq_term(ri, jac ? dinv[gi] : (IO)1, small_mult(pr, rr, cc)));
    const unsigned long long b = abs_bits(ri);
    mx = b > mx ? b : mx;
  });
  s = df_norm(s);
  small_reduce(cl, red, rc, s, mx);
  double t = df2d(s);
  double rmax = __longlong_as_double((long long)mx);
  rmax0 = rmax;
  double tprev = 1.0;
  int k = 0;
  bool nan = rmax != rmax;
  bool done = !(rmax > tol) || maxiter == 0 || nan;
  while (!done) {
    const double beta = k == 0 ? 0.0 : t / tprev;
    df dot = {0.0f, 0.0f};
    small_apply<P, N>(pr, e0, e1, Dr, Ds, U, W, nullptr, true, r, dinv, (IO)beta, p, Geo, raw, dot);
    unsigned long long none = 0ull;
    dot = df_norm(dot);
    small_reduce(cl, red, rc, dot, none);  // also the barrier after the raw stores
    double pap = df2d(dot);
    if (pr.mult_ones) {
      // unweighted dots (pcg's default mult = ones): p . Ap over every local
      // copy of the assembled Ap, which the unassembled sum does not give
      df d2 = {0.0f, 0.0f};
      small_points<N>(pr, e0, e1, [&](long long gi, long long rr, long long cc) {
        d2 = df_add_u(d2, dot_term(p[gi], small_gather(pr, raw, rr, cc)));
      });
      d2 = df_norm(d2);
      small_reduce(cl, red, rc, d2, none);
      pap = df2d(d2);
    }
    const double alpha = t / pap;
    ++k;
    df s2 = {0.0f, 0.0f};
    unsigned long long m2 = 0ull;
    small_points<N>(pr, e0, e1, [&](long long gi, long long rr, long long cc) {
      const IO ap = small_gather(pr, raw, rr, cc);
      y[gi] = y[gi] + (IO)alpha * p[gi];
      const IO ri = r[gi] - (IO)alpha * ap;
      r[gi] = ri;
      s2 = df_add_u(s2, sq_term(ri, jac ? dinv[gi] : (IO)1, small_mult(pr, rr, cc)));
      const unsigned long long b = abs_bits(ri);
      m2 = b > m2 ? b : m2;
    });
    s2 = df_norm(s2);
    small_reduce(cl, red, rc, s2, m2);  // also the barrier before the next raw stores
    tprev = t;
    t = df2d(s2);
    rmax = __longlong_as_double((long long)m2);
    nan = (rmax != rmax) || (alpha != alpha);
    done = !(rmax > tol) || k >= maxiter || nan;
  }
  iters = k;
  rmax_out = rmax;
  nan_out = nan;
}

// SEM_MIXED_RR: one FP32 CG (x32, r32, p32) whose residual is replaced by the
// FP64 residual b - A x (x += x32 first, x in FP64) whenever it has fallen by
// the factor inner_tol since the last replacement; p32 and the beta
// recurrence continue across replacements.
template <int N>
__device__ void small_rr(SmallProb& pr, cg::cluster_group& cl, SmallRed& red, int& rc, int e0, int e1,
                         const df (*Ddr)[N], const df (*Dds)[N], const float (*Dfr)[N],
                         const float (*Dfs)[N], df* Ubuf, df* Wbuf) {
  const bool jac = pr.jacobi != 0;
  float* U32 = reinterpret_cast<float*>(Ubuf);
  float* W32 = reinterpret_cast<float*>(Wbuf);
  const float* dinv32 = jac ? pr.dinv32 : nullptr;
  // x = 0, r = b (FP64)
  unsigned long long mx = 0ull;
  df z = {0.0f, 0.0f};
  small_points<N>(pr, e0, e1, [&](long long gi, long long, long long) {
    pr.x[gi] = 0.0;
    pr.r[gi] = pr.b[gi];
    const unsigned long long b = abs_bits(pr.b[gi]);
    mx = b > mx ? b : mx;
  });
  small_reduce(cl, red, rc, z, mx);
  double rmax64 = __longlong_as_double((long long)mx);
  const double res0 = rmax64;
  // r32 = (float) r, x32 = 0 (p32 = 0 the first time); t = r32 . dinv r32 . mult
  auto load_r32 = [&](bool zero_p) -> double {
    df sacc = {0.0f, 0.0f};
    unsigned long long none = 0ull;
    small_points<N>(pr, e0, e1, [&](long long gi, long long rr, long long cc) {
      const float ri = (float)pr.r[gi];
      pr.r32[gi] = ri;
      pr.x32[gi] = 0.0f;
      if (zero_p) pr.p32[gi] = 0.0f;
      sacc = df_add_u(sacc, sq_term(ri, jac ? dinv32[gi] : 1.0f, small_mult(pr, rr, cc)));
    });
    sacc = df_norm(sacc);
    small_reduce(cl, red, rc, sacc, none);
    return df2d(sacc);
  };
  double t = load_r32(true);
  double tprev = 1.0;
  double thresh = pr.inner_tol * rmax64;
  int k = 0, outer = 0;
  bool nan = rmax64 != rmax64;
  bool done = !(rmax64 > pr.tol) || pr.maxiter == 0 || nan;
  while (!done) {
    const float beta = k == 0 ? 0.0f : (float)(t / tprev);
    df dot = {0.0f, 0.0f};
    small_apply<PF32, N>(pr, e0, e1, Dfr, Dfs, U32, W32, nullptr, true, pr.r32, dinv32, beta, pr.p32, pr.Gf,
                         pr.raw32, dot);
    unsigned long long none = 0ull;
    dot = df_norm(dot);
    small_reduce(cl, red, rc, dot, none);
    double pap = df2d(dot);
    if (pr.mult_ones) {
      df d2 = {0.0f, 0.0f};
      small_points<N>(pr, e0, e1, [&](long long gi, long long rr, long long cc) {
        d2 = df_add_u(d2, dot_term(pr.p32[gi], small_gather(pr, pr.raw32, rr, cc)));
      });
      d2 = df_norm(d2);
      small_reduce(cl, red, rc, d2, none);
      pap = df2d(d2);
    }
    const double alpha = t / pap;
    const float af = (float)alpha;
    ++k;
    df s2 = {0.0f, 0.0f};
    unsigned long long m2 = 0ull;
    small_points<N>(pr, e0, e1, [&](long long gi, long long rr, long long cc) {
      const float ap = small_gather(pr, pr.raw32, rr, cc);
      pr.x32[gi] = pr.x32[gi] + af * pr.p32[gi];
      const float ri = pr.r32[gi] - af * ap;
      pr.r32[gi] = ri;
      s2 = df_add_u(s2, sq_term(ri, jac ? dinv32[gi] : 1.0f, small_mult(pr, rr, cc)));
      const unsigned long long b = abs_bits(ri);
      m2 = b > m2 ? b : m2;
    });
    s2 = df_norm(s2);
    small_reduce(cl, red, rc, s2, m2);
    tprev = t;
    t = df2d(s2);
    const double rmax32 = __longlong_as_double((long long)m2);
    const bool nan32 = (rmax32 != rmax32) || (alpha != alpha);
    if (!(rmax32 > thresh) || k >= pr.maxiter || nan32) {
      // replacement: x += x32, r = b - A x in FP64
      small_points<N>(pr, e0, e1, [&](long long gi, long long, long long) { pr.x[gi] += (double)pr.x32[gi]; });
      __syncthreads();
      df unused = {0.0f, 0.0f};
      small_apply<PDF, N>(pr, e0, e1, Ddr, Dds, Ubuf, Wbuf, pr.x, false, nullptr, nullptr, 0.0, nullptr,
                          pr.Gdf, pr.raw, unused);
      cl.sync();
      unsigned long long m3 = 0ull;
      small_points<N>(pr, e0, e1, [&](long long gi, long long rr, long long cc) {
        const double v = pr.b[gi] - small_gather(pr, pr.raw, rr, cc);
        pr.r[gi] = v;
        const unsigned long long b = abs_bits(v);
        m3 = b > m3 ? b : m3;
      });
      df z3 = {0.0f, 0.0f};
      small_reduce(cl, red, rc, z3, m3);
      rmax64 = __longlong_as_double((long long)m3);
      ++outer;
      nan = rmax64 != rmax64 || nan32;
      done = !(rmax64 > pr.tol) || k >= pr.maxiter || nan || outer >= pr.max_outer;
      if (!done) {
        t = load_r32(false);
        thresh = pr.inner_tol * rmax64;
      }
    }
  }
  if (cl.block_rank() == 0 && threadIdx.x == 0) {
    pr.iters = k;
    pr.outer = outer;
    pr.res_inf = rmax64;
    pr.res0_inf = res0;
    pr.nan = nan;
    pr.converged = !(rmax64 > pr.tol) && !nan;
  }
}

template <int N>
__global__ void __launch_bounds__(kSmallThreads, 1) k_small_pcg(const __grid_constant__ SmallArgs<N> a) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int nr = (int)cl.num_blocks();
  SmallProb& pr = *a.pr;
  __shared__ SmallRed red;
  __shared__ df Ddf[2][N][N];
  __shared__ float Df[2][N][N];
  __shared__ df Ubuf[kSmallThreads];
  __shared__ df Wbuf[kSmallThreads];
  for (int q = threadIdx.x; q < 2 * N * N; q += blockDim.x) {
    (&Ddf[0][0][0])[q] = (&a.Ddf[0][0][0])[q];
    (&Df[0][0][0])[q] = (&a.Df[0][0][0])[q];
  }
  __syncthreads();
  int rc = 0;
  int e0, e1;
  small_range(pr, rank, nr, e0, e1);
  const bool jac = pr.jacobi != 0;
  if (pr.precision == SEM_MIXED_RR) {
    small_rr<N>(pr, cl, red, rc, e0, e1, Ddf[0], Ddf[1], Df[0], Df[1], Ubuf, Wbuf);
    cl.sync();  // no CTA exits while another may still read its shared memory
    return;
  }
  if (pr.precision != SEM_MIXED) {
    int it = 0;
    double rmax = 0.0;
    bool nan = false;
    double r0 = 0.0;
    small_cg<PDF, N>(pr, cl, red, rc, e0, e1, Ddf[0], Ddf[1], Ubuf, Wbuf, pr.b, pr.x, pr.r, pr.p, pr.raw,
                     jac ? pr.dinv : nullptr, pr.Gdf, pr.tol, pr.maxiter, it, rmax, nan, r0);
    if (rank == 0 && threadIdx.x == 0) {
      pr.iters = it;
      pr.outer = 0;
      pr.res0_inf = r0;
      pr.res_inf = rmax;
      pr.nan = nan;
      pr.converged = !(rmax > pr.tol) && !nan;
    }
    cl.sync();  // no CTA exits while another may still read its shared memory
    return;
  }
  // FP64 defect correction around the FP32 inner CG: x = 0, r = b
  df z = {0.0f, 0.0f};
  unsigned long long mx = 0ull;
  small_points<N>(pr, e0, e1, [&](long long gi, long long, long long) {
    pr.x[gi] = 0.0;
    pr.r[gi] = pr.b[gi];
    const unsigned long long b = abs_bits(pr.b[gi]);
    mx = b > mx ? b : mx;
  });
  small_reduce(cl, red, rc, z, mx);
  double rmax = __longlong_as_double((long long)mx);
  const double res0 = rmax;
  int outer = 0, total = 0;
  bool nan = rmax != rmax;
  float* U32 = reinterpret_cast<float*>(Ubuf);
  float* W32 = reinterpret_cast<float*>(Wbuf);
  while (!(rmax <= pr.tol) && !nan && outer < pr.max_outer) {
    ++outer;
    int it = 0;
    double rin = 0.0;
    bool nin = false;
    double rin0 = 0.0;
    small_cg<PF32, N>(pr, cl, red, rc, e0, e1, Df[0], Df[1], U32, W32, pr.r, pr.x32, pr.r32, pr.p32,
                      pr.raw32, jac ? pr.dinv32 : nullptr, pr.Gf, pr.inner_tol * rmax, pr.maxiter, it, rin,
                      nin, rin0);
    total += it;
    // x += x32; then r = b - A x (FP64, double-float operator) and max|r|
    small_points<N>(pr, e0, e1, [&](long long gi, long long, long long) { pr.x[gi] += (double)pr.x32[gi]; });
    __syncthreads();
    df unused = {0.0f, 0.0f};
    small_apply<PDF, N>(pr, e0, e1, Ddf[0], Ddf[1], Ubuf, Wbuf, pr.x, false, nullptr, nullptr, 0.0, nullptr,
                        pr.Gdf, pr.raw, unused);
    cl.sync();
    unsigned long long m2 = 0ull;
    small_points<N>(pr, e0, e1, [&](long long gi, long long rr, long long cc) {
      const double v = pr.b[gi] - small_gather(pr, pr.raw, rr, cc);
      pr.r[gi] = v;
      const unsigned long long b = abs_bits(v);
      m2 = b > m2 ? b : m2;
    });
    df z2 = {0.0f, 0.0f};
    small_reduce(cl, red, rc, z2, m2);
    rmax = __longlong_as_double((long long)m2);
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
  cl.sync();  // no CTA exits while another may still read its shared memory
}

template <int N>
static int launch_small(SmallProb* dev, const OperatorSet& ops, cudaStream_t s) {
  SmallArgs<N> a;
  std::memset(&a, 0, sizeof(a));
  a.pr = dev;
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < N; ++k) {
      const double dr = ops.Dr[i + k * N], ds = ops.Ds[i + k * N];
      a.Ddf[0][i][k] = PDF::from_double(dr);
      a.Ddf[1][i][k] = PDF::from_double(ds);
      a.Df[0][i][k] = (float)dr;
      a.Df[1][i][k] = (float)ds;
    }
  auto kern = k_small_pcg<N>;
  SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.blockDim = dim3(((kSmallThreads / (N * N)) * N * N + 31) / 32 * 32);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  int cluster = kSmallMaxCluster;
  for (; cluster >= 2; cluster /= 2) {
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cluster);
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters >= 1) break;
    cudaGetLastError();
  }
  if (cluster < 2) return set_error(SEM_ERR_UNSUPPORTED, "no thread-block cluster fits the small-mesh solver");
  SEM_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
  return SEM_OK;
}

int launch_small_pcg(SmallProb* dev, const OperatorSet& ops, int n, cudaStream_t s) {
  switch (n) {
    case 2: return launch_small<2>(dev, ops, s);
    case 3: return launch_small<3>(dev, ops, s);
    case 4: return launch_small<4>(dev, ops, s);
    case 5: return launch_small<5>(dev, ops, s);
    case 6: return launch_small<6>(dev, ops, s);
    case 7: return launch_small<7>(dev, ops, s);
    case 8: return launch_small<8>(dev, ops, s);
    case 9: return launch_small<9>(dev, ops, s);
    case 10: return launch_small<10>(dev, ops, s);
    case 11: return launch_small<11>(dev, ops, s);
    default: return set_error(SEM_ERR_UNSUPPORTED, "the small-mesh solver serves 2 <= n <= 11");
  }
}

}  // namespace sem
