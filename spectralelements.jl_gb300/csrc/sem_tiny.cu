// Mixed-precision PCG of a whole small mesh in ONE thread block (SEM_MIXED on
// meshes whose FP32 working set fits an SM's shared memory: cfg3, 8x8
// elements, N=8, 5,184 local DOF, 187 KB).
//
// The single-cluster solver of sem_small.cu spends its ~12 us per iteration on
// cluster barriers and distributed-shared-memory reductions, in either
// arithmetic, so its FP32 inner iterations are no cheaper than FP64 ones.
// Here one CTA holds the FP32 geometry (G11, G12, G22, B), the Jacobi
// inverse diagonal and every FP32 vector of the inner CG in shared memory, and
// an iteration costs block barriers only:
//
//   p   points: p = z + beta p (z = dinv .* r)
//   P1  lines: row line -> us = Ds u, column line -> ur = Dr u (even-odd form,
//       one thread per line; the local layout's rows are coalesced across a
//       warp and its columns are stride-n, both free of bank conflicts)
//   P2  row lines: wr, ws = G (ur, us), os = Ds' ws; wr and os stored in place
//   P3  column lines: res = nu (Dr' wr + os) + k B u, unassembled, and the
//       block-wide p . A p over the unassembled products (equal to the
//       mult-weighted dot of the assembled A p for a continuous masked p)
//   P4  points: A p = QQ'(res) masked (x pairs first, the order of every other
//       kernel), x += alpha p, r -= alpha A p, r . z . mult and max|r|
//
// The FP64 defect correction runs in the same launch: x (FP64, global) +=
// x32, then r = b - A x with the double-float operator (the same phases with
// double-float line buffers in the shared memory the FP32 vectors free),
// max|r|, and the next inner solve.  Results go to the SmallProb record as the
// cluster solver writes them; the host finishes a solve whose sweeps ran out
// with the FP64 CG (sem_pcg.cu).
//
// Reference: pcg (src/pcg.jl:16-60), laplace (src/lapl.jl:70-81), hlmz
// (src/hlmz.jl:12-19), gatherScatter (src/gatherScatter.jl:8-16), mask
// (src/mask.jl:10-18).
#include <cstring>

#include "sem_apply2.cuh"

namespace sem {

constexpr int kTinyMaxThreads = 1024;

template <int N>
struct TinyArgs {
  SmallProb* pr;
  EOCoef<N, float> Dr, Drt, Ds, Dst;  // FP32 inner operator
  EOCoef<N, df> Dr2, Drt2, Ds2, Dst2;  // double-float FP64 residual
};

// shared-memory layout in 4-byte words: the persistent block (G11, G12, G22,
// [B], [dinv]) then the work block (x32, r32, p32, line buffers A and B)
struct TinyLayout {
  long long g11, g12, g22, b, dinv, x32, r32, p32, la, lb, words;
};

__host__ __device__ inline TinyLayout tiny_layout(long long L, bool mass, bool jac) {
  TinyLayout t;
  long long o = 0;
  t.g11 = o; o += L;
  t.g12 = o; o += L;
  t.g22 = o; o += L;
  t.b = o; o += mass ? L : 0;
  t.dinv = o; o += jac ? L : 0;
  o = (o + 1) & ~1LL;  // the work block holds double-float pairs in the FP64 residual
  t.x32 = o; o += L;
  t.r32 = o; o += L;
  t.p32 = o; o += L;
  t.la = o; o += L;
  t.lb = o; o += L;
  t.words = o;
  return t;
}

// fixed-order block sums: warp trees, then the warps in order; the result is
// broadcast to every thread
__device__ __forceinline__ double tiny_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = red[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    red[32] = s;
  }
  __syncthreads();
  return red[32];
}

__device__ __forceinline__ unsigned long long tiny_max(unsigned long long v, unsigned long long* red) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, v, o);
    v = y > v ? y : v;
  }
  const int w = threadIdx.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = red[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) m = red[i] > m ? red[i] : m;
    red[32] = m;
  }
  __syncthreads();
  return red[32];
}

// magnitude bits as the bits of the double of the same value (NaN orders above
// everything)
__device__ __forceinline__ unsigned long long tiny_abs_bits(float v) {
  return (unsigned long long)__double_as_longlong((double)fabsf(v)) | (v != v ? 0x7ff8000000000000ull : 0ull);
}
__device__ __forceinline__ unsigned long long tiny_abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// The operator, unassembled and unmasked, res = nu (D'G D u) + k B u, on every
// line of the mesh.  U: the input field (shared or global); A, Bf: two line
// buffers of L entries (shared); G11..Bm: the metric terms and mass (shared
// FP32 or global pre-split pairs; Bm NULL without a mass term).  The result
// is left in A; acc receives this thread's part of u . res.
template <class P, int N, class GT>
__device__ __forceinline__ void tiny_apply(const SmallProb& pr, const typename P::io* U, typename P::v* A,
                                           typename P::v* Bf, const GT* G11, const GT* G12, const GT* G22,
                                           const GT* Bm, typename P::v nu, typename P::v kk,
                                           const EOCoef<N, typename P::v>& Dr, const EOCoef<N, typename P::v>& Drt,
                                           const EOCoef<N, typename P::v>& Ds, const EOCoef<N, typename P::v>& Dst,
                                           double& acc) {
  typedef typename P::v V;
  const long long NX = pr.NX;
  const int nl = (int)(NX * pr.Ey);  // lines per direction
  const int Ex = pr.Ex;
  // P1: us on the row lines -> Bf, ur on the column lines -> A
  for (int l = threadIdx.x; l < nl; l += blockDim.x) {
    {
      const long long r = l % NX;
      const long long c0 = (long long)(l / NX) * N;
      V x[N], y[N];
#pragma unroll
      for (int j = 0; j < N; ++j) x[j] = P::cvt(U[r + (c0 + j) * NX]);
      eo_apply<P, N>(Ds, x, y);
#pragma unroll
      for (int j = 0; j < N; ++j) Bf[r + (c0 + j) * NX] = y[j];
    }
    {
      const long long ex = l % Ex;
      const long long c = l / Ex;
      const long long b0 = ex * N + c * NX;
      V x[N], y[N];
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = P::cvt(U[b0 + i]);
      eo_apply<P, N>(Dr, x, y);
#pragma unroll
      for (int i = 0; i < N; ++i) A[b0 + i] = y[i];
    }
  }
  __syncthreads();
  // P2: row lines: wr = G11 ur + G12 us -> A, ws = G12 ur + G22 us, os = Ds' ws -> Bf
  for (int l = threadIdx.x; l < nl; l += blockDim.x) {
    const long long r = l % NX;
    const long long c0 = (long long)(l / NX) * N;
    V ws[N], os[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const long long q = r + (c0 + j) * NX;
      const V ur = A[q], us = Bf[q];
      const V g11 = GeoT<P>::cvt(G11[q]), g12 = GeoT<P>::cvt(G12[q]), g22 = GeoT<P>::cvt(G22[q]);
      A[q] = P::fma(g11, ur, P::mul(g12, us));
      ws[j] = P::fma(g12, ur, P::mul(g22, us));
    }
    eo_apply<P, N>(Dst, ws, os);
#pragma unroll
    for (int j = 0; j < N; ++j) Bf[r + (c0 + j) * NX] = os[j];
  }
  __syncthreads();
  // P3: column lines: res = nu (Dr' wr + os) + k B u -> A
  for (int l = threadIdx.x; l < nl; l += blockDim.x) {
    const long long ex = l % Ex;
    const long long c = l / Ex;
    const long long b0 = ex * N + c * NX;
    V x[N], y[N];
#pragma unroll
    for (int i = 0; i < N; ++i) x[i] = A[b0 + i];
    eo_apply<P, N>(Drt, x, y);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const long long q = b0 + i;
      V res = P::fin(P::mul(nu, P::add(y[i], Bf[q])));
      if (Bm) res = P::fin(P::fma(P::mul(kk, GeoT<P>::cvt(Bm[q])), P::cvt(U[q]), res));
      A[q] = res;
      if constexpr (P::kPrecision == SEM_F32) acc += (double)U[q] * (double)res;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ float tiny_mult(const SmallProb& pr, long long r, long long c) {
  if (pr.mult_ones) return 1.0f;
  const int cc = ((pr.rinfo[r] & L_COPY2) ? 2 : 1) * ((pr.cinfo[c] & L_COPY2) ? 2 : 1);
  return cc == 1 ? 1.0f : (cc == 2 ? 0.5f : 0.25f);
}

// QQ' and mask at local point (r, c) of an unassembled field: the sum of its
// copies, x pairs first (as small_gather); each copy converted by cv first
template <class T, class F>
__device__ __forceinline__ auto tiny_gather(const SmallProb& pr, const T* raw, long long r, long long c, F&& cv,
                                            bool& zero) {
  const unsigned char br = pr.rinfo[r], bc = pr.cinfo[c];
  zero = pr.has_bc && ((br | bc) & L_ZERO);
  const long long r2 = line_partner(r, br, pr.NX);
  const long long c2 = line_partner(c, bc, pr.NY);
  const T* col = raw + c * pr.NX;
  if (c2 < 0) return r2 < 0 ? cv(col[r]) : io_add(cv(col[r]), cv(col[r2]));
  const T* col2 = raw + c2 * pr.NX;
  if (r2 < 0) return io_add(cv(col[r]), cv(col2[r]));
  return io_add(io_add(cv(col[r]), cv(col[r2])), io_add(cv(col2[r]), cv(col2[r2])));
}

template <int N>
__global__ void __launch_bounds__(kTinyMaxThreads, 1) k_tiny_pcg(const __grid_constant__ TinyArgs<N> a) {
  SmallProb& pr = *a.pr;
  extern __shared__ __align__(16) float sm[];
  __shared__ double red_d[33];
  __shared__ unsigned long long red_m[33];
  const long long NX = pr.NX, L = pr.NX * pr.NY;
  const bool jac = pr.jacobi != 0;
  const bool mass = pr.k != 0.0;
  const TinyLayout lay = tiny_layout(L, mass, jac);
  float* G11 = sm + lay.g11;
  float* G12 = sm + lay.g12;
  float* G22 = sm + lay.g22;
  float* Bs = mass ? sm + lay.b : nullptr;
  float* dinv = jac ? sm + lay.dinv : nullptr;
  float* x32 = sm + lay.x32;
  float* r32 = sm + lay.r32;
  float* p32 = sm + lay.p32;
  float* LA = sm + lay.la;
  float* LB = sm + lay.lb;
  const int T = blockDim.x;

  // persistent block: FP32 geometry and Jacobi inverse diagonal
  for (long long q = threadIdx.x; q < L; q += T) {
    G11[q] = pr.Gf[q];
    G12[q] = pr.Gf[L + q];
    G22[q] = pr.Gf[2 * L + q];
    if (mass) Bs[q] = pr.Gf[3 * L + q];
    if (jac) dinv[q] = pr.dinv32[q];
  }
  // x = 0, r = b (FP64, global), max|b|
  unsigned long long m0 = 0ull;
  for (long long q = threadIdx.x; q < L; q += T) {
    const double v = pr.b[q];
    pr.x[q] = 0.0;
    pr.r[q] = v;
    const unsigned long long bb = tiny_abs_bits(v);
    m0 = bb > m0 ? bb : m0;
  }
  double rmax = __longlong_as_double((long long)tiny_max(m0, red_m));
  const double res0 = rmax;
  int outer = 0, total = 0;
  bool nan = rmax != rmax;
  const float nu32 = (float)pr.nu, k32 = (float)pr.k;
  const df nu2 = d2df(pr.nu), k2 = d2df(pr.k);  // both inside the pair window (small_eligible)
  while (!(rmax <= pr.tol) && !nan && outer < pr.max_outer && total < pr.maxiter) {
    ++outer;
    // ---- inner FP32 CG on A d = r to inner_tol * |r|_inf: x32 = 0, r32 = r, p32 = 0
    const double thresh = pr.inner_tol * rmax;
    double tl = 0.0;
    unsigned long long ml = 0ull;
    for (long long q = threadIdx.x; q < L; q += T) {
      const float ri = (float)pr.r[q];
      r32[q] = ri;
      x32[q] = 0.0f;
      p32[q] = 0.0f;
      const long long c = q / NX, r = q - c * NX;
      const float z = jac ? ri * dinv[q] : ri;
      tl += (double)(ri * z * tiny_mult(pr, r, c));
      const unsigned long long bb = tiny_abs_bits(ri);
      ml = bb > ml ? bb : ml;
    }
    double t = tiny_sum(tl, red_d);
    double rin = __longlong_as_double((long long)tiny_max(ml, red_m));
    double tprev = 1.0;
    int k = 0;
    bool nin = rin != rin;
    bool done = !(rin > thresh) || nin || total >= pr.maxiter;
    while (!done) {
      const float beta = k == 0 ? 0.0f : (float)(t / tprev);
      for (long long q = threadIdx.x; q < L; q += T) {
        const float z = jac ? r32[q] * dinv[q] : r32[q];
        p32[q] = __fmaf_rn(beta, p32[q], z);
      }
      __syncthreads();
      double pap_l = 0.0;
      tiny_apply<PF32, N, float>(pr, p32, LA, LB, G11, G12, G22, Bs, nu32, k32, a.Dr, a.Drt, a.Ds, a.Dst,
                                 pap_l);
      const double pap = tiny_sum(pap_l, red_d);
      const double alpha = t / pap;
      const float af = (float)alpha;
      ++k;
      ++total;
      double sl = 0.0;
      unsigned long long mx = 0ull;
      for (long long q = threadIdx.x; q < L; q += T) {
        const long long c = q / NX, r = q - c * NX;
        bool zero;
        float ap = tiny_gather(pr, LA, r, c, [](float v) { return v; }, zero);
        if (zero) ap = 0.0f;
        x32[q] = __fmaf_rn(af, p32[q], x32[q]);
        const float ri = __fmaf_rn(-af, ap, r32[q]);
        r32[q] = ri;
        const float z = jac ? ri * dinv[q] : ri;
        sl += (double)(ri * z * tiny_mult(pr, r, c));
        const unsigned long long bb = tiny_abs_bits(ri);
        mx = bb > mx ? bb : mx;
      }
      tprev = t;
      t = tiny_sum(sl, red_d);
      rin = __longlong_as_double((long long)tiny_max(mx, red_m));
      nin = (rin != rin) || (alpha != alpha);
      done = !(rin > thresh) || nin || total >= pr.maxiter;
    }
    // ---- x += x32 (FP64); r = b - A x with the double-float operator
    for (long long q = threadIdx.x; q < L; q += T) pr.x[q] += (double)x32[q];
    __syncthreads();
    df* DA = reinterpret_cast<df*>(sm + lay.x32);  // the work block, free now: 2 L pairs
    df* DB = DA + L;
    double unused = 0.0;
    const df* Gdf = pr.Gdf;
    tiny_apply<PDF, N, df>(pr, pr.x, DA, DB, Gdf, Gdf + L, Gdf + 2 * L, mass ? Gdf + 3 * L : nullptr, nu2, k2,
                           a.Dr2, a.Drt2, a.Ds2, a.Dst2, unused);
    unsigned long long m2 = 0ull;
    for (long long q = threadIdx.x; q < L; q += T) {
      const long long c = q / NX, r = q - c * NX;
      bool zero;
      // each copy rounded to FP64 first, then summed in FP64 (the order of the
      // chunked path's tile stores and fixup)
      const double ax = tiny_gather(pr, DA, r, c, [](df v) { return df2d(v); }, zero);
      const double v = zero ? 0.0 : pr.b[q] - ax;
      pr.r[q] = v;
      const unsigned long long bb = tiny_abs_bits(v);
      m2 = bb > m2 ? bb : m2;
    }
    rmax = __longlong_as_double((long long)tiny_max(m2, red_m));
    nan = rmax != rmax || nin;
    __syncthreads();  // the work block is the FP32 vectors again
  }
  if (threadIdx.x == 0) {
    pr.iters = total;
    pr.outer = outer;
    pr.res_inf = rmax;
    pr.res0_inf = res0;
    pr.nan = nan;
    pr.converged = rmax <= pr.tol && !nan;
  }
}

template <class V, int N>
static void fill_eo_tiny(EOCoef<N, V>& c, const double* src, V (*cvt)(double)) {
  constexpr int M = N / 2;
  const double* A = src;
  const double* C = A + M * M;
  const double* cm = C + M * M;
  const double* mr = cm + M;
  for (int i = 0; i < M; ++i)
    for (int k = 0; k < M; ++k) {
      c.A[i][k] = cvt(A[i * M + k]);
      c.Cc[i][k] = cvt(C[i * M + k]);
    }
  for (int i = 0; i < M; ++i) {
    c.cm[i] = cvt(cm[i]);
    c.mr[i] = cvt(mr[i]);
  }
}

static float to_f32(double d) { return (float)d; }
static df to_df(double d) { return PDF::from_double(d); }

size_t tiny_smem_bytes(long long L, bool mass, bool jac) {
  return (size_t)tiny_layout(L, mass, jac).words * 4;
}

template <int N>
static int launch_tiny(SmallProb* dev, const SmallProb& host, const OperatorSet& ops, size_t smem, cudaStream_t s) {
  TinyArgs<N> a;
  std::memset(&a, 0, sizeof(a));
  a.pr = dev;
  fill_eo_tiny<float, N>(a.Dr, ops.eo[0], to_f32);
  fill_eo_tiny<float, N>(a.Drt, ops.eo[1], to_f32);
  fill_eo_tiny<float, N>(a.Ds, ops.eo[2], to_f32);
  fill_eo_tiny<float, N>(a.Dst, ops.eo[3], to_f32);
  fill_eo_tiny<df, N>(a.Dr2, ops.eo[0], to_df);
  fill_eo_tiny<df, N>(a.Drt2, ops.eo[1], to_df);
  fill_eo_tiny<df, N>(a.Ds2, ops.eo[2], to_df);
  fill_eo_tiny<df, N>(a.Dst2, ops.eo[3], to_df);
  const long long nl = host.NX * host.Ey;
  int threads = (int)((nl + 31) / 32 * 32);
  if (threads > kTinyMaxThreads) threads = kTinyMaxThreads;
  if (threads < 64) threads = 64;
  auto kern = k_tiny_pcg<N>;
  SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<1, threads, smem, s>>>(a);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int launch_tiny_pcg(SmallProb* dev, const SmallProb& host, const OperatorSet& ops, size_t smem, cudaStream_t s) {
  switch (host.n) {
    case 2: return launch_tiny<2>(dev, host, ops, smem, s);
    case 3: return launch_tiny<3>(dev, host, ops, smem, s);
    case 4: return launch_tiny<4>(dev, host, ops, smem, s);
    case 5: return launch_tiny<5>(dev, host, ops, smem, s);
    case 6: return launch_tiny<6>(dev, host, ops, smem, s);
    case 7: return launch_tiny<7>(dev, host, ops, smem, s);
    case 8: return launch_tiny<8>(dev, host, ops, smem, s);
    case 9: return launch_tiny<9>(dev, host, ops, smem, s);
    case 10: return launch_tiny<10>(dev, host, ops, smem, s);
    case 11: return launch_tiny<11>(dev, host, ops, smem, s);
    default: return set_error(SEM_ERR_UNSUPPORTED, "the single-block solver serves 2 <= n <= 11");
  }
}

}  // namespace sem
