// Mixed-precision PCG of a whole small mesh in ONE launch of a small cluster
// of thread blocks (SEM_MIXED on meshes whose FP32 working set fits the
// cluster's shared memory: cfg3, 8x8 elements, N=8, 5,184 local DOF).
//
// Each CTA of the cluster owns a strip of whole element rows and keeps, in
// its shared memory, the strip's FP32 geometry (G11, G12, G22, B), Jacobi
// inverse diagonal and every FP32 vector of the inner CG.  The element
// operator's lines lie inside one element row, so the line phases of an
// iteration touch the CTA's own shared memory only:
//
//   P1  lines: row line -> us = Ds u, column line -> ur = Dr u (even-odd form,
//       one thread per line; the local layout's rows are coalesced across a
//       warp and its columns are stride-n, both free of bank conflicts)
//   P2  row lines: wr, ws = G (ur, us), os = Ds' ws; wr and os stored in place
//   P3  column lines: res = nu (Dr' wr + os) + k B u, unassembled, and the
//       cluster-wide p . A p over the unassembled products (equal to the
//       mult-weighted dot of the assembled A p for a continuous masked p)
//   P4  points: A p = QQ'(res) masked (x pairs first, the order of every other
//       kernel; a copy across a strip boundary is read from the neighbouring
//       CTA's shared memory), x += alpha p, r -= alpha A p, r . z . mult and
//       max|r|, and p stored; the direction p = z + beta p_old is formed where
//       P1, P3 and P4 read it, so it needs no pass of its own
//
// P1 and P2 end at block barriers; each reduction (after P3 and after P4)
// costs a block barrier and one cluster barrier, which also orders the
// neighbours' reads of the unassembled result against its next writes.
//
// The FP64 defect correction runs in the same launch: x (FP64, global) +=
// x32, then r = b - A x with the double-float operator (the same phases with
// double-float line buffers in the shared memory the FP32 vectors free),
// max|r|, and the next inner solve.  Indices are 32-bit.  Results go to the
// SmallProb record as the single-cluster solver of sem_small.cu writes them;
// the host finishes a solve whose sweeps ran out with the FP64 CG (sem_pcg.cu).
//
// Reference: pcg (src/pcg.jl:16-60), laplace (src/lapl.jl:70-81), hlmz
// (src/hlmz.jl:12-19), gatherScatter (src/gatherScatter.jl:8-16), mask
// (src/mask.jl:10-18).
#include <cooperative_groups.h>

#include <cstdlib>
#include <cstring>

#include "sem_apply2.cuh"

namespace cg = cooperative_groups;

namespace sem {

// one thread per line where the strip allows; 102 registers a thread at most
constexpr int kTinyMaxThreads = 640;

template <int N>
struct TinyArgs {
  SmallProb* pr;
  EOCoef<N, float> Dr, Drt, Ds, Dst;  // FP32 inner operator
  EOCoef<N, df> Dr2, Drt2, Ds2, Dst2;  // double-float FP64 residual
};

// reduction slots: per warp a double-float sum and a maximum, and the CTA's
// folded pair that the other CTAs of the cluster read; two of each
struct TinyRed {
  df s[2][32];
  unsigned long long m[2][32];
  df cs[2];
  unsigned long long cm[2];
};

// shared-memory layout in 4-byte words for a strip of L local points: the
// persistent block (G11, G12, G22, [B], [dinv]), the work block (x32, r32,
// p32, line buffers A, B, C and D), the reduction slots and the line bits
struct TinyLayout {
  long long g11, g12, g22, b, dinv, x32, r32, p32, la, lb, lc, ld, red, bits, words;
};

__host__ __device__ inline TinyLayout tiny_layout(long long L, bool mass, bool jac, long long nbits) {
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
  t.lc = o; o += L;
  t.ld = o; o += L;
  o = (o + 1) & ~1LL;
  t.red = o; o += (long long)(sizeof(TinyRed) / 4);
  t.bits = o; o += (nbits + 3) / 4;  // line bits of the rows, then of the columns
  t.words = o;
  return t;
}

// first element row of strip k when Ey element rows are split over C CTAs,
// and the strip that holds element row e
__host__ __device__ __forceinline__ int tiny_strip_row(int k, int Ey, int C) { return (int)((long long)k * Ey / C); }
__device__ __forceinline__ int tiny_strip_of(int e, int Ey, int C) { return (int)(((long long)(e + 1) * C - 1) / Ey); }

__device__ __forceinline__ void tiny_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Cluster-wide sum and maximum.  Each thread brings an FP32 partial sum (a
// handful of products) and a magnitude as bits.  Every warp folds its lanes
// in double-float (fixed shuffle tree, FP32 pipe only: FP64 runs at 1/64 of
// the FP32 rate) and lane 0 stores the warp's pair; after a block barrier
// thread 0 folds the warps in order into the CTA's pair; after a cluster
// barrier every warp reads the CTAs' pairs (lane j: CTA j) and folds them in
// rank order with the same tree, so every thread of the cluster holds the
// same result.  Consecutive calls alternate between two slots: a slot is
// written again only after the next call's cluster barrier, which every CTA
// reaches after it has read the slot.
__device__ __forceinline__ df tiny_warp_sum(df s) {
  for (int o = 16; o > 0; o >>= 1) {
    df y;
    y.h = __shfl_down_sync(0xffffffffu, s.h, o);
    y.l = __shfl_down_sync(0xffffffffu, s.l, o);
    s = df_add(s, y);
  }
  return s;
}

__device__ __forceinline__ unsigned long long tiny_warp_max(unsigned long long m) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, m, o);
    m = y > m ? y : m;
  }
  return m;
}

__device__ __forceinline__ df tiny_cluster_fold(TinyRed& red, int slot, unsigned long long& mx) {
  const int lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    df s = red.s[slot][0];
    unsigned long long m = red.m[slot][0];
    const int nw = (int)(blockDim.x >> 5);
    for (int i = 1; i < nw; ++i) {
      s = df_add(s, red.s[slot][i]);
      m = red.m[slot][i] > m ? red.m[slot][i] : m;
    }
    red.cs[slot] = s;
    red.cm[slot] = m;
  }
  tiny_cluster_sync();
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  df s = {0.0f, 0.0f};
  unsigned long long m = 0ull;
  if (lane < C) {
    const TinyRed* rr = cl.map_shared_rank(&red, lane);
    s = rr->cs[slot];
    m = rr->cm[slot];
  }
  s = tiny_warp_sum(s);
  m = tiny_warp_max(m);
  s.h = __shfl_sync(0xffffffffu, s.h, 0);
  s.l = __shfl_sync(0xffffffffu, s.l, 0);
  mx = __shfl_sync(0xffffffffu, m, 0);
  return s;
}

// FP32 partial sum and FP32 magnitude bits (the bits of |v|; NaN orders above
// everything): returns the cluster sum (rounded to FP32: the inner CG's
// scalars are FP32), mx the cluster maximum as an FP32 bit pattern
__device__ __forceinline__ float tiny_reduce(float v, unsigned& mx, TinyRed& red, int& slot) {
  const df s = tiny_warp_sum(df{v, 0.0f});
  const unsigned m = __reduce_max_sync(0xffffffffu, mx);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red.s[slot][w] = s;
    red.m[slot][w] = m;
  }
  __syncthreads();
  unsigned long long mm;
  const df r = tiny_cluster_fold(red, slot, mm);
  mx = (unsigned)mm;
  slot ^= 1;
  return r.h + r.l;
}

// cluster maximum of FP64 magnitude bits (the FP64 residual, once per sweep)
__device__ __forceinline__ unsigned long long tiny_reduce_max64(unsigned long long mx, TinyRed& red, int& slot) {
  mx = tiny_warp_max(mx);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red.s[slot][w] = {0.0f, 0.0f};
    red.m[slot][w] = mx;
  }
  __syncthreads();
  unsigned long long mm;
  tiny_cluster_fold(red, slot, mm);
  slot ^= 1;
  return mm;
}

__device__ __forceinline__ unsigned tiny_abs_bits(float v) { return __float_as_uint(v) & 0x7fffffffu; }
__device__ __forceinline__ unsigned long long tiny_abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// The strip, the mesh sizes, line bits and this thread's line walks, held in
// registers (read once from the problem record, which stores through generic
// pointers could otherwise alias).  Local indices are the strip's: point
// (r, c) of the mesh, c in [c0, c0 + NYs), is q = r + (c - c0) NX, global
// g = q + c0 NX.  Thread t handles lines t, t + T, ...; a row line l has row
// r = l mod NX and element row e = l div NX (of the strip), a column line l
// has element column x = l mod Ex and column c = l div Ex (of the strip).
// The walks advance (r, e) and (x, c) by T without dividing.
struct TinyDims {
  int NX, NY, Ex, Ey, nl, T;
  int C, rank, c0, NYs;  // cluster size, this CTA's rank, first column and columns of its strip
  int r0, e0, dr, de;    // row-line walk
  int x0, cc0, dx, dc;   // column-line walk
  // the FP32 inner loop runs two threads per line, in two warps: warp pair k
  // takes lines 32 k + lane, 32 k + lane + T/2, ...; half h = warp & 1 owns
  // the points j < H or j >= N - H of a line (h = 0) or the others (h = 1),
  // H = ceil(N/4), and forms the contraction outputs at those points
  int pl0, pls, half;
  int pr0, pe0, pdr, pde;  // pair row-line walk
  int px0, pcc0, pdx, pdc; // pair column-line walk
  const unsigned char* rinfo;  // line bits (shared-memory copies, whole mesh)
  const unsigned char* cinfo;
};

// the points of a line that half HH owns
template <int N, int HH>
__device__ __forceinline__ constexpr bool tiny_owns(int j) {
  return (j < (N / 2 + 1) / 2 || j >= N - (N / 2 + 1) / 2) == (HH == 0);
}

// eo_apply for the outputs half h owns: the even-odd sums in full, then the
// rows i of the half's pairs (i, N-1-i), and the middle output for h = 1
template <class P, int N, int HH>
__device__ __forceinline__ void eo_apply_half(const EOCoef<N, typename P::v>& D, const typename P::v (&x)[N],
                                              typename P::v (&y)[N]) {
  typedef typename P::v V;
  constexpr int M = N / 2;
  constexpr int H = (M + 1) / 2;
  V e[M], o[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    e[k] = P::add_u(x[k], x[N - 1 - k]);
    o[k] = P::sub_u(x[k], x[N - 1 - k]);
  }
#pragma unroll
  for (int i = 0; i < M; ++i) {
    if ((i < H) != (HH == 0)) continue;
    V s = P::mul(D.A[i][0], o[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) s = P::fma(D.A[i][k], o[k], s);
    V t = P::mul(D.Cc[i][0], e[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) t = P::fma(D.Cc[i][k], e[k], t);
    if (N & 1) t = P::fma(D.cm[i], x[M], t);
    y[i] = P::add_u(s, t);
    y[N - 1 - i] = P::sub_u(s, t);
  }
  if ((N & 1) && HH == 1) {
    V s = P::mul(D.mr[0], o[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) s = P::fma(D.mr[k], o[k], s);
    y[M] = s;
  }
}

__device__ __forceinline__ void tiny_step(int& a, int& b, int da, int db, int n) {
  a += da;
  b += db;
  if (a >= n) {
    a -= n;
    ++b;
  }
}

// The operator, unassembled and unmasked, res = nu (D'G D u) + k B u, on every
// line of the strip.  ufun(q) gives the input at local point q (shared or
// global memory, or formed on the fly); A, Bf: two line buffers of the
// strip's size (shared); G11..Bm: the metric terms and mass, strip-indexed
// (shared FP32 or global pre-split pairs; Bm NULL without a mass term).  The
// result is left in A; acc receives this thread's part of u . res (FP32
// policy).
template <class P, int N, class GT, class UF>
__device__ __forceinline__ void tiny_apply(const TinyDims& d, UF&& ufun, typename P::v* A, typename P::v* Bf,
                                           const GT* G11, const GT* G12, const GT* G22, const GT* Bm,
                                           typename P::v nu, typename P::v kk, const EOCoef<N, typename P::v>& Dr,
                                           const EOCoef<N, typename P::v>& Drt, const EOCoef<N, typename P::v>& Ds,
                                           const EOCoef<N, typename P::v>& Dst, float& acc) {
  typedef typename P::v V;
  const int NX = d.NX;
  const int EN = N * NX;  // points per element row
  // P1: us on the row lines -> Bf, ur on the column lines -> A
  {
    int r = d.r0, e = d.e0, x = d.x0, c = d.cc0;
    for (int l = threadIdx.x; l < d.nl; l += d.T) {
      {
        const int q0 = r + e * EN;
        V xs[N], ys[N];
#pragma unroll
        for (int j = 0; j < N; ++j) xs[j] = ufun(q0 + j * NX);
        eo_apply<P, N>(Ds, xs, ys);
#pragma unroll
        for (int j = 0; j < N; ++j) Bf[q0 + j * NX] = ys[j];
      }
      {
        const int b0 = x * N + c * NX;
        V xs[N], ys[N];
#pragma unroll
        for (int i = 0; i < N; ++i) xs[i] = ufun(b0 + i);
        eo_apply<P, N>(Dr, xs, ys);
#pragma unroll
        for (int i = 0; i < N; ++i) A[b0 + i] = ys[i];
      }
      tiny_step(r, e, d.dr, d.de, NX);
      tiny_step(x, c, d.dx, d.dc, d.Ex);
    }
  }
  __syncthreads();
  // P2: row lines: wr = G11 ur + G12 us -> A, ws = G12 ur + G22 us, os = Ds' ws -> Bf
  {
    int r = d.r0, e = d.e0;
    for (int l = threadIdx.x; l < d.nl; l += d.T) {
      const int q0 = r + e * EN;
      V ws[N], os[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const int q = q0 + j * NX;
        const V ur = A[q], us = Bf[q];
        const V g11 = GeoT<P>::cvt(G11[q]), g12 = GeoT<P>::cvt(G12[q]), g22 = GeoT<P>::cvt(G22[q]);
        A[q] = P::fma(g11, ur, P::mul(g12, us));
        ws[j] = P::fma(g12, ur, P::mul(g22, us));
      }
      eo_apply<P, N>(Dst, ws, os);
#pragma unroll
      for (int j = 0; j < N; ++j) Bf[q0 + j * NX] = os[j];
      tiny_step(r, e, d.dr, d.de, NX);
    }
  }
  __syncthreads();
  // P3: column lines: res = nu (Dr' wr + os) + k B u -> A
  {
    int x = d.x0, c = d.cc0;
    for (int l = threadIdx.x; l < d.nl; l += d.T) {
      const int b0 = x * N + c * NX;
      V xs[N], ys[N];
#pragma unroll
      for (int i = 0; i < N; ++i) xs[i] = A[b0 + i];
      eo_apply<P, N>(Drt, xs, ys);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const int q = b0 + i;
        V res = P::fin(P::mul(nu, P::add(ys[i], Bf[q])));
        if (Bm || P::kPrecision == SEM_F32) {
          const V u = ufun(q);
          if (Bm) res = P::fin(P::fma(P::mul(kk, GeoT<P>::cvt(Bm[q])), u, res));
          if constexpr (P::kPrecision == SEM_F32) acc = __fmaf_rn(u, res, acc);
        }
        A[q] = res;
      }
      tiny_step(x, c, d.dx, d.dc, d.Ex);
    }
  }
  // no barrier here: the caller's next reduction orders these stores before
  // the gather reads them (here and in the neighbouring CTAs)
}

// one local point of a row line of the strip, with what QQ', the mask and the
// weighted dots need: local and global index, its copies' rows and columns
// (mesh columns; -1: none), 1/multiplicity, and whether the mask zeroes it
struct TinyPt {
  int q, g, r, c, r2, c2;
  float mult;
  bool zero;
};

// QQ' at a point of an unassembled strip-indexed field `raw` of this CTA: the
// sum of its copies, x pairs first (as small_gather); a copy in another strip
// is read from that CTA's `raw` (the same offset in every CTA's shared
// memory); each copy converted by cv first
template <class T, class F>
__device__ __forceinline__ auto tiny_gather(const TinyDims& d, T* raw, const TinyPt& p, F&& cv) {
  const T* col = raw + (p.c - d.c0) * d.NX;
  if (p.c2 < 0) return p.r2 < 0 ? cv(col[p.r]) : io_add(cv(col[p.r]), cv(col[p.r2]));
  const T* col2;
  if (p.c2 >= d.c0 && p.c2 < d.c0 + d.NYs) {
    col2 = raw + (p.c2 - d.c0) * d.NX;
  } else {
    const int k = tiny_strip_of(p.c2 / (d.NY / d.Ey), d.Ey, d.C);
    const int c0k = tiny_strip_row(k, d.Ey, d.C) * (d.NY / d.Ey);
    col2 = cg::this_cluster().map_shared_rank(raw, k) + (p.c2 - c0k) * d.NX;
  }
  if (p.r2 < 0) return io_add(cv(col[p.r]), cv(col2[p.r]));
  return io_add(io_add(cv(col[p.r]), cv(col[p.r2])), io_add(cv(col2[p.r]), cv(col2[p.r2])));
}

// run f(point) over the points of this thread's row lines; the row's bits
// are decoded once per line
template <int N, class F>
__device__ __forceinline__ void tiny_points(const TinyDims& d, bool ones, bool has_bc, F&& f) {
  int r = d.r0, e = d.e0;
  for (int l = threadIdx.x; l < d.nl; l += d.T) {
    const unsigned char br = d.rinfo[r];
    const int r2 = (int)line_partner(r, br, d.NX);
    const float mr = (!ones && (br & L_COPY2)) ? 0.5f : 1.0f;
    const bool zr = has_bc && (br & L_ZERO);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const int cl = e * N + j;  // strip column
      const int c = d.c0 + cl;   // mesh column
      const unsigned char bc = d.cinfo[c];
      TinyPt p;
      p.q = r + cl * d.NX;
      p.g = p.q + d.c0 * d.NX;
      p.r = r;
      p.c = c;
      p.r2 = r2;
      p.c2 = (int)line_partner(c, bc, d.NY);
      p.mult = (!ones && (bc & L_COPY2)) ? 0.5f * mr : mr;
      p.zero = zr || (has_bc && (bc & L_ZERO));
      f(p);
    }
    tiny_step(r, e, d.dr, d.de, d.NX);
  }
}

// The FP32 operator of the inner loop with two threads per line (pair walks
// of TinyDims), in three phases without barriers; the caller separates them
// with block barriers at the same program point for every warp:
// res = nu (D'G D u) + k B u, unassembled, left in A.  Each half reads whole
// lines and writes only the points it owns, so no line buffer is read and
// written by different threads in one phase: P1 writes ur to A and us to Bf,
// P2 reads them and writes wr to Cb and os to Db, P3 reads Cb and its own
// points of Db and writes res to A.  P3 adds this thread's part of u . res
// over its points to acc.
template <int N, int HH, class UF>
__device__ __forceinline__ void tiny_pair_p1(const TinyDims& d, UF&& ufun, float* A, float* Bf,
                                             const EOCoef<N, float>& Dr, const EOCoef<N, float>& Ds) {
  const int NX = d.NX;
  const int EN = N * NX;
  int r = d.pr0, e = d.pe0, x = d.px0, c = d.pcc0;
  for (int l = d.pl0; l < d.nl; l += d.pls) {
    {
      const int q0 = r + e * EN;
      float xs[N], ys[N];
#pragma unroll
      for (int j = 0; j < N; ++j) xs[j] = ufun(q0 + j * NX);
      eo_apply_half<PF32, N, HH>(Ds, xs, ys);
#pragma unroll
      for (int j = 0; j < N; ++j)
        if (tiny_owns<N, HH>(j)) Bf[q0 + j * NX] = ys[j];
    }
    {
      const int b0 = x * N + c * NX;
      float xs[N], ys[N];
#pragma unroll
      for (int i = 0; i < N; ++i) xs[i] = ufun(b0 + i);
      eo_apply_half<PF32, N, HH>(Dr, xs, ys);
#pragma unroll
      for (int i = 0; i < N; ++i)
        if (tiny_owns<N, HH>(i)) A[b0 + i] = ys[i];
    }
    tiny_step(r, e, d.pdr, d.pde, NX);
    tiny_step(x, c, d.pdx, d.pdc, d.Ex);
  }
}

template <int N, int HH>
__device__ __forceinline__ void tiny_pair_p2(const TinyDims& d, const float* A, const float* Bf, float* Cb,
                                             float* Db, const float* G11, const float* G12, const float* G22,
                                             const EOCoef<N, float>& Dst) {
  const int NX = d.NX;
  const int EN = N * NX;
  int r = d.pr0, e = d.pe0;
  for (int l = d.pl0; l < d.nl; l += d.pls) {
    const int q0 = r + e * EN;
    float ws[N], os[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const int q = q0 + j * NX;
      const float ur = A[q], us = Bf[q];
      const float g12 = G12[q];
      ws[j] = __fmaf_rn(g12, ur, G22[q] * us);
      if (tiny_owns<N, HH>(j)) Cb[q] = __fmaf_rn(G11[q], ur, g12 * us);
    }
    eo_apply_half<PF32, N, HH>(Dst, ws, os);
#pragma unroll
    for (int j = 0; j < N; ++j)
      if (tiny_owns<N, HH>(j)) Db[q0 + j * NX] = os[j];
    tiny_step(r, e, d.pdr, d.pde, NX);
  }
}

template <int N, int HH, class UF>
__device__ __forceinline__ void tiny_pair_p3(const TinyDims& d, UF&& ufun, float* A, const float* Cb,
                                             const float* Db, const float* Bm, float nu, float kk,
                                             const EOCoef<N, float>& Drt, float& acc) {
  const int NX = d.NX;
  int x = d.px0, c = d.pcc0;
  for (int l = d.pl0; l < d.nl; l += d.pls) {
    const int b0 = x * N + c * NX;
    float xs[N], ys[N];
#pragma unroll
    for (int i = 0; i < N; ++i) xs[i] = Cb[b0 + i];
    eo_apply_half<PF32, N, HH>(Drt, xs, ys);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      if (!tiny_owns<N, HH>(i)) continue;
      const int q = b0 + i;
      float res = nu * (ys[i] + Db[q]);
      const float u = ufun(q);
      if (Bm) res = __fmaf_rn(kk * Bm[q], u, res);
      acc = __fmaf_rn(u, res, acc);
      A[q] = res;
    }
    tiny_step(x, c, d.pdx, d.pdc, d.Ex);
  }
}

// a thread's partial sum and maximum (FP32 magnitude bits) over its points
struct TinyAcc {
  float s;
  unsigned m;
};

// run f(point, acc) over the points this half owns of its pair's row lines;
// returns the accumulated partials (f captures values only, so nothing of
// the caller needs an address)
template <int N, int HH, class F>
__device__ __forceinline__ TinyAcc tiny_points_pair(const TinyDims& d, bool ones, bool has_bc, F f) {
  TinyAcc acc = {0.0f, 0u};
  int r = d.pr0, e = d.pe0;
  for (int l = d.pl0; l < d.nl; l += d.pls) {
    const unsigned char br = d.rinfo[r];
    const int r2 = (int)line_partner(r, br, d.NX);
    const float mr = (!ones && (br & L_COPY2)) ? 0.5f : 1.0f;
    const bool zr = has_bc && (br & L_ZERO);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      if (!tiny_owns<N, HH>(j)) continue;
      const int cl = e * N + j;
      const int c = d.c0 + cl;
      const unsigned char bc = d.cinfo[c];
      TinyPt p;
      p.q = r + cl * d.NX;
      p.g = p.q + d.c0 * d.NX;
      p.r = r;
      p.c = c;
      p.r2 = r2;
      p.c2 = (int)line_partner(c, bc, d.NY);
      p.mult = (!ones && (bc & L_COPY2)) ? 0.5f * mr : mr;
      p.zero = zr || (has_bc && (bc & L_ZERO));
      f(p, acc);
    }
    tiny_step(r, e, d.pdr, d.pde, d.NX);
  }
  return acc;
}

// The FP64 defect-correction step of a sweep: x += x32 (FP64, global), then
// r = b - A x with the double-float operator in the work block (free while no
// inner solve runs), and the cluster maximum of |r|.  A separate function, so
// that the double-float registers do not crowd the FP32 inner loop.  Its
// arguments are values (no address of a caller's register variable is taken);
// it uses reduction slot `slot`, so the caller flips its slot after the call.
template <int N>
__device__ __noinline__ double tiny_residual(const TinyArgs<N>& a, SmallProb* prp, TinyDims d, float* sm,
                                             TinyLayout lay, TinyRed* redp, int slot, bool mass, bool has_bc) {
  SmallProb& pr = *prp;
  TinyRed& red = *redp;
  const int L = d.NX * d.NYs;  // the strip's points
  const int off = d.c0 * d.NX;
  const long long LG = (long long)d.NX * d.NY;
  const float* x32 = sm + lay.x32;
  for (int q = threadIdx.x; q < L; q += d.T) pr.x[off + q] += (double)x32[q];
  __syncthreads();
  // two strip-sized pair buffers in the work block (5 strip sizes of words),
  // at the same offsets in every CTA
  df* DA = reinterpret_cast<df*>(sm + lay.x32);
  df* DB = DA + (lay.r32 - lay.x32);
  float unused = 0.0f;
  const df* Gdf = pr.Gdf + off;
  const double* X = pr.x + off;
  const df nu2 = d2df(pr.nu), k2 = d2df(pr.k);  // both inside the pair window (small_eligible)
  tiny_apply<PDF, N, df>(d, [&](int q) { return PDF::cvt(X[q]); }, DA, DB, Gdf, Gdf + LG, Gdf + 2 * LG,
                         mass ? Gdf + 3 * LG : nullptr, nu2, k2, a.Dr2, a.Drt2, a.Ds2, a.Dst2, unused);
  // the neighbours' copies are read below: a cluster barrier
  tiny_cluster_sync();
  unsigned long long m2 = 0ull;
  tiny_points<N>(d, true, has_bc, [&](const TinyPt& p) {
    // each copy rounded to FP64 first, then summed in FP64 (the order of the
    // chunked path's tile stores and fixup)
    const double ax = tiny_gather(d, DA, p, [](df v) { return df2d(v); });
    const double v = p.zero ? 0.0 : pr.b[p.g] - ax;
    pr.r[p.g] = v;
    const unsigned long long bb = tiny_abs_bits(v);
    m2 = bb > m2 ? bb : m2;
  });
  // the reduction's cluster barrier also ends the neighbours' reads of DA
  // before the work block holds FP32 vectors again
  m2 = tiny_reduce_max64(m2, red, slot);
  return __longlong_as_double((long long)m2);
}

template <int N>
__global__ void __launch_bounds__(kTinyMaxThreads, 1) k_tiny_pcg(const __grid_constant__ TinyArgs<N> a) {
  SmallProb& pr = *a.pr;
  extern __shared__ __align__(16) float sm[];
  int slot = 0;
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks();
  const int rank = (int)cl.block_rank();
  const int NX = (int)pr.NX, NY = (int)pr.NY;
  const int Ey = pr.Ey;
  const int maxiter = pr.maxiter;
  const bool jac = pr.jacobi != 0;
  const bool mass = pr.k != 0.0;
  const bool ones = pr.mult_ones != 0;
  const bool has_bc = pr.has_bc;
  const int e0 = tiny_strip_row(rank, Ey, C), e1 = tiny_strip_row(rank + 1, Ey, C);
  const int Ls_max = NX * N * (int)((Ey + C - 1) / C);
  const TinyLayout lay = tiny_layout(Ls_max, mass, jac, NX + NY);  // the same offsets in every CTA
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
  float* LC = sm + lay.lc;
  float* LD = sm + lay.ld;
  TinyRed& red = *reinterpret_cast<TinyRed*>(sm + lay.red);
  unsigned char* bits = reinterpret_cast<unsigned char*>(sm + lay.bits);
  const int T = blockDim.x;
  TinyDims dm;
  dm.NX = NX;
  dm.NY = NY;
  dm.Ex = pr.Ex;
  dm.Ey = Ey;
  dm.C = C;
  dm.rank = rank;
  dm.c0 = e0 * N;
  dm.NYs = (e1 - e0) * N;
  dm.nl = NX * (e1 - e0);
  dm.T = T;
  dm.r0 = (int)threadIdx.x % NX;
  dm.e0 = (int)threadIdx.x / NX;
  dm.dr = T % NX;
  dm.de = T / NX;
  dm.x0 = (int)threadIdx.x % dm.Ex;
  dm.cc0 = (int)threadIdx.x / dm.Ex;
  dm.dx = T % dm.Ex;
  dm.dc = T / dm.Ex;
  {  // pair walks: T is a multiple of 64
    const int w = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    dm.half = w & 1;
    dm.pl0 = (w >> 1) * 32 + lane;
    dm.pls = T / 2;
    dm.pr0 = dm.pl0 % NX;
    dm.pe0 = dm.pl0 / NX;
    dm.pdr = dm.pls % NX;
    dm.pde = dm.pls / NX;
    dm.px0 = dm.pl0 % dm.Ex;
    dm.pcc0 = dm.pl0 / dm.Ex;
    dm.pdx = dm.pls % dm.Ex;
    dm.pdc = dm.pls / dm.Ex;
  }
  dm.rinfo = bits;
  dm.cinfo = bits + NX;
  const int Ls = NX * dm.NYs;     // this strip's points
  const int off = dm.c0 * NX;     // its first global index
  const long long LG = (long long)NX * NY;

  // persistent block: the strip's FP32 geometry and Jacobi inverse diagonal,
  // and the mesh's line bits
  for (int q = threadIdx.x; q < Ls; q += T) {
    G11[q] = pr.Gf[off + q];
    G12[q] = pr.Gf[LG + off + q];
    G22[q] = pr.Gf[2 * LG + off + q];
    if (mass) Bs[q] = pr.Gf[3 * LG + off + q];
    if (jac) dinv[q] = pr.dinv32[off + q];
  }
  for (int i = threadIdx.x; i < NX + NY; i += T) bits[i] = i < NX ? pr.rinfo[i] : pr.cinfo[i - NX];
  // x = 0, r = b (FP64, global), max|b|
  unsigned long long m0 = 0ull;
  for (int q = threadIdx.x; q < Ls; q += T) {
    const double v = pr.b[off + q];
    pr.x[off + q] = 0.0;
    pr.r[off + q] = v;
    const unsigned long long bb = tiny_abs_bits(v);
    m0 = bb > m0 ? bb : m0;
  }
  m0 = tiny_reduce_max64(m0, red, slot);  // its barriers also publish the staged blocks
  double rmax = __longlong_as_double((long long)m0);
  const double res0 = rmax;
  int outer = 0, total = 0;
  bool nan = rmax != rmax;
  const float nu32 = (float)pr.nu, k32 = (float)pr.k;
  while (!(rmax <= pr.tol) && !nan && outer < pr.max_outer && total < maxiter) {
    ++outer;
    // ---- inner FP32 CG on A d = r to inner_tol * |r|_inf: x32 = 0, r32 = r, p32 = 0
    const float thresh = (float)(pr.inner_tol * rmax);
    float tl = 0.0f;
    unsigned ml = 0u;
    const double* rg = pr.r;
    auto init_point = [=](const TinyPt& p, TinyAcc& ac) {
      const float ri = (float)rg[p.g];
      r32[p.q] = ri;
      x32[p.q] = 0.0f;
      p32[p.q] = 0.0f;
      const float z = jac ? ri * dinv[p.q] : ri;
      ac.s = __fmaf_rn(ri * p.mult, z, ac.s);
      const unsigned bb = tiny_abs_bits(ri);
      ac.m = bb > ac.m ? bb : ac.m;
    };
    const TinyAcc ia = dm.half == 0 ? tiny_points_pair<N, 0>(dm, ones, has_bc, init_point)
                                    : tiny_points_pair<N, 1>(dm, ones, has_bc, init_point);
    tl = ia.s;
    ml = ia.m;
    float t = tiny_reduce(tl, ml, red, slot);
    float rin = __uint_as_float(ml);
    float tprev = 1.0f;
    int k = 0;
    bool nin = rin != rin;
    bool done = !(rin > thresh) || nin || total >= maxiter;
    while (!done) {
      // the new direction p = z + beta p_old is formed where it is read; the
      // update pass stores it
      const float beta = k == 0 ? 0.0f : t / tprev;
      auto pnew = [=](int q) {
        const float rr = r32[q];
        return __fmaf_rn(beta, p32[q], jac ? rr * dinv[q] : rr);
      };
      float papl = 0.0f;
      // the operator in three phases; the branches hold no barrier, so every
      // warp meets the block barriers at the same program point
      if (dm.half == 0)
        tiny_pair_p1<N, 0>(dm, pnew, LA, LB, a.Dr, a.Ds);
      else
        tiny_pair_p1<N, 1>(dm, pnew, LA, LB, a.Dr, a.Ds);
      __syncthreads();
      if (dm.half == 0)
        tiny_pair_p2<N, 0>(dm, LA, LB, LC, LD, G11, G12, G22, a.Dst);
      else
        tiny_pair_p2<N, 1>(dm, LA, LB, LC, LD, G11, G12, G22, a.Dst);
      __syncthreads();
      if (dm.half == 0)
        tiny_pair_p3<N, 0>(dm, pnew, LA, LC, LD, Bs, nu32, k32, a.Drt, papl);
      else
        tiny_pair_p3<N, 1>(dm, pnew, LA, LC, LD, Bs, nu32, k32, a.Drt, papl);
      // the reduction's barriers order P3's stores before the gather reads them
      unsigned none = 0u;
      const float pap = tiny_reduce(papl, none, red, slot);
      const float af = t / pap;
      ++k;
      ++total;
      float sl = 0.0f;
      unsigned mx = 0u;
      const TinyDims dmc = dm;
      auto update_point = [=](const TinyPt& p, TinyAcc& ac) {
        float ap = tiny_gather(dmc, LA, p, [](float v) { return v; });
        if (p.zero) ap = 0.0f;
        const float pk = pnew(p.q);
        x32[p.q] = __fmaf_rn(af, pk, x32[p.q]);
        const float ri = __fmaf_rn(-af, ap, r32[p.q]);
        r32[p.q] = ri;
        p32[p.q] = pk;
        const float z = jac ? ri * dinv[p.q] : ri;
        ac.s = __fmaf_rn(ri * p.mult, z, ac.s);
        const unsigned bb = tiny_abs_bits(ri);
        ac.m = bb > ac.m ? bb : ac.m;
      };
      const TinyAcc ua = dm.half == 0 ? tiny_points_pair<N, 0>(dm, ones, has_bc, update_point)
                                      : tiny_points_pair<N, 1>(dm, ones, has_bc, update_point);
      sl = ua.s;
      mx = ua.m;
      tprev = t;
      t = tiny_reduce(sl, mx, red, slot);
      rin = __uint_as_float(mx);
      nin = (rin != rin) || (af != af);
      done = !(rin > thresh) || nin || total >= maxiter;
    }
    rmax = tiny_residual<N>(a, &pr, dm, sm, lay, &red, slot, mass, has_bc);
    slot ^= 1;
    nan = rmax != rmax || nin;
  }
  if (rank == 0 && threadIdx.x == 0) {
    pr.iters = total;
    pr.outer = outer;
    pr.res_inf = rmax;
    pr.res0_inf = res0;
    pr.nan = nan;
    pr.converged = rmax <= pr.tol && !nan;
  }
  // no CTA leaves while another may still read its shared memory
  tiny_cluster_sync();
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

// CTAs of the cluster for an Ey-element-row mesh: SEM_TINY_CLUSTER (1, 2, 4
// or 8) when set, else 8 (at most one strip per element row).  cfg3 (8x8
// elements, N=8) takes 4.04, 3.38 and 3.11 ms with 2, 4 and 8 CTAs.
int tiny_cluster_size(int Ey) {
  int c = 8;
  if (const char* e = std::getenv("SEM_TINY_CLUSTER")) {
    const int v = std::atoi(e);
    if (v == 1 || v == 2 || v == 4 || v == 8) c = v;
  }
  while (c > 1 && c > Ey) c >>= 1;
  return c;
}

size_t tiny_smem_bytes(int n, int Ex, int Ey, bool mass, bool jac) {
  const int C = tiny_cluster_size(Ey);
  const long long NX = (long long)n * Ex, NY = (long long)n * Ey;
  const long long Ls_max = NX * n * ((Ey + C - 1) / C);
  return (size_t)tiny_layout(Ls_max, mass, jac, NX + NY).words * 4;
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
  const int C = tiny_cluster_size(host.Ey);
  const long long nl = host.NX * ((host.Ey + C - 1) / C);  // lines of the largest strip
  int threads = (int)((nl + 31) / 32 * 64);                 // two threads per line (pair walks)
  if (threads > kTinyMaxThreads) threads = kTinyMaxThreads;   // a multiple of 64
  if (threads < 64) threads = 64;
  auto kern = k_tiny_pcg<N>;
  SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)C);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  SEM_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
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
