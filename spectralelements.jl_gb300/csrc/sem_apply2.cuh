// Second-generation fused element operator (kernel variants 2 and 3).
//
// Differences from k_apply:
//  * one in-place shared-memory work buffer: in every phase a thread reads and
//    writes only its own line (row or column) of its element, so the x- and
//    y-direction contractions can overwrite their input; a second buffer keeps
//    u for the mass term (no registers held across the phases for it);
//  * geometry read through GeoT: for the double-float policy the mesh handle
//    stores G11/G12/G22/B pre-split into (h, l) float pairs (same 8 bytes per
//    value), so no per-load double -> pair conversion is executed;
//  * variant 3 stages G11/G12/G22 with cp.async at kernel start.
// Reference: laplace (src/lapl.jl:70-81), hlmz (src/hlmz.jl:12-19),
// gatherScatter (src/gatherScatter.jl:8-16), mask (src/mask.jl:10-18).
#pragma once

#include "sem_apply_kernels.cuh"

namespace sem {

// storage type of the geometry fields read by k_apply2 and its conversion to
// the arithmetic type
template <class P>
struct GeoT {
  typedef typename P::io type;
  static __device__ __forceinline__ typename P::v ld(const type* p) { return P::ld(p); }
  static __device__ __forceinline__ typename P::v cvt(type x) { return P::cvt(x); }
};
template <>
struct GeoT<PDF> {
  typedef df type;  // split on the device by d2df when the mesh is set up
  static __device__ __forceinline__ df ld(const df* p) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return {v.x, v.y};
  }
  static __device__ __forceinline__ df cvt(df x) { return x; }
};

template <class P, int N>
struct Apply2Args {
  typedef typename P::io io;
  typedef typename P::v v;
  typedef typename GeoT<P>::type gt;
  const io* u;
  io* out;
  const gt* G11;
  const gt* G12;
  const gt* G22;
  const gt* B;
  const io* nu;
  v nu_s;
  v k_s;
  // range guard (double-float policy): *rflag = rtag when an input row or a
  // result leaves the pair format's range; a gated launch (gate non-NULL)
  // does nothing unless *gate == gate_tag
  unsigned* rflag;
  unsigned rtag;
  const unsigned* gate;
  unsigned gate_tag;
  int Ex, Ey;
  long long NX;
  unsigned mode;
  const int* skip;
  unsigned* ctr;          // interface arrival counters (in-kernel completion), or NULL
  int tiles_x, tiles_y;   // element tiles of the launch (in-kernel completion)
  int ty0;                // first element-tile row of the launch (a window of the grid)
  // CG-fused launch: u = p = dinv .* r + beta p_old is formed here (p read and
  // written in place) and every CTA stores its share of p . A p in dpart
  const io* r;
  const io* dinv;
  io* p;
  const double* beta;
  df* dpart;
  EOCoef<N, v> Dr, Drt, Ds, Dst;
};


// In-kernel completion of the cross-tile QQ' (kernel variant 5).  Every tile
// edge and every tile corner on a cross-tile interface has an arrival counter
// (three per tile: the edge to its right, the edge above it, their corner).
// A CTA that has stored its tile counts itself in at the counters of the up to
// four edges and four corners it touches; the CTA that arrives last at an edge
// (second of two) or corner (fourth of four) sums its copies, with the
// operations and order of k_dss_fixup, so the result is bit-identical to a
// separate fixup launch.  Counters are never reset: an edge completes when its
// count is odd after the increment, a corner when it is 3 mod 4, so every
// launch that runs to its end leaves them consistent for the next.  Stores are
// made device-visible (__threadfence) before the arrival, and the last arriver
// reads the other tiles' copies from L2.  Needs two distinct tiles across every
// periodic direction (tiles_x >= 2 if x is periodic, likewise y).
template <class IO, int TX, int TY>
__device__ __forceinline__ void finish_tile_interfaces(IO* out, int n, int Ex, int Ey, long long NX,
                                                       unsigned mode, unsigned* ctr, int tiles_x,
                                                       int tiles_y, int bx, int by) {
  __shared__ int s_last[8];
  __shared__ long long s_a[8], s_b[8];
  const bool perx = (mode & M_PERX) != 0, pery = (mode & M_PERY) != 0;
  __threadfence();
  __syncthreads();
  if (threadIdx.x < 8) {
    const int k = threadIdx.x;
    const int lx = (bx + tiles_x - 1) % tiles_x, ly = (by + tiles_y - 1) % tiles_y;
    const bool left = bx > 0 || perx, right = bx + 1 < tiles_x || perx;
    const bool below = by > 0 || pery, above = by + 1 < tiles_y || pery;
    // segment k: 0 left edge, 1 right edge, 2 lower edge, 3 upper edge,
    // 4..7 corners lower-left, lower-right, upper-left, upper-right
    int tx = bx, ty = by, kind = 0;
    bool exists = false;
    switch (k) {
      case 0: tx = lx; kind = 0; exists = left; break;
      case 1: kind = 0; exists = right; break;
      case 2: ty = ly; kind = 1; exists = below; break;
      case 3: kind = 1; exists = above; break;
      case 4: tx = lx; ty = ly; kind = 2; exists = left && below; break;
      case 5: ty = ly; kind = 2; exists = right && below; break;
      case 6: tx = lx; kind = 2; exists = left && above; break;
      default: kind = 2; exists = right && above; break;
    }
    int last = 0;
    if (exists) {
      const unsigned old = atomicAdd(ctr + 3 * ((long long)ty * tiles_x + tx) + kind, 1u);
      last = kind == 2 ? ((old & 3u) == 3u) : ((old & 1u) == 1u);
      if (last) __threadfence();
    }
    // interface element indices right of / above the owner tile (0: the wrap)
    const long long a = (long long)(tx + 1) * TX >= Ex ? 0 : (long long)(tx + 1) * TX;
    const long long b = (long long)(ty + 1) * TY >= Ey ? 0 : (long long)(ty + 1) * TY;
    s_last[k] = last ? kind + 1 : 0;
    s_a[k] = kind == 1 ? (long long)tx : a;  // y edge: owner tile column
    s_b[k] = kind == 0 ? (long long)ty : b;  // x edge: owner tile row
  }
  __syncthreads();
  FixArgs f;
  f.n = n;
  f.Ex = Ex;
  f.Ey = Ey;
  f.TX = TX;
  f.TY = TY;
  f.NX = NX;
  f.NY = (long long)Ey * n;
  f.mode = mode;
  f.skip = nullptr;
  f.key_lo = 0;
  f.key_hi = 1LL << 62;
  f.nxi = f.nyi = 0;
  f.gate = nullptr;
  f.gate_tag = 0;
  auto none = [](long long, long long, IO) {};
  for (int k = 0; k < 8; ++k) {
    const int kind = s_last[k] - 1;
    if (kind == 0) {
      const long long ty = s_b[k];
      const long long c1 = ((ty + 1) * TY < Ey ? (ty + 1) * TY : (long long)Ey) * n;
      fix_xline(out, f, s_a[k], ty * TY * n + threadIdx.x, c1, (long long)blockDim.x, none);
    } else if (kind == 1) {
      const long long tx = s_a[k];
      const long long r1 = ((tx + 1) * TX < Ex ? (tx + 1) * TX : (long long)Ex) * n;
      fix_yline(out, f, s_b[k], tx * TX * n + threadIdx.x, r1, (long long)blockDim.x, none);
    } else if (kind == 2 && threadIdx.x == (k - 4) * (blockDim.x / 4)) {
      fix_corner(out, f, s_a[k], s_b[k], none);
    }
  }
}

// y = D x with x in registers and y stored to shared memory at the given
// stride: the operations and order of eo_apply, with the output pairs formed
// one at a time in a loop that is not unrolled (coefficients indexed at run
// time from the parameter block).  From 13 points on, the four inlined
// double-float line products of a kernel no longer fit the instruction cache;
// in this form each shrinks by a factor of n/2.  y may overwrite the line x
// was read from (x is held in registers).
template <class P, int N>
__device__ __forceinline__ void eo_apply_to(const EOCoef<N, typename P::v>& D, const typename P::v (&x)[N],
                                            typename P::v* y, int stride) {
  typedef typename P::v V;
  constexpr int M = N / 2;
  V e[M], o[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    e[k] = P::add_u(x[k], x[N - 1 - k]);
    o[k] = P::sub_u(x[k], x[N - 1 - k]);
  }
  const V xm = (N & 1) ? x[M] : P::zero();
#pragma unroll 1
  for (int i = 0; i < M; ++i) {
    V s = P::mul(D.A[i][0], o[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) s = P::fma(D.A[i][k], o[k], s);
    V t = P::mul(D.Cc[i][0], e[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) t = P::fma(D.Cc[i][k], e[k], t);
    if (N & 1) t = P::fma(D.cm[i], xm, t);
    y[i * stride] = P::add_u(s, t);
    y[(N - 1 - i) * stride] = P::sub_u(s, t);
  }
  if (N & 1) {
    V s = P::mul(D.mr[0], o[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) s = P::fma(D.mr[k], o[k], s);
    y[M * stride] = s;
  }
}

// the same on a column line held in shared memory (stride 1), in place
template <class P, int N>
__device__ __forceinline__ void eo_apply_col(const EOCoef<N, typename P::v>& D, typename P::v* line) {
  typename P::v x[N];
#pragma unroll
  for (int i = 0; i < N; ++i) x[i] = line[i];
  eo_apply_to<P, N>(D, x, line, 1);
}

// resident blocks per SM asked of the register allocator: without the
// register copy of u the double-float kernel fits five blocks up to n = 9
// (56 registers at n = 9, with a few words spilled to L1; 3 % faster than
// four blocks at 72 registers without spills on the 256^2 n = 9 apply); at
// n = 8 the 256-thread tile would spill more, so it keeps four
template <class P, int N, bool STAGE>
struct MinBlocks2 {
  static constexpr int value =
      (!STAGE && P::kPrecision == SEM_F64_DF && N <= 9)
          ? (N == 8 ? 4 : 5)
          // from 15 points the line products of all four phases loop over
          // their output pairs and the row phases' outputs live in shared
          // memory, which frees the registers for a third resident CTA
          // (shared memory allows three)
          : ((!STAGE && P::kPrecision == SEM_F64_DF && N >= 15) ? 3 : MinBlocks<P, N, STAGE>::value);
};

// CG: the launch is one CG iteration's operator application (src/pcg.jl:40-47):
// it forms the direction p from r and the previous p, applies the operator to
// it and writes each CTA's part of p . A p.  The denominator is summed over the
// unassembled local products p_i (A_e p)_i, which equals the reference's
// sum(p .* Ap .* mult) for a continuous, masked p (QQ' is the transpose of the
// scatter and mask zeroes p where it zeroes Ap), so the cross-tile completion
// does not enter it and the sum is deterministic.
template <class P, int N, int TX, int TY, bool STAGE, bool FUSE = false, bool CG = false>
__global__ void __launch_bounds__(TX* TY* N, (MinBlocks2<P, N, STAGE>::value))
    k_apply2(const __grid_constant__ Apply2Args<P, N> a) {
  typedef typename P::v V;
  typedef typename P::io IO;
  typedef typename GeoT<P>::type GT;
  constexpr int SP = N | 1;
  constexpr int ES = N * SP;
  constexpr int TE = TX * TY * ES;
  // line products in loop form (see eo_apply_to): the column phases from 13
  // points, the row phases as well from 15 (at 13 points the looped row
  // phases measured 6 % slower: 0.157 against 0.148 ms on 167^2 elements; at
  // 17 points 3 % faster with a third resident CTA)
  constexpr bool kColLoop = N >= 13 && P::kPrecision == SEM_F64_DF;
  constexpr bool kRowLoop = N >= 15 && P::kPrecision == SEM_F64_DF;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S0 = reinterpret_cast<V*>(smem_raw);  // u (mass term), later the y exchange
  V* S1 = S0 + TE;                         // in-place work buffer
  GT* R = reinterpret_cast<GT*>(S1 + TE);  // staged G11, G12, G22 (variant 3)

  pdl_trigger();  // the next kernel (the cross-tile fixup) may be scheduled now
  pdl_wait();     // a no-op unless this launch is a programmatic dependent
  if (a.skip && *a.skip) return;
  if (a.gate && *a.gate != a.gate_tag) return;  // gated re-run not needed
  const int t = threadIdx.x;
  const int elem = t / N;
  const int lane = t - elem * N;
  const int exl = elem % TX;
  const int eyl = elem / TX;
  const int ex = blockIdx.x * TX + exl;
  const int ey = (blockIdx.y + a.ty0) * TY + eyl;
  const bool valid = ex < a.Ex && ey < a.Ey;
  const long long NX = a.NX;
  const long long base = (long long)ex * N + lane + (long long)ey * N * NX;
  const unsigned mode = a.mode;
  const bool stiff = (mode & M_STIFF) != 0;
  V* s0 = S0 + elem * ES;
  V* s1 = S1 + elem * ES;
  const int rofs = elem * ES + lane;
  bool kbad = false;  // range guard: a tiny stiffness row or a tiny k B product

  if (STAGE) {
    if (valid && stiff) {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const long long gi = base + (long long)j * NX;
        cp_async(R + 0 * TE + rofs + j * SP, a.G11 + gi);
        cp_async(R + 1 * TE + rofs + j * SP, a.G12 + gi);
        cp_async(R + 2 * TE + rofs + j * SP, a.G22 + gi);
      }
    }
    cp_async_commit();
  }
  auto ldg = [&](const GT* src, int slot, int j) -> V {
    if (!valid) return P::zero();
    if (STAGE) return GeoT<P>::cvt(R[slot * TE + rofs + j * SP]);
    return GeoT<P>::ld(src + base + (long long)j * NX);
  };

  // ---- A: row `lane` of u; y-direction derivative
  V res[N];
  {
    V u[N];
    if constexpr (CG) {
      const IO beta = (IO)*a.beta;
      const bool jac = a.dinv != nullptr;
#pragma unroll
      for (int j = 0; j < N; ++j) {
        IO pn = (IO)0;
        if (valid) {
          const long long gi = base + (long long)j * NX;
          if constexpr (P::kPrecision == SEM_F64)  // native FP64 direction (the whole double range)
            pn = __fma_rn(beta, a.p[gi], jac ? __dmul_rn(a.r[gi], a.dinv[gi]) : a.r[gi]);
          else
            pn = cg_direction(a.r[gi], jac ? a.dinv[gi] : (IO)1, beta, a.p[gi], jac);
          a.p[gi] = pn;
        }
        u[j] = P::cvt(pn);
        s0[j * SP + lane] = u[j];
      }
    } else {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        u[j] = valid ? P::ld(a.u + base + (long long)j * NX) : P::zero();
        s0[j * SP + lane] = u[j];
      }
    }
    if (stiff) {
      // with kRowLoop the y-derivative us and later the transposed
      // y-product os live in this thread's row of s0 (u is reloaded for the
      // mass term); otherwise in registers
      V us[kRowLoop ? 1 : N];
#pragma unroll
      for (int j = 0; j < N; ++j) s1[j * SP + lane] = u[j];
      if constexpr (kRowLoop)
        eo_apply_to<P, N>(a.Ds, u, s0 + lane, SP);
      else
        eo_apply<P, N>(a.Ds, u, us);
      __syncthreads();
      // ---- B: column `lane` in place; x-direction derivative
      if constexpr (kColLoop) {
        eo_apply_col<P, N>(a.Dr, s1 + lane * SP);
      } else {
        V col[N], ur[N];
#pragma unroll
        for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
        eo_apply<P, N>(a.Dr, col, ur);
#pragma unroll
        for (int i = 0; i < N; ++i) s1[lane * SP + i] = ur[i];
      }
      __syncthreads();
      // ---- C: row `lane` in place; metric terms, transposed y-derivative
      if (STAGE) cp_async_wait_all();
      V os[kRowLoop ? 1 : N];
      {
        V ws[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const V g11 = ldg(a.G11, 0, j);
          const V g12 = ldg(a.G12, 1, j);
          const V g22 = ldg(a.G22, 2, j);
          const V ur = s1[j * SP + lane];
          const V usj = kRowLoop ? s0[j * SP + lane] : us[kRowLoop ? 0 : j];
          V wr = P::fma(g11, ur, P::mul(g12, usj));
          ws[j] = P::fma(g12, ur, P::mul(g22, usj));
          if (mode & M_NUG) {
            const V nu = valid ? P::ld(a.nu + base + (long long)j * NX) : P::zero();
            wr = P::mul(nu, wr);
            ws[j] = P::mul(nu, ws[j]);
          }
          s1[j * SP + lane] = wr;
        }
        if constexpr (kRowLoop)
          eo_apply_to<P, N>(a.Dst, ws, s0 + lane, SP);  // os over us, same thread's row
        else
          eo_apply<P, N>(a.Dst, ws, os);
      }
      __syncthreads();
      // ---- D: column `lane` in place; transposed x-derivative
      if constexpr (kColLoop) {
        eo_apply_col<P, N>(a.Drt, s1 + lane * SP);
      } else {
        V col[N], o[N];
#pragma unroll
        for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
        eo_apply<P, N>(a.Drt, col, o);
#pragma unroll
        for (int i = 0; i < N; ++i) s1[lane * SP + i] = o[i];
      }
      __syncthreads();
      // ---- E: assemble
#pragma unroll
      for (int j = 0; j < N; ++j) res[j] = P::add(s1[j * SP + lane], kRowLoop ? s0[j * SP + lane] : os[kRowLoop ? 0 : j]);
      if constexpr (P::kPrecision == SEM_F64_DF) kbad |= df_row_tiny(res);  // the stiffness sum, before nu
      if (mode & M_NU) {
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const V nu = valid ? P::ld(a.nu + base + (long long)j * NX) : P::zero();
          res[j] = P::fin(P::mul(nu, res[j]));
        }
      } else {
#pragma unroll
        for (int j = 0; j < N; ++j) res[j] = P::fin((mode & M_NUFOLD) ? res[j] : P::mul(a.nu_s, res[j]));
      }
    } else {
#pragma unroll
      for (int j = 0; j < N; ++j) res[j] = P::zero();
    }
  }
  // this thread's row of u: s0, or (kRowLoop with the stiffness part, which
  // reused s0) the input reloaded and converted exactly as phase A did
  auto u_at = [&](int j) -> V {
    if (!(kRowLoop && stiff)) return s0[j * SP + lane];
    if (!valid) return P::zero();
    const long long gi = base + (long long)j * NX;
    if constexpr (CG) return P::cvt(a.p[gi]);
    else return P::ld(a.u + gi);
  };
  if (mode & M_MASS) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const V b = valid ? GeoT<P>::ld(a.B + base + (long long)j * NX) : P::zero();
      const V kb = (mode & M_KB) ? b : P::mul(a.k_s, b);
      if constexpr (P::kPrecision == SEM_F64_DF) kbad |= df_tiny_nz(kb, kKbTiny);
      res[j] = P::fin(P::fma(kb, u_at(j), res[j]));
    }
  }

  if constexpr (P::kPrecision == SEM_F64_DF) {
    // range guard: a tiny stiffness or result row, a tiny k B or a NaN/Inf
    // result flags the call (degenerate metric terms arrive as NaN pairs)
    bool bad = kbad || df_row_tiny(res);
#pragma unroll
    for (int j = 0; j < N; ++j) bad |= df_bad(res[j]);
    if (bad && a.rflag) *a.rflag = a.rtag;
  }
  if constexpr (CG)
    store_dot_part<P, N>([&](int j) { return u_at(j); }, [&](int j) { return res[j]; }, a.dpart,
                         blockIdx.y * gridDim.x + blockIdx.x);
  static_assert(sizeof(V) == sizeof(IO), "line buffers are reused for stored values");
  tile_dss_store<P, N, TX, TY>(res, reinterpret_cast<IO*>(S1), reinterpret_cast<IO*>(S0), elem, lane,
                               ex, ey, valid, base, a.Ex, a.Ey, NX, mode, a.out);
  if constexpr (FUSE) {
    if (mode & M_GS)
      finish_tile_interfaces<IO, TX, TY>(a.out, N, a.Ex, a.Ey, NX, mode, a.ctr, a.tiles_x, a.tiles_y,
                                         blockIdx.x, blockIdx.y);
  }
}

}  // namespace sem
