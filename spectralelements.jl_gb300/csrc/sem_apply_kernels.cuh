// Fused element operator kernel: mask(QQ'(nu .* D'GD u + k B u)) on the
// reference's column-major local layout.
//
// Work decomposition.  One CTA owns a tile of TX x TY elements and N threads
// per element.  A thread alternately owns one local row i (x-direction line
// inside its element) and one local column j; the lines are exchanged through
// shared memory.  The 1D operators are applied in even-odd form (GLL
// derivative matrices are centro-antisymmetric), which cuts the multiply-adds
// of an N-point line from N^2 to about N^2/2; the coefficients live in the
// kernel parameter block (constant bank), so every multiply-add takes its
// coefficient as a constant operand and no shared-memory read is spent on it.
//
//   A  row i   : load u(i,:) (coalesced across the tile), us = Ds u(i,:)
//   B  column j: ur = Dr u(:,j)
//   C  row i   : wr = G11 ur + G12 us, ws = G12 ur + G22 us, os = Ds' ws
//   D  column j: or = Dr' wr(:,j)
//   E  row i   : res = nu (or + os) + k B u, then QQ' inside the tile
//                (x pairs, then y pairs) and the mask; points whose copies
//                live in another tile are written unsummed and finished by
//                k_dss_fixup.
//
// Reference: laplace (src/lapl.jl:70-81), hlmz (src/hlmz.jl:12-19),
// gatherScatter (src/gatherScatter.jl:8-16 with src/semq.jl:6-25),
// mask (src/mask.jl:10-18).
#pragma once

#include "sem_arith.cuh"

namespace sem {

template <class P, int N>
struct ApplyArgs {
  typedef typename P::io io;
  typedef typename P::v v;
  const io* u;
  io* out;
  const io* G11;
  const io* G12;
  const io* G22;
  const io* B;
  const io* nu;
  v nu_s;
  v k_s;
  int Ex, Ey;
  long long NX;
  unsigned mode;
  const int* skip;
  int slot_g, slot_b, slot_nu;  // staged-variant shared-memory slots (-1: not staged)
  int ty0;                      // first element-tile row of the launch (a window of the grid)
  df* dpart;                    // DOT launches: each CTA's part of u . (A u), unassembled
  // range guard (double-float policy): *rflag = rtag when an input row or a
  // result leaves the pair format's range; a gated launch (gate non-NULL)
  // does nothing unless *gate == gate_tag
  unsigned* rflag;
  unsigned rtag;
  const unsigned* gate;
  unsigned gate_tag;
  EOCoef<N, v> Dr, Drt, Ds, Dst;
};

template <int N>
struct TileShape {
  static constexpr int TX = 8;
  static constexpr int TY = N <= 4 ? 8 : (N <= 8 ? 4 : (N <= 12 ? 3 : 2));
  static constexpr int SP = N | 1;  // odd line stride: conflict-free 8-byte accesses
  static constexpr int ES = N * SP;
  static constexpr int THREADS = TX * TY * N;
};

// resident blocks per SM requested from the register allocator: the
// double-float kernels are latency bound, so they trade a few spilled
// registers for more resident warps.  Up to n = 9: a third block.  At n = 13
// three blocks of 208 threads (80 registers, about 50 bytes spilled per
// thread) run the 167^2 apply in 0.159 ms against 0.214 ms with two blocks and
// 0.288 ms with one (255 registers); at n = 17 two blocks (96 registers) take
// 0.241 ms against 0.319 ms with one.  Four blocks at n = 13 and three at
// n = 17 would spill 200 and 900 bytes with the line products inlined; the
// second-generation kernel (MinBlocks2) loops over them from 13 points and
// runs three blocks from 15.
template <class P, int N, bool STAGE>
struct MinBlocks {
  static constexpr int value =
      STAGE ? (N <= 9 ? 2 : 1)
            : ((P::kPrecision == SEM_F64_DF) ? (N <= 9 ? 3 : (N <= 12 ? 2 : (N == 13 ? 3 : 2)))
                                              : (N <= 10 ? 3 : (N <= 12 ? 2 : 1)));
};

// asynchronous global -> shared copies (LDGSTS); each thread later reads only
// the entries it copied itself, so cp.async.wait_all is the only fence needed
template <class IO>
__device__ __forceinline__ void cp_async(IO* dst_smem, const IO* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  if (sizeof(IO) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// y = D x for a centro-antisymmetric D given in even-odd form
template <class P, int N>
__device__ __forceinline__ void eo_apply(const EOCoef<N, typename P::v>& D,
                                         const typename P::v (&x)[N], typename P::v (&y)[N]) {
  typedef typename P::v V;
  constexpr int M = N / 2;
  V e[M], o[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    e[k] = P::add_u(x[k], x[N - 1 - k]);
    o[k] = P::sub_u(x[k], x[N - 1 - k]);
  }
#pragma unroll
  for (int i = 0; i < M; ++i) {
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
  if (N & 1) {
    V s = P::mul(D.mr[0], o[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) s = P::fma(D.mr[k], o[k], s);
    y[M] = s;
  }
}

__host__ __device__ inline bool xcross_row(int ex, int i, int n, int Ex, int TX, bool perx) {
  const int exl = ex % TX;
  if (i == 0 && exl == 0 && (ex > 0 || perx)) return true;
  if (i == n - 1 && (exl == TX - 1 || ex == Ex - 1) && (ex < Ex - 1 || perx)) return true;
  return false;
}

// QQ' inside the tile, the mask, and the store of one thread's row.  Each
// local value is first rounded to the storage type; the copies of a node are
// then summed in storage arithmetic, x pairs before y pairs, so every node
// gets exactly the sums of k_gather_scatter on the rounded values, whatever
// the tile shape.  A row on a cross-tile x interface takes no in-tile y pair:
// k_dss_fixup finishes its corners in the same x-first order.  Points with
// copies in another tile are stored unsummed and unmasked; finished(j, value)
// is called for every other point of the row.  X1 and X0 are two tile-sized
// shared buffers free for reuse; every thread of the block calls this (it
// holds barriers).
struct NoFinish {
  template <class IO>
  __device__ __forceinline__ void operator()(int, IO) const {}
};

template <class P, int N, int TX, int TY, class F = NoFinish>
__device__ __forceinline__ void tile_dss_store(const typename P::v (&res)[N], typename P::io* X1,
                                               typename P::io* X0, int elem, int lane, int ex,
                                               int ey, bool valid, long long base, int Ex, int Ey,
                                               long long NX, unsigned mode, typename P::io* out,
                                               F&& finished = F()) {
  typedef typename P::io IO;
  constexpr int SP = N | 1;
  constexpr int ES = N * SP;
  const int exl = elem % TX;
  const int eyl = elem / TX;
  const bool gs = (mode & M_GS) != 0;
  const bool perx = (mode & M_PERX) != 0;
  const bool pery = (mode & M_PERY) != 0;
  IO rv[N];
#pragma unroll
  for (int j = 0; j < N; ++j) rv[j] = P::st(res[j]);
  const bool xrow = gs && xcross_row(ex, lane, N, Ex, TX, perx);
  if (gs) {
    // x pairs inside the tile: row n-1 of element exl with row 0 of exl+1
    IO* x1 = X1 + elem * ES;
#pragma unroll
    for (int j = 0; j < N; ++j) x1[j * SP + lane] = rv[j];
    __syncthreads();
    if (lane == N - 1 && exl + 1 < TX && ex + 1 < Ex) {
      const IO* nb = X1 + (elem + 1) * ES;
#pragma unroll
      for (int j = 0; j < N; ++j) rv[j] = io_add(rv[j], nb[j * SP]);
    }
    if (lane == 0 && exl > 0) {
      const IO* nb = X1 + (elem - 1) * ES;
#pragma unroll
      for (int j = 0; j < N; ++j) rv[j] = io_add(nb[j * SP + N - 1], rv[j]);
    }
    // y pairs inside the tile: column n-1 of element eyl with column 0 of eyl+1
    IO* x0 = X0 + elem * ES;
    x0[lane] = rv[0];
    x0[(N - 1) * SP + lane] = rv[N - 1];
    __syncthreads();
    if (!xrow && eyl + 1 < TY && ey + 1 < Ey) rv[N - 1] = io_add(rv[N - 1], X0[(elem + TX) * ES + lane]);
    if (!xrow && eyl > 0) rv[0] = io_add(X0[(elem - TX) * ES + (N - 1) * SP + lane], rv[0]);
  }
  if (!valid) return;
  const long long row = (long long)ex * N + lane;
  const long long NY = (long long)Ey * N;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    bool raw = xrow;
    if (gs) {
      if (j == 0 && eyl == 0 && (ey > 0 || pery)) raw = true;
      if (j == N - 1 && (eyl == TY - 1 || ey == Ey - 1) && (ey < Ey - 1 || pery)) raw = true;
    }
    IO val = rv[j];
    if (!raw) {
      const long long col = (long long)ey * N + j;
      if ((mode & M_MASK) && !mask_keep(row, col, NX, NY, mode)) val = masked_zero(val);
      finished(j, val);
    }
    out[base + (long long)j * NX] = val;
  }
}

// DOT: the launch is a CG iteration's operator application on the direction
// u = p and every CTA also writes its part of p . A p, summed over the
// unassembled local products (equal to the mult-weighted dot of the assembled
// A p for a continuous, masked p; the same sum as the CG-fused k_apply2)
template <class P, int N, int TX, int TY, bool STAGE, bool DOT = false>
__global__ void __launch_bounds__(TX* TY* N, (MinBlocks<P, N, STAGE>::value))
    k_apply(const __grid_constant__ ApplyArgs<P, N> a) {
  typedef typename P::v V;
  typedef typename P::io IO;
  constexpr int SP = N | 1;
  constexpr int ES = N * SP;
  constexpr int TE = TX * TY * ES;  // entries of one tile-sized buffer
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S1 = reinterpret_cast<V*>(smem_raw);
  V* S2 = S1 + TE;
  IO* R = reinterpret_cast<IO*>(S2 + TE);  // staged raw inputs (STAGE): slot * TE + ...

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
  V* s1 = S1 + elem * ES;
  V* s2 = S2 + elem * ES;
  const int rofs = elem * ES + lane;  // this thread's row inside a staged slot (+ j*SP)
  bool gbad = false;  // range guard: degenerate metric terms, a tiny row or a tiny k B

  // ---- staged variant: issue every later global read of this row now
  if (STAGE) {
    if (valid) {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const long long gi = base + (long long)j * NX;
        if (a.slot_g >= 0) {
          cp_async(R + (a.slot_g + 0) * TE + rofs + j * SP, a.G11 + gi);
          cp_async(R + (a.slot_g + 1) * TE + rofs + j * SP, a.G12 + gi);
          cp_async(R + (a.slot_g + 2) * TE + rofs + j * SP, a.G22 + gi);
        }
        if (a.slot_b >= 0) cp_async(R + a.slot_b * TE + rofs + j * SP, a.B + gi);
        if (a.slot_nu >= 0) cp_async(R + a.slot_nu * TE + rofs + j * SP, a.nu + gi);
      }
    }
    cp_async_commit();
  }
  auto ldx = [&](const IO* gsrc, int slot, int j) -> V {
    if (!valid) return P::zero();
    if (STAGE && slot >= 0) return P::cvt(R[slot * TE + rofs + j * SP]);
    return P::ld(gsrc + base + (long long)j * NX);
  };

  // ---- A: row `lane` of u; y-direction derivative
  V u[N];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    u[j] = valid ? P::ld(a.u + base + (long long)j * NX) : P::zero();
  }

  V res[N];
  if (stiff) {
    V us[N];
#pragma unroll
    for (int j = 0; j < N; ++j) s1[j * SP + lane] = u[j];
    eo_apply<P, N>(a.Ds, u, us);
    __syncthreads();
    // ---- B: column `lane`; x-direction derivative
    {
      V col[N], ur[N];
#pragma unroll
      for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
      eo_apply<P, N>(a.Dr, col, ur);
#pragma unroll
      for (int i = 0; i < N; ++i) s2[lane * SP + i] = ur[i];
    }
    __syncthreads();
    // ---- C: row `lane`; metric terms, transposed y-derivative
    if (STAGE) cp_async_wait_all();
    V os[N];
    {
      V ws[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        V g11 = ldx(a.G11, a.slot_g, j);
        V g12 = ldx(a.G12, a.slot_g < 0 ? -1 : a.slot_g + 1, j);
        V g22 = ldx(a.G22, a.slot_g < 0 ? -1 : a.slot_g + 2, j);
        if constexpr (P::kPrecision == SEM_F64_DF) gbad |= geo_tiny(g11, g22);
        V ur = s2[j * SP + lane];
        V wr = P::fma(g11, ur, P::mul(g12, us[j]));
        ws[j] = P::fma(g12, ur, P::mul(g22, us[j]));
        if (mode & M_NUG) {
          V nu = ldx(a.nu, a.slot_nu, j);
          wr = P::mul(nu, wr);
          ws[j] = P::mul(nu, ws[j]);
        }
        s1[j * SP + lane] = wr;
      }
      eo_apply<P, N>(a.Dst, ws, os);
    }
    __syncthreads();
    // ---- D: column `lane`; transposed x-derivative
    {
      V col[N], o[N];
#pragma unroll
      for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
      eo_apply<P, N>(a.Drt, col, o);
#pragma unroll
      for (int i = 0; i < N; ++i) s2[lane * SP + i] = o[i];
    }
    __syncthreads();
    // ---- E: assemble
#pragma unroll
    for (int j = 0; j < N; ++j) res[j] = P::add(s2[j * SP + lane], os[j]);
    if constexpr (P::kPrecision == SEM_F64_DF) gbad |= df_row_tiny(res);  // the stiffness sum, before nu
    if (mode & M_NU) {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        V nu = ldx(a.nu, a.slot_nu, j);
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
  if (mode & M_MASS) {
    if (STAGE && !stiff) cp_async_wait_all();
#pragma unroll
    for (int j = 0; j < N; ++j) {
      V b = ldx(a.B, a.slot_b, j);
      V kb = (mode & M_KB) ? b : P::mul(a.k_s, b);
      if constexpr (P::kPrecision == SEM_F64_DF) gbad |= df_tiny_nz(kb, kKbTiny);
      res[j] = P::fin(P::fma(kb, u[j], res[j]));
    }
  }
  if constexpr (P::kPrecision == SEM_F64_DF) {
    // range guard: a tiny stiffness or result row, degenerate metric terms, a
    // tiny k B or a NaN/Inf result flags the call
    bool bad = gbad || df_row_tiny(res);
#pragma unroll
    for (int j = 0; j < N; ++j) bad |= df_bad(res[j]);
    if (bad && a.rflag) *a.rflag = a.rtag;
  }
  if constexpr (DOT)
    store_dot_part<P, N>([&](int j) { return u[j]; }, [&](int j) { return res[j]; }, a.dpart,
                         blockIdx.y * gridDim.x + blockIdx.x);

  static_assert(sizeof(V) == sizeof(IO), "line buffers are reused for stored values");
  tile_dss_store<P, N, TX, TY>(res, reinterpret_cast<IO*>(S1), reinterpret_cast<IO*>(S2), elem, lane,
                               ex, ey, valid, base, a.Ex, a.Ey, NX, mode, a.out);
}

// Finishes QQ' (and the mask) at the points whose copies sit in different
// tiles: x interfaces every TX elements (+ the periodic wrap), y interfaces
// every TY elements (+ wrap), and the corners on them.  Every node with four
// copies is summed x pairs first, ((rl,cl) + (rr,cl)) + ((rl,cr) + (rr,cr)),
// the order the in-tile pass and k_gather_scatter use, so the result does not
// depend on the tile shape.  blockIdx.y walks the interfaces (x interfaces,
// then y interfaces, then one row for the corners of two cross-tile
// interfaces), blockIdx.x/threadIdx.x the points along one interface.
struct FixArgs {
  int n, Ex, Ey, TX, TY;
  long long NX, NY;
  unsigned mode;
  long long nxi, nyi;  // number of cross-tile interfaces in x and y
  const int* skip;
  // only the interface points whose highest copy column lies in [key_lo, key_hi)
  // (a pipeline finishes the columns of one slab of tile rows at a time)
  long long key_lo, key_hi;
  const unsigned* gate;  // gated re-run: nothing to do unless *gate == gate_tag
  unsigned gate_tag;
};

__device__ __forceinline__ bool fix_key_in(long long key, long long lo, long long hi) {
  return key >= lo && key < hi;
}

__host__ __device__ inline long long fix_iface(long long q, int T, bool per) {
  return per ? q * T : (q + 1) * T;  // interface index a: between elements a-1 and a
}

template <class IO>
__device__ __forceinline__ IO fix_value(long long r, long long c, IO s, const FixArgs& f, bool msk) {
  return (msk && !mask_keep(r, c, f.NX, f.NY, f.mode)) ? masked_zero(s) : s;
}

// Number of interface rows of k_dss_fixup's index space: x interfaces, then
// y interfaces, then one row for the corners of two cross-tile interfaces.
__host__ __device__ inline long long fix_rows(const FixArgs& f) {
  return f.nxi + f.nyi + (f.nxi * f.nyi > 0 ? 1 : 0);
}

// Loads of values another CTA may have stored during the same launch go to L2
// (ld.global.cg), never to a possibly stale L1 line.
template <class IO>
__device__ __forceinline__ IO fix_ld(const IO* p) {
  return __ldcg(p);
}

// The copies on the x interface left of element column a (a == 0: the
// periodic wrap between the last and the first column), columns c_begin,
// c_begin + stride, ... below c_end.  Columns on cross-tile y interfaces are
// corners (fix_corner); on an in-tile y interface the four copies are summed,
// x pairs first.  done(r, c, value) is called for every copy stored.
template <class IO, class F>
__device__ __forceinline__ void fix_xline(IO* out, const FixArgs& f, long long a, long long c_begin,
                                          long long c_end, long long stride, F&& done) {
  const bool pery = (f.mode & M_PERY) != 0;
  const bool msk = (f.mode & M_MASK) != 0;
  const unsigned n = (unsigned)f.n;
  const long long rl = a == 0 ? f.NX - 1 : a * f.n - 1;
  const long long rr = a * f.n;
  auto put = [&](long long r, long long c, IO s) {
    const IO v = fix_value(r, c, s, f, msk);
    out[r + c * f.NX] = v;
    done(r, c, v);
  };
  for (long long c = c_begin; c < c_end; c += stride) {
    const int ey = (int)((unsigned)c / n);  // NX, NY < 2^31 (checked at launch)
    const int j = (int)(c - (long long)ey * f.n);
    if (xcross_row(ey, j, f.n, f.Ey, f.TY, pery)) continue;  // corner of two cross-tile interfaces
    if (j == 0 && ey > 0) continue;                            // in-tile y pair, done from column c-1
    const bool quad = j == f.n - 1 && ey + 1 < f.Ey;
    if (!fix_key_in(quad ? c + 1 : c, f.key_lo, f.key_hi)) continue;
    if (quad) {
      const long long c2 = c + 1;
      const IO s = io_add(io_add(fix_ld(out + rl + c * f.NX), fix_ld(out + rr + c * f.NX)),
                          io_add(fix_ld(out + rl + c2 * f.NX), fix_ld(out + rr + c2 * f.NX)));
      put(rl, c, s);
      put(rr, c, s);
      put(rl, c2, s);
      put(rr, c2, s);
      continue;
    }
    const IO s = io_add(fix_ld(out + rl + c * f.NX), fix_ld(out + rr + c * f.NX));
    put(rl, c, s);
    put(rr, c, s);
  }
}

// The copies on the y interface below element row b (b == 0: the wrap), rows
// r_begin, r_begin + stride, ... below r_end; rows on cross-tile x interfaces
// are corners.
template <class IO, class F>
__device__ __forceinline__ void fix_yline(IO* out, const FixArgs& f, long long b, long long r_begin,
                                          long long r_end, long long stride, F&& done) {
  const bool perx = (f.mode & M_PERX) != 0;
  const bool msk = (f.mode & M_MASK) != 0;
  const unsigned n = (unsigned)f.n;
  const long long cl = b == 0 ? f.NY - 1 : b * f.n - 1;
  const long long cr = b * f.n;
  if (!fix_key_in(cl > cr ? cl : cr, f.key_lo, f.key_hi)) return;
  for (long long r = r_begin; r < r_end; r += stride) {
    const int ex = (int)((unsigned)r / n);
    const int i = (int)(r - (long long)ex * f.n);
    if (xcross_row(ex, i, f.n, f.Ex, f.TX, perx)) continue;
    const IO s = io_add(fix_ld(out + r + cl * f.NX), fix_ld(out + r + cr * f.NX));
    const IO vl = fix_value(r, cl, s, f, msk);
    const IO vr = fix_value(r, cr, s, f, msk);
    out[r + cl * f.NX] = vl;
    out[r + cr * f.NX] = vr;
    done(r, cl, vl);
    done(r, cr, vr);
  }
}

// The four copies where the cross-tile x interface left of element column a
// meets the cross-tile y interface below element row b.
template <class IO, class F>
__device__ __forceinline__ void fix_corner(IO* out, const FixArgs& f, long long a, long long b, F&& done) {
  const bool msk = (f.mode & M_MASK) != 0;
  const long long rl = a == 0 ? f.NX - 1 : a * f.n - 1;
  const long long rr = a * f.n;
  const long long cl = b == 0 ? f.NY - 1 : b * f.n - 1;
  const long long cr = b * f.n;
  if (!fix_key_in(cl > cr ? cl : cr, f.key_lo, f.key_hi)) return;
  const IO s = io_add(io_add(fix_ld(out + rl + cl * f.NX), fix_ld(out + rr + cl * f.NX)),
                      io_add(fix_ld(out + rl + cr * f.NX), fix_ld(out + rr + cr * f.NX)));
  const long long rs[2] = {rl, rr};
  const long long cs[2] = {cl, cr};
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const IO val = fix_value(rs[u], cs[v], s, f, msk);
      out[rs[u] + cs[v] * f.NX] = val;
      done(rs[u], cs[v], val);
    }
}

// Finishes interface row q of k_dss_fixup's index space at the points first,
// first + stride, ...
template <class IO, class F>
__device__ __forceinline__ void fix_interface(IO* __restrict__ out, const FixArgs& f, long long q,
                                              long long first, long long stride, F&& done) {
  const bool perx = (f.mode & M_PERX) != 0;
  const bool pery = (f.mode & M_PERY) != 0;
  if (q < f.nxi) {
    // the columns whose unit key can lie in [key_lo, key_hi): a unit spans
    // columns c or c, c + 1 and its key is the higher one
    const long long c_lo = f.key_lo > 0 ? f.key_lo - 1 : 0;
    const long long c_hi = f.key_hi < f.NY ? f.key_hi : f.NY;
    fix_xline(out, f, fix_iface(q, f.TX, perx), c_lo + first, c_hi, stride, done);
  } else if (q < f.nxi + f.nyi) {
    fix_yline(out, f, fix_iface(q - f.nxi, f.TY, pery), first, f.NX, stride, done);
  } else {
    for (long long id = first; id < f.nxi * f.nyi; id += stride) {
      const long long qx = id / f.nyi;
      const long long qy = id - qx * f.nyi;
      fix_corner(out, f, fix_iface(qx, f.TX, perx), fix_iface(qy, f.TY, pery), done);
    }
  }
}

template <class IO>
__global__ void k_dss_fixup(IO* __restrict__ out, const FixArgs f) {
  pdl_wait();  // launched as a programmatic dependent of the operator kernel
  if (f.skip && *f.skip) return;
  if (f.gate && *f.gate != f.gate_tag) return;
  const long long nI = fix_rows(f);
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long first = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long q = blockIdx.y; q < nI; q += gridDim.y)
    fix_interface(out, f, q, first, stride, [](long long, long long, IO) {});
}

}  // namespace sem
