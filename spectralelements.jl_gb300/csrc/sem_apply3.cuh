// Third-generation fused element operator (kernel variant 4): a persistent
// grid whose CTAs walk the element tiles and prefetch the next tile's inputs
// while they compute the current one.
//
// The arithmetic, the phases and their order are those of k_apply2 (and so
// the results are bit-identical); what changes is where the inputs come from.
// Each thread copies the entries of u, G11, G12, G22 and B it will read itself
// (its row of its element) into a private shared-memory stage with cp.async,
// and each field's stage is refilled for the next tile as soon as the current
// tile has read it: u after phase A, the metric terms after phase C, B after
// the mass term.  Every wait is cp.async.wait_group 2 (three groups per tile,
// committed in the same order by every thread), so no DRAM latency is exposed
// after the first tile and no CTA waits at a barrier for another CTA's loads.
//
// Tile shapes are chosen so that two CTAs fit on one SM (stage + line buffers
// of about 110 KB at most for 8-byte fields).
//
// Reference: laplace (src/lapl.jl:70-81), hlmz (src/hlmz.jl:12-19),
// gatherScatter (src/gatherScatter.jl:8-16), mask (src/mask.jl:10-18).
#pragma once

#include "sem_apply2.cuh"

namespace sem {

template <int N>
struct PTile {
  static constexpr int TX = N <= 11 ? 8 : (N <= 15 ? 4 : 2);
  static constexpr int TY = N <= 5 ? 8 : (N <= 7 ? 4 : (N <= 9 ? 3 : (N <= 11 ? 2 : (N == 12 ? 3 : (N <= 15 ? 2 : 3)))));
  static constexpr int SP = N | 1;
  static constexpr int ES = N * SP;
  static constexpr int THREADS = TX * TY * N;
};

template <int NPEND>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND) : "memory");
}

template <class P, int N, int TX, int TY>
__global__ void __launch_bounds__(TX* TY* N, 2) k_apply3(const __grid_constant__ Apply2Args<P, N> a,
                                                         const int tiles_x, const int tiles) {
  typedef typename P::v V;
  typedef typename P::io IO;
  typedef typename GeoT<P>::type GT;
  static_assert(sizeof(V) == sizeof(IO), "line buffers are reused for stored values");
  constexpr int SP = N | 1;
  constexpr int ES = N * SP;
  constexpr int TE = TX * TY * ES;
  constexpr int T = TX * TY * N;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S0 = reinterpret_cast<V*>(smem_raw);  // u of the current tile (mass term), then the y exchange
  V* S1 = S0 + TE;                         // in-place work buffer
  GT* RG = reinterpret_cast<GT*>(S1 + TE);  // stage: G11, G12, G22, B  [slot][j][thread]
  IO* RU = reinterpret_cast<IO*>(RG + 4 * N * T);  // stage: u [j][thread]

  pdl_trigger();  // the next kernel (the cross-tile fixup) may be scheduled now
  pdl_wait();     // a no-op unless this launch is a programmatic dependent
  if (a.skip && *a.skip) return;
  if (a.gate && *a.gate != a.gate_tag) return;  // gated re-run not needed
  const int t = threadIdx.x;
  const int elem = t / N;
  const int lane = t - elem * N;
  const int exl = elem % TX;
  const int eyl = elem / TX;
  const long long NX = a.NX;
  const unsigned mode = a.mode;
  const bool stiff = (mode & M_STIFF) != 0;
  const bool mass = (mode & M_MASS) != 0;
  V* s0 = S0 + elem * ES;
  V* s1 = S1 + elem * ES;

  // this thread's element and row start for a tile index
  auto where = [&](int tile, int& ex, int& ey, long long& base) -> bool {
    const int ty = tile / tiles_x;
    const int tx = tile - ty * tiles_x;
    ex = tx * TX + exl;
    ey = ty * TY + eyl;
    base = (long long)ex * N + lane + (long long)ey * N * NX;
    return tile < tiles && ex < a.Ex && ey < a.Ey;
  };
  auto fetch_u = [&](int tile) {
    int ex, ey;
    long long base;
    if (where(tile, ex, ey, base)) {
      const IO* src = a.u + base;
#pragma unroll 1
      for (int j = 0; j < N; ++j, src += NX) cp_async(RU + j * T + t, src);
    }
    cp_async_commit();
  };
  auto fetch_g = [&](int tile) {
    int ex, ey;
    long long base;
    if (stiff && where(tile, ex, ey, base)) {
      long long gi = base;
#pragma unroll 1
      for (int j = 0; j < N; ++j, gi += NX) {
        cp_async(RG + (0 * N + j) * T + t, a.G11 + gi);
        cp_async(RG + (1 * N + j) * T + t, a.G12 + gi);
        cp_async(RG + (2 * N + j) * T + t, a.G22 + gi);
      }
    }
    cp_async_commit();
  };
  auto fetch_b = [&](int tile) {
    int ex, ey;
    long long base;
    if (mass && where(tile, ex, ey, base)) {
      const GT* src = a.B + base;
#pragma unroll 1
      for (int j = 0; j < N; ++j, src += NX) cp_async(RG + (3 * N + j) * T + t, src);
    }
    cp_async_commit();
  };

  int tile = blockIdx.x;
  fetch_u(tile);
  fetch_g(tile);
  fetch_b(tile);
  for (; tile < tiles; tile += gridDim.x) {
    const int next = tile + gridDim.x;
    int ex, ey;
    long long base;
    const bool valid = where(tile, ex, ey, base);

    // ---- A: row `lane` of u; y-direction derivative
    V res[N];
    bool kbad = false;  // range guard: a tiny stiffness row or a tiny k B product
    cp_async_wait_group<2>();  // u(tile); G(tile), B(tile) may be in flight
    {
      V u[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        u[j] = valid ? P::cvt(RU[j * T + t]) : P::zero();
        s0[j * SP + lane] = u[j];
      }
      fetch_u(next);
      if (stiff) {
        V us[N];
#pragma unroll
        for (int j = 0; j < N; ++j) s1[j * SP + lane] = u[j];
        eo_apply<P, N>(a.Ds, u, us);
        __syncthreads();
        // ---- B: column `lane` in place; x-direction derivative
        {
          V col[N], ur[N];
#pragma unroll
          for (int i = 0; i < N; ++i) col[i] = s1[lane * SP + i];
          eo_apply<P, N>(a.Dr, col, ur);
#pragma unroll
          for (int i = 0; i < N; ++i) s1[lane * SP + i] = ur[i];
        }
        __syncthreads();
        // ---- C: row `lane` in place; metric terms, transposed y-derivative
        cp_async_wait_group<2>();  // G(tile); B(tile), u(next) may be in flight
        V os[N];
        {
          V ws[N];
#pragma unroll
          for (int j = 0; j < N; ++j) {
            const V g11 = valid ? GeoT<P>::cvt(RG[(0 * N + j) * T + t]) : P::zero();
            const V g12 = valid ? GeoT<P>::cvt(RG[(1 * N + j) * T + t]) : P::zero();
            const V g22 = valid ? GeoT<P>::cvt(RG[(2 * N + j) * T + t]) : P::zero();
            const V ur = s1[j * SP + lane];
            V wr = P::fma(g11, ur, P::mul(g12, us[j]));
            ws[j] = P::fma(g12, ur, P::mul(g22, us[j]));
            if (mode & M_NUG) {
              const V nu = valid ? P::ld(a.nu + base + (long long)j * NX) : P::zero();
              wr = P::mul(nu, wr);
              ws[j] = P::mul(nu, ws[j]);
            }
            s1[j * SP + lane] = wr;
          }
          fetch_g(next);
          eo_apply<P, N>(a.Dst, ws, os);
        }
        __syncthreads();
        // ---- D: column `lane` in place; transposed x-derivative
        {
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
        for (int j = 0; j < N; ++j) res[j] = P::add(s1[j * SP + lane], os[j]);
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
        cp_async_wait_group<2>();
        fetch_g(next);
#pragma unroll
        for (int j = 0; j < N; ++j) res[j] = P::zero();
      }
    }
    cp_async_wait_group<2>();  // B(tile); u(next), G(next) may be in flight
    if (mass) {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const V b = valid ? GeoT<P>::cvt(RG[(3 * N + j) * T + t]) : P::zero();
        const V kb = (mode & M_KB) ? b : P::mul(a.k_s, b);
        if constexpr (P::kPrecision == SEM_F64_DF) kbad |= df_tiny_nz(kb, kKbTiny);
        res[j] = P::fin(P::fma(kb, s0[j * SP + lane], res[j]));
      }
    }
    fetch_b(next);

    if constexpr (P::kPrecision == SEM_F64_DF) {
      // range guard: a tiny stiffness or result row, a tiny k B or a NaN/Inf
      // result flags the call (degenerate metric terms arrive as NaN pairs)
      bool bad = kbad || df_row_tiny(res);
#pragma unroll
      for (int j = 0; j < N; ++j) bad |= df_bad(res[j]);
      if (bad && a.rflag) *a.rflag = a.rtag;
    }
    tile_dss_store<P, N, TX, TY>(res, reinterpret_cast<IO*>(S1), reinterpret_cast<IO*>(S0), elem, lane,
                                 ex, ey, valid, base, a.Ex, a.Ey, NX, mode, a.out);
    __syncthreads();  // the next tile overwrites s0 and s1
  }
  cp_async_wait_all();
}

}  // namespace sem
