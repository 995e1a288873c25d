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
  int Ex, Ey;
  long long NX;
  unsigned mode;
  const int* skip;
  EOCoef<N, v> Dr, Drt, Ds, Dst;
};

// resident blocks per SM asked of the register allocator: without the
// register copy of u the double-float kernel fits four blocks (72 registers,
// no spills) up to n = 9
template <class P, int N, bool STAGE>
struct MinBlocks2 {
  static constexpr int value =
      (!STAGE && P::kPrecision == SEM_F64_DF && N <= 9) ? 4 : MinBlocks<P, N, STAGE>::value;
};

template <class P, int N, int TX, int TY, bool STAGE>
__global__ void __launch_bounds__(TX* TY* N, (MinBlocks2<P, N, STAGE>::value))
    k_apply2(const __grid_constant__ Apply2Args<P, N> a) {
  typedef typename P::v V;
  typedef typename P::io IO;
  typedef typename GeoT<P>::type GT;
  constexpr int SP = N | 1;
  constexpr int ES = N * SP;
  constexpr int TE = TX * TY * ES;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* S0 = reinterpret_cast<V*>(smem_raw);  // u (mass term), later the y exchange
  V* S1 = S0 + TE;                         // in-place work buffer
  GT* R = reinterpret_cast<GT*>(S1 + TE);  // staged G11, G12, G22 (variant 3)

  if (a.skip && *a.skip) return;
  const int t = threadIdx.x;
  const int elem = t / N;
  const int lane = t - elem * N;
  const int exl = elem % TX;
  const int eyl = elem / TX;
  const int ex = blockIdx.x * TX + exl;
  const int ey = blockIdx.y * TY + eyl;
  const bool valid = ex < a.Ex && ey < a.Ey;
  const long long NX = a.NX;
  const long long base = (long long)ex * N + lane + (long long)ey * N * NX;
  const unsigned mode = a.mode;
  const bool stiff = (mode & M_STIFF) != 0;
  V* s0 = S0 + elem * ES;
  V* s1 = S1 + elem * ES;
  const int rofs = elem * ES + lane;

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
#pragma unroll
    for (int j = 0; j < N; ++j) {
      u[j] = valid ? P::ld(a.u + base + (long long)j * NX) : P::zero();
      s0[j * SP + lane] = u[j];
    }
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
      if (STAGE) cp_async_wait_all();
      V os[N];
      {
        V ws[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const V g11 = ldg(a.G11, 0, j);
          const V g12 = ldg(a.G12, 1, j);
          const V g22 = ldg(a.G22, 2, j);
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
      if (mode & M_NU) {
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const V nu = valid ? P::ld(a.nu + base + (long long)j * NX) : P::zero();
          res[j] = P::fin(P::mul(nu, res[j]));
        }
      } else {
#pragma unroll
        for (int j = 0; j < N; ++j) res[j] = P::fin(P::mul(a.nu_s, res[j]));
      }
    } else {
#pragma unroll
      for (int j = 0; j < N; ++j) res[j] = P::zero();
    }
  }
  if (mode & M_MASS) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const V b = valid ? GeoT<P>::ld(a.B + base + (long long)j * NX) : P::zero();
      res[j] = P::fin(P::fma(P::mul(a.k_s, b), s0[j * SP + lane], res[j]));
    }
  }

  static_assert(sizeof(V) == sizeof(IO), "line buffers are reused for stored values");
  tile_dss_store<P, N, TX, TY>(res, reinterpret_cast<IO*>(S1), reinterpret_cast<IO*>(S0), elem, lane,
                               ex, ey, valid, base, a.Ex, a.Ey, NX, mode, a.out);
}

}  // namespace sem
