// Fourth-generation fused element operator (kernel variant 6): the persistent
// grid of k_apply3, with every input tile moved by the tensor memory
// accelerator (TMA) instead of per-thread copies.
//
// One thread of each CTA issues, per element tile, five 2-D tensor copies
// (cp.async.bulk.tensor) of the tile's TX*n x TY*n box of u, G11, G12, G22 and
// B from HBM into shared memory; each copy signals an mbarrier with its byte
// count (complete_tx).  A field's box is refilled for the next tile as soon as
// every thread has read it (u after phase A, the metric terms after phase C,
// B after the mass term: the block barriers that end those phases order the
// reads before the refill), so the next tile's bytes stream in while the
// current tile computes, and the per-thread load instructions of the other
// variants (and their address arithmetic) leave the issue stream.
//
// Shared-memory box layout is the tensor's own: point (x, y) of the box at
// y * TX*n + x.  A thread reads its row of its element (fixed x, n values of
// y) at a stride of TX*n, so a warp reads consecutive addresses.
//
// The arithmetic, the phases and their order are those of k_apply2 and
// k_apply3, so the results are bit-identical to every other variant.
//
// Every mbarrier wait is bounded (about two seconds of %globaltimer).  A wait
// that runs out makes the whole CTA leave at the next block barrier: one
// thread adds 1 to the caller's timeout word, waits (again bounded) for the
// copies this CTA still has in flight, and for the double-float policy sets
// the call's range-guard word, so the gated native FP64 re-run (variant 4)
// recomputes the result.
//
// Reference: laplace (src/lapl.jl:70-81), hlmz (src/hlmz.jl:12-19),
// gatherScatter (src/gatherScatter.jl:8-16), mask (src/mask.jl:10-18).
#pragma once

#include <cuda.h>  // CUtensorMap (the type only; the encoder is reached through the runtime)

#include "sem_apply3.cuh"

namespace sem {

// tensor maps of one launch: u, G11, G12, G22, B (NX x NY, x contiguous)
struct TmaSet {
  CUtensorMap m[5];
};

constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // bound of one mbarrier wait

// shared-memory layout of k_apply4 (byte offsets from a 128-byte aligned base)
template <class P, int N, int TX, int TY>
struct K4Layout {
  static constexpr size_t al(size_t x) { return (x + 127) / 128 * 128; }
  static constexpr int TE = TX * TY * N * (N | 1);
  static constexpr int BOX = TX * N * TY * N;
  static constexpr size_t ubytes = (size_t)BOX * sizeof(typename P::io);
  static constexpr size_t gbytes = (size_t)BOX * sizeof(typename GeoT<P>::type);
  static constexpr size_t u = al(2 * (size_t)TE * sizeof(typename P::v));
  static constexpr size_t g = u + al(ubytes);
  static constexpr size_t b = g + 3 * al(gbytes);
  static constexpr size_t bar = b + al(gbytes);
  static constexpr size_t total = bar + 3 * sizeof(unsigned long long) + 128;  // + base alignment slack
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make the initialised barriers visible to the async proxy (the TMA unit)
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// wait for the phase of the given parity; false once kWaitLimitNs have passed
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kWaitLimitNs) return false;
  }
}

// 2-D tensor copy of the box at element coordinates (x, y) into shared memory
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, unsigned long long* bar, int x,
                                            int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

template <class P, int N, int TX, int TY>
__global__ void __launch_bounds__(TX* TY* N, 2)
    k_apply4(const __grid_constant__ Apply2Args<P, N> a, const __grid_constant__ TmaSet maps, const int tiles_x,
             const int tiles, unsigned* werr) {
  typedef typename P::v V;
  typedef typename P::io IO;
  typedef typename GeoT<P>::type GT;
  typedef K4Layout<P, N, TX, TY> L;
  static_assert(sizeof(V) == sizeof(IO), "line buffers are reused for stored values");
  constexpr int SP = N | 1;
  constexpr int ES = N * SP;
  constexpr int TE = TX * TY * ES;
  constexpr int BX = TX * N;  // box row length (x)
  constexpr int BY = TY * N;  // box rows (y)
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<size_t>(smem_raw) + 127) & ~(size_t)127);
  V* S0 = reinterpret_cast<V*>(sm);  // u of the current tile (mass term), then the y exchange
  V* S1 = S0 + TE;                   // in-place work buffer
  IO* SU = reinterpret_cast<IO*>(sm + L::u);
  GT* SG = reinterpret_cast<GT*>(sm + L::g);  // G11, G12, G22 boxes, al(gbytes) apart
  GT* SB = reinterpret_cast<GT*>(sm + L::b);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(sm + L::bar);  // u, G, B
  constexpr int GSTRIDE = (int)(L::al(L::gbytes) / sizeof(GT));

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
  const int srow = eyl * N * BX + exl * N + lane;  // this thread's row in a box; + j * BX

  if (t == 0) {
    for (int i = 0; i < 3; ++i) mbar_init(bar + i, 1);
    mbar_fence_init();
  }
  __syncthreads();

  // loads issued per barrier (thread 0 only): the k-th load completes phase k
  unsigned nu_iss = 0, ng_iss = 0, nb_iss = 0;
  auto issue_u = [&](int tile) {
    if (t != 0 || tile >= tiles) return;
    const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
    mbar_expect_tx(bar + 0, (unsigned)L::ubytes);
    tma_load_2d(SU, &maps.m[0], bar + 0, tx * BX, ty * BY);
    ++nu_iss;
  };
  auto issue_g = [&](int tile) {
    if (t != 0 || tile >= tiles || !stiff) return;
    const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
    mbar_expect_tx(bar + 1, (unsigned)(3 * L::gbytes));
    for (int f = 0; f < 3; ++f) tma_load_2d(SG + f * GSTRIDE, &maps.m[1 + f], bar + 1, tx * BX, ty * BY);
    ++ng_iss;
  };
  auto issue_b = [&](int tile) {
    if (t != 0 || tile >= tiles || !mass) return;
    const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
    mbar_expect_tx(bar + 2, (unsigned)L::gbytes);
    tma_load_2d(SB, &maps.m[4], bar + 2, tx * BX, ty * BY);
    ++nb_iss;
  };
  auto where = [&](int tile, int& ex, int& ey, long long& base) -> bool {
    const int ty = tile / tiles_x;
    const int tx = tile - ty * tiles_x;
    ex = tx * TX + exl;
    ey = ty * TY + eyl;
    base = (long long)ex * N + lane + (long long)ey * N * NX;
    return tile < tiles && ex < a.Ex && ey < a.Ey;
  };

  int tile = blockIdx.x;
  issue_u(tile);
  issue_g(tile);
  issue_b(tile);
  bool failed = false;
  for (unsigned it = 0; tile < tiles; tile += gridDim.x, ++it) {
    const int next = tile + gridDim.x;
    const unsigned ph = it & 1u;
    int ex, ey;
    long long base;
    const bool valid = where(tile, ex, ey, base);

    // ---- A: row `lane` of u; y-direction derivative
    V res[N];
    bool kbad = false;  // range guard: a tiny stiffness row or a tiny k B product
    bool ok = mbar_wait(bar + 0, ph);
    {
      V u[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        u[j] = valid ? P::cvt(SU[srow + j * BX]) : P::zero();
        s0[j * SP + lane] = u[j];
      }
      if (stiff) {
        V us[N];
#pragma unroll
        for (int j = 0; j < N; ++j) s1[j * SP + lane] = u[j];
        eo_apply<P, N>(a.Ds, u, us);
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
        issue_u(next);  // every thread has read the u box
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
        ok = mbar_wait(bar + 1, ph);
        V os[N];
        {
          V ws[N];
#pragma unroll
          for (int j = 0; j < N; ++j) {
            const V g11 = valid ? GeoT<P>::cvt(SG[srow + j * BX]) : P::zero();
            const V g12 = valid ? GeoT<P>::cvt(SG[GSTRIDE + srow + j * BX]) : P::zero();
            const V g22 = valid ? GeoT<P>::cvt(SG[2 * GSTRIDE + srow + j * BX]) : P::zero();
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
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
        issue_g(next);  // every thread has read the metric boxes
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
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
        issue_u(next);
#pragma unroll
        for (int j = 0; j < N; ++j) res[j] = P::zero();
      }
    }
    ok = true;
    if (mass) {
      ok = mbar_wait(bar + 2, ph);
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const V b = valid ? GeoT<P>::cvt(SB[srow + j * BX]) : P::zero();
        const V kb = (mode & M_KB) ? b : P::mul(a.k_s, b);
        if constexpr (P::kPrecision == SEM_F64_DF) kbad |= df_tiny_nz(kb, kKbTiny);
        res[j] = P::fin(P::fma(kb, s0[j * SP + lane], res[j]));
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
    tile_dss_store<P, N, TX, TY>(res, reinterpret_cast<IO*>(S1), reinterpret_cast<IO*>(S0), elem, lane, ex, ey,
                                 valid, base, a.Ex, a.Ey, NX, mode, a.out);
    if (__syncthreads_or(!ok)) {  // the next tile overwrites s0 and s1
      failed = true;
      break;
    }
    issue_b(next);  // every thread has read the B box
  }
  if (failed && t == 0) {
    // a copy did not arrive in time: report it, let the copies still in
    // flight land (bounded) before the CTA's shared memory is released, and
    // have the double-float call recomputed by its native FP64 re-run
    atomicAdd(werr, 1u);
    if (nu_iss) mbar_wait(bar + 0, (nu_iss - 1) & 1u);
    if (ng_iss) mbar_wait(bar + 1, (ng_iss - 1) & 1u);
    if (nb_iss) mbar_wait(bar + 2, (nb_iss - 1) & 1u);
    if constexpr (P::kPrecision == SEM_F64_DF)
      if (a.rflag) *a.rflag = a.rtag;
  }
}

}  // namespace sem
