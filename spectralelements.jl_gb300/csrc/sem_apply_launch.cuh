// Launch templates of the fused element-operator kernel, instantiated once per
// arithmetic policy in sem_apply_{f64,df,f32}.cu (parallel compilation).
#pragma once

#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "sem_apply2.cuh"
#include "sem_apply3.cuh"
#include "sem_apply4.cuh"
#include "sem_apply_kernels.cuh"

namespace sem {

std::pair<cudaEvent_t, cudaEvent_t>* timing_slot();
size_t max_smem_optin();
int num_sms();
// 2-D tensor map of an NX x NY field of elem-byte values (x contiguous) with a
// bx x by box; false when TMA cannot serve it (alignment, strides, a field not
// in device memory, no encoder)
bool encode_tile_map(CUtensorMap* map, const void* ptr, size_t elem, long long NX, long long NY, int bx, int by);

// per-policy launchers, one translation unit each for n <= 9 and n >= 10; tile
// receives the element tile (TX, TY) of the launched kernel for k_dss_fixup
int launch_apply_f64_lo(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s, int* tile);
int launch_apply_f64_hi(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s, int* tile);
int launch_apply_df_lo(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s, int* tile);
int launch_apply_df_hi(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s, int* tile);
int launch_apply_f32_lo(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s, int* tile);
int launch_apply_f32_hi(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s, int* tile);

template <class P, int N>
static void fill_eo(EOCoef<N, typename P::v>& c, const double* src, double scale = 1.0) {
  constexpr int M = N / 2;
  const double* A = src;
  const double* C = A + M * M;
  const double* cm = C + M * M;
  const double* mr = cm + M;
  for (int i = 0; i < M; ++i)
    for (int k = 0; k < M; ++k) {
      c.A[i][k] = P::from_double(scale * A[i * M + k]);
      c.Cc[i][k] = P::from_double(scale * C[i * M + k]);
    }
  for (int i = 0; i < M; ++i) {
    c.cm[i] = P::from_double(scale * cm[i]);
    c.mr[i] = P::from_double(scale * mr[i]);
  }
}

// The scalar nu of a call without a nu field multiplies the stiffness part
// after the last contraction; it is folded into the coefficients of the
// transposed derivatives instead (D' -> nu D'), which saves one multiply per
// point (M_NUFOLD).  The scaled coefficients are rounded once, so the results
// differ from nu .* (D'GD u) by rounding only; every kernel variant folds the
// same way, so the variants stay bit-identical.
static inline bool fold_nu(unsigned mode) { return !(mode & M_NU) && (mode & M_STIFF); }

// kern<<<grid, block, smem, s>>>(args...), as a programmatic dependent of
// the previous kernel on s when pdl is set
template <class... KArgs, class... Args>
static int launch_kernel(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool pdl,
                         Args... args) {
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  SEM_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
  return SEM_OK;
}

template <class P, int N, bool STAGE, bool DOT = false>
static int launch_apply_v(const Grid& g, const OperatorSet* ops, const ApplyCall& c,
                          cudaStream_t s) {
  typedef TileShape<N> TS;
  typedef typename P::io io;
  ApplyArgs<P, N> a;
  std::memset(&a, 0, sizeof(a));
  a.u = static_cast<const io*>(c.u);
  a.out = static_cast<io*>(c.out);
  a.G11 = static_cast<const io*>(c.G11);
  a.G12 = static_cast<const io*>(c.G12);
  a.G22 = static_cast<const io*>(c.G22);
  a.B = static_cast<const io*>(c.B);
  a.nu = static_cast<const io*>(c.nu);
  const bool fold = fold_nu(c.mode);
  a.nu_s = P::from_double(fold ? 1.0 : c.nu_s);
  a.k_s = P::from_double(c.k_s);
  a.Ex = g.Ex;
  a.Ey = g.Ey;
  a.NX = g.NX;
  a.mode = c.mode | (fold ? M_NUFOLD : 0u);
  a.skip = c.skip;
  a.rflag = c.rflag;
  a.rtag = c.rtag;
  a.gate = c.gate;
  a.gate_tag = c.gate_tag;
  int nslot = 0;
  a.slot_g = a.slot_b = a.slot_nu = -1;
  if (STAGE) {
    if (c.mode & M_STIFF) {
      a.slot_g = nslot;
      nslot += 3;
    }
    if (c.mode & M_MASS) a.slot_b = nslot++;
    if (c.mode & (M_NU | M_NUG)) a.slot_nu = nslot++;
  }
  fill_eo<P, N>(a.Dr, ops->eo[0]);
  fill_eo<P, N>(a.Drt, ops->eo[1], fold ? c.nu_s : 1.0);
  fill_eo<P, N>(a.Ds, ops->eo[2]);
  fill_eo<P, N>(a.Dst, ops->eo[3], fold ? c.nu_s : 1.0);
  const size_t te = (size_t)TS::TX * TS::TY * TS::ES;
  const size_t smem = 2 * te * sizeof(typename P::v) + nslot * te * sizeof(io);
  a.dpart = static_cast<df*>(c.cg_dpart);
  auto kern = k_apply<P, N, TS::TX, TS::TY, STAGE, DOT>;
  if (smem > 48 * 1024) SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((g.Ex + TS::TX - 1) / TS::TX, c.tyn > 0 ? c.tyn : (g.Ey + TS::TY - 1) / TS::TY);
  a.ty0 = c.ty0;
  auto* ev = c.gate ? nullptr : timing_slot();  // gated re-runs are not timed
  if (ev) SEM_CUDA(cudaEventRecord(ev->first, s));
  SEM_CHECK(launch_kernel(kern, grid, TS::THREADS, smem, s, c.pdl != 0, a));
  if (ev) SEM_CUDA(cudaEventRecord(ev->second, s));
  return SEM_OK;
}

template <class P, int N>
static void fill_args2(Apply2Args<P, N>& a, const Grid& g, const OperatorSet* ops, const ApplyCall& c) {
  typedef typename P::io io;
  typedef typename GeoT<P>::type gt;
  std::memset(&a, 0, sizeof(a));
  a.u = static_cast<const io*>(c.u);
  a.out = static_cast<io*>(c.out);
  if (P::kPrecision == SEM_F64_DF) {
    const long long L = g.NX * g.NY;
    const gt* G = static_cast<const gt*>(c.Gdf);
    a.G11 = G;
    a.G12 = G + L;
    a.G22 = G + 2 * L;
    a.B = G + 3 * L;
  } else {
    a.G11 = static_cast<const gt*>(c.G11);
    a.G12 = static_cast<const gt*>(c.G12);
    a.G22 = static_cast<const gt*>(c.G22);
    a.B = static_cast<const gt*>(c.B);
  }
  a.nu = static_cast<const io*>(c.nu);
  const bool fold = fold_nu(c.mode);
  a.nu_s = P::from_double(fold ? 1.0 : c.nu_s);
  a.k_s = P::from_double(c.k_s);
  a.rflag = c.rflag;
  a.rtag = c.rtag;
  a.gate = c.gate;
  a.gate_tag = c.gate_tag;
  a.Ex = g.Ex;
  a.Ey = g.Ey;
  a.NX = g.NX;
  a.mode = c.mode | (fold ? M_NUFOLD : 0u);
  a.skip = c.skip;
  fill_eo<P, N>(a.Dr, ops->eo[0]);
  fill_eo<P, N>(a.Drt, ops->eo[1], fold ? c.nu_s : 1.0);
  fill_eo<P, N>(a.Ds, ops->eo[2]);
  fill_eo<P, N>(a.Dst, ops->eo[3], fold ? c.nu_s : 1.0);
}

template <class P, int N, bool STAGE, bool FUSE = false, bool CG = false>
static int launch_apply_v2(const Grid& g, const OperatorSet* ops, const ApplyCall& c,
                           cudaStream_t s) {
  typedef TileShape<N> TS;
  typedef typename GeoT<P>::type gt;
  typedef typename P::io io;
  Apply2Args<P, N> a;
  fill_args2<P, N>(a, g, ops, c);
  if (CG) {
    a.r = static_cast<const io*>(c.cg_r);
    a.dinv = static_cast<const io*>(c.cg_dinv);
    a.p = static_cast<io*>(c.cg_p);
    a.beta = c.cg_beta;
    a.dpart = static_cast<df*>(c.cg_dpart);
  }
  if (FUSE) {
    a.ctr = c.ctr;
    a.tiles_x = (g.Ex + TS::TX - 1) / TS::TX;
    a.tiles_y = (g.Ey + TS::TY - 1) / TS::TY;
  }
  const size_t te = (size_t)TS::TX * TS::TY * TS::ES;
  const size_t smem = 2 * te * sizeof(typename P::v) + (STAGE ? 3 * te * sizeof(gt) : 0);
  auto kern = k_apply2<P, N, TS::TX, TS::TY, STAGE, FUSE, CG>;
  if (smem > 48 * 1024) SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((g.Ex + TS::TX - 1) / TS::TX, c.tyn > 0 ? c.tyn : (g.Ey + TS::TY - 1) / TS::TY);
  a.ty0 = c.ty0;
  auto* ev = c.gate ? nullptr : timing_slot();  // gated re-runs are not timed
  if (ev) SEM_CUDA(cudaEventRecord(ev->first, s));
  SEM_CHECK(launch_kernel(kern, grid, TS::THREADS, smem, s, c.pdl != 0, a));
  if (ev) SEM_CUDA(cudaEventRecord(ev->second, s));
  return SEM_OK;
}

// persistent prefetching kernel: grid = resident CTAs, balanced so that every
// CTA walks the same number of tiles (up to one)
template <class P, int N>
static int launch_apply_v3(const Grid& g, const OperatorSet* ops, const ApplyCall& c,
                           cudaStream_t s) {
  typedef PTile<N> TS;
  typedef typename GeoT<P>::type gt;
  Apply2Args<P, N> a;
  fill_args2<P, N>(a, g, ops, c);
  const size_t te = (size_t)TS::TX * TS::TY * TS::ES;
  const size_t smem = 2 * te * sizeof(typename P::v) +
                      (size_t)N * TS::THREADS * (4 * sizeof(gt) + sizeof(typename P::io));
  auto kern = k_apply3<P, N, TS::TX, TS::TY>;
  if (smem > 48 * 1024) SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  SEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TS::THREADS, smem));
  if (per_sm < 1) return set_error(SEM_ERR_UNSUPPORTED, "persistent operator kernel does not fit an SM (n = %d)", N);
  const int tiles_x = (g.Ex + TS::TX - 1) / TS::TX;
  const int tiles_y = (g.Ey + TS::TY - 1) / TS::TY;
  const long long tiles = (long long)tiles_x * tiles_y;
  if (tiles > 2147483647LL) return set_error(SEM_ERR_UNSUPPORTED, "too many element tiles");
  const long long slots = (long long)per_sm * num_sms();
  const long long rounds = (tiles + slots - 1) / slots;
  const long long grid = (tiles + rounds - 1) / rounds;
  auto* ev = c.gate ? nullptr : timing_slot();  // gated re-runs are not timed
  if (ev) SEM_CUDA(cudaEventRecord(ev->first, s));
  SEM_CHECK(launch_kernel(kern, dim3((unsigned)grid), TS::THREADS, smem, s, c.pdl != 0, a, tiles_x, (int)tiles));
  if (ev) SEM_CUDA(cudaEventRecord(ev->second, s));
  return SEM_OK;
}

// TMA persistent kernel (variant 6); *served = false, with nothing launched,
// when the call's fields cannot be described by tensor maps
template <class P, int N>
static int launch_apply_v4(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s,
                           bool* served) {
  typedef PTile<N> TS;
  typedef typename GeoT<P>::type gt;
  typedef typename P::io io;
  typedef K4Layout<P, N, TS::TX, TS::TY> L;
  *served = false;
  if (L::total > max_smem_optin()) return SEM_OK;
  Apply2Args<P, N> a;
  fill_args2<P, N>(a, g, ops, c);
  TmaSet maps;
  std::memset(&maps, 0, sizeof(maps));
  const int bx = TS::TX * N, by = TS::TY * N;
  if (!encode_tile_map(&maps.m[0], a.u, sizeof(io), g.NX, g.NY, bx, by)) return SEM_OK;
  if (c.mode & M_STIFF) {
    if (!encode_tile_map(&maps.m[1], a.G11, sizeof(gt), g.NX, g.NY, bx, by) ||
        !encode_tile_map(&maps.m[2], a.G12, sizeof(gt), g.NX, g.NY, bx, by) ||
        !encode_tile_map(&maps.m[3], a.G22, sizeof(gt), g.NX, g.NY, bx, by))
      return SEM_OK;
  }
  if ((c.mode & M_MASS) && !encode_tile_map(&maps.m[4], a.B, sizeof(gt), g.NX, g.NY, bx, by)) return SEM_OK;
  // the word is made outside launches (variant selection, the autotuner, an
  // uncaptured stream); a launch on a capturing stream before then runs as
  // variant 4
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;  // unknown: do not allocate
  }
  unsigned* werr = wait_timeout_word(cap == cudaStreamCaptureStatusNone);
  if (!werr) {
    if (cap != cudaStreamCaptureStatusNone) return SEM_OK;
    return set_error(SEM_ERR_CUDA, "cannot make the TMA timeout word");
  }
  auto kern = k_apply4<P, N, TS::TX, TS::TY>;
  SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::total));
  int per_sm = 0;
  SEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TS::THREADS, L::total));
  if (per_sm < 1) return SEM_OK;
  const int tiles_x = (g.Ex + TS::TX - 1) / TS::TX;
  const int tiles_y = (g.Ey + TS::TY - 1) / TS::TY;
  const long long tiles = (long long)tiles_x * tiles_y;
  if (tiles > 2147483647LL) return set_error(SEM_ERR_UNSUPPORTED, "too many element tiles");
  const long long slots = (long long)per_sm * num_sms();
  const long long rounds = (tiles + slots - 1) / slots;
  const long long grid = (tiles + rounds - 1) / rounds;
  auto* ev = c.gate ? nullptr : timing_slot();  // gated re-runs are not timed
  if (ev) SEM_CUDA(cudaEventRecord(ev->first, s));
  SEM_CHECK(launch_kernel(kern, dim3((unsigned)grid), TS::THREADS, L::total, s, c.pdl != 0, a, maps, tiles_x,
                          (int)tiles, werr));
  if (ev) SEM_CUDA(cudaEventRecord(ev->second, s));
  *served = true;
  return SEM_OK;
}

// variant 0: k_apply, direct loads; 1: k_apply, cp.async-staged inputs;
// 2: k_apply2, direct loads; 3: k_apply2, cp.async-staged metric terms;
// 4: k_apply3, persistent CTAs prefetching the next tile; 5: k_apply2 with
// the cross-tile QQ' completed inside the kernel (tile = {0, 0}: no fixup);
// 6: k_apply4, persistent CTAs whose element tiles arrive by TMA copies (runs
// as variant 4 where tensor maps cannot describe the call's fields).
// Variants 2-5 of the double-float policy read the pre-split geometry
// (ApplyCall::Gdf) and run as variant 0 when the call carries none; variant 5
// runs as variant 2 without counters (ApplyCall::ctr) or with a single tile
// across a periodic direction; a staged variant whose shared memory exceeds
// the opt-in limit runs unstaged.
template <class P, int N>
static int launch_apply_n(const Grid& g, const OperatorSet* ops, const ApplyCall& c,
                          cudaStream_t s, int* tile) {
  const bool geo_ok = P::kPrecision != SEM_F64_DF || c.Gdf;
  const bool cg = c.cg_p != nullptr;
  // DOT launches (p . A p parts without the direction update) are served by
  // the k_apply variants 0 and 1
  const bool dot = !cg && c.cg_dpart != nullptr;
  if (dot && !(c.variant <= 1 || (P::kPrecision == SEM_F64_DF && !geo_ok)))
    return set_error(SEM_ERR_UNSUPPORTED, "a p.Ap launch needs kernel variant 0 or 1");
  if (c.tyn > 0) {  // a window of tile rows: the non-persistent kernels with the fixup outside
    if (cg) return set_error(SEM_ERR_UNSUPPORTED, "a tile-row window takes no CG fusion");
    if (c.variant >= 4) {
      ApplyCall c2 = c;
      c2.variant = 2;
      return launch_apply_n<P, N>(g, ops, c2, s, tile);
    }
  }
  if (cg && !(geo_ok && (c.variant == 2 || c.variant == 5) && (c.mode & M_STIFF)))
    return set_error(SEM_ERR_UNSUPPORTED, "CG-fused operator launch needs kernel variant 2 or 5");
  if (c.variant == 5 && geo_ok && c.ctr && (c.mode & M_GS)) {
    typedef TileShape<N> TS;
    const bool one_x = (g.Ex + TS::TX - 1) / TS::TX < 2, one_y = (g.Ey + TS::TY - 1) / TS::TY < 2;
    if (!((c.mode & M_PERX) && one_x) && !((c.mode & M_PERY) && one_y)) {
      tile[0] = tile[1] = 0;
      return cg ? launch_apply_v2<P, N, false, true, true>(g, ops, c, s)
                : launch_apply_v2<P, N, false, true>(g, ops, c, s);
    }
  }
  if (cg) {
    tile[0] = TileShape<N>::TX;
    tile[1] = TileShape<N>::TY;
    return launch_apply_v2<P, N, false, false, true>(g, ops, c, s);
  }
  if ((c.variant == 4 || c.variant == 6) && geo_ok) {
    tile[0] = PTile<N>::TX;
    tile[1] = PTile<N>::TY;
    if (c.variant == 6) {
      bool served = false;
      const int st = launch_apply_v4<P, N>(g, ops, c, s, &served);
      if (st != SEM_OK) return st;
      if (served) return SEM_OK;
    }
    return launch_apply_v3<P, N>(g, ops, c, s);
  }
  typedef TileShape<N> TS;
  tile[0] = TS::TX;
  tile[1] = TS::TY;
  if (c.variant >= 2 && c.variant != 4 && c.variant != 6 && geo_ok) {
    const size_t te = (size_t)TS::TX * TS::TY * TS::ES;
    const size_t smem = 2 * te * sizeof(typename P::v) + 3 * te * sizeof(typename GeoT<P>::type);
    if (c.variant == 3 && smem <= max_smem_optin()) return launch_apply_v2<P, N, true>(g, ops, c, s);
    return launch_apply_v2<P, N, false>(g, ops, c, s);
  }
  if (c.variant == 1) {
    const size_t te = (size_t)TS::TX * TS::TY * TS::ES;
    const int nslot = ((c.mode & M_STIFF) ? 3 : 0) + ((c.mode & M_MASS) ? 1 : 0) +
                      ((c.mode & (M_NU | M_NUG)) ? 1 : 0);
    const size_t smem = 2 * te * sizeof(typename P::v) + nslot * te * sizeof(typename P::io);
    if (smem <= max_smem_optin())
      return dot ? launch_apply_v<P, N, true, true>(g, ops, c, s) : launch_apply_v<P, N, true>(g, ops, c, s);
  }
  return dot ? launch_apply_v<P, N, false, true>(g, ops, c, s) : launch_apply_v<P, N, false>(g, ops, c, s);
}

// element tile (TX, TY) of the non-persistent kernels for n points (host)
inline void tile_shape(int n, int* tx, int* ty) {
  switch (n) {
#define SEM_CASE(NN)            \
  case NN:                      \
    *tx = TileShape<NN>::TX;    \
    *ty = TileShape<NN>::TY;    \
    return;
    SEM_CASE(2) SEM_CASE(3) SEM_CASE(4) SEM_CASE(5) SEM_CASE(6) SEM_CASE(7) SEM_CASE(8)
    SEM_CASE(9) SEM_CASE(10) SEM_CASE(11) SEM_CASE(12) SEM_CASE(13) SEM_CASE(14)
    SEM_CASE(15) SEM_CASE(16) SEM_CASE(17)
#undef SEM_CASE
    default:
      *tx = *ty = 1;
  }
}

// the orders LO..HI of one policy (one translation unit)
template <class P, int LO, int HI>
static int launch_apply_range(const Grid& g, const OperatorSet* ops, const ApplyCall& c,
                              cudaStream_t s, int* tile) {
  switch (g.n) {
#define SEM_CASE(NN)                                                            \
  case NN:                                                                      \
    if constexpr (NN >= LO && NN <= HI) return launch_apply_n<P, NN>(g, ops, c, s, tile); \
    break;
    SEM_CASE(2) SEM_CASE(3) SEM_CASE(4) SEM_CASE(5) SEM_CASE(6) SEM_CASE(7) SEM_CASE(8)
    SEM_CASE(9) SEM_CASE(10) SEM_CASE(11) SEM_CASE(12) SEM_CASE(13) SEM_CASE(14)
    SEM_CASE(15) SEM_CASE(16) SEM_CASE(17)
#undef SEM_CASE
    default:
      break;
  }
  return set_error(SEM_ERR_UNSUPPORTED, "no fused kernel for n = %d", g.n);
}

}  // namespace sem
