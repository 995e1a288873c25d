// Host side of the fused operator kernels: coefficient sets and launches.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include <cudaTypedefs.h>

#include "sem_apply_launch.cuh"

namespace sem {

// ---- event timing of the fused kernel launches (instrumentation)
std::mutex g_tmu;
bool g_timing = false;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_pool;  // recycled event pairs
size_t g_used = 0;

std::pair<cudaEvent_t, cudaEvent_t>* timing_slot() {
  std::lock_guard<std::mutex> lk(g_tmu);
  if (!g_timing) return nullptr;
  if (g_used == g_pool.size()) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess) return nullptr;
    if (cudaEventCreate(&b) != cudaSuccess) {
      cudaEventDestroy(a);
      return nullptr;
    }
    g_pool.emplace_back(a, b);
  }
  return &g_pool[g_used++];
}

bool timing_enabled() {
  std::lock_guard<std::mutex> lk(g_tmu);
  return g_timing;
}

size_t max_smem_optin() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 48 * 1024;
  if (!cached[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) v = 48 * 1024;
    cached[dev] = v;
  }
  return (size_t)cached[dev];
}

bool is_centro_antisymmetric(const double* D, int n, double rel_tol) {
  double mx = 0.0;
  for (int i = 0; i < n * n; ++i) mx = std::fmax(mx, std::fabs(D[i]));
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < n; ++i) {
      const double a = D[i + k * n];
      const double b = D[(n - 1 - i) + (n - 1 - k) * n];
      if (!(std::fabs(a + b) <= rel_tol * mx)) return false;
    }
  return true;
}

void eo_from_dense(const double* D, int n, bool transpose, double* A, double* C, double* cm,
                   double* mr) {
  const int m = n / 2;
  auto at = [&](int i, int k) { return transpose ? D[k + i * n] : D[i + k * n]; };
  // exactly centro-antisymmetric part of D
  auto ds = [&](int i, int k) { return 0.5 * (at(i, k) - at(n - 1 - i, n - 1 - k)); };
  for (int i = 0; i < m; ++i)
    for (int k = 0; k < m; ++k) {
      A[i * m + k] = 0.5 * (ds(i, k) - ds(i, n - 1 - k));
      C[i * m + k] = 0.5 * (ds(i, k) + ds(i, n - 1 - k));
    }
  for (int i = 0; i < m; ++i) {
    cm[i] = (n & 1) ? ds(i, m) : 0.0;
    mr[i] = (n & 1) ? ds(m, i) : 0.0;
  }
}

int init_operator_set(const double* Dr, const double* Ds, int n, OperatorSet* o) {
  if (n < 2 || n > kMaxN) return set_error(SEM_ERR_UNSUPPORTED, "fused operators serve 2 <= n <= %d GLL points, got %d", kMaxN, n);
  if (!is_centro_antisymmetric(Dr, n, 1e-12) || !is_centro_antisymmetric(Ds, n, 1e-12))
    return set_error(SEM_ERR_UNSUPPORTED,
                     "derivative matrices must be centro-antisymmetric (GLL derivative "
                     "matrices are); a general matrix is served by sem_abu");
  std::memset(o, 0, sizeof(*o));
  o->n = n;
  std::memcpy(o->Dr, Dr, sizeof(double) * n * n);
  std::memcpy(o->Ds, Ds, sizeof(double) * n * n);
  const int m = n / 2;
  for (int b = 0; b < 4; ++b) {
    const double* D = b < 2 ? Dr : Ds;
    double* p = o->eo[b];
    eo_from_dense(D, n, (b & 1) != 0, p, p + m * m, p + 2 * m * m, p + 2 * m * m + m);
  }
  return SEM_OK;
}

int make_operator_set(const double* Dr, const double* Ds, int n, OperatorSet** out) {
  OperatorSet* o = new OperatorSet;
  const int st = init_operator_set(Dr, Ds, n, o);
  if (st != SEM_OK) {
    delete o;
    return st;
  }
  *out = o;
  return SEM_OK;
}

void free_operator_set(OperatorSet* o) { delete o; }

int num_sms() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cached[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) v = 152;
    cached[dev] = v;
  }
  return cached[dev];
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library), looked up once per process
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

bool encode_tile_map(CUtensorMap* map, const void* ptr, size_t elem, long long NX, long long NY, int bx, int by) {
  // TMA rules: 16-byte aligned base, row pitch and box row; box sides <= 256
  if (!ptr || (reinterpret_cast<uintptr_t>(ptr) & 15) || ((size_t)NX * elem) % 16 || ((size_t)bx * elem) % 16 ||
      bx < 1 || by < 1 || bx > 256 || by > 256 || NX < 1 || NY < 1 || NX >= (1LL << 32) || NY >= (1LL << 32))
    return false;
  if (elem != 4 && elem != 8) return false;
  cudaPointerAttributes pa;
  if (cudaPointerGetAttributes(&pa, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (pa.type != cudaMemoryTypeDevice) return false;  // TMA here reads this GPU's own memory only
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || pa.device != dev) return false;
  auto enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)NX, (cuuint64_t)NY};
  const cuuint64_t strides[1] = {(cuuint64_t)NX * elem};
  const cuuint32_t box[2] = {(cuuint32_t)bx, (cuuint32_t)by};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r =
      enc(map, elem == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(ptr),
          dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

unsigned* wait_timeout_word(bool may_alloc) {
  static std::mutex mu;
  static unsigned* words[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!words[dev] && may_alloc) {
    unsigned* p = nullptr;
    if (cudaMalloc(&p, sizeof(unsigned)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, sizeof(unsigned)) != cudaSuccess) {
      cudaFree(p);
      return nullptr;
    }
    words[dev] = p;
  }
  return words[dev];
}

int launch_dss_fixup(const Grid& g, void* out, unsigned mode, int precision, const int* skip, int TX,
                     int TY, cudaStream_t s, long long key_lo, long long key_hi, const unsigned* gate,
                     unsigned gate_tag) {
  if (!(mode & M_GS)) return SEM_OK;
  if (g.NX >= (1LL << 31) || g.NY >= (1LL << 31))
    return set_error(SEM_ERR_UNSUPPORTED, "local dimensions must be below 2^31");
  FixArgs f;
  f.n = g.n;
  f.Ex = g.Ex;
  f.Ey = g.Ey;
  f.TX = TX;
  f.TY = TY;
  f.NX = g.NX;
  f.NY = g.NY;
  f.mode = mode;
  f.skip = skip;
  f.key_lo = key_lo;
  f.key_hi = key_hi;
  f.gate = gate;
  f.gate_tag = gate_tag;
  const bool perx = (mode & M_PERX) != 0, pery = (mode & M_PERY) != 0;
  f.nxi = (g.Ex - 1) / f.TX + (perx ? 1 : 0);
  f.nyi = (g.Ey - 1) / f.TY + (pery ? 1 : 0);
  const long long nI = f.nxi + f.nyi + (f.nxi * f.nyi > 0 ? 1 : 0);
  if (nI == 0) return SEM_OK;
  const int threads = 256;
  long long along = std::max(std::max(f.NX, f.NY), f.nxi * f.nyi);
  long long bx = (along + threads - 1) / threads;
  if (bx > 64) bx = 64;
  long long by = std::min(nI, 65535LL);
  if (gate) {  // a gated re-run: a small grid (it exits at once unless the guard fired)
    bx = std::min(bx, 4LL);
    by = std::min(by, std::max(1LL, 2LL * num_sms() / bx));
  }
  // a programmatic dependent of the operator kernel before it on the stream:
  // its CTAs are scheduled once every operator CTA has started, and wait
  // (griddepcontrol.wait) for the operator grid's completion
  cudaLaunchConfig_t cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)bx, (unsigned)by);
  cfg.blockDim = dim3(threads);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (precision == SEM_F32)
    SEM_CUDA(cudaLaunchKernelEx(&cfg, k_dss_fixup<float>, static_cast<float*>(out), f));
  else
    SEM_CUDA(cudaLaunchKernelEx(&cfg, k_dss_fixup<double>, static_cast<double*>(out), f));
  return SEM_OK;
}

// A double-float call whose scalar coefficients lie outside the pair format's
// window runs in native FP64 (tiles with out-of-window field values are
// recomputed in FP64 inside the kernels).
static ApplyCall scalar_window(const ApplyCall& c) {
  ApplyCall r = c;
  if (c.precision == SEM_F64_DF && !(df_window_ok(c.nu_s) && df_window_ok(c.k_s))) r.precision = SEM_F64;
  return r;
}

// The native FP64 re-run of a guarded double-float call: the persistent
// kernel (variant 4, one CTA per resident slot) and its fixup on a small grid,
// launched after the double-float kernels and gated on the call's flag word
// (every CTA returns at once unless the word holds the call's tag), so that an
// unflagged call pays two short launches.
static int launch_gated_f64(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s,
                            long long key_lo, long long key_hi) {
  ApplyCall r = c;
  r.precision = SEM_F64;
  r.variant = 4;
  r.ctr = nullptr;
  r.rflag = nullptr;
  r.gate = c.rflag;
  r.gate_tag = c.rtag;
  r.cg_dpart = nullptr;
  r.cg_p = nullptr;
  r.pdl = 1;
  int tile[2] = {0, 0};
  SEM_CHECK(g.n >= 10 ? launch_apply_f64_hi(g, ops, r, s, tile) : launch_apply_f64_lo(g, ops, r, s, tile));
  if (tile[0] == 0) return SEM_OK;
  return launch_dss_fixup(g, r.out, r.mode, SEM_F64, r.skip, tile[0], tile[1], s, key_lo, key_hi, c.rflag, c.rtag);
}

int launch_apply(const Grid& g, const OperatorSet* ops, const ApplyCall& c0, cudaStream_t s) {
  ApplyCall c = scalar_window(c0);
  if (c.precision != SEM_F64_DF) c.rflag = nullptr;
  int st;
  int tile[2] = {0, 0};
  const bool hi = g.n >= 10;
  if (c.precision == SEM_F64)
    st = hi ? launch_apply_f64_hi(g, ops, c, s, tile) : launch_apply_f64_lo(g, ops, c, s, tile);
  else if (c.precision == SEM_F64_DF)
    st = hi ? launch_apply_df_hi(g, ops, c, s, tile) : launch_apply_df_lo(g, ops, c, s, tile);
  else if (c.precision == SEM_F32)
    st = hi ? launch_apply_f32_hi(g, ops, c, s, tile) : launch_apply_f32_lo(g, ops, c, s, tile);
  else
    return set_error(SEM_ERR_BAD_ARG, "unknown precision %d", c.precision);
  if (st != SEM_OK) return st;
  if (tile[0] != 0)  // otherwise completed inside the kernel
    SEM_CHECK(launch_dss_fixup(g, c.out, c.mode, c.precision, c.skip, tile[0], tile[1], s));
  if (c.rflag) SEM_CHECK(launch_gated_f64(g, ops, c, s, 0, 1LL << 62));
  return SEM_OK;
}

int launch_apply_window(const Grid& g, const OperatorSet* ops, const ApplyCall& c0, long long key_lo,
                        long long key_hi, cudaStream_t s) {
  ApplyCall c = scalar_window(c0);
  if (c.precision != SEM_F64_DF) c.rflag = nullptr;
  if (c.tyn <= 0) return set_error(SEM_ERR_BAD_ARG, "empty tile-row window");
  int st;
  int tile[2] = {0, 0};
  const bool hi = g.n >= 10;
  if (c.precision == SEM_F64)
    st = hi ? launch_apply_f64_hi(g, ops, c, s, tile) : launch_apply_f64_lo(g, ops, c, s, tile);
  else if (c.precision == SEM_F64_DF)
    st = hi ? launch_apply_df_hi(g, ops, c, s, tile) : launch_apply_df_lo(g, ops, c, s, tile);
  else
    return set_error(SEM_ERR_BAD_ARG, "tile-row windows serve SEM_F64 and SEM_F64_DF");
  if (st != SEM_OK) return st;
  SEM_CHECK(launch_dss_fixup(g, c.out, c.mode, c.precision, c.skip, tile[0], tile[1], s, key_lo, key_hi));
  // the range guard's re-run covers the whole field once every window is
  // done (launch_guard_rerun): a window's fixup has already summed the
  // interface copies of the window before it
  return SEM_OK;
}

int launch_guard_rerun(const Grid& g, const OperatorSet* ops, const ApplyCall& c0, cudaStream_t s) {
  ApplyCall c = scalar_window(c0);
  if (c.precision != SEM_F64_DF || !c.rflag) return SEM_OK;
  c.ty0 = 0;
  c.tyn = 0;
  return launch_gated_f64(g, ops, c, s, 0, 1LL << 62);
}

// the device's own guard word, for calls without a mesh handle (one per
// device, made on first use)
static unsigned* device_guard_word() {
  static std::mutex mu;
  static unsigned* words[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!words[dev]) {
    unsigned* p = nullptr;
    if (cudaMalloc(&p, sizeof(unsigned)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, sizeof(unsigned)) != cudaSuccess) {
      cudaFree(p);
      return nullptr;
    }
    words[dev] = p;
  }
  return words[dev];
}

int arm_range_guard(sem_mesh* m, ApplyCall& c) {
  if (c.precision != SEM_F64_DF) return SEM_OK;
  static std::atomic<unsigned> dev_tag{0};
  if (m) {
    if (!m->rflag) {
      SEM_CUDA(cudaMalloc(&m->rflag, sizeof(unsigned)));
      SEM_CUDA(cudaMemset(m->rflag, 0, sizeof(unsigned)));
    }
    if (++m->rtag == 0) ++m->rtag;  // tags are never 0 (the word's initial value)
    c.rflag = m->rflag;
    c.rtag = m->rtag;
    return SEM_OK;
  }
  unsigned* w = device_guard_word();
  if (!w) return set_error(SEM_ERR_CUDA, "cannot make the range-guard word");
  unsigned t = ++dev_tag;
  if (t == 0) t = ++dev_tag;
  c.rflag = w;
  c.rtag = t;
  return SEM_OK;
}

void tile_shape_of(int n, int* tx, int* ty) { tile_shape(n, tx, ty); }

long long cg_apply_parts(const Grid& g) {
  int tx = 1, ty = 1;
  tile_shape(g.n, &tx, &ty);
  return (long long)((g.Ex + tx - 1) / tx) * ((g.Ey + ty - 1) / ty);
}

__global__ void k_scale_into(const double* __restrict__ B, double k, double* __restrict__ out, long long L) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < L; i += (long long)gridDim.x * blockDim.x)
    out[i] = __dmul_rn(k, B[i]);
}

int use_kB(sem_mesh* m, ApplyCall& c, cudaStream_t s) {
  if (c.precision != SEM_F64 || !(c.mode & M_MASS) || c.B != m->B || c.k_s == 1.0) return SEM_OK;
  const long long L = m->g.NX * m->g.NY;
  if (!m->kB) {
    SEM_CUDA(cudaMalloc(&m->kB, sizeof(double) * (size_t)L));
    m->kB_k = std::nan("");  // not yet made
  }
  if (!(m->kB_k == c.k_s)) {
    long long blocks = (L + 255) / 256;
    if (blocks > 152LL * 16) blocks = 152LL * 16;
    k_scale_into<<<(unsigned)blocks, 256, 0, s>>>(m->B, c.k_s, m->kB, L);
    SEM_CUDA(cudaGetLastError());
    m->kB_k = c.k_s;
  }
  c.B = m->kB;
  c.k_s = 1.0;
  c.mode |= M_KB;
  return SEM_OK;
}

int ensure_fix_counters(sem_mesh* m) {
  if (m->fix_ctr) return SEM_OK;
  int tx = 1, ty = 1;
  tile_shape(m->g.n, &tx, &ty);
  const long long tiles = (long long)((m->g.Ex + tx - 1) / tx) * ((m->g.Ey + ty - 1) / ty);
  unsigned* p = nullptr;
  SEM_CUDA(cudaMalloc(&p, sizeof(unsigned) * 3 * (size_t)tiles));
  const cudaError_t e = cudaMemset(p, 0, sizeof(unsigned) * 3 * (size_t)tiles);
  if (e != cudaSuccess) {
    cudaFree(p);
    return cuda_error(e, "cudaMemset(interface counters)");
  }
  m->fix_ctr = p;
  return SEM_OK;
}

}  // namespace sem

using sem::cuda_error;

extern "C" {

int sem_timing_enable(int on) {
  std::lock_guard<std::mutex> lk(sem::g_tmu);
  sem::g_timing = on != 0;
  return SEM_OK;
}

int sem_wait_timeouts(int reset, unsigned* count) {
  if (!count) return sem::set_error(SEM_ERR_BAD_ARG, "NULL count");
  unsigned* w = sem::wait_timeout_word(true);
  if (!w) return sem::set_error(SEM_ERR_CUDA, "cannot make the TMA timeout word");
  SEM_CUDA(cudaDeviceSynchronize());
  SEM_CUDA(cudaMemcpy(count, w, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (reset) SEM_CUDA(cudaMemset(w, 0, sizeof(unsigned)));
  return SEM_OK;
}

int sem_timing_read(double* total_ms, int* launches) {
  std::lock_guard<std::mutex> lk(sem::g_tmu);
  double tot = 0.0;
  for (size_t i = 0; i < sem::g_used; ++i) {
    float ms = 0.f;
    SEM_CUDA(cudaEventSynchronize(sem::g_pool[i].second));
    SEM_CUDA(cudaEventElapsedTime(&ms, sem::g_pool[i].first, sem::g_pool[i].second));
    tot += ms;
  }
  if (total_ms) *total_ms = tot;
  if (launches) *launches = (int)sem::g_used;
  sem::g_used = 0;
  return SEM_OK;
}

}  // extern "C"
