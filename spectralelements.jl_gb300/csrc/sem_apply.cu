// Host side of the fused operator kernels: coefficient sets and launches.
#include <cmath>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "sem_apply_kernels.cuh"

namespace sem {

// ---- event timing of the fused kernel launches (instrumentation)
namespace {
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
}  // namespace

struct OperatorSet {
  int n;
  // even-odd coefficients in double for Dr, Dr', Ds, Ds' (index 0..3); each
  // block holds A (m*m), C (m*m), cm (m), mr (m)
  std::vector<double> eo[4];
  std::vector<double> Dr, Ds;  // dense, column-major
};

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

int make_operator_set(const double* Dr, const double* Ds, int n, OperatorSet** out) {
  if (n < 2 || n > kMaxN) return set_error(SEM_ERR_UNSUPPORTED, "fused operators serve 2 <= n <= %d GLL points, got %d", kMaxN, n);
  if (!is_centro_antisymmetric(Dr, n, 1e-12) || !is_centro_antisymmetric(Ds, n, 1e-12))
    return set_error(SEM_ERR_UNSUPPORTED,
                     "derivative matrices must be centro-antisymmetric (GLL derivative "
                     "matrices are); a general matrix is served by sem_abu");
  OperatorSet* o = new OperatorSet;
  o->n = n;
  o->Dr.assign(Dr, Dr + n * n);
  o->Ds.assign(Ds, Ds + n * n);
  const int m = n / 2;
  for (int b = 0; b < 4; ++b) {
    o->eo[b].assign(2 * m * m + 2 * m, 0.0);
    const double* D = b < 2 ? Dr : Ds;
    double* p = o->eo[b].data();
    eo_from_dense(D, n, (b & 1) != 0, p, p + m * m, p + 2 * m * m, p + 2 * m * m + m);
  }
  *out = o;
  return SEM_OK;
}

void free_operator_set(OperatorSet* o) { delete o; }

template <class P, int N>
static void fill_eo(EOCoef<N, typename P::v>& c, const std::vector<double>& src) {
  constexpr int M = N / 2;
  const double* A = src.data();
  const double* C = A + M * M;
  const double* cm = C + M * M;
  const double* mr = cm + M;
  for (int i = 0; i < M; ++i)
    for (int k = 0; k < M; ++k) {
      c.A[i][k] = P::from_double(A[i * M + k]);
      c.Cc[i][k] = P::from_double(C[i * M + k]);
    }
  for (int i = 0; i < M; ++i) {
    c.cm[i] = P::from_double(cm[i]);
    c.mr[i] = P::from_double(mr[i]);
  }
}

template <class P, int N>
static int launch_apply_n(const Grid& g, const OperatorSet* ops, const ApplyCall& c,
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
  a.nu_s = P::from_double(c.nu_s);
  a.k_s = P::from_double(c.k_s);
  a.Ex = g.Ex;
  a.Ey = g.Ey;
  a.NX = g.NX;
  a.mode = c.mode;
  a.skip = c.skip;
  fill_eo<P, N>(a.Dr, ops->eo[0]);
  fill_eo<P, N>(a.Drt, ops->eo[1]);
  fill_eo<P, N>(a.Ds, ops->eo[2]);
  fill_eo<P, N>(a.Dst, ops->eo[3]);
  const size_t smem = 2ull * TS::TX * TS::TY * TS::ES * sizeof(typename P::v);
  auto kern = k_apply<P, N, TS::TX, TS::TY>;
  if (smem > 48 * 1024) SEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((g.Ex + TS::TX - 1) / TS::TX, (g.Ey + TS::TY - 1) / TS::TY);
  auto* ev = timing_slot();
  if (ev) SEM_CUDA(cudaEventRecord(ev->first, s));
  kern<<<grid, TS::THREADS, smem, s>>>(a);
  SEM_CUDA(cudaGetLastError());
  if (ev) SEM_CUDA(cudaEventRecord(ev->second, s));
  return SEM_OK;
}

template <class P>
static int launch_apply_p(const Grid& g, const OperatorSet* ops, const ApplyCall& c,
                          cudaStream_t s) {
  switch (g.n) {
#define SEM_CASE(NN) \
  case NN:           \
    return launch_apply_n<P, NN>(g, ops, c, s);
    SEM_CASE(2) SEM_CASE(3) SEM_CASE(4) SEM_CASE(5) SEM_CASE(6) SEM_CASE(7) SEM_CASE(8)
    SEM_CASE(9) SEM_CASE(10) SEM_CASE(11) SEM_CASE(12) SEM_CASE(13) SEM_CASE(14)
    SEM_CASE(15) SEM_CASE(16) SEM_CASE(17)
#undef SEM_CASE
    default:
      return set_error(SEM_ERR_UNSUPPORTED, "no fused kernel for n = %d", g.n);
  }
}

// tile shape of the fused kernel for a given n (host mirror of TileShape)
static void tile_of(int n, int* TX, int* TY) {
  *TX = 8;
  *TY = n <= 4 ? 8 : (n <= 8 ? 4 : (n <= 12 ? 3 : 2));
}

int launch_dss_fixup(const Grid& g, const OperatorSet* ops, void* out, unsigned mode,
                     int precision, const int* skip, cudaStream_t s) {
  (void)ops;
  if (!(mode & M_GS)) return SEM_OK;
  FixArgs f;
  f.n = g.n;
  f.Ex = g.Ex;
  f.Ey = g.Ey;
  tile_of(g.n, &f.TX, &f.TY);
  f.NX = g.NX;
  f.NY = g.NY;
  f.mode = mode;
  f.skip = skip;
  const bool perx = (mode & M_PERX) != 0, pery = (mode & M_PERY) != 0;
  f.nxi = (g.Ex - 1) / f.TX + (perx ? 1 : 0);
  f.nyi = (g.Ey - 1) / f.TY + (pery ? 1 : 0);
  const long long total = f.nxi * f.NY + f.nyi * f.NX + f.nxi * f.nyi;
  if (total == 0) return SEM_OK;
  const int threads = 256;
  long long blocks = (total + threads - 1) / threads;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (precision == SEM_F32)
    k_dss_fixup<float><<<(unsigned)blocks, threads, 0, s>>>(static_cast<float*>(out), f);
  else
    k_dss_fixup<double><<<(unsigned)blocks, threads, 0, s>>>(static_cast<double*>(out), f);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int launch_apply(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s) {
  int st;
  if (c.precision == SEM_F64)
    st = launch_apply_p<PF64>(g, ops, c, s);
  else if (c.precision == SEM_F64_DF)
    st = launch_apply_p<PDF>(g, ops, c, s);
  else if (c.precision == SEM_F32)
    st = launch_apply_p<PF32>(g, ops, c, s);
  else
    return set_error(SEM_ERR_BAD_ARG, "unknown precision %d", c.precision);
  if (st != SEM_OK) return st;
  return launch_dss_fixup(g, ops, c.out, c.mode, c.precision, c.skip, s);
}

}  // namespace sem

using sem::cuda_error;

extern "C" {

int sem_timing_enable(int on) {
  std::lock_guard<std::mutex> lk(sem::g_tmu);
  sem::g_timing = on != 0;
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
