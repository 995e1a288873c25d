// Operators beside the fused hot path, composed from the tensor-product
// kernel (launch_abu) and pointwise kernels on the device:
//   * the dealiased (over-integrated) Laplacian, laplace(u,Jr,Js,Dr,Ds,G11,G12,G22)
//     (src/lapl.jl:83-103), with the metric terms on the fine quadrature grid;
//   * the functional mass with interpolation, J'(B .* (J u)) (src/mass.jl:32-50);
//   * grad and grad' (src/grad.jl:16-63);
//   * advection B .* (u.grad T), plain and dealiased (src/advect.jl:27-64).
// Each follows the reference's sequence of ABu calls and broadcasts; the
// broadcasts are separate multiplies and adds (no fused multiply-add), as
// Julia's @. evaluates them.  Temporaries are stream-ordered allocations.
#include <cstring>

#include "sem_internal.cuh"

namespace sem {
namespace {

constexpr int kThreadsX = 256;

unsigned grid_of(long long n) {
  long long b = (n + kThreadsX - 1) / kThreadsX;
  if (b < 1) b = 1;
  if (b > 152LL * 32) b = 152LL * 32;
  return (unsigned)b;
}

// o1 = A .* x + B .* y, o2 = C .* x + D .* y
__global__ void k_mix2(const double* __restrict__ A, const double* __restrict__ Bf,
                       const double* __restrict__ C, const double* __restrict__ D,
                       const double* __restrict__ x, const double* __restrict__ y,
                       double* __restrict__ o1, double* __restrict__ o2, long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x) {
    const double xi = x[i], yi = y[i];
    o1[i] = __dadd_rn(__dmul_rn(A[i], xi), __dmul_rn(Bf[i], yi));
    o2[i] = __dadd_rn(__dmul_rn(C[i], xi), __dmul_rn(D[i], yi));
  }
}

// o = a .* x (a NULL: o = x)
__global__ void k_mul(const double* __restrict__ a, const double* __restrict__ x, double* __restrict__ o,
                      long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x)
    o[i] = a ? __dmul_rn(a[i], x[i]) : x[i];
}

// o = x + y
__global__ void k_add(const double* __restrict__ x, const double* __restrict__ y, double* __restrict__ o,
                      long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x)
    o[i] = __dadd_rn(x[i], y[i]);
}

// o = (ux .* Tx + uy .* Ty) .* B
__global__ void k_advect_mix(const double* __restrict__ ux, const double* __restrict__ Tx,
                             const double* __restrict__ uy, const double* __restrict__ Ty,
                             const double* __restrict__ B, double* __restrict__ o, long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x)
    o[i] = __dmul_rn(__dadd_rn(__dmul_rn(ux[i], Tx[i]), __dmul_rn(uy[i], Ty[i])), B[i]);
}

// transpose of a column-major r x c host matrix
void transpose(const double* A, int r, int c, double* At) {
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < c; ++j) At[j + i * c] = A[i + j * r];
}

// stream-ordered scratch fields, released on the stream when the set dies
struct Scratch {
  cudaStream_t s;
  double* p[8] = {nullptr};
  int n = 0;
  explicit Scratch(cudaStream_t st) : s(st) {}
  int get(long long len, double** out) {
    SEM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p[n]), sizeof(double) * (size_t)len, s));
    *out = p[n++];
    return SEM_OK;
  }
  ~Scratch() {
    for (int i = 0; i < n; ++i) cudaFreeAsync(p[i], s);
  }
};

int check_block(const double* A, int r, int c, const char* name) {
  if (!A) return set_error(SEM_ERR_BAD_ARG, "NULL %s", name);
  if (r < 1 || c < 1 || r > kMaxBlock || c > kMaxBlock)
    return set_error(SEM_ERR_UNSUPPORTED, "%s must be at most %dx%d (got %dx%d)", name, kMaxBlock, kMaxBlock, r, c);
  return SEM_OK;
}

}  // namespace
}  // namespace sem

using namespace sem;

extern "C" {

int sem_laplace_dealiased(int n, int mr, int ms, int Ex, int Ey, const double* Jr, const double* Js,
                          const double* Dr, const double* Ds, const double* G11, const double* G12,
                          const double* G22, const double* u, double* out, sem_stream_t stream) {
  if (!G11 || !G12 || !G22 || !u || !out) return set_error(SEM_ERR_BAD_ARG, "NULL field");
  if (Ex < 1 || Ey < 1) return set_error(SEM_ERR_BAD_ARG, "Ex and Ey must be positive");
  if (u == out) return set_error(SEM_ERR_BAD_ARG, "output must not alias the input");
  SEM_CHECK(check_block(Dr, n, n, "Dr"));
  SEM_CHECK(check_block(Ds, n, n, "Ds"));
  SEM_CHECK(check_block(Jr, mr, n, "Jr"));
  SEM_CHECK(check_block(Js, ms, n, "Js"));
  cudaStream_t s = (cudaStream_t)stream;
  const int NX = n * Ex, NY = n * Ey, MX = mr * Ex, MY = ms * Ey;
  const long long Lc = (long long)NX * NY, Lf = (long long)MX * MY;
  double Drt[kMaxBlock * kMaxBlock], Dst[kMaxBlock * kMaxBlock], Jrt[kMaxBlock * kMaxBlock],
      Jst[kMaxBlock * kMaxBlock];
  transpose(Dr, n, n, Drt);
  transpose(Ds, n, n, Dst);
  transpose(Jr, mr, n, Jrt);
  transpose(Js, ms, n, Jst);
  Scratch t(s);
  double *ur, *us, *Jur, *Jus, *vr, *vs, *wr, *ws;
  SEM_CHECK(t.get(Lc, &ur));
  SEM_CHECK(t.get(Lc, &us));
  SEM_CHECK(t.get(Lf, &Jur));
  SEM_CHECK(t.get(Lf, &Jus));
  SEM_CHECK(t.get(Lf, &vr));
  SEM_CHECK(t.get(Lf, &vs));
  SEM_CHECK(t.get(Lc, &wr));
  SEM_CHECK(t.get(Lc, &ws));
  // ur = ABu([],Dr,u), us = ABu(Ds,[],u)
  SEM_CHECK(launch_abu(nullptr, 0, 0, Dr, n, n, u, NX, NY, ur, s));
  SEM_CHECK(launch_abu(Ds, n, n, nullptr, 0, 0, u, NX, NY, us, s));
  // Jur = ABu(Js,Jr,ur), Jus = ABu(Js,Jr,us)
  SEM_CHECK(launch_abu(Js, ms, n, Jr, mr, n, ur, NX, NY, Jur, s));
  SEM_CHECK(launch_abu(Js, ms, n, Jr, mr, n, us, NX, NY, Jus, s));
  // vr = G11 Jur + G12 Jus, vs = G12 Jur + G22 Jus (fine grid)
  k_mix2<<<grid_of(Lf), kThreadsX, 0, s>>>(G11, G12, G12, G22, Jur, Jus, vr, vs, Lf);
  SEM_CUDA(cudaGetLastError());
  // wr = ABu(Js',Jr',vr), ws = ABu(Js',Jr',vs)
  SEM_CHECK(launch_abu(Jst, n, ms, Jrt, n, mr, vr, MX, MY, wr, s));
  SEM_CHECK(launch_abu(Jst, n, ms, Jrt, n, mr, vs, MX, MY, ws, s));
  // Au = ABu([],Dr',wr) + ABu(Ds',[],ws)
  SEM_CHECK(launch_abu(nullptr, 0, 0, Drt, n, n, wr, NX, NY, ur, s));
  SEM_CHECK(launch_abu(Dst, n, n, nullptr, 0, 0, ws, NX, NY, us, s));
  k_add<<<grid_of(Lc), kThreadsX, 0, s>>>(ur, us, out, Lc);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int sem_mass_dealiased(int n, int mr, int ms, int Ex, int Ey, const double* Jr, const double* Js,
                       const double* B, const double* u, double* out, sem_stream_t stream) {
  if (!u || !out) return set_error(SEM_ERR_BAD_ARG, "NULL field");
  if (Ex < 1 || Ey < 1) return set_error(SEM_ERR_BAD_ARG, "Ex and Ey must be positive");
  if (u == out) return set_error(SEM_ERR_BAD_ARG, "output must not alias the input");
  SEM_CHECK(check_block(Jr, mr, n, "Jr"));
  SEM_CHECK(check_block(Js, ms, n, "Js"));
  cudaStream_t s = (cudaStream_t)stream;
  const int NX = n * Ex, NY = n * Ey, MX = mr * Ex, MY = ms * Ey;
  const long long Lf = (long long)MX * MY;
  double Jrt[kMaxBlock * kMaxBlock], Jst[kMaxBlock * kMaxBlock];
  transpose(Jr, mr, n, Jrt);
  transpose(Js, ms, n, Jst);
  Scratch t(s);
  double *Ju, *BJu;
  SEM_CHECK(t.get(Lf, &Ju));
  SEM_CHECK(t.get(Lf, &BJu));
  // Ju = ABu(Js,Jr,u); BJu = B .* Ju (B = []: Ju); Bu = ABu(Js',Jr',BJu)
  SEM_CHECK(launch_abu(Js, ms, n, Jr, mr, n, u, NX, NY, Ju, s));
  k_mul<<<grid_of(Lf), kThreadsX, 0, s>>>(B, Ju, BJu, Lf);
  SEM_CUDA(cudaGetLastError());
  SEM_CHECK(launch_abu(Jst, n, ms, Jrt, n, mr, BJu, MX, MY, out, s));
  return SEM_OK;
}

int sem_grad(sem_mesh_t* m, const double* u, double* ux, double* uy, sem_stream_t stream) {
  if (!m || !u || !ux || !uy) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (u == ux || u == uy || ux == uy) return set_error(SEM_ERR_BAD_ARG, "outputs must not alias");
  cudaStream_t s = (cudaStream_t)stream;
  const int n = m->g.n;
  const int NX = (int)m->g.NX, NY = (int)m->g.NY;
  const long long L = (long long)NX * NY;
  Scratch t(s);
  double *ur, *us, *rx, *ry, *sx, *sy;
  SEM_CHECK(t.get(L, &ur));
  SEM_CHECK(t.get(L, &us));
  SEM_CHECK(t.get(L, &rx));
  SEM_CHECK(t.get(L, &ry));
  SEM_CHECK(t.get(L, &sx));
  SEM_CHECK(t.get(L, &sy));
  SEM_CHECK(export_field(m, SEM_FIELD_RX, rx, s));
  SEM_CHECK(export_field(m, SEM_FIELD_RY, ry, s));
  SEM_CHECK(export_field(m, SEM_FIELD_SX, sx, s));
  SEM_CHECK(export_field(m, SEM_FIELD_SY, sy, s));
  // ur = ABu([],Dr,u), us = ABu(Ds,[],u); ux = rx ur + sx us, uy = ry ur + sy us
  SEM_CHECK(launch_abu(nullptr, 0, 0, m->Dr_h, n, n, u, NX, NY, ur, s));
  SEM_CHECK(launch_abu(m->Ds_h, n, n, nullptr, 0, 0, u, NX, NY, us, s));
  k_mix2<<<grid_of(L), kThreadsX, 0, s>>>(rx, sx, ry, sy, ur, us, ux, uy, L);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int sem_grad_t(sem_mesh_t* m, const double* u, double* ux, double* uy, sem_stream_t stream) {
  if (!m || !u || !ux || !uy) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (u == ux || u == uy || ux == uy) return set_error(SEM_ERR_BAD_ARG, "outputs must not alias");
  cudaStream_t s = (cudaStream_t)stream;
  const int n = m->g.n;
  const int NX = (int)m->g.NX, NY = (int)m->g.NY;
  const long long L = (long long)NX * NY;
  double Drt[kMaxBlock * kMaxBlock], Dst[kMaxBlock * kMaxBlock];
  transpose(m->Dr_h, n, n, Drt);
  transpose(m->Ds_h, n, n, Dst);
  Scratch t(s);
  double *g, *a, *b;
  SEM_CHECK(t.get(L, &g));
  SEM_CHECK(t.get(L, &a));
  SEM_CHECK(t.get(L, &b));
  // ux = ABu(Dr',[],rx.*u) + ABu([],Ds',sx.*u); uy likewise with ry, sy
  // (src/grad.jl:55-61: As = Dr', Br = Ds', as written there)
  const int fields[2][2] = {{SEM_FIELD_RX, SEM_FIELD_SX}, {SEM_FIELD_RY, SEM_FIELD_SY}};
  double* outs[2] = {ux, uy};
  for (int q = 0; q < 2; ++q) {
    SEM_CHECK(export_field(m, fields[q][0], g, s));
    k_mul<<<grid_of(L), kThreadsX, 0, s>>>(g, u, b, L);
    SEM_CUDA(cudaGetLastError());
    SEM_CHECK(launch_abu(Drt, n, n, nullptr, 0, 0, b, NX, NY, a, s));
    SEM_CHECK(export_field(m, fields[q][1], g, s));
    k_mul<<<grid_of(L), kThreadsX, 0, s>>>(g, u, b, L);
    SEM_CUDA(cudaGetLastError());
    SEM_CHECK(launch_abu(nullptr, 0, 0, Dst, n, n, b, NX, NY, g, s));
    k_add<<<grid_of(L), kThreadsX, 0, s>>>(a, g, outs[q], L);
    SEM_CUDA(cudaGetLastError());
  }
  return SEM_OK;
}

int sem_advect(sem_mesh_t* m, const double* T, const double* ux, const double* uy, double* out,
               sem_stream_t stream) {
  if (!m || !T || !ux || !uy || !out) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  const long long L = m->g.NX * m->g.NY;
  Scratch t(s);
  double *Tx, *Ty;
  SEM_CHECK(t.get(L, &Tx));
  SEM_CHECK(t.get(L, &Ty));
  SEM_CHECK(sem_grad(m, T, Tx, Ty, stream));
  k_advect_mix<<<grid_of(L), kThreadsX, 0, s>>>(ux, Tx, uy, Ty, m->B, out, L);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int sem_advect_dealiased(sem_mesh_t* m, int mr, int ms, const double* Jr, const double* Js,
                         const double* Bd, const double* T, const double* ux, const double* uy,
                         double* out, sem_stream_t stream) {
  if (!m || !Bd || !T || !ux || !uy || !out) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  const int n = m->g.n;
  SEM_CHECK(check_block(Jr, mr, n, "Jr"));
  SEM_CHECK(check_block(Js, ms, n, "Js"));
  cudaStream_t s = (cudaStream_t)stream;
  const int NX = (int)m->g.NX, NY = (int)m->g.NY, MX = mr * m->g.Ex, MY = ms * m->g.Ey;
  const long long L = (long long)NX * NY, Lf = (long long)MX * MY;
  double Jrt[kMaxBlock * kMaxBlock], Jst[kMaxBlock * kMaxBlock];
  transpose(Jr, mr, n, Jrt);
  transpose(Js, ms, n, Jst);
  Scratch t(s);
  double *Tx, *Ty, *JTx, *JTy, *Jux, *Juy, *JCu;
  SEM_CHECK(t.get(L, &Tx));
  SEM_CHECK(t.get(L, &Ty));
  SEM_CHECK(t.get(Lf, &JTx));
  SEM_CHECK(t.get(Lf, &JTy));
  SEM_CHECK(t.get(Lf, &Jux));
  SEM_CHECK(t.get(Lf, &Juy));
  SEM_CHECK(t.get(Lf, &JCu));
  SEM_CHECK(sem_grad(m, T, Tx, Ty, stream));
  // JTx = ABu(Js,Jr,Tx), JTy, Jux, Juy likewise
  SEM_CHECK(launch_abu(Js, ms, n, Jr, mr, n, Tx, NX, NY, JTx, s));
  SEM_CHECK(launch_abu(Js, ms, n, Jr, mr, n, Ty, NX, NY, JTy, s));
  SEM_CHECK(launch_abu(Js, ms, n, Jr, mr, n, ux, NX, NY, Jux, s));
  SEM_CHECK(launch_abu(Js, ms, n, Jr, mr, n, uy, NX, NY, Juy, s));
  // JCu = (Jux JTx + Juy JTy) .* Bd; Cu = ABu(Js',Jr',JCu)
  k_advect_mix<<<grid_of(Lf), kThreadsX, 0, s>>>(Jux, JTx, Juy, JTy, Bd, JCu, Lf);
  SEM_CUDA(cudaGetLastError());
  SEM_CHECK(launch_abu(Jst, n, ms, Jrt, n, mr, JCu, MX, MY, out, s));
  return SEM_OK;
}

}  // extern "C"
