// Single-domain spectral operator algebra on the device
// (src/Spectral/Operators.jl, src/Spectral/OperatorBasics.jl): the matrix,
// diagonal and tensor-product operators of the Spectral module applied to
// batches of fields.
//
// Every tensor-product apply is a sequence of mode products: along one
// dimension d of a column-major array of shape (inner, n, outer),
//   V[a, i, b] = sum_k M[i, k] U[a, k, b],
// which is one GEMM of M (m x n) with the n x (inner*outer) matrix of the
// fibres.  The kernel tiles it in shared memory (32 rows of M, 64 fibres,
// chunks of 16 along k) with FP64 fused multiply-adds in increasing k.
#include <cstring>

#include "sem_internal.cuh"

namespace sem {
namespace {

constexpr int kTM = 32, kTF = 64, kTK = 16;
constexpr int kModeThreads = 256;  // each thread: 2 rows x 4 fibres

__global__ void __launch_bounds__(kModeThreads) k_mode_product(const double* __restrict__ M, int m, int n,
                                                               const double* __restrict__ U,
                                                               double* __restrict__ V, long long inner,
                                                               long long nfib) {
  __shared__ double sM[kTK][kTM + 1];
  __shared__ double sU[kTK][kTF + 1];
  const int tid = threadIdx.x;
  const int ti = tid / 16, tf = tid % 16;  // rows ti, ti+16; fibres tf + 16 q
  const long long f0 = (long long)blockIdx.x * kTF;
  const int i0 = blockIdx.y * kTM;
  double acc[2][4] = {{0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}};
  for (int k0 = 0; k0 < n; k0 += kTK) {
    // M tile: rows i0..i0+31 (contiguous), columns k0..k0+15
    for (int e = tid; e < kTM * kTK; e += kModeThreads) {
      const int r = e % kTM, c = e / kTM;
      const int i = i0 + r, k = k0 + c;
      sM[c][r] = (i < m && k < n) ? M[i + (long long)k * m] : 0.0;
    }
    // U tile: fibres f0..f0+63, k0..k0+15; contiguous along k when inner == 1
    if (inner == 1) {
      for (int e = tid; e < kTK * kTF; e += kModeThreads) {
        const int c = e % kTK, q = e / kTK;
        const long long f = f0 + q;
        const int k = k0 + c;
        sU[c][q] = (f < nfib && k < n) ? U[k + f * n] : 0.0;
      }
    } else {
      for (int e = tid; e < kTK * kTF; e += kModeThreads) {
        const int q = e % kTF, c = e / kTF;
        const long long f = f0 + q;
        const int k = k0 + c;
        double v = 0.0;
        if (f < nfib && k < n) {
          const long long a = f % inner, b = f / inner;
          v = U[a + (long long)k * inner + b * inner * n];
        }
        sU[c][q] = v;
      }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < kTK; ++c) {
      const double m0 = sM[c][ti], m1 = sM[c][ti + 16];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double u = sU[c][tf + 16 * q];
        acc[0][q] = fma(m0, u, acc[0][q]);
        acc[1][q] = fma(m1, u, acc[1][q]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = i0 + ti + 16 * h;
    if (i >= m) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long f = f0 + tf + 16 * q;
      if (f >= nfib) continue;
      const long long a = f % inner, b = f / inner;
      V[a + (long long)i * inner + b * inner * m] = acc[h][q];
    }
  }
}

__global__ void k_axpby(double alpha, const double* __restrict__ x, double beta, const double* __restrict__ y,
                        double* __restrict__ out, long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x) {
    const double a = x ? alpha * x[i] : 0.0;
    out[i] = y ? fma(beta, y[i], a) : a;
  }
}

__global__ void k_diag(const double* __restrict__ d, const double* __restrict__ u, double* __restrict__ v,
                       long long len, int invert) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x)
    v[i] = invert ? u[i] / d[i] : d[i] * u[i];
}

unsigned grid_1d(long long len) {
  long long b = (len + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152LL * 32) b = 152LL * 32;
  return (unsigned)b;
}

int mode_product(const double* M, int m, int n, const double* U, double* V, long long inner, long long outer,
                 cudaStream_t s) {
  const long long nfib = inner * outer;
  if (nfib == 0 || m == 0) return SEM_OK;
  const long long gx = (nfib + kTF - 1) / kTF;
  const int gy = (m + kTM - 1) / kTM;
  if (gx > 2147483647LL || gy > 65535) return set_error(SEM_ERR_UNSUPPORTED, "mode product too large");
  k_mode_product<<<dim3((unsigned)gx, (unsigned)gy), kModeThreads, 0, s>>>(M, m, n, U, V, inner, nfib);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int check_dims(std::initializer_list<int> d) {
  for (int v : d)
    if (v < 1) return set_error(SEM_ERR_BAD_ARG, "dimensions must be positive");
  return SEM_OK;
}

}  // namespace
}  // namespace sem

using namespace sem;

extern "C" {

int sem_mode_product(const double* M, int m, int n, const double* U, double* V, int64_t inner,
                     int64_t outer, sem_stream_t stream) {
  if (!M || !U || !V) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (U == V) return set_error(SEM_ERR_BAD_ARG, "V must not alias U");
  SEM_CHECK(check_dims({m, n}));
  if (inner < 1 || outer < 0) return set_error(SEM_ERR_BAD_ARG, "inner must be positive, outer >= 0");
  return mode_product(M, m, n, U, V, inner, outer, (cudaStream_t)stream);
}

int sem_tp2d(const double* A, int ma, int na, const double* B, int mb, int nb, const double* U, double* V,
             int batch, sem_stream_t stream) {
  if (!U || !V) return set_error(SEM_ERR_BAD_ARG, "NULL field");
  if (U == V) return set_error(SEM_ERR_BAD_ARG, "V must not alias U");
  if (!A) ma = na;
  if (!B) mb = nb;
  SEM_CHECK(check_dims({ma, na, mb, nb, batch}));
  cudaStream_t s = (cudaStream_t)stream;
  const long long lin = (long long)na * nb * batch, lmid = (long long)ma * nb * batch;
  if (!A && !B) {
    SEM_CUDA(cudaMemcpyAsync(V, U, sizeof(double) * lin, cudaMemcpyDeviceToDevice, s));
    return SEM_OK;
  }
  if (!B) return mode_product(A, ma, na, U, V, 1, (long long)nb * batch, s);
  if (!A) return mode_product(B, mb, nb, U, V, na, batch, s);
  double* tmp = nullptr;
  SEM_CUDA(cudaMallocAsync(&tmp, sizeof(double) * lmid, s));
  int st = mode_product(A, ma, na, U, tmp, 1, (long long)nb * batch, s);
  if (st == SEM_OK) st = mode_product(B, mb, nb, tmp, V, ma, batch, s);
  cudaFreeAsync(tmp, s);
  return st;
}

int sem_tp3d(const double* A, int ma, int na, const double* B, int mb, int nb, const double* C, int mc, int nc,
             const double* U, double* V, int batch, sem_stream_t stream) {
  if (!U || !V) return set_error(SEM_ERR_BAD_ARG, "NULL field");
  if (U == V) return set_error(SEM_ERR_BAD_ARG, "V must not alias U");
  if (!A) ma = na;
  if (!B) mb = nb;
  if (!C) mc = nc;
  SEM_CHECK(check_dims({ma, na, mb, nb, mc, nc, batch}));
  cudaStream_t s = (cudaStream_t)stream;
  const double* mats[3] = {A, B, C};
  const int ms[3] = {ma, mb, mc}, ns[3] = {na, nb, nc};
  int steps = 0;
  for (int d = 0; d < 3; ++d) steps += mats[d] ? 1 : 0;
  if (steps == 0) {
    SEM_CUDA(cudaMemcpyAsync(V, U, sizeof(double) * (long long)na * nb * nc * batch, cudaMemcpyDeviceToDevice, s));
    return SEM_OK;
  }
  // shape after each applied mode; intermediates in two scratch buffers
  long long cur[3] = {na, nb, nc};
  long long maxlen = 0;
  for (int d = 0; d < 3; ++d) {
    if (!mats[d]) continue;
    cur[d] = ms[d];
    const long long len = cur[0] * cur[1] * cur[2] * batch;
    if (len > maxlen) maxlen = len;
  }
  double* tmp[2] = {nullptr, nullptr};
  const int ntmp = steps > 2 ? 2 : steps - 1;
  for (int t = 0; t < ntmp; ++t) SEM_CUDA(cudaMallocAsync(&tmp[t], sizeof(double) * maxlen, s));
  long long shape[3] = {na, nb, nc};
  const double* src = U;
  int done = 0, st = SEM_OK;
  for (int d = 0; d < 3 && st == SEM_OK; ++d) {
    if (!mats[d]) continue;
    ++done;
    double* dst = done == steps ? V : tmp[(done - 1) % 2];
    long long inner = 1, outer = batch;
    for (int j = 0; j < d; ++j) inner *= shape[j];
    for (int j = d + 1; j < 3; ++j) outer *= shape[j];
    st = mode_product(mats[d], ms[d], ns[d], src, dst, inner, outer, s);
    shape[d] = ms[d];
    src = dst;
  }
  for (int t = 0; t < ntmp; ++t) cudaFreeAsync(tmp[t], s);
  return st;
}

int sem_axpby(double alpha, const double* x, double beta, const double* y, double* out, int64_t len,
              sem_stream_t stream) {
  if (!out) return set_error(SEM_ERR_BAD_ARG, "NULL output");
  if (len < 0) return set_error(SEM_ERR_BAD_ARG, "negative length");
  if (len == 0) return SEM_OK;
  k_axpby<<<grid_1d(len), 256, 0, (cudaStream_t)stream>>>(alpha, x, beta, y, out, len);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int sem_diag_apply(const double* d, const double* u, double* v, int64_t len, int invert, sem_stream_t stream) {
  if (!d || !u || !v) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (len < 0) return set_error(SEM_ERR_BAD_ARG, "negative length");
  if (len == 0) return SEM_OK;
  k_diag<<<grid_1d(len), 256, 0, (cudaStream_t)stream>>>(d, u, v, len, invert ? 1 : 0);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

}  // extern "C"
