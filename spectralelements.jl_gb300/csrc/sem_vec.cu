// Structured, memory-bound kernels: standalone QQ', masks, mass, mult and the
// generic tensor-product apply ABu.
#include <cstring>

#include "sem_internal.cuh"

namespace sem {

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(long long n, int threads = kThreads, long long cap = 152LL * 32) {
  long long b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

// QQ' u: x sums in increasing row order, then y sums in increasing column
// order, so every copy of a global node receives bit-identical values
// (src/gatherScatter.jl:8-16 applies QQtx then QQty).
__global__ void k_gather_scatter(const double* __restrict__ u, double* __restrict__ out, Grid g,
                                 unsigned mode) {
  const long long NX = g.NX;
  for_each_point(g, [&](unsigned r, unsigned c, long long idx) {
    const unsigned char rb = g.rinfo[r], cb = g.cinfo[c];
    const long long pr = line_partner(r, rb, g.NX);
    const long long pc = line_partner(c, cb, g.NY);
    const long long r0 = (pr >= 0 && pr < r) ? pr : r;
    const long long r1 = (pr >= 0 && pr < r) ? (long long)r : pr;
    auto xsum = [&](long long cc) {
      double s = u[r0 + cc * NX];
      if (r1 >= 0) s += u[r1 + cc * NX];
      return s;
    };
    double v;
    if (pc < 0) {
      v = xsum(c);
    } else {
      const long long c0 = pc < c ? pc : (long long)c, c1 = pc < c ? (long long)c : pc;
      v = xsum(c0) + xsum(c1);
    }
    if ((mode & M_MASK) && ((rb | cb) & L_ZERO)) v = v * 0.0;
    out[idx] = v;
  });
}

// QQ' u on a grid described by its sizes alone (no mesh handle): the
// functional gatherScatter(u,QQtx,QQty) (src/gatherScatter.jl:8-16), which
// may have nr != ns.  Same sums in the same order as k_gather_scatter.
struct GsGrid {
  long long NX, NY;
  int nr, ns, Ex, Ey;
  bool perx, pery;
};

__global__ void k_gather_scatter_grid(const double* __restrict__ u, double* __restrict__ out, GsGrid q) {
  const long long NX = q.NX, total = q.NX * q.NY;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long c = idx / NX, r = idx - c * NX;
    const long long pr = line_partner(r, line_info(r, q.nr, q.Ex, q.perx, false, false), q.NX);
    const long long pc = line_partner(c, line_info(c, q.ns, q.Ey, q.pery, false, false), q.NY);
    const long long r0 = (pr >= 0 && pr < r) ? pr : r;
    const long long r1 = (pr >= 0 && pr < r) ? r : pr;
    auto xsum = [&](long long cc) {
      double s = u[r0 + cc * NX];
      if (r1 >= 0) s += u[r1 + cc * NX];
      return s;
    };
    double v;
    if (pc < 0) {
      v = xsum(c);
    } else {
      const long long c0 = pc < c ? pc : c, c1 = pc < c ? c : pc;
      v = xsum(c0) + xsum(c1);
    }
    out[idx] = v;
  }
}

__global__ void k_mask_bc(const double* __restrict__ u, double* __restrict__ out, Grid g) {
  for_each_point(g, [&](unsigned r, unsigned c, long long idx) {
    const double v = u[idx];
    out[idx] = ((g.rinfo[r] | g.cinfo[c]) & L_ZERO) ? v * 0.0 : v;
  });
}

__global__ void k_mask_array(const double* __restrict__ M, const double* __restrict__ u,
                             double* __restrict__ out, long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = M ? M[i] * u[i] : u[i];
}

__global__ void k_mass(const double* __restrict__ B, const double* __restrict__ u,
                       double* __restrict__ out, long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = B[i] * u[i];
}

// mult = 1 ./ QQ'(ones) (src/mesh.jl:94-96): 1 / (copies_x * copies_y)
__global__ void k_mult(double* __restrict__ out, Grid g) {
  for_each_point(g, [&](unsigned r, unsigned c, long long idx) {
    const int cc = copies_at(g, r, c);
    out[idx] = cc == 1 ? 1.0 : (cc == 2 ? 0.5 : 0.25);
  });
}

// ---------------------------------------------------------------------------
// ABu (src/ABu.jl:9-37)
// ---------------------------------------------------------------------------
struct Mat32 {
  double a[kMaxBlock * kMaxBlock];  // row-major a[p*cols + k]
  int rows, cols;
};

// Br side: Br applied to consecutive chunks of nb entries of the column-major
// flattening of u (reshape(u, nb, :)), output reshaped back
__global__ void k_abu_br(const __grid_constant__ Mat32 Br, const double* __restrict__ u,
                         double* __restrict__ v, long long nchunks) {
  const int mb = Br.rows, nb = Br.cols;
  const long long total = nchunks * mb;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long ch = idx / mb;
    const int p = (int)(idx - ch * mb);
    const double* src = u + ch * nb;
    double s = 0.0;
    for (int k = 0; k < nb; ++k) s = fma(Br.a[p * nb + k], src[k], s);
    v[idx] = s;
  }
}

// As side: out[:, b*ma + q] = sum_l As[q,l] u[:, b*na + l]
__global__ void k_abu_as(const __grid_constant__ Mat32 As, const double* __restrict__ u,
                         double* __restrict__ v, long long m, long long nblk) {
  const int ma = As.rows, na = As.cols;
  const long long total = m * nblk * ma;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long col = idx / m;
    const long long r = idx - col * m;
    const long long b = col / ma;
    const int q = (int)(col - b * ma);
    const double* src = u + r + b * na * m;
    double s = 0.0;
    for (int l = 0; l < na; ++l) s = fma(As.a[q * na + l], src[(long long)l * m], s);
    v[idx] = s;
  }
}

// both sides, one output block (mb x ma) per block of u (nb x na), staged in
// shared memory: out_blk = Br * u_blk * As'
__global__ void k_abu_both(const __grid_constant__ Mat32 As, const __grid_constant__ Mat32 Br,
                           const double* __restrict__ u, double* __restrict__ v, long long m,
                           long long nbx, long long nby) {
  extern __shared__ double sh[];
  const int ma = As.rows, na = As.cols, mb = Br.rows, nb = Br.cols;
  double* ub = sh;            // nb x na
  double* tb = sh + nb * na;  // mb x na
  const long long mo = m / nb * mb;
  for (long long blk = blockIdx.x; blk < nbx * nby; blk += gridDim.x) {
    const long long by = blk / nbx, bx = blk - by * nbx;
    for (int t = threadIdx.x; t < nb * na; t += blockDim.x) {
      const int k = t % nb, l = t / nb;
      ub[t] = u[bx * nb + k + (by * na + l) * m];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < mb * na; t += blockDim.x) {
      const int p = t % mb, l = t / mb;
      double s = 0.0;
      for (int k = 0; k < nb; ++k) s = fma(Br.a[p * nb + k], ub[k + l * nb], s);
      tb[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < mb * ma; t += blockDim.x) {
      const int p = t % mb, q = t / mb;
      double s = 0.0;
      for (int l = 0; l < na; ++l) s = fma(As.a[q * na + l], tb[p + l * mb], s);
      v[bx * mb + p + (by * ma + q) * mo] = s;
    }
    __syncthreads();
  }
}

// Large factors (a side above kMaxBlock): C_b = A_b B_b for b < batch, every
// operand addressed through (row, column, batch) strides, in 64 x 64 output
// tiles of 256 threads (4 x 4 outputs each) with 16-deep k slices staged in
// shared memory.  Each output is one FMA chain over k in increasing order,
// the order of the small-block kernels above.
struct GemmArgs {
  const double* A;
  const double* B;
  double* C;
  long long M, N, K, batch;
  long long a_rs, a_cs, a_bs, b_rs, b_cs, b_bs, c_rs, c_cs, c_bs;
};

constexpr int kGT = 64, kGK = 16;

__global__ void __launch_bounds__(256) k_abu_gemm(const __grid_constant__ GemmArgs g) {
  __shared__ double sa[kGK][kGT + 1];
  __shared__ double sb[kGK][kGT + 1];
  const long long tiles_m = (g.M + kGT - 1) / kGT, tiles_n = (g.N + kGT - 1) / kGT;
  const long long tiles = tiles_m * tiles_n * g.batch;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const long long b = tile / (tiles_m * tiles_n);
    const long long rem = tile - b * tiles_m * tiles_n;
    const long long i0 = (rem % tiles_m) * kGT, j0 = (rem / tiles_m) * kGT;
    const double* A = g.A + b * g.a_bs;
    const double* B = g.B + b * g.b_bs;
    double acc[4][4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = 0.0;
    for (long long k0 = 0; k0 < g.K; k0 += kGK) {
      for (int t = threadIdx.x; t < kGK * kGT; t += blockDim.x) {
        const int kk = t / kGT, ii = t - kk * kGT;  // A: ii along rows; B: ii along columns
        const long long k = k0 + kk;
        sa[kk][ii] = (k < g.K && i0 + ii < g.M) ? A[(i0 + ii) * g.a_rs + k * g.a_cs] : 0.0;
        sb[kk][ii] = (k < g.K && j0 + ii < g.N) ? B[k * g.b_rs + (j0 + ii) * g.b_cs] : 0.0;
      }
      __syncthreads();
      const int kn = (int)(g.K - k0 < kGK ? g.K - k0 : kGK);
      for (int kk = 0; kk < kn; ++kk) {
        double av[4], bv[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) av[p] = sa[kk][ty + 16 * p];
#pragma unroll
        for (int q = 0; q < 4; ++q) bv[q] = sb[kk][tx + 16 * q];
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[p][q] = fma(av[p], bv[q], acc[p][q]);
      }
      __syncthreads();
    }
    double* C = g.C + b * g.c_bs;
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const long long i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
        if (i < g.M && j < g.N) C[i * g.c_rs + j * g.c_cs] = acc[p][q];
      }
  }
}

void load_mat(Mat32& M, const double* colmajor, int rows, int cols) {
  std::memset(&M, 0, sizeof(M));
  M.rows = rows;
  M.cols = cols;
  for (int p = 0; p < rows; ++p)
    for (int k = 0; k < cols; ++k) M.a[p * cols + k] = colmajor[p + (long long)k * rows];
}

}  // namespace

unsigned topo_bits(const Grid& g) { return g.topo; }

int launch_gather_scatter(const Grid& g, const double* u, double* out, unsigned mode,
                          cudaStream_t s) {
  if (!g.rinfo) return set_error(SEM_ERR_BAD_ARG, "gather-scatter needs a mesh handle");
  k_gather_scatter<<<grid_for(g.NX * g.NY), kThreads, 0, s>>>(u, out, g, mode);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int launch_gather_scatter_grid(int nr, int ns, int Ex, int Ey, bool perx, bool pery, const double* u,
                               double* out, cudaStream_t s) {
  GsGrid q;
  q.NX = (long long)nr * Ex;
  q.NY = (long long)ns * Ey;
  q.nr = nr;
  q.ns = ns;
  q.Ex = Ex;
  q.Ey = Ey;
  q.perx = perx;
  q.pery = pery;
  k_gather_scatter_grid<<<grid_for(q.NX * q.NY), kThreads, 0, s>>>(u, out, q);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int launch_mask_bc(const Grid& g, const double* u, double* out, unsigned topo, cudaStream_t s) {
  (void)topo;
  k_mask_bc<<<grid_for(g.NX * g.NY), kThreads, 0, s>>>(u, out, g);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int launch_mask_array(const double* M, const double* u, double* out, int64_t len,
                      cudaStream_t s) {
  if (len == 0) return SEM_OK;
  k_mask_array<<<grid_for(len), kThreads, 0, s>>>(M, u, out, len);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int launch_mass(const Grid& g, const double* B, const double* u, double* out, cudaStream_t s) {
  const long long len = g.NX * g.NY;
  k_mass<<<grid_for(len), kThreads, 0, s>>>(B, u, out, len);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int launch_mult(const Grid& g, double* out, cudaStream_t s) {
  k_mult<<<grid_for(g.NX * g.NY), kThreads, 0, s>>>(out, g);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

// ABu with a factor larger than kMaxBlock: the factors are copied to
// stream-ordered device buffers and applied as strided GEMMs, Br first on the
// column-major chunks of reshape(u, nb, :), then As on the column blocks
// (src/ABu.jl:13-34), through a temporary field when both are given
static int launch_abu_large(const double* As, int ma, int na, const double* Br, int mb, int nb,
                            const double* u, int m, int n, double* v, cudaStream_t s) {
  double* dA = nullptr;
  double* dB = nullptr;
  double* tmp = nullptr;
  int st = SEM_OK;
  auto alloc = [&](double** p, size_t count) {
    const cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(p), sizeof(double) * count, s);
    if (e != cudaSuccess) st = cuda_error(e, "cudaMallocAsync(ABu operand)");
    return e == cudaSuccess;
  };
  auto upload = [&](double* d, const double* h, size_t count) {
    const cudaError_t e = cudaMemcpyAsync(d, h, sizeof(double) * count, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) st = cuda_error(e, "cudaMemcpyAsync(ABu factor)");
    return e == cudaSuccess;
  };
  auto gemm = [&](const GemmArgs& g) {
    const long long tiles = ((g.M + kGT - 1) / kGT) * ((g.N + kGT - 1) / kGT) * g.batch;
    const unsigned blocks = (unsigned)(tiles < 152LL * 8 ? tiles : 152LL * 8);
    k_abu_gemm<<<blocks, 256, 0, s>>>(g);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = cuda_error(e, "k_abu_gemm");
  };
  const long long m1 = Br ? (long long)m * mb / nb : m;  // rows after the Br side
  do {
    if (Br && !(alloc(&dB, (size_t)mb * nb) && upload(dB, Br, (size_t)mb * nb))) break;
    if (As && !(alloc(&dA, (size_t)ma * na) && upload(dA, As, (size_t)ma * na))) break;
    const double* src = u;
    if (Br) {
      double* dst = v;
      if (As) {
        if (!alloc(&tmp, (size_t)m1 * n)) break;
        dst = tmp;
      }
      // (mb x nb) times reshape(u, nb, :) -> reshape(dst, mb, :)
      GemmArgs g{dB, u, dst, mb, (long long)m * n / nb, nb, 1, 1, mb, 0, 1, nb, 0, 1, mb, 0};
      gemm(g);
      if (st != SEM_OK) break;
      src = dst;
    }
    if (As) {
      // column block b: (m1 x na) times As' (na x ma) -> (m1 x ma)
      GemmArgs g{src, dA, v, m1, ma, na, n / na, 1, m1, (long long)na * m1, ma, 1, 0, 1, m1,
                 (long long)ma * m1};
      gemm(g);
    }
  } while (false);
  if (tmp) cudaFreeAsync(tmp, s);
  if (dA) cudaFreeAsync(dA, s);
  if (dB) cudaFreeAsync(dB, s);
  return st;
}

int launch_abu(const double* As, int ma, int na, const double* Br, int mb, int nb,
               const double* u, int m, int n, double* v, cudaStream_t s) {
  if (m <= 0 || n <= 0) return SEM_OK;
  if (As == nullptr && Br == nullptr) {
    SEM_CUDA(cudaMemcpyAsync(v, u, sizeof(double) * (size_t)m * n, cudaMemcpyDeviceToDevice, s));
    return SEM_OK;
  }
  // factors above kMaxBlock, or both factors on a u whose rows are not whole
  // chunks of nb (the one-pass kernel below tiles u into nb x na blocks)
  if ((Br && (mb > kMaxBlock || nb > kMaxBlock)) || (As && (ma > kMaxBlock || na > kMaxBlock)) ||
      (As && Br && m % nb != 0))
    return launch_abu_large(As, ma, na, Br, mb, nb, u, m, n, v, s);
  if (Br != nullptr && As == nullptr) {
    Mat32 B;
    load_mat(B, Br, mb, nb);
    const long long nchunks = (long long)m * n / nb;
    k_abu_br<<<grid_for(nchunks * mb), kThreads, 0, s>>>(B, u, v, nchunks);
    SEM_CUDA(cudaGetLastError());
    return SEM_OK;
  }
  if (As != nullptr && Br == nullptr) {
    Mat32 A;
    load_mat(A, As, ma, na);
    const long long nblk = n / na;
    k_abu_as<<<grid_for((long long)m * nblk * ma), kThreads, 0, s>>>(A, u, v, m, nblk);
    SEM_CUDA(cudaGetLastError());
    return SEM_OK;
  }
  Mat32 A, B;
  load_mat(A, As, ma, na);
  load_mat(B, Br, mb, nb);
  const long long nbx = m / nb, nby = n / na;
  const size_t smem = sizeof(double) * (size_t)(nb * na + mb * na);
  unsigned blocks = grid_for(nbx * nby, 1, 152LL * 16);
  k_abu_both<<<blocks, 128, smem, s>>>(A, B, u, v, m, nbx, nby);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

}  // namespace sem
