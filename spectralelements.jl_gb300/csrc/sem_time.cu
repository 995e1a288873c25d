// BDFk/EXTk time stepping of the diffusion equation with the histories and
// the right-hand side on the device (src/time.jl:31-112,
// src/diffusion.jl:36-137).
//
// One step of the reference (evolve!, src/diffusion.jl:81-106) is: shift the
// histories (uh[i] <- uh[i-1], uh[1] <- u), advance the time history and
// recompute the BDF coefficients, set ub and f at the new time, build
// rhs = QQ'(mask(B f - nu lapl(ub) - sum_i bdfB[1+i] B uh_i)), solve
// mask(QQ'(hlmz(u, nu, bdfB[1]))) u = rhs by pcg from u = 0, then u += ub.
//
// Here the right-hand side is one gather kernel (the mass terms combined per
// local copy, summed over the copies of each global node in the x-first order
// of the standalone QQ'), plus one fused operator launch for the lapl(ub)
// term when boundary data is given.  sem_bdf_run queues whole runs: where the
// single-launch small-mesh solver serves the mesh, no step waits for the
// host; results are read back once per block of steps.
#include <cstring>

#include "sem_internal.cuh"

namespace sem {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxTerms = 16;   // fields in one combination (forcing modes + histories)
constexpr int kMaxModes = 8;    // forcing or boundary-data modes of sem_bdf_run
constexpr int kBlockSteps = 128;  // small-path steps queued before the host reads results

inline unsigned grid_for(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  if (b > 152LL * 32) b = 152LL * 32;
  return (unsigned)b;
}

struct Comb {
  int nterms;
  double coef[kMaxTerms];
  const double* fld[kMaxTerms];
};

struct RhsArgs {
  Grid g;
  Comb w;              // w = sum_m coef_m fld_m, multiplied by B per local copy
  const double* B;
  const double* extra;  // assembled field added as extra_coef * extra (or NULL)
  double extra_coef;
  int mask;
};

__device__ __forceinline__ double comb_at(const Comb& c, long long i) {
  double w = 0.0;
  for (int m = 0; m < c.nterms; ++m) w = fma(c.coef[m], __ldg(c.fld[m] + i), w);
  return w;
}

// rhs(p) = mask(p) * sum over the copies c of p's node of B(c) w(c)
//          (+ extra_coef * extra(p))
__global__ void __launch_bounds__(kThreads) k_bdf_rhs(const __grid_constant__ RhsArgs a,
                                                      double* __restrict__ out) {
  const Grid g = a.g;
  const long long NX = g.NX;
  for_each_point(g, [&](unsigned r, unsigned c, long long idx) {
    const unsigned char rb = g.rinfo[r], cb = g.cinfo[c];
    const long long pr = line_partner(r, rb, g.NX);
    const long long pc = line_partner(c, cb, g.NY);
    const long long r0 = (pr >= 0 && pr < r) ? pr : r;
    const long long r1 = (pr >= 0 && pr < r) ? (long long)r : pr;
    auto bw = [&](long long i) { return __ldg(a.B + i) * comb_at(a.w, i); };
    auto xsum = [&](long long cc) {
      double s = bw(r0 + cc * NX);
      if (r1 >= 0) s += bw(r1 + cc * NX);
      return s;
    };
    double v;
    if (pc < 0) {
      v = xsum(c);
    } else {
      const long long c0 = pc < c ? pc : (long long)c, c1 = pc < c ? (long long)c : pc;
      v = xsum(c0) + xsum(c1);
    }
    if (a.mask && ((rb | cb) & L_ZERO)) v = v * 0.0;
    if (a.extra) v = fma(a.extra_coef, a.extra[idx], v);
    out[idx] = v;
  });
}

// out = sum_m coef_m fld_m (out may be one of the fields)
__global__ void __launch_bounds__(kThreads) k_comb(const __grid_constant__ Comb c, double* out,
                                                   long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x) {
    double w = 0.0;
    for (int m = 0; m < c.nterms; ++m) w = fma(c.coef[m], c.fld[m][i], w);
    out[i] = w;
  }
}

int launch_comb(const Comb& c, double* out, long long len, cudaStream_t s) {
  k_comb<<<grid_for(len), kThreads, 0, s>>>(c, out, len);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

// out = mask(QQ'(lapl(u))) through the fused operator of the mesh
int lapl_gs(sem_mesh* m, const double* u, double* out, cudaStream_t s) {
  ApplyCall c;
  std::memset(&c, 0, sizeof(c));
  c.u = u;
  c.out = out;
  c.G11 = m->G11;
  c.G12 = m->G12;
  c.G22 = m->G22;
  c.B = m->B;
  c.nu_s = 1.0;
  c.k_s = 0.0;
  c.mode = m->g.topo | M_STIFF | M_GS | (m->has_bc ? M_MASK : 0u);
  c.precision = m->precision;
  c.variant = m->variant[m->precision];
  c.Gdf = m->Gdf;
  c.ctr = m->fix_ctr;
  SEM_CHECK(arm_range_guard(m, c));
  return launch_apply(m->g, m->ops, c, s);
}

// rhs from the prepared combination w (mass terms) and, when lub is given,
// the assembled -nu * mask(QQ'(lapl(ub)))
int launch_rhs(sem_mesh* m, const Comb& w, const double* lub, double nu, double* rhs, cudaStream_t s) {
  RhsArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = m->g;
  a.w = w;
  a.B = m->B;
  a.extra = lub;
  a.extra_coef = -nu;
  a.mask = m->has_bc ? 1 : 0;
  k_bdf_rhs<<<grid_for(m->g.NX * m->g.NY), kThreads, 0, s>>>(a, rhs);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

struct DevScratch {
  cudaStream_t s;
  void* p[4] = {nullptr};
  int n = 0;
  explicit DevScratch(cudaStream_t st) : s(st) {}
  template <class T>
  int get(size_t count, T** out) {
    SEM_CUDA(cudaMallocAsync(&p[n], sizeof(T) * (count ? count : 1), s));
    *out = static_cast<T*>(p[n++]);
    return SEM_OK;
  }
  ~DevScratch() {
    for (int i = 0; i < n; ++i) cudaFreeAsync(p[i], s);
  }
};

// pinned host records of queued small-mesh solves; freed only after the
// stream has consumed them (an error return may leave copies queued)
struct PinnedRecords {
  SmallProb* h = nullptr;
  cudaStream_t s = nullptr;
  ~PinnedRecords() {
    if (!h) return;
    cudaStreamSynchronize(s);
    cudaFreeHost(h);
  }
};

// Lagrange weights on the nodes x[0..n-1]: lambda_i = 1 / prod_{j != i} (x_i - x_j)
void bary_weights(const double* x, int n, double* lam) {
  for (int i = 0; i < n; ++i) {
    double p = 1.0;
    for (int j = 0; j < n; ++j)
      if (j != i) p *= (x[i] - x[j]);
    lam[i] = 1.0 / p;
  }
}

}  // namespace

// BDFk/EXTk coefficients (src/time.jl:31-53).  With u = the distinct times
// (first occurrences, in order) and kk = len(u) - 1: b = row 1 of the
// Lagrange derivative matrix on u (src/derivMat.jl:9-35: the derivative of
// basis j at u_1 is lambda_j / (lambda_1 (u_1 - u_j)), and the diagonal
// sum_{j != 1} 1 / (u_1 - u_j)); a = the Lagrange weights of u_2..u_{kk+1}
// at u_1 (src/interp.jl:10-35); both zero-padded to k and k+1 entries or
// truncated; a_1 = 1 when every time is equal (the steady branch).
int bdf_coeffs(int k, const double* t, double* a, double* b) {
  double u[SEM_BDF_MAX_ORDER + 1];
  int nu = 0;
  for (int i = 0; i <= k; ++i) {
    bool seen = false;
    for (int j = 0; j < nu; ++j) seen = seen || (u[j] == t[i]);
    if (!seen) u[nu++] = t[i];
  }
  const int kk = nu - 1;
  for (int i = 0; i < k; ++i) a[i] = 0.0;
  for (int i = 0; i <= k; ++i) b[i] = 0.0;
  double lam[SEM_BDF_MAX_ORDER + 1];
  bary_weights(u, nu, lam);
  double diag = 0.0;
  for (int j = 1; j < nu; ++j) diag += 1.0 / (u[0] - u[j]);
  b[0] = diag;
  for (int j = 1; j < nu && j <= k; ++j) b[j] = lam[j] / (lam[0] * (u[0] - u[j]));
  if (kk > 0) {
    double lam0[SEM_BDF_MAX_ORDER];
    bary_weights(u + 1, kk, lam0);
    for (int j = 0; j < kk && j < k; ++j) {
      // prod_{m != j} (u_1 - u0_m) as the product of the left and right
      // partial products, the order src/interp.jl:10-35 forms them in
      double sl = 1.0, sr = 1.0;
      for (int m = 0; m < j; ++m) sl *= (u[0] - u[1 + m]);
      for (int m = kk - 1; m > j; --m) sr *= (u[0] - u[1 + m]);
      a[j] = lam0[j] * sl * sr;
    }
  } else {
    a[0] = 1.0;
  }
  return SEM_OK;
}

}  // namespace sem

using namespace sem;

extern "C" {

int sem_bdf_coeffs(int k, const double* t, double* a, double* b) {
  if (!t || !a || !b) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (k < 1 || k > SEM_BDF_MAX_ORDER)
    return set_error(SEM_ERR_BAD_ARG, "order k must be in 1..%d (got %d)", SEM_BDF_MAX_ORDER, k);
  return bdf_coeffs(k, t, a, b);
}

int sem_bdf_rhs(sem_mesh_t* m, double nu, int order, const double* bdfB, const double* f,
                const double* ub, const double* const* uh, double* rhs, sem_stream_t stream) {
  if (!m || !bdfB || !rhs) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (order < 0 || order > SEM_BDF_MAX_ORDER)
    return set_error(SEM_ERR_BAD_ARG, "order must be in 0..%d (got %d)", SEM_BDF_MAX_ORDER, order);
  if (order > 0 && !uh) return set_error(SEM_ERR_BAD_ARG, "NULL history list");
  cudaStream_t s = (cudaStream_t)stream;
  Comb w;
  std::memset(&w, 0, sizeof(w));
  if (f) {
    if (f == rhs) return set_error(SEM_ERR_BAD_ARG, "rhs must not alias an input");
    w.coef[w.nterms] = 1.0;
    w.fld[w.nterms++] = f;
  }
  for (int i = 0; i < order; ++i) {
    if (!uh[i]) return set_error(SEM_ERR_BAD_ARG, "NULL history %d", i);
    if (uh[i] == rhs) return set_error(SEM_ERR_BAD_ARG, "rhs must not alias an input");
    if (bdfB[1 + i] == 0.0) continue;  // the zero-padded terms of the first BDFk steps
    w.coef[w.nterms] = -bdfB[1 + i];
    w.fld[w.nterms++] = uh[i];
  }
  DevScratch sc(s);
  double* lub = nullptr;
  if (ub) {
    if (ub == rhs) return set_error(SEM_ERR_BAD_ARG, "rhs must not alias an input");
    SEM_CHECK(sc.get(m->g.NX * m->g.NY, &lub));
    SEM_CHECK(lapl_gs(m, ub, lub, s));
  }
  return launch_rhs(m, w, lub, nu, rhs, s);
}

int sem_bdf_run(sem_mesh_t* m, const sem_bdf_desc* d, double* time, double* u, double* const* uh,
                sem_solve_info* info, sem_stream_t stream) {
  if (!m || !d || !time || !u) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  const int k = d->order;
  if (k < 1 || k > SEM_BDF_MAX_ORDER)
    return set_error(SEM_ERR_BAD_ARG, "order must be in 1..%d (got %d)", SEM_BDF_MAX_ORDER, k);
  if (!uh) return set_error(SEM_ERR_BAD_ARG, "NULL history list");
  for (int i = 0; i < k; ++i) {
    if (!uh[i]) return set_error(SEM_ERR_BAD_ARG, "NULL history %d", i);
    if (uh[i] == u) return set_error(SEM_ERR_BAD_ARG, "a history must not alias u");
  }
  if (d->nsteps < 0) return set_error(SEM_ERR_BAD_ARG, "nsteps must be >= 0");
  if (d->nf < 0 || d->nf > kMaxModes || d->nb < 0 || d->nb > kMaxModes)
    return set_error(SEM_ERR_BAD_ARG, "at most %d forcing and %d boundary modes", kMaxModes, kMaxModes);
  if ((d->nf && (!d->F || !d->fcoef)) || (d->nb && (!d->UB || !d->bcoef)))
    return set_error(SEM_ERR_BAD_ARG, "NULL mode list or coefficient table");
  for (int j = 0; j < d->nf; ++j)
    if (!d->F[j]) return set_error(SEM_ERR_BAD_ARG, "NULL forcing mode %d", j);
  for (int j = 0; j < d->nb; ++j)
    if (!d->UB[j]) return set_error(SEM_ERR_BAD_ARG, "NULL boundary mode %d", j);
  if (d->solve.nu_field)
    return set_error(SEM_ERR_UNSUPPORTED, "the time loop takes a scalar nu");
  if (d->nsteps == 0) return SEM_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const long long L = m->g.NX * m->g.NY;
  const size_t bytes = sizeof(double) * (size_t)L;

  DevScratch sc(s);
  double *rhs = nullptr, *ub = nullptr, *lub = nullptr;
  SEM_CHECK(sc.get(L, &rhs));
  if (d->nb) {
    SEM_CHECK(sc.get(L, &ub));
    SEM_CHECK(sc.get(L, &lub));
  }
  sem_pcg_opts o = d->solve;
  o.nu = d->nu;
  o.nu_field = nullptr;
  o.k = 0.0;  // set per step
  const bool small = small_path_taken(m, &o);
  SmallProb* rec_dev = nullptr;
  PinnedRecords rec_h;
  rec_h.s = s;
  if (small) {
    SEM_CHECK(sc.get(kBlockSteps, &rec_dev));
    SEM_CUDA(cudaMallocHost(&rec_h.h, sizeof(SmallProb) * kBlockSteps));
  }
  int status = SEM_OK;
  int first_bad = -1;
  auto record = [&](int step, const sem_solve_info& si, int st) -> int {
    if (info) info[step] = si;
    if (st == SEM_ERR_NAN) return set_error(SEM_ERR_NAN, "NaN/Inf in the residual of step %d", step);
    if (st == SEM_ERR_NOT_CONVERGED) {
      if (first_bad < 0) first_bad = step;
      status = SEM_ERR_NOT_CONVERGED;
      return SEM_OK;
    }
    return st;
  };

  int block_start = 0, nblock = 0;
  auto flush = [&]() -> int {
    if (!nblock) return SEM_OK;
    SEM_CUDA(cudaMemcpyAsync(rec_h.h, rec_dev, sizeof(SmallProb) * nblock, cudaMemcpyDeviceToHost, s));
    SEM_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < nblock; ++i) {
      const SmallProb& r = rec_h.h[i];
      sem_solve_info si;
      si.iters = r.iters;
      si.outer = r.outer;
      si.res_inf = r.res_inf;
      si.res0_inf = r.res0_inf;
      si.converged = r.converged;
      const int st = r.nan ? SEM_ERR_NAN : (r.converged ? SEM_OK : SEM_ERR_NOT_CONVERGED);
      SEM_CHECK(record(block_start + i, si, st));
    }
    block_start += nblock;
    nblock = 0;
    return SEM_OK;
  };

  for (int step = 0; step < d->nsteps; ++step) {
    // updateHist!(fld): uh[k-1] <- uh[k-2] <- ... <- uh[0] <- u
    for (int i = k - 1; i > 0; --i)
      SEM_CUDA(cudaMemcpyAsync(uh[i], uh[i - 1], bytes, cudaMemcpyDeviceToDevice, s));
    SEM_CUDA(cudaMemcpyAsync(uh[0], u, bytes, cudaMemcpyDeviceToDevice, s));
    // updateHist!(time); time[1] += dt; bdfExtK!
    for (int i = k; i > 0; --i) time[i] = time[i - 1];
    time[0] += d->dt;
    double bA[SEM_BDF_MAX_ORDER], bB[SEM_BDF_MAX_ORDER + 1];
    SEM_CHECK(bdf_coeffs(k, time, bA, bB));
    // setBC!: ub = sum_j bcoef[step, j] UB_j, and its lapl term
    if (d->nb) {
      Comb c;
      std::memset(&c, 0, sizeof(c));
      for (int j = 0; j < d->nb; ++j) {
        c.coef[c.nterms] = d->bcoef[(long long)step * d->nb + j];
        c.fld[c.nterms++] = d->UB[j];
      }
      SEM_CHECK(launch_comb(c, ub, L, s));
      SEM_CHECK(lapl_gs(m, ub, lub, s));
    }
    // makeRHS!: mass terms of the forcing modes and the histories
    Comb w;
    std::memset(&w, 0, sizeof(w));
    for (int j = 0; j < d->nf; ++j) {
      w.coef[w.nterms] = d->fcoef[(long long)step * d->nf + j];
      w.fld[w.nterms++] = d->F[j];
    }
    for (int i = 0; i < k; ++i) {
      if (bB[1 + i] == 0.0) continue;
      w.coef[w.nterms] = -bB[1 + i];
      w.fld[w.nterms++] = uh[i];
    }
    SEM_CHECK(launch_rhs(m, w, d->nb ? lub : nullptr, d->nu, rhs, s));
    // solve!: pcg from u = 0 on opLHS with k = bdfB[1]
    o.k = bB[0];
    if (small) {
      SmallProb& r = rec_h.h[nblock];
      SEM_CHECK(small_prepare(m, &o, rhs, u, &r, s));
      SEM_CUDA(cudaMemcpyAsync(rec_dev + nblock, &r, sizeof(SmallProb), cudaMemcpyHostToDevice, s));
      SEM_CHECK(launch_small_pcg(rec_dev + nblock, *m->ops, m->g.n, s));
      ++nblock;
    } else {
      sem_solve_info si;
      std::memset(&si, 0, sizeof(si));
      const int st = sem_pcg(m, &o, rhs, u, &si, stream);
      if (st != SEM_OK && st != SEM_ERR_NOT_CONVERGED && st != SEM_ERR_NAN) return st;
      SEM_CHECK(record(step, si, st));
      ++block_start;
    }
    // u .+= ub
    if (d->nb) {
      Comb c;
      std::memset(&c, 0, sizeof(c));
      c.nterms = 2;
      c.coef[0] = 1.0;
      c.fld[0] = u;
      c.coef[1] = 1.0;
      c.fld[1] = ub;
      SEM_CHECK(launch_comb(c, u, L, s));
    }
    if (small && nblock == kBlockSteps) SEM_CHECK(flush());
  }
  if (small) SEM_CHECK(flush());
  if (status == SEM_ERR_NOT_CONVERGED)
    return set_error(SEM_ERR_NOT_CONVERGED, "step %d (and possibly later ones) reached maxiter", first_bad);
  return SEM_OK;
}

}  // extern "C"
