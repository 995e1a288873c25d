// Host side of the batched solver: per-problem workspace and Jacobi set-up,
// problems grouped by polynomial order (largest estimated work first inside a
// group), and one persistent cluster launch per order on its own stream, all
// joined back into the caller's stream.  Each group's launch shape (cluster
// size, register budget, cluster count) and problem order come from its
// configuration, which the autotuner below chooses from measured per-problem
// timelines.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <queue>
#include <string>
#include <vector>

#include "sem_batch_kernel.cuh"

namespace sem {
#define SEM_BATCH_UNIT(u)                                                                  \
  int launch_batch_##u(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s); \
  int max_clusters_##u(int n, int csize);
SEM_BATCH_UNIT(ka)
SEM_BATCH_UNIT(kb)
SEM_BATCH_UNIT(kc)
SEM_BATCH_UNIT(kd)
SEM_BATCH_UNIT(ke)
SEM_BATCH_UNIT(kf)
#undef SEM_BATCH_UNIT
int batch_diag(sem_mesh* m, double nu, double k, double* dinv, double* tmp, cudaStream_t s);

namespace {
// the translation unit of order n at register budget c.ctas_per_sm
int launch_group(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  if (c.ctas_per_sm != 1 && c.ctas_per_sm != 2)
    return set_error(SEM_ERR_BAD_ARG, "batch CTAs per SM %d (1 or 2)", c.ctas_per_sm);
  const bool two = c.ctas_per_sm == 2;
  if (n <= 6) return two ? launch_batch_ka(n, c, ops, s) : launch_batch_kd(n, c, ops, s);
  if (n <= 9) return two ? launch_batch_kb(n, c, ops, s) : launch_batch_ke(n, c, ops, s);
  return two ? launch_batch_kc(n, c, ops, s) : launch_batch_kf(n, c, ops, s);
}

// clusters of the given shape that fit the device at once (0: none)
int max_clusters(int n, int csize, int mb) {
  if (mb != 1 && mb != 2) return 0;
  const bool two = mb == 2;
  if (n <= 6) return two ? max_clusters_ka(n, csize) : max_clusters_kd(n, csize);
  if (n <= 9) return two ? max_clusters_kb(n, csize) : max_clusters_ke(n, csize);
  return two ? max_clusters_kc(n, csize) : max_clusters_kf(n, csize);
}

// makespan of list-scheduling durations d (queue order) onto k identical
// clusters: each problem goes to the cluster that frees first
double list_makespan(const std::vector<double>& d, int k) {
  if (d.empty()) return 0.0;
  std::priority_queue<double, std::vector<double>, std::greater<double>> free_at;
  for (int i = 0; i < std::max(1, k); ++i) free_at.push(0.0);
  double end = 0.0;
  for (double x : d) {
    const double t = free_at.top() + x;
    free_at.pop();
    free_at.push(t);
    end = std::max(end, t);
  }
  return end;
}

// FNV-1a over the bytes of a value
void fnv(unsigned long long& h, const void* p, size_t n) {
  const unsigned char* c = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= c[i];
    h *= 1099511628211ull;
  }
}

__global__ void k_d2f_copy(const double* __restrict__ a, float* __restrict__ b, long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// estimated CG work of a problem: local DOF times a Jacobi-PCG iteration-count proxy
double work_of(const BProb& q) { return (double)q.NX * q.NY * (double)(q.Ex + q.Ey) * q.n; }
}  // namespace
}  // namespace sem

using namespace sem;

struct sem_batch {
  struct Group {
    int n, first, count;
    double work;
    const OperatorSet* ops;
    cudaStream_t stream;
    cudaEvent_t done;
    // launch configuration: CTAs per cluster, resident CTAs per SM (register
    // budget), persistent clusters (0: the work-proportional share)
    int csize, mb, clusters;
  };
  int count = 0;
  int device = 0;
  int jacobi = 0;
  std::vector<BProb> host;  // per problem, creation order (device pointers inside)
  std::vector<sem_mesh*> meshes;  // per problem (solves outside the pair format's range)
  std::vector<int> order;   // device slot -> problem index
  std::vector<Group> groups;
  BProb* dev = nullptr;     // device descriptors in slot order
  int* queues = nullptr;    // one work-queue counter per group
  void* ws = nullptr;       // all per-problem vectors
  cudaEvent_t start = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;  // timing of the last solve
  cudaEvent_t w0 = nullptr, w1 = nullptr;  // timing of one wide problem
  // timeline of the last solve, per problem in creation order
  std::vector<long long> t_start, t_end;
  std::vector<int> cluster;  // group index * 65536 + the cluster's index in its launch
  double last_ms = 0.0;
  // problems solved on the whole GPU (sem_pcg's chunked path) before the
  // persistent launches, and their last solve times
  std::vector<char> wide;
  std::vector<double> wide_ms;
};

extern "C" {

int sem_batch_create(sem_mesh_t* const* meshes, const double* nu, const double* k, int count,
                     int precond, sem_batch_t** out) {
  if (!meshes || !nu || !k || !out || count <= 0) return set_error(SEM_ERR_BAD_ARG, "bad batch arguments");
  *out = nullptr;
  if (precond != SEM_PRECOND_NONE && precond != SEM_PRECOND_JACOBI)
    return set_error(SEM_ERR_BAD_ARG, "unknown preconditioner %d", precond);
  int dev = 0;
  SEM_CUDA(cudaGetDevice(&dev));
  const OperatorSet* first[kBatchMaxN + 1] = {nullptr};
  size_t total = 0;
  for (int i = 0; i < count; ++i) {
    const sem_mesh* m = meshes[i];
    if (!m) return set_error(SEM_ERR_BAD_ARG, "NULL mesh %d", i);
    if (m->device != dev) return set_error(SEM_ERR_BAD_ARG, "mesh %d lives on another device", i);
    const int n = m->g.n;
    if (n < 2 || n > kBatchMaxN)
      return set_error(SEM_ERR_UNSUPPORTED,
                       "the batch kernels serve 2 <= n <= %d (mesh %d has n = %d); solve it with sem_pcg",
                       kBatchMaxN, i, n);
    if (!first[n])
      first[n] = m->ops;
    else if (std::memcmp(first[n]->eo, m->ops->eo, sizeof(m->ops->eo)) != 0)
      return set_error(SEM_ERR_UNSUPPORTED, "meshes with n = %d use different derivative matrices", n);
    total += (size_t)(m->g.NX * m->g.NY);
  }
  sem_batch* b = new sem_batch;
  b->count = count;
  b->device = dev;
  b->jacobi = precond == SEM_PRECOND_JACOBI;
  const size_t bytes = total * (4 * sizeof(double) + 5 * sizeof(float)) + (size_t)count * 9 * 256;
  cudaError_t e = cudaMalloc(&b->ws, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&b->dev, sizeof(BProb) * count);
  if (e == cudaSuccess) e = cudaMalloc(&b->queues, sizeof(int) * (kBatchMaxN + 1));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->start, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->t1);
  if (e == cudaSuccess) e = cudaEventCreate(&b->w0);
  if (e == cudaSuccess) e = cudaEventCreate(&b->w1);
  if (e != cudaSuccess) {
    sem_batch_destroy(b);
    return cuda_error(e, "batch allocation");
  }
  b->host.resize(count);
  b->meshes.assign(meshes, meshes + count);
  b->wide.assign(count, 0);
  b->wide_ms.assign(count, 0.0);
  char* p = static_cast<char*>(b->ws);
  auto take = [&](size_t nbytes) {
    char* q = p;
    p += (nbytes + 255) & ~(size_t)255;
    return q;
  };
  int st = SEM_OK;
  for (int i = 0; i < count && st == SEM_OK; ++i) {
    sem_mesh* m = meshes[i];
    const long long L = m->g.NX * m->g.NY;
    BProb& q = b->host[i];
    std::memset(&q, 0, sizeof(q));
    q.n = m->g.n;
    q.Ex = m->g.Ex;
    q.Ey = m->g.Ey;
    q.NX = m->g.NX;
    q.NY = m->g.NY;
    q.topo = m->g.topo | (m->has_bc ? M_MASK : 0u);
    q.nu = nu[i];
    q.k = k[i];
    q.r = (double*)take(L * 8);
    q.p = (double*)take(L * 8);
    q.Ap = (double*)take(L * 8);
    q.dinv = (double*)take(L * 8);
    q.r32 = (float*)take(L * 4);
    q.p32 = (float*)take(L * 4);
    q.Ap32 = (float*)take(L * 4);
    q.x32 = (float*)take(L * 4);
    q.dinv32 = (float*)take(L * 4);
    st = ensure_f32_geometry(m, 0);
    if (st == SEM_OK) st = ensure_df_geometry(m, 0);
    q.Gdf = m->Gdf;
    q.G11f = m->G11_f;
    q.G12f = m->G12_f;
    q.G22f = m->G22_f;
    q.Bf = m->B_f;
    if (st == SEM_OK && b->jacobi) {
      st = batch_diag(m, nu[i], k[i], q.dinv, q.r, 0);
      if (st == SEM_OK) {
        k_d2f_copy<<<(unsigned)std::min<long long>((L + 255) / 256, 4096), 256>>>(q.dinv, q.dinv32, L);
        if ((e = cudaGetLastError()) != cudaSuccess) st = cuda_error(e, "batch Jacobi copy");
      }
    }
  }
  if (st == SEM_OK && (e = cudaStreamSynchronize(0)) != cudaSuccess) st = cuda_error(e, "batch set-up");
  if (st != SEM_OK) {
    sem_batch_destroy(b);
    return st;
  }
  // slots: grouped by order, largest estimated work first inside a group
  for (int n = 2; n <= kBatchMaxN; ++n) {
    if (!first[n]) continue;
    sem_batch::Group gr;
    gr.n = n;
    gr.first = (int)b->order.size();
    gr.work = 0.0;
    gr.ops = first[n];
    for (int i = 0; i < count; ++i)
      if (b->host[i].n == n) {
        b->order.push_back(i);
        gr.work += work_of(b->host[i]);
      }
    gr.count = (int)b->order.size() - gr.first;
    std::stable_sort(b->order.begin() + gr.first, b->order.end(),
                     [&](int x, int y) { return work_of(b->host[x]) > work_of(b->host[y]); });
    gr.stream = nullptr;
    gr.done = nullptr;
    gr.csize = 8;
    gr.mb = 2;
    gr.clusters = 0;
    if ((e = cudaStreamCreateWithFlags(&gr.stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&gr.done, cudaEventDisableTiming)) != cudaSuccess) {
      b->groups.push_back(gr);
      sem_batch_destroy(b);
      return cuda_error(e, "batch streams");
    }
    b->groups.push_back(gr);
  }
  *out = b;
  return SEM_OK;
}

int sem_batch_destroy(sem_batch_t* b) {
  if (!b) return SEM_OK;
  for (auto& g : b->groups) {
    if (g.stream) cudaStreamDestroy(g.stream);
    if (g.done) cudaEventDestroy(g.done);
  }
  if (b->start) cudaEventDestroy(b->start);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  if (b->w0) cudaEventDestroy(b->w0);
  if (b->w1) cudaEventDestroy(b->w1);
  if (b->ws) cudaFree(b->ws);
  if (b->dev) cudaFree(b->dev);
  if (b->queues) cudaFree(b->queues);
  delete b;
  return SEM_OK;
}

int sem_batch_pcg(sem_batch_t* b, const double* const* rhs, double* const* x, const double* tol,
                  const int* maxiter, int precision, double inner_tol, int max_outer,
                  sem_solve_info* info, sem_stream_t stream) {
  if (!b || !rhs || !x || !tol) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (precision != SEM_F64_DF && precision != SEM_MIXED && precision != SEM_MIXED_RR)
    return set_error(SEM_ERR_BAD_ARG, "the batch kernels take SEM_F64_DF, SEM_MIXED or SEM_MIXED_RR");
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<BProb> q(b->count);
  for (int j = 0; j < b->count; ++j) {
    const int i = b->order[j];
    q[j] = b->host[i];
    if (!rhs[i] || !x[i]) return set_error(SEM_ERR_BAD_ARG, "NULL b or x for problem %d", i);
    if (rhs[i] == x[i]) return set_error(SEM_ERR_BAD_ARG, "x aliases b for problem %d", i);
    q[j].b = rhs[i];
    q[j].x = x[i];
    q[j].tol = tol[i];
    const long long L = q[j].NX * q[j].NY;
    q[j].maxiter = (maxiter && maxiter[i] > 0) ? maxiter[i] : (int)(L > 2147483647LL ? 2147483647LL : L);
    // a problem whose nu or k lies outside the double-float window is solved
    // in native FP64 after the launch (none of its iterations run in it)
    if (!(df_window_ok(q[j].nu) && df_window_ok(q[j].k))) q[j].maxiter = -1;
    // a wide problem is solved on the whole GPU before the launch
    else if (b->wide[i]) q[j].maxiter = -2;
  }
  SEM_CUDA(cudaMemcpyAsync(b->dev, q.data(), sizeof(BProb) * b->count, cudaMemcpyHostToDevice, s));
  SEM_CUDA(cudaMemsetAsync(b->queues, 0, sizeof(int) * (kBatchMaxN + 1), s));
  SEM_CUDA(cudaEventRecord(b->t0, s));
  // ---- the wide problems, one after another on the whole GPU (sem_pcg's
  // chunked path, the batch's arithmetic), each timed on the stream
  double wide_total_ms = 0.0;
  for (int j = 0; j < b->count; ++j) {
    if (q[j].maxiter != -2) continue;
    const int i = b->order[j];
    sem_pcg_opts o;
    std::memset(&o, 0, sizeof(o));
    o.nu = q[j].nu;
    o.k = q[j].k;
    o.precond = b->jacobi ? SEM_PRECOND_JACOBI : SEM_PRECOND_NONE;
    o.precision = precision;
    o.tol = tol[i];
    o.maxiter = (maxiter && maxiter[i] > 0) ? maxiter[i] : 0;
    o.inner_tol = inner_tol;
    o.max_outer = max_outer;
    o.path = SEM_PATH_CHUNKED;
    sem_solve_info si;
    std::memset(&si, 0, sizeof(si));
    SEM_CUDA(cudaEventRecord(b->w0, s));
    const int st = sem_pcg(b->meshes[i], &o, rhs[i], x[i], &si, stream);
    if (st != SEM_OK && st != SEM_ERR_NOT_CONVERGED && st != SEM_ERR_NAN) return st;
    SEM_CUDA(cudaEventRecord(b->w1, s));
    SEM_CUDA(cudaEventSynchronize(b->w1));
    float wms = 0.0f;
    SEM_CUDA(cudaEventElapsedTime(&wms, b->w0, b->w1));
    b->wide_ms[i] = wms;
    wide_total_ms += wms;
    q[j].iters = si.iters;
    q[j].outer = si.outer;
    q[j].res_inf = si.res_inf;
    q[j].res0_inf = si.res0_inf;
    q[j].converged = si.converged;
    q[j].nan = st == SEM_ERR_NAN;
  }
  SEM_CUDA(cudaEventRecord(b->start, s));
  double wtot = 0.0;
  for (auto& g : b->groups) wtot += g.work;
  // the heaviest group launches first; each group's default cluster count is
  // its share of the estimated work times the clusters of its shape that fit
  // the device at once, so that every group's clusters are resident together
  // (clusters are placed within one GPC each, so 38 clusters of 8 do not fit
  // 152 SMs at two CTAs each)
  std::vector<int> launch_order(b->groups.size());
  for (size_t gi = 0; gi < b->groups.size(); ++gi) launch_order[gi] = (int)gi;
  std::stable_sort(launch_order.begin(), launch_order.end(),
                   [&](int p, int q) { return b->groups[p].work > b->groups[q].work; });
  for (int gi : launch_order) {
    auto& g = b->groups[gi];
    BatchCommon c;
    c.probs = b->dev + g.first;
    c.count = g.count;
    c.queue = b->queues + gi;
    c.precision = precision;
    c.jacobi = b->jacobi;
    const bool rr = precision == SEM_MIXED_RR;
    c.inner_tol = inner_tol > 0 ? inner_tol : (rr ? 0.3 : 1e-4);
    c.max_outer = max_outer > 0 ? max_outer : (rr ? 100 : 6);
    c.cluster_size = g.csize;
    c.ctas_per_sm = g.mb;
    c.clusters = g.clusters > 0 ? g.clusters
                 : std::max(1, (int)(max_clusters(g.n, g.csize, g.mb) * g.work / wtot));
    SEM_CUDA(cudaStreamWaitEvent(g.stream, b->start, 0));
    SEM_CHECK(launch_group(g.n, c, *g.ops, g.stream));
    SEM_CUDA(cudaEventRecord(g.done, g.stream));
    SEM_CUDA(cudaStreamWaitEvent(s, g.done, 0));
  }
  SEM_CUDA(cudaEventRecord(b->t1, s));
  std::vector<int> wanted(b->count);
  for (int j = 0; j < b->count; ++j) wanted[j] = q[j].maxiter;
  std::vector<BProb> wide_res;
  for (int j = 0; j < b->count; ++j)
    if (wanted[j] == -2) wide_res.push_back(q[j]);
  SEM_CUDA(cudaMemcpyAsync(q.data(), b->dev, sizeof(BProb) * b->count, cudaMemcpyDeviceToHost, s));
  SEM_CUDA(cudaStreamSynchronize(s));
  for (int j = 0, w = 0; j < b->count; ++j)  // the wide problems' results (the kernel skipped them)
    if (wanted[j] == -2) {
      const BProb& r = wide_res[w++];
      q[j].iters = r.iters;
      q[j].outer = r.outer;
      q[j].res_inf = r.res_inf;
      q[j].res0_inf = r.res0_inf;
      q[j].converged = r.converged;
      q[j].nan = r.nan;
    }
  float ms = 0.0f;
  SEM_CUDA(cudaEventElapsedTime(&ms, b->t0, b->t1));
  b->last_ms = ms;
  b->t_start.assign(b->count, 0);
  b->t_end.assign(b->count, 0);
  b->cluster.assign(b->count, -1);
  auto gi_of_slot = [&](int j) {
    int gi = 0;
    while (gi + 1 < (int)b->groups.size() && j >= b->groups[gi + 1].first) ++gi;
    return gi;
  };
  long long tmin = 0;
  bool any = false;
  for (int j = 0; j < b->count; ++j)
    if (wanted[j] >= 0 && (!any || q[j].t_start < tmin)) {
      tmin = q[j].t_start;
      any = true;
    }
  // the wide phase comes first (cluster -2), then the launches' problems
  const long long woff = (long long)(wide_total_ms * 1e6);
  long long wt = 0;
  for (int j = 0; j < b->count; ++j) {
    const int i = b->order[j];
    if (wanted[j] == -2) {
      const long long d = (long long)(b->wide_ms[i] * 1e6);
      b->t_start[i] = wt;
      b->t_end[i] = wt + d;
      b->cluster[i] = -2;
      wt += d;
      continue;
    }
    if (wanted[j] < 0) continue;  // left to the host's FP64 solve
    b->t_start[i] = q[j].t_start - tmin + woff;
    b->t_end[i] = q[j].t_end - tmin + woff;
    b->cluster[i] = gi_of_slot(j) * 65536 + q[j].cluster;
  }
  int bad = 0, nanc = 0;
  for (int j = 0; j < b->count; ++j) {
    const int i = b->order[j];
    // range guard: a problem outside the double-float window, one that ended
    // in NaN/Inf with a finite b, or one whose b lies below 2^-60, is solved
    // again by the native FP64 sem_pcg
    const double r0 = q[j].res0_inf;
    const bool finite_b = r0 == r0 && r0 <= 1.7976931348623157e308;
    const bool tiny_b = wanted[j] >= 0 && r0 > 0.0 && r0 < 0x1p-60;  // as pcg_guarded
    if (wanted[j] == -1 || (q[j].nan && finite_b) || tiny_b) {
      sem_pcg_opts o;
      std::memset(&o, 0, sizeof(o));
      o.nu = q[j].nu;
      o.k = q[j].k;
      o.precond = b->jacobi ? SEM_PRECOND_JACOBI : SEM_PRECOND_NONE;
      o.precision = SEM_F64;
      o.tol = tol[i];
      o.maxiter = (maxiter && maxiter[i] > 0) ? maxiter[i] : 0;
      o.path = SEM_PATH_CHUNKED;
      sem_solve_info si;
      std::memset(&si, 0, sizeof(si));
      const int st = sem_pcg(b->meshes[i], &o, rhs[i], x[i], &si, stream);
      if (st != SEM_OK && st != SEM_ERR_NOT_CONVERGED && st != SEM_ERR_NAN) return st;
      q[j].iters = si.iters;
      q[j].outer = si.outer;
      q[j].res_inf = si.res_inf;
      q[j].res0_inf = si.res0_inf;
      q[j].converged = si.converged;
      q[j].nan = st == SEM_ERR_NAN;
    }
    if (info) {
      info[i].iters = q[j].iters;
      info[i].outer = q[j].outer;
      info[i].res_inf = q[j].res_inf;
      info[i].res0_inf = q[j].res0_inf;
      info[i].converged = q[j].converged;
    }
    bad += !q[j].converged;
    nanc += q[j].nan;
  }
  if (nanc) return set_error(SEM_ERR_NAN, "%d of %d problems hit NaN/Inf", nanc, b->count);
  if (bad) return set_error(SEM_ERR_NOT_CONVERGED, "%d of %d problems reached maxiter", bad, b->count);
  return SEM_OK;
}

int sem_batch_group_count(const sem_batch_t* b) { return b ? (int)b->groups.size() : 0; }

int sem_batch_get_config(const sem_batch_t* b, sem_batch_group_config* cfg, int count) {
  if (!b || !cfg || count < (int)b->groups.size()) return set_error(SEM_ERR_BAD_ARG, "bad batch config arguments");
  for (size_t gi = 0; gi < b->groups.size(); ++gi) {
    const auto& g = b->groups[gi];
    cfg[gi].n = g.n;
    cfg[gi].problems = g.count;
    cfg[gi].cluster_size = g.csize;
    cfg[gi].ctas_per_sm = g.mb;
    cfg[gi].clusters = g.clusters;
  }
  return SEM_OK;
}

int sem_batch_set_config(sem_batch_t* b, const sem_batch_group_config* cfg, int count) {
  if (!b || !cfg || count != (int)b->groups.size()) return set_error(SEM_ERR_BAD_ARG, "one config per group");
  for (int gi = 0; gi < count; ++gi) {
    const auto& c = cfg[gi];
    if (c.n != b->groups[gi].n) return set_error(SEM_ERR_BAD_ARG, "config %d is for n = %d, the group has n = %d", gi, c.n, b->groups[gi].n);
    if (c.cluster_size != 2 && c.cluster_size != 4 && c.cluster_size != 8 && c.cluster_size != 16)
      return set_error(SEM_ERR_BAD_ARG, "cluster size %d (2, 4, 8 or 16)", c.cluster_size);
    if (c.ctas_per_sm != 1 && c.ctas_per_sm != 2) return set_error(SEM_ERR_BAD_ARG, "CTAs per SM %d (1 or 2)", c.ctas_per_sm);
    if (c.clusters < 0) return set_error(SEM_ERR_BAD_ARG, "negative cluster count");
    const int fit = max_clusters(c.n, c.cluster_size, c.ctas_per_sm);
    if (fit < 1) return set_error(SEM_ERR_UNSUPPORTED, "clusters of %d CTAs (%d per SM) do not fit for n = %d", c.cluster_size, c.ctas_per_sm, c.n);
  }
  for (int gi = 0; gi < count; ++gi) {
    auto& g = b->groups[gi];
    g.csize = cfg[gi].cluster_size;
    g.mb = cfg[gi].ctas_per_sm;
    g.clusters = cfg[gi].clusters;
  }
  return SEM_OK;
}

int sem_batch_get_order(const sem_batch_t* b, int* order, int count) {
  if (!b || !order || count != b->count) return set_error(SEM_ERR_BAD_ARG, "order takes one entry per problem");
  std::memcpy(order, b->order.data(), sizeof(int) * b->count);
  return SEM_OK;
}

int sem_batch_set_order(sem_batch_t* b, const int* order, int count) {
  if (!b || !order || count != b->count) return set_error(SEM_ERR_BAD_ARG, "order takes one entry per problem");
  // a permutation that keeps every group's problems in the group's slots
  std::vector<char> seen(b->count, 0);
  for (const auto& g : b->groups)
    for (int j = g.first; j < g.first + g.count; ++j) {
      const int i = order[j];
      if (i < 0 || i >= b->count || seen[i] || b->host[i].n != g.n)
        return set_error(SEM_ERR_BAD_ARG, "order[%d] = %d is not a problem of order n = %d", j, i, g.n);
      seen[i] = 1;
    }
  b->order.assign(order, order + count);
  return SEM_OK;
}

int sem_batch_get_wide(const sem_batch_t* b, int* wide, int count) {
  if (!b || !wide || count != b->count) return set_error(SEM_ERR_BAD_ARG, "wide takes one entry per problem");
  for (int i = 0; i < count; ++i) wide[i] = b->wide[i];
  return SEM_OK;
}

int sem_batch_set_wide(sem_batch_t* b, const int* wide, int count) {
  if (!b || !wide || count != b->count) return set_error(SEM_ERR_BAD_ARG, "wide takes one entry per problem");
  for (int i = 0; i < count; ++i) b->wide[i] = wide[i] != 0;
  return SEM_OK;
}

int sem_batch_timeline(const sem_batch_t* b, long long* start_ns, long long* end_ns, int* cluster, int count,
                       double* total_ms) {
  if (!b || count != b->count) return set_error(SEM_ERR_BAD_ARG, "the timeline has one entry per problem");
  if (b->t_start.empty()) return set_error(SEM_ERR_BAD_ARG, "no solve has run on this batch");
  for (int i = 0; i < count; ++i) {
    if (start_ns) start_ns[i] = b->t_start[i];
    if (end_ns) end_ns[i] = b->t_end[i];
    if (cluster) cluster[i] = b->cluster[i];
  }
  if (total_ms) *total_ms = b->last_ms;
  return SEM_OK;
}

}  // extern "C"

namespace {

// the batch's signature: device, arithmetic and every problem's shape,
// coefficients and tolerance
unsigned long long batch_signature(const sem_batch* b, const double* tol, const int* maxiter, int precision,
                                   double inner_tol, int max_outer) {
  unsigned long long h = 1469598103934665603ull;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  fnv(h, &sms, sizeof(sms));
  fnv(h, &precision, sizeof(precision));
  fnv(h, &inner_tol, sizeof(inner_tol));
  fnv(h, &max_outer, sizeof(max_outer));
  fnv(h, &b->jacobi, sizeof(b->jacobi));
  for (int i = 0; i < b->count; ++i) {
    const BProb& q = b->host[i];
    fnv(h, &q.n, sizeof(q.n));
    fnv(h, &q.Ex, sizeof(q.Ex));
    fnv(h, &q.Ey, sizeof(q.Ey));
    fnv(h, &q.topo, sizeof(q.topo));
    fnv(h, &q.nu, sizeof(q.nu));
    fnv(h, &q.k, sizeof(q.k));
    fnv(h, &tol[i], sizeof(double));
    const int mi = maxiter ? maxiter[i] : 0;
    fnv(h, &mi, sizeof(mi));
  }
  return h;
}

// cache file: one line per signature,
//   <hex signature> <groups> {n csize mb clusters}... <count> order... wide...
bool load_tuned(sem_batch* b, const char* path, unsigned long long sig) {
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  bool found = false;
  std::vector<sem_batch_group_config> cfg;
  std::vector<int> order, wide;
  char hex[32];
  while (std::fscanf(f, "%31s", hex) == 1) {
    unsigned long long s = std::strtoull(hex, nullptr, 16);
    int ng = 0;
    if (std::fscanf(f, "%d", &ng) != 1 || ng < 0 || ng > 64) break;
    std::vector<sem_batch_group_config> c(ng);
    bool ok = true;
    for (int gi = 0; gi < ng && ok; ++gi) {
      ok = std::fscanf(f, "%d %d %d %d", &c[gi].n, &c[gi].cluster_size, &c[gi].ctas_per_sm, &c[gi].clusters) == 4;
      c[gi].problems = 0;
    }
    int cnt = 0;
    ok = ok && std::fscanf(f, "%d", &cnt) == 1 && cnt >= 0 && cnt <= (1 << 24);
    if (!ok) break;
    std::vector<int> o(cnt), w(cnt);
    for (int j = 0; j < cnt && ok; ++j) ok = std::fscanf(f, "%d", &o[j]) == 1;
    for (int j = 0; j < cnt && ok; ++j) ok = std::fscanf(f, "%d", &w[j]) == 1;
    if (!ok) break;
    if (s == sig && ng == (int)b->groups.size() && cnt == b->count) {
      found = true;
      cfg = c;
      order = o;
      wide = w;
    }
  }
  std::fclose(f);
  if (!found) return false;
  for (int gi = 0; gi < (int)cfg.size(); ++gi) cfg[gi].problems = b->groups[gi].count;
  if (sem_batch_set_config(b, cfg.data(), (int)cfg.size()) != SEM_OK) return false;
  if (sem_batch_set_wide(b, wide.data(), (int)wide.size()) != SEM_OK) return false;
  return sem_batch_set_order(b, order.data(), (int)order.size()) == SEM_OK;
}

void store_tuned(const sem_batch* b, const char* path, unsigned long long sig) {
  FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%016llx %d", sig, (int)b->groups.size());
  for (const auto& g : b->groups) std::fprintf(f, " %d %d %d %d", g.n, g.csize, g.mb, g.clusters);
  std::fprintf(f, " %d", b->count);
  for (int i : b->order) std::fprintf(f, " %d", i);
  for (char w : b->wide) std::fprintf(f, " %d", (int)w);
  std::fprintf(f, "\n");
  std::fclose(f);
}

}  // namespace

extern "C" {

int sem_batch_autotune(sem_batch_t* b, const double* const* rhs, double* const* x, const double* tol,
                       const int* maxiter, int precision, double inner_tol, int max_outer, const char* cache_path,
                       int* runs_out, double* best_ms, sem_stream_t stream) {
  if (!b || !rhs || !x || !tol) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (runs_out) *runs_out = 0;
  const unsigned long long sig = batch_signature(b, tol, maxiter, precision, inner_tol, max_outer);
  if (cache_path && load_tuned(b, cache_path, sig)) {
    if (best_ms) *best_ms = 0.0;
    return SEM_OK;
  }
  const int G = (int)b->groups.size();
  // ---- measure every launch shape that fits every group, all groups alike,
  // with the default (work-proportional) cluster counts and the estimated order
  struct Opt {
    int csize, mb;
  };
  const Opt cand[] = {{8, 2}, {4, 2}, {16, 2}, {2, 2}, {8, 1}, {4, 1}, {16, 1}};
  const std::vector<int> order0 = b->order;
  b->wide.assign(b->count, 0);
  std::vector<Opt> opts;
  std::vector<double> wall;
  std::vector<std::vector<double>> dur;  // per option, per problem (creation order), ns
  int runs = 0;
  for (const Opt& o : cand) {
    bool fits = true;
    for (const auto& g : b->groups) fits = fits && max_clusters(g.n, o.csize, o.mb) > 0;
    if (!fits) continue;
    for (auto& g : b->groups) {
      g.csize = o.csize;
      g.mb = o.mb;
      g.clusters = 0;
    }
    b->order = order0;
    const int st = sem_batch_pcg(b, rhs, x, tol, maxiter, precision, inner_tol, max_outer, nullptr, stream);
    ++runs;
    if (st != SEM_OK && st != SEM_ERR_NOT_CONVERGED && st != SEM_ERR_NAN) return st;
    opts.push_back(o);
    wall.push_back(b->last_ms);
    std::vector<double> d(b->count);
    for (int i = 0; i < b->count; ++i) d[i] = (double)(b->t_end[i] - b->t_start[i]);
    dur.push_back(d);
  }
  if (opts.empty()) return set_error(SEM_ERR_UNSUPPORTED, "no batch launch shape fits");
  // ---- model: per group and shape, the makespan of k clusters under list
  // scheduling of the measured durations, largest first; a cluster costs the
  // fraction 1/fit of the device, fit being the clusters of that shape that
  // the device holds at once.  The smallest makespan T whose cheapest
  // per-group choices fit the device together wins.
  struct Choice {
    double T, cost;
    int opt, k;
  };
  std::vector<std::vector<Choice>> ch(G);
  std::vector<double> Ts;
  for (int gi = 0; gi < G; ++gi) {
    const auto& g = b->groups[gi];
    for (size_t oi = 0; oi < opts.size(); ++oi) {
      std::vector<double> d;
      for (int j = g.first; j < g.first + g.count; ++j) d.push_back(dur[oi][b->order[j]]);
      std::sort(d.begin(), d.end(), std::greater<double>());
      const int fit = max_clusters(g.n, opts[oi].csize, opts[oi].mb);
      const int kmax = std::min(g.count, fit);
      for (int k = 1; k <= kmax; ++k) {
        const double T = list_makespan(d, k);
        ch[gi].push_back({T, (double)k / fit, (int)oi, k});
        Ts.push_back(T);
      }
    }
  }
  std::sort(Ts.begin(), Ts.end());
  std::vector<Choice> pick(G);
  bool feasible = false;
  for (double T : Ts) {
    double total = 0.0;
    for (int gi = 0; gi < G; ++gi) {
      const Choice* best = nullptr;
      for (const Choice& c : ch[gi])
        if (c.T <= T && (!best || c.cost < best->cost)) best = &c;
      if (!best) {
        total = 1e300;
        break;
      }
      pick[gi] = *best;
      total += best->cost;
    }
    if (total <= 1.0) {
      feasible = true;
      break;
    }
  }
  // ---- the model's shapes, measured against the best uniform shape
  size_t best_uniform = 0;
  for (size_t oi = 1; oi < opts.size(); ++oi)
    if (wall[oi] < wall[best_uniform]) best_uniform = oi;
  double best = wall[best_uniform];
  std::vector<sem_batch_group_config> keep(G);
  std::vector<int> keep_order = order0;
  std::vector<char> keep_wide(b->count, 0);
  for (int gi = 0; gi < G; ++gi)
    keep[gi] = {b->groups[gi].n, b->groups[gi].count, opts[best_uniform].csize, opts[best_uniform].mb, 0};
  // per group: the shape (option), its cluster count and the durations the model uses
  std::vector<int> g_opt(G, (int)best_uniform), g_k(G, 0);
  auto apply_shapes = [&](const std::vector<char>& wide) {
    std::vector<int> ord = order0;
    for (int gi = 0; gi < G; ++gi) {
      const auto& g = b->groups[gi];
      const auto& d = dur[g_opt[gi]];
      std::stable_sort(ord.begin() + g.first, ord.begin() + g.first + g.count,
                       [&](int p, int q) { return d[p] > d[q]; });
      auto& gg = b->groups[gi];
      gg.csize = opts[g_opt[gi]].csize;
      gg.mb = opts[g_opt[gi]].mb;
      gg.clusters = g_k[gi];
    }
    b->order = ord;
    b->wide.assign(wide.begin(), wide.end());
  };
  auto run_and_keep = [&]() -> int {
    const int st = sem_batch_pcg(b, rhs, x, tol, maxiter, precision, inner_tol, max_outer, nullptr, stream);
    ++runs;
    if (st != SEM_OK && st != SEM_ERR_NOT_CONVERGED && st != SEM_ERR_NAN) return st;
    if (b->last_ms < best) {
      best = b->last_ms;
      keep_order = b->order;
      keep_wide = b->wide;
      for (int gi = 0; gi < G; ++gi)
        keep[gi] = {b->groups[gi].n, b->groups[gi].count, b->groups[gi].csize, b->groups[gi].mb, b->groups[gi].clusters};
    }
    return SEM_OK;
  };
  if (feasible) {
    for (int gi = 0; gi < G; ++gi) {
      g_opt[gi] = pick[gi].opt;
      g_k[gi] = pick[gi].k;
    }
    apply_shapes(std::vector<char>(b->count, 0));
    SEM_CHECK(run_and_keep());
  }
  // ---- wide problems: the candidates are the problems whose clusters took
  // longest; one solve puts them all on the whole GPU and times each, then
  // the model picks how many of them (largest first) to keep wide:
  // sum of their whole-GPU times + the makespan of the rest on the clusters
  std::vector<int> byd(b->count);
  for (int i = 0; i < b->count; ++i) byd[i] = i;
  std::vector<double> dmodel(b->count);
  for (int gi = 0; gi < G; ++gi)
    for (int j = b->groups[gi].first; j < b->groups[gi].first + b->groups[gi].count; ++j)
      dmodel[order0[j]] = dur[g_opt[gi]][order0[j]];
  std::stable_sort(byd.begin(), byd.end(), [&](int p, int q) { return dmodel[p] > dmodel[q]; });
  const int K = std::min(b->count, 32);
  std::vector<char> cand_wide(b->count, 0);
  for (int r = 0; r < K; ++r) cand_wide[byd[r]] = 1;
  apply_shapes(cand_wide);
  SEM_CHECK(run_and_keep());
  std::vector<double> wms(b->wide_ms.begin(), b->wide_ms.end());
  auto group_of = [&](int i) {
    for (int gi = 0; gi < G; ++gi)
      if (b->host[i].n == b->groups[gi].n) return gi;
    return 0;
  };
  double bestT = 1e300;
  int bestk = 0;
  for (int k = 0; k <= K; ++k) {
    double T = 0.0;
    for (int r = 0; r < k; ++r) T += wms[byd[r]] * 1e6;
    std::vector<std::vector<double>> rest(G);
    std::vector<char> isw(b->count, 0);
    for (int r = 0; r < k; ++r) isw[byd[r]] = 1;
    for (int i = 0; i < b->count; ++i)
      if (!isw[i]) rest[group_of(i)].push_back(dmodel[i]);
    double M = 0.0;
    for (int gi = 0; gi < G; ++gi) {
      std::sort(rest[gi].begin(), rest[gi].end(), std::greater<double>());
      const auto& o = opts[g_opt[gi]];
      int kc = g_k[gi];
      if (kc == 0) {  // the default share the launch would take
        double wtot = 0.0;
        for (const auto& g : b->groups) wtot += g.work;
        kc = std::max(1, (int)(max_clusters(b->groups[gi].n, o.csize, o.mb) * b->groups[gi].work / wtot));
      }
      M = std::max(M, list_makespan(rest[gi], std::max(1, kc)));
    }
    T += M;
    if (T < bestT) {
      bestT = T;
      bestk = k;
    }
  }
  if (bestk > 0 && bestk < K) {
    std::vector<char> w(b->count, 0);
    for (int r = 0; r < bestk; ++r) w[byd[r]] = 1;
    apply_shapes(w);
    SEM_CHECK(run_and_keep());
  }
  SEM_CHECK(sem_batch_set_config(b, keep.data(), G));
  b->order = keep_order;
  b->wide = keep_wide;
  if (cache_path) store_tuned(b, cache_path, sig);
  if (runs_out) *runs_out = runs;
  if (best_ms) *best_ms = best;
  return SEM_OK;
}

}  // extern "C"
