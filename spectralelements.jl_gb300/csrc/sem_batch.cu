// Host side of the batched solver: per-problem workspace and Jacobi set-up,
// problems grouped by polynomial order (largest estimated work first inside a
// group), and one persistent cluster launch per order on its own stream, all
// joined back into the caller's stream.
#include <algorithm>
#include <cstring>
#include <vector>

#include "sem_batch_kernel.cuh"

namespace sem {
int launch_batch_group_a(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s);
int launch_batch_group_b(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s);
int launch_batch_group_c(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s);
int batch_diag(sem_mesh* m, double nu, double k, double* dinv, double* tmp, cudaStream_t s);

namespace {
int launch_group(int n, const BatchCommon& c, const OperatorSet& ops, cudaStream_t s) {
  if (n <= 6) return launch_batch_group_a(n, c, ops, s);
  if (n <= 9) return launch_batch_group_b(n, c, ops, s);
  return launch_batch_group_c(n, c, ops, s);
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
  if (e != cudaSuccess) {
    sem_batch_destroy(b);
    return cuda_error(e, "batch allocation");
  }
  b->host.resize(count);
  b->meshes.assign(meshes, meshes + count);
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
  }
  SEM_CUDA(cudaMemcpyAsync(b->dev, q.data(), sizeof(BProb) * b->count, cudaMemcpyHostToDevice, s));
  SEM_CUDA(cudaMemsetAsync(b->queues, 0, sizeof(int) * (kBatchMaxN + 1), s));
  SEM_CUDA(cudaEventRecord(b->start, s));
  double wtot = 0.0;
  for (auto& g : b->groups) wtot += g.work;
  int sms = 0;
  SEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
  const int budget = std::max(1, sms * kBatchCtasPerSm / kCluster);  // resident clusters
  for (size_t gi = 0; gi < b->groups.size(); ++gi) {
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
    c.clusters = b->groups.size() == 1 ? 0 : std::max(1, (int)(budget * g.work / wtot + 0.5));
    SEM_CUDA(cudaStreamWaitEvent(g.stream, b->start, 0));
    SEM_CHECK(launch_group(g.n, c, *g.ops, g.stream));
    SEM_CUDA(cudaEventRecord(g.done, g.stream));
    SEM_CUDA(cudaStreamWaitEvent(s, g.done, 0));
  }
  std::vector<int> wanted(b->count);
  for (int j = 0; j < b->count; ++j) wanted[j] = q[j].maxiter;
  SEM_CUDA(cudaMemcpyAsync(q.data(), b->dev, sizeof(BProb) * b->count, cudaMemcpyDeviceToHost, s));
  SEM_CUDA(cudaStreamSynchronize(s));
  int bad = 0, nanc = 0;
  for (int j = 0; j < b->count; ++j) {
    const int i = b->order[j];
    // range guard: a problem outside the double-float window, or one that ended
    // in NaN/Inf with a finite b, is solved again by the native FP64 sem_pcg
    const double r0 = q[j].res0_inf;
    const bool finite_b = r0 == r0 && r0 <= 1.7976931348623157e308;
    if (wanted[j] < 0 || (q[j].nan && finite_b)) {
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

}  // extern "C"
