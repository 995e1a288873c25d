// The fused operator on HOST buffers: mask(QQ'(hlmz(u))) for a field that
// lives in host memory and a result that goes back to it.
//
// The field moves in and out in slabs of element-tile rows (whole columns of
// the column-major layout, so each slab is one contiguous copy).  The copy
// in of slab k+1 overlaps the operator kernel of slab k, and the copy out of
// slab k starts once its columns are final, which is after the fixup of
// slab k+1 has summed the copies on their shared interface.  Copies in and
// out run on two streams of their own; the caller's stream joins them at the
// end.  The result is bit-identical to sem_hlmz on device buffers: the same
// tiles are computed, and every interface point is summed once, in the same
// order, by the fixup of the slab that holds its highest copy column.
#include <cstring>

#include "sem_internal.cuh"

namespace sem {

struct HostPipe {
  static constexpr int kMaxSlabs = 16;
  cudaStream_t in = nullptr, out = nullptr;
  cudaEvent_t start = nullptr, done = nullptr;
  cudaEvent_t ev_in[kMaxSlabs] = {}, ev_fix[kMaxSlabs] = {};
  double* u = nullptr;
  double* o = nullptr;
  long long cap = 0;  // doubles per buffer
};

namespace {

int make_pipe(HostPipe* p) {
  SEM_CUDA(cudaStreamCreateWithFlags(&p->in, cudaStreamNonBlocking));
  SEM_CUDA(cudaStreamCreateWithFlags(&p->out, cudaStreamNonBlocking));
  SEM_CUDA(cudaEventCreateWithFlags(&p->start, cudaEventDisableTiming));
  SEM_CUDA(cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming));
  for (int i = 0; i < HostPipe::kMaxSlabs; ++i) {
    SEM_CUDA(cudaEventCreateWithFlags(&p->ev_in[i], cudaEventDisableTiming));
    SEM_CUDA(cudaEventCreateWithFlags(&p->ev_fix[i], cudaEventDisableTiming));
  }
  return SEM_OK;
}

int get_pipe(sem_mesh* m, long long L, HostPipe** out) {
  HostPipe* p = static_cast<HostPipe*>(m->host_pipe);
  if (!p) {
    p = new HostPipe();
    m->host_pipe = p;
    SEM_CHECK(make_pipe(p));
  }
  if (p->cap < L) {
    SEM_CUDA(cudaDeviceSynchronize());  // earlier calls may still use the old buffers
    if (p->u) cudaFree(p->u);
    if (p->o) cudaFree(p->o);
    p->u = p->o = nullptr;
    p->cap = 0;
    SEM_CUDA(cudaMalloc(&p->u, sizeof(double) * (size_t)L));
    SEM_CUDA(cudaMalloc(&p->o, sizeof(double) * (size_t)L));
    p->cap = L;
  }
  *out = p;
  return SEM_OK;
}

}  // namespace

void free_host_pipe(sem_mesh* m) {
  HostPipe* p = static_cast<HostPipe*>(m->host_pipe);
  if (!p) return;
  if (p->in) cudaStreamSynchronize(p->in);
  if (p->out) cudaStreamSynchronize(p->out);
  if (p->u) cudaFree(p->u);
  if (p->o) cudaFree(p->o);
  for (int i = 0; i < HostPipe::kMaxSlabs; ++i) {
    if (p->ev_in[i]) cudaEventDestroy(p->ev_in[i]);
    if (p->ev_fix[i]) cudaEventDestroy(p->ev_fix[i]);
  }
  if (p->start) cudaEventDestroy(p->start);
  if (p->done) cudaEventDestroy(p->done);
  if (p->in) cudaStreamDestroy(p->in);
  if (p->out) cudaStreamDestroy(p->out);
  delete p;
  m->host_pipe = nullptr;
}

}  // namespace sem

using namespace sem;

extern "C" int sem_hlmz_host(sem_mesh_t* m, const double* nu_field, double nu, double k,
                             const double* u_host, double* out_host, unsigned flags, int slabs,
                             sem_stream_t stream) {
  if (!m || !u_host || !out_host) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (u_host == out_host) return set_error(SEM_ERR_BAD_ARG, "output must not alias the input");
  if (slabs < 0) return set_error(SEM_ERR_BAD_ARG, "slabs must be >= 0");
  int dev = -1;
  SEM_CUDA(cudaGetDevice(&dev));
  if (dev != m->device) return set_error(SEM_ERR_BAD_ARG, "mesh handle lives on device %d", m->device);
  cudaStream_t s = (cudaStream_t)stream;
  const Grid& g = m->g;
  const long long NX = g.NX, L = g.NX * g.NY;
  if (m->precision == SEM_F64_DF) SEM_CHECK(ensure_df_geometry(m, s));
  HostPipe* p = nullptr;
  SEM_CHECK(get_pipe(m, L, &p));

  int TX = 1, TY = 1;
  tile_shape_of(g.n, &TX, &TY);
  const int tiles_y = (g.Ey + TY - 1) / TY;
  int K = slabs > 0 ? slabs : 8;
  if (K > HostPipe::kMaxSlabs) K = HostPipe::kMaxSlabs;
  if (K > tiles_y) K = tiles_y;
  long long t0[HostPipe::kMaxSlabs + 1], c0[HostPipe::kMaxSlabs + 1];
  for (int i = 0; i <= K; ++i) {
    t0[i] = (long long)tiles_y * i / K;
    const long long ey = t0[i] * TY < g.Ey ? t0[i] * TY : g.Ey;
    c0[i] = ey * g.n;
  }

  unsigned mode = g.topo | M_STIFF | M_MASS;
  if (flags & SEM_GS) mode |= M_GS;
  if ((flags & SEM_MASK) && m->has_bc) mode |= M_MASK;
  if (nu_field) mode |= M_NU;
  if (k == 0.0) mode &= ~M_MASS;
  ApplyCall c;
  std::memset(&c, 0, sizeof(c));
  c.u = p->u;
  c.out = p->o;
  c.G11 = m->G11;
  c.G12 = m->G12;
  c.G22 = m->G22;
  c.B = m->B;
  c.nu = nu_field;
  c.nu_s = nu;
  c.k_s = k;
  c.mode = mode;
  c.precision = m->precision;
  c.variant = m->variant[m->precision];
  c.Gdf = m->Gdf;

  // the copies start after everything queued on the caller's stream
  SEM_CUDA(cudaEventRecord(p->start, s));
  SEM_CUDA(cudaStreamWaitEvent(p->in, p->start, 0));
  SEM_CUDA(cudaStreamWaitEvent(p->out, p->start, 0));
  for (int i = 0; i < K; ++i) {
    const size_t bytes = sizeof(double) * (size_t)((c0[i + 1] - c0[i]) * NX);
    SEM_CUDA(cudaMemcpyAsync(p->u + c0[i] * NX, u_host + c0[i] * NX, bytes, cudaMemcpyHostToDevice, p->in));
    SEM_CUDA(cudaEventRecord(p->ev_in[i], p->in));
  }
  const bool gs = (mode & M_GS) != 0;
  for (int i = 0; i < K; ++i) {
    SEM_CUDA(cudaStreamWaitEvent(s, p->ev_in[i], 0));
    c.ty0 = (int)t0[i];
    c.tyn = (int)(t0[i + 1] - t0[i]);
    const long long key_hi = i + 1 < K ? c0[i + 1] : (1LL << 62);
    SEM_CHECK(launch_apply_window(g, m->ops, c, c0[i], key_hi, s));
    SEM_CUDA(cudaEventRecord(p->ev_fix[i], s));
  }
  // slab i is final after the fixup of slab i + 1 (their shared interface);
  // with a periodic y direction slab 0 also waits for the last slab (the wrap)
  const bool wrap = gs && (mode & M_PERY) && K > 1;
  for (int q = 0; q < K; ++q) {
    const int i = wrap ? (q + 1) % K : q;  // slab 0 last when it waits for the wrap
    int after = gs ? (i + 1 < K ? i + 1 : K - 1) : i;
    if (wrap && i == 0) after = K - 1;
    SEM_CUDA(cudaStreamWaitEvent(p->out, p->ev_fix[after], 0));
    const size_t bytes = sizeof(double) * (size_t)((c0[i + 1] - c0[i]) * NX);
    SEM_CUDA(cudaMemcpyAsync(out_host + c0[i] * NX, p->o + c0[i] * NX, bytes, cudaMemcpyDeviceToHost, p->out));
  }
  SEM_CUDA(cudaEventRecord(p->done, p->out));
  SEM_CUDA(cudaStreamWaitEvent(s, p->done, 0));
  return SEM_OK;
}
