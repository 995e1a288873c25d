// The fused operator on HOST buffers: mask(QQ'(hlmz(u))) for a field that
// lives in host memory and a result that goes back to it.
//
// Direct access (slabs = SEM_HOST_DIRECT): the operator kernel reads u_host
// and writes out_host in place over the coherent CPU-GPU link (about 200 GB/s
// each way on GB300), and the cross-tile fixup finishes the interface points
// there.  Measured on the 256^2, N=8 apply it is slower than the slab pipeline
// below (0.53 against 0.46 ms in FP64): every CTA waits for its inputs from the
// link at its start.  It serves buffers the copy engines cannot reach in place
// (pageable memory read through the host page tables).  Otherwise:
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

// Whether the device can read and write p in place: pinned or registered host
// memory mapped at the same address (unified addressing), or any host memory
// when `pageable` is set and the device reads pageable memory through the host
// page tables (Grace-Blackwell's coherent CPU-GPU link).
bool device_can_address(const void* p, bool pageable) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeHost) return a.devicePointer == p;
  if (a.type == cudaMemoryTypeUnregistered && pageable) {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) return false;
    return v != 0;
  }
  return false;
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
  if (slabs < SEM_HOST_DIRECT) return set_error(SEM_ERR_BAD_ARG, "slabs must be >= SEM_HOST_DIRECT (-1)");
  if ((flags & SEM_NU_IN_G) && !nu_field) return set_error(SEM_ERR_BAD_ARG, "SEM_NU_IN_G needs nu_field");
  int dev = -1;
  SEM_CUDA(cudaGetDevice(&dev));
  if (dev != m->device) return set_error(SEM_ERR_BAD_ARG, "mesh handle lives on device %d", m->device);
  cudaStream_t s = (cudaStream_t)stream;
  const Grid& g = m->g;
  const long long NX = g.NX, L = g.NX * g.NY;
  if (m->precision == SEM_F64_DF) SEM_CHECK(ensure_df_geometry(m, s));

  unsigned mode = g.topo | M_STIFF | M_MASS;
  if (flags & SEM_GS) mode |= M_GS;
  if ((flags & SEM_MASK) && m->has_bc) mode |= M_MASK;
  if (nu_field) mode |= (flags & SEM_NU_IN_G) ? M_NUG : M_NU;
  if (k == 0.0) mode &= ~M_MASS;
  ApplyCall c;
  std::memset(&c, 0, sizeof(c));
  c.G11 = m->G11;
  c.G12 = m->G12;
  c.G22 = m->G22;
  c.B = m->B;
  c.nu = nu_field;
  c.nu_s = (flags & SEM_NU_IN_G) ? 1.0 : nu;
  c.k_s = k;
  c.mode = mode;
  c.precision = m->precision;
  c.variant = m->variant[m->precision];
  c.Gdf = m->Gdf;
  SEM_CHECK(use_kB(m, c, s));
  SEM_CHECK(arm_range_guard(m, c));

  // direct access: the operator kernels read u_host and write out_host over
  // the CPU-GPU link while they compute (no staging buffers, no copy engines)
  const bool direct =
      slabs == SEM_HOST_DIRECT && device_can_address(u_host, true) && device_can_address(out_host, true);
  if (slabs == SEM_HOST_DIRECT && !direct)
    return set_error(SEM_ERR_UNSUPPORTED, "the device cannot address these host buffers in place");
  if (direct) {
    c.u = u_host;
    c.out = out_host;
    if (c.variant == 5) c.variant = 2;  // the cross-tile sums run in the fixup launch
    return launch_apply(g, m->ops, c, s);
  }

  HostPipe* p = nullptr;
  SEM_CHECK(get_pipe(m, L, &p));
  c.u = p->u;
  c.out = p->o;

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
  if (!c.rflag) return SEM_OK;
  // range guard: a flagged call is recomputed in native FP64 over the whole
  // field from the uploaded input, after every slab has been copied out; the
  // re-run writes the host buffer in place when the device can address it
  c.u = p->u;
  if (device_can_address(out_host, false)) {
    c.out = out_host;
    return launch_guard_rerun(g, m->ops, c, s);
  }
  unsigned word = 0;
  SEM_CUDA(cudaMemcpyAsync(&word, c.rflag, sizeof(word), cudaMemcpyDeviceToHost, s));
  SEM_CUDA(cudaStreamSynchronize(s));
  if (word != c.rtag) return SEM_OK;
  c.out = p->o;
  SEM_CHECK(launch_guard_rerun(g, m->ops, c, s));
  SEM_CUDA(cudaMemcpyAsync(out_host, p->o, sizeof(double) * (size_t)L, cudaMemcpyDeviceToHost, s));
  SEM_CUDA(cudaStreamSynchronize(s));
  return SEM_OK;
}
