// C ABI entry points: errors, mesh handles, operators.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "sem_internal.cuh"

namespace sem {

static thread_local char g_err[512] = "";

int set_error(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return status;
}

int cuda_error(cudaError_t e, const char* what) {
  const int st = (e == cudaErrorMemoryAllocation) ? SEM_ERR_NO_MEMORY : SEM_ERR_CUDA;
  return set_error(st, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

static int check_device(const sem_mesh* m) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  if (dev != m->device)
    return set_error(SEM_ERR_BAD_ARG, "mesh handle lives on device %d but device %d is current",
                     m->device, dev);
  return SEM_OK;
}

static unsigned bc_bits(const char* bc) {
  unsigned b = 0;
  if (bc[0] == 'D') b |= M_DXMIN;
  if (bc[1] == 'D') b |= M_DXMAX;
  if (bc[2] == 'D') b |= M_DYMIN;
  if (bc[3] == 'D') b |= M_DYMAX;
  return b;
}

static int valid_bc(const char* bc) {
  for (int i = 0; i < 4; ++i)
    if (bc[i] != 'D' && bc[i] != 'N') return 0;
  return 1;
}

static unsigned op_mode(const sem_mesh* m, unsigned flags) {
  unsigned mode = m->g.topo;
  if (flags & SEM_GS) mode |= M_GS;
  if ((flags & SEM_MASK) && m->has_bc) mode |= M_MASK;
  return mode;
}

int upload_line_info(sem_mesh* m) {
  const int64_t NX = m->g.NX, NY = m->g.NY;
  if (!m->info) SEM_CUDA(cudaMalloc(&m->info, (size_t)(NX + NY)));
  unsigned char* h = (unsigned char*)std::malloc((size_t)(NX + NY));
  const unsigned t = m->g.topo;
  const bool bc = m->has_bc;
  for (int64_t r = 0; r < NX; ++r)
    h[r] = line_info(r, m->g.n, m->g.Ex, (t & M_PERX) != 0, bc && (t & M_DXMIN), bc && (t & M_DXMAX));
  for (int64_t c = 0; c < NY; ++c)
    h[NX + c] = line_info(c, m->g.n, m->g.Ey, (t & M_PERY) != 0, bc && (t & M_DYMIN), bc && (t & M_DYMAX));
  cudaError_t e = cudaMemcpy(m->info, h, (size_t)(NX + NY), cudaMemcpyHostToDevice);
  std::free(h);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemcpy(line info)");
  m->g.rinfo = m->info;
  m->g.cinfo = m->info + NX;
  return SEM_OK;
}

}  // namespace sem

using namespace sem;

extern "C" {

const char* sem_last_error(void) { return g_err; }

int sem_abi_version(void) { return SEM_ABI_VERSION; }

int sem_mesh_create(const sem_mesh_desc* d, sem_mesh_t** out) {
  if (!d || !out) return set_error(SEM_ERR_BAD_ARG, "NULL descriptor or output");
  *out = nullptr;
  if (d->nr < 2 || d->ns < 2 || d->Ex < 1 || d->Ey < 1)
    return set_error(SEM_ERR_BAD_ARG, "bad mesh sizes nr=%d ns=%d Ex=%d Ey=%d", d->nr, d->ns,
                     d->Ex, d->Ey);
  if (d->nr != d->ns)
    return set_error(SEM_ERR_UNSUPPORTED, "nr != ns is not served (nr=%d ns=%d)", d->nr, d->ns);
  if (d->nr > kMaxN)
    return set_error(SEM_ERR_UNSUPPORTED, "at most %d GLL points per direction", kMaxN);
  if (!d->Dr || !d->Ds || !d->wr || !d->ws || !d->x || !d->y)
    return set_error(SEM_ERR_BAD_ARG, "Dr, Ds, wr, ws, x and y are required");
  const int ng = (d->G11 != nullptr) + (d->G12 != nullptr) + (d->G22 != nullptr) + (d->B != nullptr);
  if (ng != 0 && ng != 4) return set_error(SEM_ERR_BAD_ARG, "give all of G11, G12, G22, B or none");
  if (d->bc && !valid_bc(d->bc)) return set_error(SEM_ERR_BAD_ARG, "bc must be 4 chars of 'D'/'N'");
  int dev = 0;
  SEM_CUDA(cudaGetDevice(&dev));

  const int n = d->nr;
  OperatorSet* ops = nullptr;
  SEM_CHECK(make_operator_set(d->Dr, d->Ds, n, &ops));

  sem_mesh* m = (sem_mesh*)std::calloc(1, sizeof(sem_mesh));
  m->device = dev;
  m->g.n = n;
  m->g.Ex = d->Ex;
  m->g.Ey = d->Ey;
  m->g.NX = (int64_t)n * d->Ex;
  m->g.NY = (int64_t)n * d->Ey;
  m->g.topo = (d->periodic_x ? M_PERX : 0u) | (d->periodic_y ? M_PERY : 0u);
  m->has_bc = d->bc != nullptr;
  if (d->bc) m->g.topo |= bc_bits(d->bc);
  m->precision = SEM_F64_DF;
  // default kernel variants until sem_mesh_autotune measures them: the
  // in-place double-float kernel on pre-split geometry (2) and the staged FP32
  // kernel (1) are the fastest on a GB300 across the orders measured; the
  // native FP64 variants lie within 2 % of each other
  m->variant[SEM_F64_DF] = 2;
  m->variant[SEM_F32] = 1;
  m->ops = ops;
  m->Dr_h = (double*)std::malloc(sizeof(double) * n * n);
  m->Ds_h = (double*)std::malloc(sizeof(double) * n * n);
  m->wr_h = (double*)std::malloc(sizeof(double) * n);
  m->ws_h = (double*)std::malloc(sizeof(double) * n);
  std::memcpy(m->Dr_h, d->Dr, sizeof(double) * n * n);
  std::memcpy(m->Ds_h, d->Ds, sizeof(double) * n * n);
  std::memcpy(m->wr_h, d->wr, sizeof(double) * n);
  std::memcpy(m->ws_h, d->ws, sizeof(double) * n);

  const long long L = m->g.NX * m->g.NY;
  const size_t bytes = sizeof(double) * (size_t)L;
  double* blk = nullptr;
  cudaError_t e = cudaMalloc(&blk, 6 * bytes);
  if (e != cudaSuccess) {
    sem_mesh_destroy(m);
    return cuda_error(e, "cudaMalloc(mesh geometry)");
  }
  m->x = blk;
  m->y = blk + L;
  m->B = blk + 2 * L;
  m->G11 = blk + 3 * L;
  m->G12 = blk + 4 * L;
  m->G22 = blk + 5 * L;
  int st = SEM_OK;
  if ((e = cudaMemcpy(m->x, d->x, bytes, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(m->y, d->y, bytes, cudaMemcpyHostToDevice)) != cudaSuccess) {
    st = cuda_error(e, "cudaMemcpy(grid)");
  } else if (ng == 4) {
    if ((e = cudaMemcpy(m->B, d->B, bytes, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m->G11, d->G11, bytes, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m->G12, d->G12, bytes, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m->G22, d->G22, bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
      st = cuda_error(e, "cudaMemcpy(geometry)");
  } else {
    st = build_geometry(m, d->x, d->y, 0);
    if (st == SEM_OK && (e = cudaStreamSynchronize(0)) != cudaSuccess)
      st = cuda_error(e, "geometry kernel");
  }
  if (st == SEM_OK) st = upload_line_info(m);
  // the pre-split geometry of the double-float kernels, made once here so
  // that every double-float apply and solve finds it
  if (st == SEM_OK) st = ensure_df_geometry(m, 0);
  if (st == SEM_OK && (e = cudaStreamSynchronize(0)) != cudaSuccess) st = cuda_error(e, "geometry split");
  if (st != SEM_OK) {
    sem_mesh_destroy(m);
    return st;
  }
  *out = m;
  return SEM_OK;
}

int sem_mesh_destroy(sem_mesh_t* m) {
  if (!m) return SEM_OK;
  if (m->x) cudaFree(m->x);
  if (m->G11_f) cudaFree(m->G11_f);
  if (m->Gdf) cudaFree(m->Gdf);
  if (m->fix_ctr) cudaFree(m->fix_ctr);
  if (m->kB) cudaFree(m->kB);
  if (m->rflag) cudaFree(m->rflag);
  free_graph_cache(m);
  free_host_pipe(m);
  if (m->ws) cudaFree(m->ws);
  if (m->info) cudaFree(m->info);
  if (m->ops) free_operator_set(m->ops);
  std::free(m->Dr_h);
  std::free(m->Ds_h);
  std::free(m->wr_h);
  std::free(m->ws_h);
  std::free(m);
  return SEM_OK;
}

int sem_mesh_set_bc(sem_mesh_t* m, const char* bc) {
  if (!m) return set_error(SEM_ERR_BAD_ARG, "NULL mesh");
  m->g.topo &= ~(M_DXMIN | M_DXMAX | M_DYMIN | M_DYMAX);
  if (!bc) {
    m->has_bc = false;
    return upload_line_info(m);
  }
  if (!valid_bc(bc)) return set_error(SEM_ERR_BAD_ARG, "bc must be 4 chars of 'D'/'N'");
  m->g.topo |= bc_bits(bc);
  m->has_bc = true;
  return upload_line_info(m);
}

int sem_mesh_set_precision(sem_mesh_t* m, int precision) {
  if (!m) return set_error(SEM_ERR_BAD_ARG, "NULL mesh");
  if (precision != SEM_F64 && precision != SEM_F64_DF)
    return set_error(SEM_ERR_BAD_ARG, "fused FP64 operators take SEM_F64 or SEM_F64_DF");
  m->precision = precision;
  return SEM_OK;
}

int sem_mesh_set_variant(sem_mesh_t* m, int precision, int variant) {
  if (!m) return set_error(SEM_ERR_BAD_ARG, "NULL mesh");
  if (precision < SEM_F64 || precision > SEM_F32) return set_error(SEM_ERR_BAD_ARG, "bad precision");
  if (variant < 0 || variant >= kVariants) return set_error(SEM_ERR_BAD_ARG, "bad variant");
  if ((precision == SEM_F64_DF && variant >= 2) || variant == 5 || variant == 6) {
    SEM_CHECK(check_device(m));
    if (precision == SEM_F64_DF) SEM_CHECK(ensure_df_geometry(m, nullptr));
    if (variant == 5) SEM_CHECK(ensure_fix_counters(m));
    // the TMA kernel's timeout word, made here rather than inside a later
    // launch that a CUDA-graph capture (the CG chunks) may enclose
    if (variant == 6 && !wait_timeout_word(true)) return set_error(SEM_ERR_CUDA, "cannot make the TMA timeout word");
    SEM_CUDA(cudaStreamSynchronize(nullptr));  // later launches may use any stream
  }
  m->variant[precision] = variant;
  return SEM_OK;
}

int sem_mesh_autotune(sem_mesh_t* m, int precision, double* ms_out, int* chosen) {
  if (!m) return set_error(SEM_ERR_BAD_ARG, "NULL mesh");
  if (precision < SEM_F64 || precision > SEM_F32) return set_error(SEM_ERR_BAD_ARG, "bad precision");
  SEM_CHECK(check_device(m));
  cudaStream_t s = nullptr;
  SEM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const long long L = m->g.NX * m->g.NY;
  const bool f32 = precision == SEM_F32;
  if (f32) SEM_CHECK(ensure_f32_geometry(m, s));
  if (precision == SEM_F64_DF) SEM_CHECK(ensure_df_geometry(m, s));
  SEM_CHECK(ensure_fix_counters(m));
  void* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int st = SEM_OK;
  double best = 1e30;
  int bestv = 0;
  cudaError_t e = cudaMalloc(&out, (size_t)L * (f32 ? 4 : 8));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) st = cuda_error(e, "autotune set-up");
  ApplyCall c;
  std::memset(&c, 0, sizeof(c));
  c.u = f32 ? (const void*)m->G11_f : (const void*)m->x;  // any smooth non-zero field
  c.out = out;
  c.G11 = f32 ? (const void*)m->G11_f : (const void*)m->G11;
  c.G12 = f32 ? (const void*)m->G12_f : (const void*)m->G12;
  c.G22 = f32 ? (const void*)m->G22_f : (const void*)m->G22;
  c.B = f32 ? (const void*)m->B_f : (const void*)m->B;
  c.Gdf = m->Gdf;
  c.ctr = m->fix_ctr;
  c.nu_s = 0.5;
  c.k_s = 1.0;
  c.mode = m->g.topo | M_STIFF | M_MASS | M_GS | (m->has_bc ? M_MASK : 0u);
  c.precision = precision;
  for (int v = 0; v < kVariants && st == SEM_OK; ++v) {
    c.variant = v;
    for (int w = 0; w < 2 && st == SEM_OK; ++w) st = launch_apply(m->g, m->ops, c, s);
    if (st != SEM_OK) break;
    if ((e = cudaEventRecord(e0, s)) != cudaSuccess) { st = cuda_error(e, "event"); break; }
    for (int r = 0; r < 5 && st == SEM_OK; ++r) st = launch_apply(m->g, m->ops, c, s);
    if (st != SEM_OK) break;
    float ms = 0.f;
    if ((e = cudaEventRecord(e1, s)) != cudaSuccess || (e = cudaEventSynchronize(e1)) != cudaSuccess ||
        (e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) {
      st = cuda_error(e, "autotune timing");
      break;
    }
    const double t = ms / 5.0;
    if (ms_out) ms_out[v] = t;
    if (t < best) {
      best = t;
      bestv = v;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  cudaStreamDestroy(s);
  if (st != SEM_OK) return st;
  m->variant[precision] = bestv;
  if (chosen) *chosen = bestv;
  return SEM_OK;
}

int sem_mesh_field(sem_mesh_t* m, int which, double* out, sem_stream_t stream) {
  if (!m || !out) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  SEM_CHECK(check_device(m));
  return export_field(m, which, out, (cudaStream_t)stream);
}

int sem_mesh_dims(const sem_mesh_t* m, int64_t* nx, int64_t* ny) {
  if (!m || !nx || !ny) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  *nx = m->g.NX;
  *ny = m->g.NY;
  return SEM_OK;
}

int sem_abu(const double* As, int ma, int na, const double* Br, int mb, int nb,
            const double* u, int m, int n, double* v, sem_stream_t stream) {
  if (!u || !v) return set_error(SEM_ERR_BAD_ARG, "NULL field");
  if (m < 0 || n < 0) return set_error(SEM_ERR_BAD_ARG, "negative size");
  if (u == v) return set_error(SEM_ERR_BAD_ARG, "ABu output must not alias its input");
  if (Br) {
    if (mb < 1 || nb < 1) return set_error(SEM_ERR_BAD_ARG, "Br must not be empty (got %dx%d)", mb, nb);
    if (((long long)m * n) % nb != 0)
      return set_error(SEM_ERR_BAD_ARG, "length(u) = %lld is not a multiple of size(Br,2) = %d", (long long)m * n, nb);
    if (((long long)m * mb) % nb != 0)
      return set_error(SEM_ERR_BAD_ARG, "m*mb/nb is not an integer");
  }
  if (As) {
    if (ma < 1 || na < 1) return set_error(SEM_ERR_BAD_ARG, "As must not be empty (got %dx%d)", ma, na);
    if (n % na != 0) return set_error(SEM_ERR_BAD_ARG, "size(u,2) = %d is not a multiple of size(As,2) = %d", n, na);
  }
  return launch_abu(As, ma, na, Br, mb, nb, u, m, n, v, (cudaStream_t)stream);
}

static int fused(sem_mesh_t* m, const double* u, double* out, unsigned mode, const double* nu,
                 double nu_s, double k, sem_stream_t stream) {
  if (!m || !u || !out) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (u == out || (nu && nu == out))
    return set_error(SEM_ERR_BAD_ARG, "output must not alias an input of a fused operator");
  SEM_CHECK(check_device(m));
  ApplyCall c;
  std::memset(&c, 0, sizeof(c));
  c.u = u;
  c.out = out;
  c.G11 = m->G11;
  c.G12 = m->G12;
  c.G22 = m->G22;
  c.B = m->B;
  c.nu = nu;
  c.nu_s = nu_s;
  c.k_s = k;
  c.mode = mode | (nu ? M_NU : 0u);
  c.precision = m->precision;
  c.skip = nullptr;
  c.variant = m->variant[m->precision];
  c.Gdf = m->Gdf;
  c.ctr = m->fix_ctr;
  SEM_CHECK(use_kB(m, c, (cudaStream_t)stream));
  SEM_CHECK(arm_range_guard(m, c));
  return launch_apply(m->g, m->ops, c, (cudaStream_t)stream);
}

int sem_lapl(sem_mesh_t* m, const double* u, double* out, unsigned flags, sem_stream_t stream) {
  if (!m) return set_error(SEM_ERR_BAD_ARG, "NULL mesh");
  return fused(m, u, out, op_mode(m, flags) | M_STIFF, nullptr, 1.0, 0.0, stream);
}

int sem_lapl_nu(sem_mesh_t* m, const double* nu, const double* u, double* out, unsigned flags,
                sem_stream_t stream) {
  if (!m || !nu) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  return fused(m, u, out, op_mode(m, flags) | M_STIFF, nu, 1.0, 0.0, stream);
}

int sem_hlmz(sem_mesh_t* m, const double* nu_field, double nu, double k, const double* u,
             double* out, unsigned flags, sem_stream_t stream) {
  if (!m) return set_error(SEM_ERR_BAD_ARG, "NULL mesh");
  return fused(m, u, out, op_mode(m, flags) | M_STIFF | M_MASS, nu_field, nu, k, stream);
}

int sem_varcoef(sem_mesh_t* m, const double* nu_field, double k, const double* u, double* out,
                unsigned flags, sem_stream_t stream) {
  if (!m || !nu_field) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  unsigned mode = op_mode(m, flags) | M_STIFF | M_NUG | (k != 0.0 ? M_MASS : 0u);
  // fused() adds M_NU for a non-NULL nu; the G-folded form replaces it
  if (!u || !out) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (u == out || nu_field == out)
    return set_error(SEM_ERR_BAD_ARG, "output must not alias an input of a fused operator");
  SEM_CHECK(check_device(m));
  ApplyCall c;
  std::memset(&c, 0, sizeof(c));
  c.u = u;
  c.out = out;
  c.G11 = m->G11;
  c.G12 = m->G12;
  c.G22 = m->G22;
  c.B = m->B;
  c.nu = nu_field;
  c.nu_s = 1.0;
  c.k_s = k;
  c.mode = mode;
  c.precision = m->precision;
  c.variant = m->variant[m->precision];
  c.Gdf = m->Gdf;
  c.ctr = m->fix_ctr;
  SEM_CHECK(use_kB(m, c, (cudaStream_t)stream));
  SEM_CHECK(arm_range_guard(m, c));
  return launch_apply(m->g, m->ops, c, (cudaStream_t)stream);
}

int sem_mass(sem_mesh_t* m, const double* u, double* out, unsigned flags, sem_stream_t stream) {
  if (!m || !u || !out) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  SEM_CHECK(check_device(m));
  if (!(flags & (SEM_GS | SEM_MASK))) return launch_mass(m->g, m->B, u, out, (cudaStream_t)stream);
  return fused(m, u, out, op_mode(m, flags) | M_MASS, nullptr, 1.0, 1.0, stream);
}

int sem_gather_scatter(sem_mesh_t* m, const double* u, double* out, sem_stream_t stream) {
  if (!m || !u || !out) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (u == out) return set_error(SEM_ERR_BAD_ARG, "gatherScatter output must not alias its input");
  SEM_CHECK(check_device(m));
  return launch_gather_scatter(m->g, u, out, m->g.topo, (cudaStream_t)stream);
}

int sem_gather_scatter_grid(int nr, int ns, int Ex, int Ey, int periodic_x, int periodic_y, const double* u,
                            double* out, sem_stream_t stream) {
  if (nr < 1 || ns < 1 || Ex < 1 || Ey < 1) return set_error(SEM_ERR_BAD_ARG, "bad sizes");
  if ((long long)nr * Ex >= (1LL << 31) || (long long)ns * Ey >= (1LL << 31))
    return set_error(SEM_ERR_UNSUPPORTED, "local dimensions must be below 2^31");
  if (!u || !out) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (u == out) return set_error(SEM_ERR_BAD_ARG, "gatherScatter output must not alias its input");
  return launch_gather_scatter_grid(nr, ns, Ex, Ey, periodic_x != 0, periodic_y != 0, u, out,
                                    (cudaStream_t)stream);
}

int sem_mask(const double* M, const double* u, double* out, int64_t len, sem_stream_t stream) {
  if (len < 0) return set_error(SEM_ERR_BAD_ARG, "negative length");
  if (len > 0 && (!u || !out)) return set_error(SEM_ERR_BAD_ARG, "NULL field");
  return launch_mask_array(M, u, out, len, (cudaStream_t)stream);
}

int sem_mask_bc(sem_mesh_t* m, const double* u, double* out, sem_stream_t stream) {
  if (!m || !u || !out) return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  SEM_CHECK(check_device(m));
  if (!m->has_bc) return set_error(SEM_ERR_BAD_ARG, "the mesh handle has no bc (sem_mesh_set_bc)");
  return launch_mask_bc(m->g, u, out, m->g.topo, (cudaStream_t)stream);
}

int sem_lapl_geom(int nr, int ns, int Ex, int Ey, int periodic_x, int periodic_y, const char* bc,
                  const double* Dr, const double* Ds, const double* G11, const double* G12,
                  const double* G22, const double* u, double* out, unsigned flags,
                  int precision, sem_stream_t stream) {
  if (nr < 2 || ns < 2 || Ex < 1 || Ey < 1) return set_error(SEM_ERR_BAD_ARG, "bad sizes");
  if (nr != ns) return set_error(SEM_ERR_UNSUPPORTED, "nr != ns is not served");
  if (!Dr || !Ds || !G11 || !G12 || !G22 || !u || !out)
    return set_error(SEM_ERR_BAD_ARG, "NULL argument");
  if (u == out) return set_error(SEM_ERR_BAD_ARG, "output must not alias an input");
  if (bc && !valid_bc(bc)) return set_error(SEM_ERR_BAD_ARG, "bc must be 4 chars of 'D'/'N'");
  if (precision != SEM_F64 && precision != SEM_F64_DF)
    return set_error(SEM_ERR_BAD_ARG, "precision must be SEM_F64 or SEM_F64_DF");
  OperatorSet* ops = nullptr;
  SEM_CHECK(make_operator_set(Dr, Ds, nr, &ops));
  Grid g;
  std::memset(&g, 0, sizeof(g));
  g.n = nr;
  g.Ex = Ex;
  g.Ey = Ey;
  g.NX = (int64_t)nr * Ex;
  g.NY = (int64_t)nr * Ey;
  g.topo = (periodic_x ? M_PERX : 0u) | (periodic_y ? M_PERY : 0u) | (bc ? bc_bits(bc) : 0u);
  unsigned mode = g.topo | M_STIFF;
  if (flags & SEM_GS) mode |= M_GS;
  if ((flags & SEM_MASK) && bc) mode |= M_MASK;
  ApplyCall c;
  std::memset(&c, 0, sizeof(c));
  c.u = u;
  c.out = out;
  c.G11 = G11;
  c.G12 = G12;
  c.G22 = G22;
  c.nu_s = 1.0;
  c.mode = mode;
  c.precision = precision;
  int st = arm_range_guard(nullptr, c);
  if (st == SEM_OK) st = launch_apply(g, ops, c, (cudaStream_t)stream);
  free_operator_set(ops);
  return st;
}

}  // extern "C"
