// Device-side geometry of a mesh handle: Jacobian, inverse metrics, mass
// matrix and the Laplacian metric factors from the deformed grid
// (src/jac.jl:24-40, src/mesh.jl:111-123).
#include <cstring>

#include "sem_arith.cuh"
#include "sem_internal.cuh"

namespace sem {

namespace {

struct GeomArgs {
  double Dr[kMaxN * kMaxN];  // column-major
  double Ds[kMaxN * kMaxN];
  double wr[kMaxN];
  double ws[kMaxN];
  int n, Ex, Ey;
  long long NX, NY;
};

enum GeomOut { G_ALL = -1 };

// which = -1: write B, G11, G12, G22; otherwise one sem_field into out0
__global__ void k_geometry(const __grid_constant__ GeomArgs a, const double* __restrict__ x,
                           const double* __restrict__ y, int which, double* __restrict__ out0,
                           double* __restrict__ o_B, double* __restrict__ o_G11,
                           double* __restrict__ o_G12, double* __restrict__ o_G22) {
  const long long total = a.NX * a.NY;
  const int n = a.n;
  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long c = idx / a.NX;
    const long long r = idx - c * a.NX;
    const long long ex = r / n, ey = c / n;
    const int i = (int)(r - ex * n), j = (int)(c - ey * n);
    const long long r0 = ex * n, c0 = ey * n;
    double xr = 0, xs = 0, yr = 0, ys = 0;
    for (int k = 0; k < n; ++k) {
      const double dr = a.Dr[i + k * n];
      const double ds = a.Ds[j + k * n];
      const long long pr = (r0 + k) + c * a.NX;  // (k, j) in this element
      const long long ps = r + (c0 + k) * a.NX;  // (i, k)
      xr = fma(dr, x[pr], xr);
      yr = fma(dr, y[pr], yr);
      xs = fma(ds, x[ps], xs);
      ys = fma(ds, y[ps], ys);
    }
    const double J = __dsub_rn(__dmul_rn(xr, ys), __dmul_rn(xs, yr));
    const double Ji = 1.0 / J;
    const double rx = __dmul_rn(Ji, ys);
    const double ry = -__dmul_rn(Ji, xs);
    const double sx = -__dmul_rn(Ji, yr);
    const double sy = __dmul_rn(Ji, xr);
    const double B = __dmul_rn(J, __dmul_rn(a.wr[i], a.ws[j]));
    const double g11 = __dmul_rn(B, __dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)));
    const double g12 = __dmul_rn(B, __dadd_rn(__dmul_rn(rx, sx), __dmul_rn(ry, sy)));
    const double g22 = __dmul_rn(B, __dadd_rn(__dmul_rn(sx, sx), __dmul_rn(sy, sy)));
    if (which == G_ALL) {
      o_B[idx] = B;
      o_G11[idx] = g11;
      o_G12[idx] = g12;
      o_G22[idx] = g22;
    } else {
      double v = 0.0;
      switch (which) {
        case SEM_FIELD_JAC: v = J; break;
        case SEM_FIELD_JACI: v = Ji; break;
        case SEM_FIELD_RX: v = rx; break;
        case SEM_FIELD_RY: v = ry; break;
        case SEM_FIELD_SX: v = sx; break;
        case SEM_FIELD_SY: v = sy; break;
        case SEM_FIELD_B: v = B; break;
        case SEM_FIELD_BI: v = 1.0 / B; break;
        case SEM_FIELD_G11: v = g11; break;
        case SEM_FIELD_G12: v = g12; break;
        case SEM_FIELD_G22: v = g22; break;
        default: break;
      }
      out0[idx] = v;
    }
  }
}

__global__ void k_d2f(const double* __restrict__ a, float* __restrict__ b, long long len) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// the geometry's split, with the range guard's poisoning: a point whose G11
// and G22 both lie below 2^-40 gets NaN metric pairs, and a nonzero mass entry
// below 2^-100 a NaN pair, so that every double-float apply on the mesh is
// flagged and re-run in native FP64
__global__ void k_geo_d2df(const double* __restrict__ G11, const double* __restrict__ G12,
                           const double* __restrict__ G22, const double* __restrict__ B, df* __restrict__ out,
                           long long len) {
  const df nan = {__uint_as_float(0x7fc00000u), 0.0f};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (long long)gridDim.x * blockDim.x) {
    const double g11 = G11[i], g22 = G22[i], b = B[i];
    const bool gt = geo_tiny(g11, g22);
    out[i] = gt ? nan : d2df_op(g11);
    out[len + i] = gt ? nan : d2df_op(G12[i]);
    out[2 * len + i] = gt ? nan : d2df_op(g22);
    out[3 * len + i] = (b != 0.0 && fabs(b) < (double)kKbTiny) ? nan : d2df_op(b);
  }
}

__global__ void k_maskfield(double* __restrict__ out, Grid g) {
  for_each_point(g, [&](unsigned r, unsigned c, long long idx) {
    out[idx] = ((g.rinfo[r] | g.cinfo[c]) & L_ZERO) ? 0.0 : 1.0;
  });
}

void fill_geom_args(GeomArgs& a, const sem_mesh* m) {
  std::memset(&a, 0, sizeof(a));
  const int n = m->g.n;
  a.n = n;
  a.Ex = m->g.Ex;
  a.Ey = m->g.Ey;
  a.NX = m->g.NX;
  a.NY = m->g.NY;
  std::memcpy(a.Dr, m->Dr_h, sizeof(double) * n * n);
  std::memcpy(a.Ds, m->Ds_h, sizeof(double) * n * n);
  std::memcpy(a.wr, m->wr_h, sizeof(double) * n);
  std::memcpy(a.ws, m->ws_h, sizeof(double) * n);
}

unsigned blocks_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152LL * 32) b = 152LL * 32;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

int build_geometry(sem_mesh* m, const double* x_h, const double* y_h, cudaStream_t s) {
  (void)x_h;
  (void)y_h;
  GeomArgs a;
  fill_geom_args(a, m);
  k_geometry<<<blocks_for(m->g.NX * m->g.NY), 256, 0, s>>>(a, m->x, m->y, G_ALL, nullptr, m->B,
                                                           m->G11, m->G12, m->G22);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int export_field(const sem_mesh* m, int which, double* out, cudaStream_t s) {
  const size_t bytes = sizeof(double) * (size_t)(m->g.NX * m->g.NY);
  switch (which) {
    case SEM_FIELD_X:
      SEM_CUDA(cudaMemcpyAsync(out, m->x, bytes, cudaMemcpyDeviceToDevice, s));
      return SEM_OK;
    case SEM_FIELD_Y:
      SEM_CUDA(cudaMemcpyAsync(out, m->y, bytes, cudaMemcpyDeviceToDevice, s));
      return SEM_OK;
    case SEM_FIELD_B:
      SEM_CUDA(cudaMemcpyAsync(out, m->B, bytes, cudaMemcpyDeviceToDevice, s));
      return SEM_OK;
    case SEM_FIELD_G11:
      SEM_CUDA(cudaMemcpyAsync(out, m->G11, bytes, cudaMemcpyDeviceToDevice, s));
      return SEM_OK;
    case SEM_FIELD_G12:
      SEM_CUDA(cudaMemcpyAsync(out, m->G12, bytes, cudaMemcpyDeviceToDevice, s));
      return SEM_OK;
    case SEM_FIELD_G22:
      SEM_CUDA(cudaMemcpyAsync(out, m->G22, bytes, cudaMemcpyDeviceToDevice, s));
      return SEM_OK;
    case SEM_FIELD_MULT:
      return launch_mult(m->g, out, s);
    case SEM_FIELD_MASK:
      k_maskfield<<<blocks_for(m->g.NX * m->g.NY), 256, 0, s>>>(out, m->g);
      SEM_CUDA(cudaGetLastError());
      return SEM_OK;
    case SEM_FIELD_JAC:
    case SEM_FIELD_JACI:
    case SEM_FIELD_RX:
    case SEM_FIELD_RY:
    case SEM_FIELD_SX:
    case SEM_FIELD_SY:
    case SEM_FIELD_BI: {
      GeomArgs a;
      fill_geom_args(a, m);
      k_geometry<<<blocks_for(m->g.NX * m->g.NY), 256, 0, s>>>(a, m->x, m->y, which, out, nullptr,
                                                               nullptr, nullptr, nullptr);
      SEM_CUDA(cudaGetLastError());
      return SEM_OK;
    }
    default:
      return set_error(SEM_ERR_BAD_ARG, "unknown field %d", which);
  }
}

int ensure_f32_geometry(sem_mesh* m, cudaStream_t s) {
  if (m->G11_f) return SEM_OK;
  const long long len = m->g.NX * m->g.NY;
  const size_t bytes = sizeof(float) * (size_t)len;
  float* p = nullptr;
  SEM_CUDA(cudaMalloc(&p, 4 * bytes));
  m->G11_f = p;
  m->G12_f = p + len;
  m->G22_f = p + 2 * len;
  m->B_f = p + 3 * len;
  k_d2f<<<blocks_for(len), 256, 0, s>>>(m->G11, m->G11_f, len);
  k_d2f<<<blocks_for(len), 256, 0, s>>>(m->G12, m->G12_f, len);
  k_d2f<<<blocks_for(len), 256, 0, s>>>(m->G22, m->G22_f, len);
  k_d2f<<<blocks_for(len), 256, 0, s>>>(m->B, m->B_f, len);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

int ensure_df_geometry(sem_mesh* m, cudaStream_t s) {
  if (m->Gdf) return SEM_OK;
  const long long len = m->g.NX * m->g.NY;
  df* p = nullptr;
  SEM_CUDA(cudaMalloc(&p, 4 * sizeof(df) * (size_t)len));
  m->Gdf = p;
  k_geo_d2df<<<blocks_for(len), 256, 0, s>>>(m->G11, m->G12, m->G22, m->B, p, len);
  SEM_CUDA(cudaGetLastError());
  return SEM_OK;
}

}  // namespace sem
