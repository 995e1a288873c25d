// Internal declarations shared by the translation units of libsem_b200.so.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <cstring>
#include <string>

#include "../../include/sem_b200.h"

namespace sem {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
int set_error(int status, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

#define SEM_CUDA(call)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_error(e_, #call); \
  } while (0)

#define SEM_CHECK(status_expr)          \
  do {                                  \
    int s_ = (status_expr);             \
    if (s_ != SEM_OK) return s_;        \
  } while (0)

constexpr int kMaxN = 17;       // GLL points per direction served by the fused kernels
constexpr int kMaxBlock = 32;   // block size limit of the generic ABu kernel

// ---------------------------------------------------------------------------
// structured mesh description used by the kernels
// ---------------------------------------------------------------------------
// mode bits of the fused operators
enum : unsigned {
  M_MASS = 1u << 0,    // add k * B .* u
  M_NU = 1u << 1,      // multiply the stiffness part by a nu field
  M_GS = 1u << 2,      // direct-stiffness summation QQ'
  M_MASK = 1u << 3,    // Dirichlet mask
  M_PERX = 1u << 4,    // periodic in x
  M_PERY = 1u << 5,    // periodic in y
  M_DXMIN = 1u << 6,   // Dirichlet at xmin (only meaningful without M_PERX)
  M_DXMAX = 1u << 7,
  M_DYMIN = 1u << 8,
  M_DYMAX = 1u << 9,
  M_STIFF = 1u << 10,  // include the stiffness (lapl) part
  M_NUG = 1u << 11,    // variable coefficient folded into G: D'(nu G)D
  M_MULT1 = 1u << 12,  // solver dots without the SEM multiplicity weights
  M_NUFOLD = 1u << 13, // the scalar nu is folded into the transposed derivative coefficients
  M_KB = 1u << 14,     // B already holds k .* B (no k multiply in the mass term)
};

// per-row / per-column structure bits (device tables of a mesh handle)
enum : unsigned char {
  L_LEFT = 1,    // partner copy is the previous row/column
  L_RIGHT = 2,   // partner copy is the next row/column
  L_WRAPE = 4,   // partner copy is the last row/column (periodic wrap)
  L_WRAPS = 8,   // partner copy is the first row/column (periodic wrap)
  L_ZERO = 16,   // Dirichlet row/column under the handle's bc
};
constexpr unsigned char L_COPY2 = L_LEFT | L_RIGHT | L_WRAPE | L_WRAPS;

struct Grid {
  int n;        // GLL points per direction (nr == ns)
  int Ex, Ey;
  int64_t NX, NY;  // local rows n*Ex, local columns n*Ey
  unsigned topo;   // M_PERX | M_PERY | M_D* bits
  const unsigned char* rinfo;  // device, NX entries of L_* bits (may be NULL off-handle)
  const unsigned char* cinfo;  // device, NY entries
};

// host: L_* bits of local line l (row or column) of a direction with E
// elements of n points; zero_first/zero_last mark Dirichlet ends
__host__ __device__ inline unsigned char line_info(int64_t l, int n, int E, bool per, bool zero_first, bool zero_last) {
  const int64_t NL = (int64_t)n * E;
  const int64_t e = l / n;
  const int i = (int)(l - e * n);
  unsigned char b = 0;
  if (i == 0) b |= e > 0 ? L_LEFT : (per ? L_WRAPE : 0);
  if (i == n - 1) b |= e < E - 1 ? L_RIGHT : (per ? L_WRAPS : 0);
  if (!per && ((zero_first && l == 0) || (zero_last && l == NL - 1))) b |= L_ZERO;
  return b;
}

// partner line of l under the L_* bits, or -1
__host__ __device__ inline int64_t line_partner(int64_t l, unsigned char b, int64_t NL) {
  if (b & L_LEFT) return l - 1;
  if (b & L_RIGHT) return l + 1;
  if (b & L_WRAPE) return NL - 1;
  if (b & L_WRAPS) return 0;
  return -1;
}

// mask value of local point (r, c) under the topology bits
__host__ __device__ inline bool mask_keep(int64_t r, int64_t c, int64_t NX, int64_t NY,
                                          unsigned topo) {
  if (!(topo & M_PERX)) {
    if ((topo & M_DXMIN) && r == 0) return false;
    if ((topo & M_DXMAX) && r == NX - 1) return false;
  }
  if (!(topo & M_PERY)) {
    if ((topo & M_DYMIN) && c == 0) return false;
    if ((topo & M_DYMAX) && c == NY - 1) return false;
  }
  return true;
}

// number of local copies of the global node behind local row r (1 or 2)
__host__ __device__ inline int copies_1d(int64_t r, int n, int E, bool per) {
  int64_t e = r / n;
  int i = (int)(r - e * n);
  int c = 1;
  if (i == 0 && (e > 0 || per)) c = 2;
  if (i == n - 1 && (e < E - 1 || per)) c = 2;
  return c;
}

// ---------------------------------------------------------------------------
// even-odd (centro-antisymmetric) 1D operator coefficients
// ---------------------------------------------------------------------------
// y = D x with D[n-1-i][n-1-k] = -D[i][k]:  e_k = x_k + x_{n-1-k},
// o_k = x_k - x_{n-1-k} (k < m = n/2);  S_i = sum_k A[i][k] o_k,
// T_i = sum_k C[i][k] e_k (+ cm[i] x_m for odd n);  y_i = S_i + T_i,
// y_{n-1-i} = S_i - T_i;  odd n: y_m = sum_k mr[k] o_k.
template <int N, class C>
struct EOCoef {
  static constexpr int M = N / 2;
  C A[M][M];
  C Cc[M][M];
  C cm[M];
  C mr[M];
};

template <int N, class C>
struct DenseCoef {
  C D[N][N];  // D[i][k]
};

// double-float value: h + l with |l| <= ulp(h)/2
struct df {
  float h, l;
};

// host helpers building coefficient sets from a column-major double matrix
bool is_centro_antisymmetric(const double* D, int n, double rel_tol);
void eo_from_dense(const double* D, int n, bool transpose, double* A, double* C, double* cm,
                   double* mr);

// ---------------------------------------------------------------------------
// the mesh handle
// ---------------------------------------------------------------------------
// coefficient blocks of the fused kernels for one pair of derivative matrices
// (fixed size, no heap storage: it can live on the stack of a call)
struct OperatorSet {
  int n;
  // even-odd coefficients in double for Dr, Dr', Ds, Ds' (index 0..3); each
  // block holds A (m*m), C (m*m), cm (m), mr (m) with m = n/2
  double eo[4][2 * (kMaxN / 2) * (kMaxN / 2) + 2 * (kMaxN / 2)];
  double Dr[kMaxN * kMaxN], Ds[kMaxN * kMaxN];  // dense, column-major
};
int init_operator_set(const double* Dr, const double* Ds, int n, OperatorSet* o);

}  // namespace sem

struct sem_mesh {
  int device;
  sem::Grid g;
  bool has_bc;
  int precision;           // SEM_F64 or SEM_F64_DF for the fused operators
  double* Dr_h;            // host copies (n*n, column-major)
  double* Ds_h;
  double* wr_h;
  double* ws_h;
  // device geometry, local layout, double
  double *x, *y, *B, *G11, *G12, *G22;
  // FP32 copies for the mixed-precision inner solve (lazily created)
  float *B_f, *G11_f, *G12_f, *G22_f;
  // G11, G12, G22, B split into double-float pairs by d2df (lazily created,
  // read by the double-float kernel variants 2 and 3)
  sem::df* Gdf;
  sem::OperatorSet* ops;   // coefficient blocks for the kernels
  // solver workspace (lazily created)
  void* ws;
  size_t ws_bytes;
  unsigned char* info;     // device L_* tables: NX row entries then NY column entries
  int variant[4];          // autotuned kernel variant per precision (SEM_F64, SEM_F64_DF, SEM_F32)
  void* graphs;            // CUDA graphs of the CG iteration chunks (sem_pcg.cu), or NULL
  unsigned* fix_ctr;       // interface arrival counters of kernel variant 5 (3 per tile), or NULL
  void* host_pipe;         // streams, events and buffers of sem_hlmz_host (sem_host.cu), or NULL
  double* kB;              // k .* B for the native FP64 operator (lazily created), and its k
  double kB_k;
  unsigned* rflag;         // range-guard word of the double-float calls (lazily created)
  unsigned rtag;           // tag of the latest guarded call
};

namespace sem {

// geometry (sem_geom.cu)
int build_geometry(sem_mesh* m, const double* x_h, const double* y_h, cudaStream_t s);
int export_field(const sem_mesh* m, int which, double* out, cudaStream_t s);
int ensure_f32_geometry(sem_mesh* m, cudaStream_t s);
int ensure_df_geometry(sem_mesh* m, cudaStream_t s);
int ensure_fix_counters(sem_mesh* m);  // sem_apply.cu

// operator coefficients (sem_apply.cu)
int make_operator_set(const double* Dr, const double* Ds, int n, OperatorSet** out);
void free_operator_set(OperatorSet* o);

struct ApplyCall {
  const void* u;
  void* out;
  const void* G11;
  const void* G12;
  const void* G22;
  const void* B;
  const void* nu;
  double nu_s;
  double k_s;
  unsigned mode;   // M_* bits (topology bits included)
  int precision;   // SEM_F64, SEM_F64_DF, SEM_F32
  const int* skip; // device flag: when non-zero the launch does nothing (solver loops)
  int variant;     // kernel variant 0..kVariants-1 (launch_apply_n in sem_apply_launch.cuh)
  const void* Gdf; // G11, G12, G22, B split into double-float pairs (4 blocks of NX*NY), or NULL
  unsigned* ctr;   // interface arrival counters of the mesh (variant 5), or NULL
  // CG-fused launch (variants 2 and 5; cg_p non-NULL): u = p = dinv.*r + beta p
  // formed in the kernel, per-CTA parts of p.Ap written to cg_dpart
  const void* cg_r;
  const void* cg_dinv;
  void* cg_p;
  const double* cg_beta;
  void* cg_dpart;
  int pdl;         // launch as a programmatic dependent of the previous kernel on the stream
  // a window of element-tile rows [ty0, ty0 + tyn) instead of the whole grid
  // (tyn = 0: all); variants 0-3 only, no CG fusion, the fixup left to the caller
  int ty0, tyn;
  // range guard of a double-float call (rflag non-NULL): the kernels set
  // *rflag = rtag when a value leaves the pair format's range, and
  // launch_apply follows them with a native FP64 re-run of the whole call,
  // gated on that word (gate, gate_tag: the gated launch itself)
  unsigned* rflag;
  unsigned rtag;
  const unsigned* gate;
  unsigned gate_tag;
};
// arm the range guard of a double-float call on mesh m (the mesh's flag word)
// or, without a mesh, on the device's own word
int arm_range_guard(sem_mesh* m, ApplyCall& c);
// the device's timeout word of the TMA operator kernel (variant 6), or NULL;
// made on first use when may_alloc (never inside a launch that a stream
// capture may enclose)
unsigned* wait_timeout_word(bool may_alloc);

// launch kern<<<grid, block, 0, s>>>(args...) as a programmatic dependent of
// the previous kernel on s (the kernel must call griddepcontrol.wait before it
// touches memory)
template <class... KArgs, class... Args>
int launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  SEM_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
  return SEM_OK;
}

// number of CTAs (element tiles) of a CG-fused operator launch on grid g
long long cg_apply_parts(const Grid& g);

// Problem description of the single-launch small-mesh PCG (sem_small.cu),
// filled by the host and read and updated by the kernel.
struct SmallProb {
  int n, Ex, Ey;
  long long NX, NY;
  const unsigned char* rinfo;  // L_* bits of the local rows and columns
  const unsigned char* cinfo;
  bool has_bc;
  int jacobi;
  int mult_ones;  // 1: unweighted dots
  double nu, k, tol;
  int maxiter;
  int precision;  // SEM_F64_DF (or SEM_F64: same vectors, double-float operator) or SEM_MIXED
  double inner_tol;
  int max_outer;
  const double* b;
  double* x;
  double *r, *p, *raw, *dinv;
  float *r32, *p32, *raw32, *x32, *dinv32;
  const df* Gdf;   // G11, G12, G22, B split into double-float pairs (4 blocks of NX*NY)
  const float* Gf; // G11, G12, G22, B in FP32 (4 blocks)
  // results
  int iters, outer, converged, nan;
  double res_inf, res0_inf;
};

int launch_small_pcg(SmallProb* dev, const OperatorSet& ops, int n, cudaStream_t s);  // sem_small.cu
// the SEM_MIXED solve of a small mesh in one launch of a small cluster whose
// CTAs hold the FP32 working set of a strip of element rows each in shared
// memory (sem_tiny.cu); host is the record copied to dev, smem the per-CTA
// shared memory tiny_smem_bytes gives
int launch_tiny_pcg(SmallProb* dev, const SmallProb& host, const OperatorSet& ops, size_t smem, cudaStream_t s);
size_t tiny_smem_bytes(int n, int Ex, int Ey, bool mass, bool jac);
size_t max_smem_optin();  // the device's opt-in shared memory per block (sem_apply.cu)

// results at the tail of a SmallProb, in the same order
struct SmallOut {
  int iters, outer, converged, nan;
  double res_inf, res0_inf;
};
static_assert(sizeof(SmallProb) - offsetof(SmallProb, iters) == sizeof(SmallOut),
              "SmallOut mirrors the result fields of SmallProb");

// sem_pcg.cu, for callers that queue several small-mesh solves without
// waiting on each: whether sem_pcg would take the single-launch path for o on
// m, and the record of one such solve (the Jacobi diagonal it reads is
// enqueued on s into the mesh's workspace)
bool small_path_taken(const sem_mesh* m, const sem_pcg_opts* o);
int small_prepare(sem_mesh* m, const sem_pcg_opts* o, const double* b, double* x, SmallProb* rec,
                  cudaStream_t s);

constexpr int kVariants = SEM_VARIANTS;

int launch_apply(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s);
// native FP64 calls with a mass term read the mesh's k .* B (one multiply fewer
// per point); made or refreshed on s when k changes
int use_kB(sem_mesh* m, ApplyCall& c, cudaStream_t s);
bool timing_enabled();                 // sem_timing_enable state (sem_apply.cu)
void free_graph_cache(sem_mesh* m);    // sem_pcg.cu
void free_host_pipe(sem_mesh* m);      // sem_host.cu
void tile_shape_of(int n, int* tx, int* ty);  // element tile of the fused kernels (sem_apply.cu)
int launch_dss_fixup(const Grid& g, void* out, unsigned mode, int precision, const int* skip, int TX,
                     int TY, cudaStream_t s, long long key_lo = 0, long long key_hi = 1LL << 62,
                     const unsigned* gate = nullptr, unsigned gate_tag = 0);
// the operator kernel on a window of tile rows (ApplyCall::ty0, tyn) and the
// fixup of the interface points whose highest copy column is in [key_lo, key_hi)
int launch_apply_window(const Grid& g, const OperatorSet* ops, const ApplyCall& c, long long key_lo,
                        long long key_hi, cudaStream_t s);
// the range guard's native FP64 re-run of a whole double-float call, gated on
// the call's flag word (for callers that ran the call in windows)
int launch_guard_rerun(const Grid& g, const OperatorSet* ops, const ApplyCall& c, cudaStream_t s);

// elementwise / structured kernels (sem_vec.cu)
int launch_gather_scatter(const Grid& g, const double* u, double* out, unsigned mode, cudaStream_t s);
int launch_gather_scatter_grid(int nr, int ns, int Ex, int Ey, bool perx, bool pery, const double* u,
                               double* out, cudaStream_t s);
int launch_mask_bc(const Grid& g, const double* u, double* out, unsigned topo, cudaStream_t s);
int launch_mask_array(const double* M, const double* u, double* out, int64_t len, cudaStream_t s);
int launch_mass(const Grid& g, const double* B, const double* u, double* out, cudaStream_t s);
int launch_mult(const Grid& g, double* out, cudaStream_t s);
int launch_abu(const double* As, int ma, int na, const double* Br, int mb, int nb,
               const double* u, int m, int n, double* v, cudaStream_t s);

unsigned topo_bits(const Grid& g);
int upload_line_info(sem_mesh* m);

// Visit every local point (r, c) of g with a block-uniform loop (all threads
// of a block run the same number of trips, so block reductions may follow):
// blocks walk chunks of blockDim.x consecutive rows of one column.
template <class F>
__device__ __forceinline__ void for_each_point(const Grid& g, F&& f) {
  const unsigned NX = (unsigned)g.NX, NY = (unsigned)g.NY;
  const unsigned nrc = (NX + blockDim.x - 1) / blockDim.x;
  const unsigned total = nrc * NY;
  for (unsigned b = blockIdx.x; b < total; b += gridDim.x) {
    const unsigned c = b / nrc;
    const unsigned r = (b - c * nrc) * blockDim.x + threadIdx.x;
    if (r < NX) f(r, c, (long long)r + (long long)c * NX);
  }
}

__device__ __forceinline__ int copies_at(const Grid& g, unsigned r, unsigned c) {
  return ((g.rinfo[r] & L_COPY2) ? 2 : 1) * ((g.cinfo[c] & L_COPY2) ? 2 : 1);
}
}  // namespace sem
