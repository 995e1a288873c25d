/*
 * sem_b200.h — C ABI of libsem_b200.so, the GB300 (sm_103a) implementation
 * of the spectral-element operator-apply and solve hot path of
 * SpectralElements.jl (ABu, lapl, mass, hlmz, gatherScatter, mask, pcg).
 *
 * Conventions
 *  - Every entry point returns an int status (enum sem_status).  On failure
 *    sem_last_error() returns a message for the calling host thread.
 *  - Fields ("local" vectors) are DEVICE pointers to column-major
 *    (nr*Ex) x (ns*Ey) arrays of double: element (ex,ey) occupies rows
 *    ex*nr .. ex*nr+nr-1 and columns ey*ns .. ey*ns+ns-1 (0-based), the
 *    layout of the reference (src/semmesh.jl:19, src/ndgrid.jl:8-13).
 *  - Small operator matrices (derivative / interpolation matrices, at most
 *    32x32) are HOST pointers to column-major arrays.
 *  - Calls are asynchronous on the given stream (a cudaStream_t, NULL = the
 *    legacy default stream) except sem_mesh_create / sem_mesh_destroy and
 *    the solvers, which synchronise the stream to return their result.
 *  - The library never frees caller memory.  A mesh handle is not safe for
 *    concurrent use from several host threads or streams at once.
 *  - No entry point falls back to the CPU: without a usable CUDA device every
 *    compute call returns SEM_ERR_CUDA.
 */
#ifndef SEM_B200_H
#define SEM_B200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEM_ABI_VERSION 1

typedef struct sem_mesh sem_mesh_t;
typedef void* sem_stream_t; /* cudaStream_t */

enum sem_status {
  SEM_OK = 0,
  SEM_ERR_BAD_ARG = 1,       /* invalid sizes, NULL pointers, aliasing   */
  SEM_ERR_NOT_CONVERGED = 2, /* pcg reached maxiter (x is still returned) */
  SEM_ERR_NAN = 3,           /* a NaN/Inf appeared in a solver residual   */
  SEM_ERR_TIMEOUT = 4,       /* a bounded device wait ran out             */
  SEM_ERR_CUDA = 5,          /* a CUDA runtime call failed                */
  SEM_ERR_UNSUPPORTED = 6,   /* a valid request this build cannot serve   */
  SEM_ERR_NO_MEMORY = 7      /* device allocation failed                  */
};

/* operator flags: the fused operators compose mask(QQ'(op(u))) on request */
#define SEM_GS 1u   /* apply direct-stiffness summation QQ' (gatherScatter) */
#define SEM_MASK 2u /* apply the handle's Dirichlet mask R'R afterwards     */
#define SEM_NU_IN_G 4u /* sem_hlmz_host: nu_field is folded into G11/G12/G22,
                          the variable-coefficient operator of sem_varcoef */

/* arithmetic of the fused operators and of the solver */
enum sem_precision {
  SEM_F64 = 0,    /* native FP64 arithmetic                                  */
  SEM_F64_DF = 1, /* FP64 in/out, double-float (FP32 pair) arithmetic, ~47 bit */
  SEM_F32 = 2,    /* FP32 geometry copy and FP32 arithmetic (solver inner loop) */
  SEM_MIXED = 3,  /* solver only: FP32 inner CG inside FP64 defect correction */
  SEM_MIXED_RR = 4 /* solver only: one FP32 CG whose residual is replaced by the
                      FP64 residual b - A x (x kept in FP64) whenever it has
                      fallen by the factor inner_tol (default 0.3) since the
                      last replacement; the search direction is kept, so the
                      iteration count stays near that of the FP64 CG */
};

/* geometry fields that sem_mesh_field can export */
enum sem_field {
  SEM_FIELD_X = 0, SEM_FIELD_Y = 1, SEM_FIELD_JAC = 2, SEM_FIELD_JACI = 3,
  SEM_FIELD_RX = 4, SEM_FIELD_RY = 5, SEM_FIELD_SX = 6, SEM_FIELD_SY = 7,
  SEM_FIELD_B = 8, SEM_FIELD_BI = 9, SEM_FIELD_G11 = 10, SEM_FIELD_G12 = 11,
  SEM_FIELD_G22 = 12, SEM_FIELD_MULT = 13, SEM_FIELD_MASK = 14
};

typedef struct {
  int nr, ns, Ex, Ey;         /* GLL points per direction, elements        */
  int periodic_x, periodic_y; /* Mesh(...,ifperiodic) (src/mesh.jl:66-68)   */
  const double* Dr;           /* host nr x nr derivative matrix            */
  const double* Ds;           /* host ns x ns                              */
  const double* wr;           /* host GLL weights (nr)                     */
  const double* ws;           /* host GLL weights (ns)                     */
  const double* x;            /* host deformed grid, local layout          */
  const double* y;
  /* optional host geometry: all four or none.  When given they are uploaded
   * verbatim (the Julia Mesh already holds them); otherwise the Jacobian,
   * B and G11/G12/G22 are computed on the device from x, y (src/jac.jl:24-40,
   * src/mesh.jl:111-123). */
  const double* G11;
  const double* G12;
  const double* G22;
  const double* B;
  const char* bc; /* 4 chars 'D'/'N' for xmin,xmax,ymin,ymax, or NULL = no mask */
} sem_mesh_desc;

/* ---- handle lifecycle: replaces the device-side image of Mesh (src/mesh.jl:25-133) */
int sem_mesh_create(const sem_mesh_desc* desc, sem_mesh_t** out);
int sem_mesh_destroy(sem_mesh_t* mesh);
/* generateMask(bc,msh) (src/mesh.jl:149-175): set the handle's Dirichlet mask */
int sem_mesh_set_bc(sem_mesh_t* mesh, const char* bc);
/* select the arithmetic of the fused FP64 operators (SEM_F64 or SEM_F64_DF) */
int sem_mesh_set_precision(sem_mesh_t* mesh, int precision);
/* number of fused element-operator kernel variants:
 *   0  two shared-memory line buffers, every input read directly;
 *   1  as 0, with the geometry, B and nu fields staged by cp.async;
 *   2  one in-place line buffer, u kept in shared memory for the mass term;
 *      for SEM_F64_DF the geometry is read pre-split into float pairs (the
 *      mesh then holds 4 more fields of NX*NY*8 bytes);
 *   3  as 2, with G11, G12, G22 staged by cp.async;
 *   4  as 2, in a persistent grid whose CTAs prefetch the next element tile's
 *      inputs (cp.async) while they compute the current one;
 *   5  as 2, with the cross-tile QQ' finished inside the same launch (the
 *      last CTA to reach a tile edge or corner sums its copies; the mesh
 *      holds 3 arrival counters per element tile).  Fused calls on one mesh
 *      handle must then not run concurrently on the GPU;
 *   6  as 4, with each element tile's u, G11, G12, G22 and B moved into shared
 *      memory by tensor (TMA) copies that one thread issues, completing on
 *      mbarriers; runs as 4 where TMA cannot serve the call (a row of n*Ex
 *      values or a tile row not a multiple of 16 bytes, a field not 16-byte
 *      aligned or not in device memory).
 * All variants compute the same operations in the same order: their results
 * are bit-identical. */
#define SEM_VARIANTS 7
/* autotuner (no counterpart in the reference): time every variant of the fused
 * element-operator kernel on this mesh, running mask(QQ'(hlmz)) on scratch
 * fields in the given precision (SEM_F64, SEM_F64_DF or SEM_F32), and keep the
 * fastest for all later calls of that precision.  ms_out (nullable) receives
 * SEM_VARIANTS times, one per variant; chosen (nullable) the variant kept.
 * Synchronous. */
int sem_mesh_autotune(sem_mesh_t* mesh, int precision, double* ms_out, int* chosen);
/* pin a kernel variant (0 .. SEM_VARIANTS-1) for one precision; synchronous */
int sem_mesh_set_variant(sem_mesh_t* mesh, int precision, int variant);
/* copy one geometry field (enum sem_field) into a caller device buffer */
int sem_mesh_field(sem_mesh_t* mesh, int which, double* out, sem_stream_t stream);
/* sizes: local rows (nr*Ex), local columns (ns*Ey) */
int sem_mesh_dims(const sem_mesh_t* mesh, int64_t* nx, int64_t* ny);

const char* sem_last_error(void);
int sem_abi_version(void);

/* ---- ABu(As,Br,u) (src/ABu.jl:9-37): v = (As (x) Br) u.
 * As (ma x na) and Br (mb x nb) are host matrices (column-major), NULL =
 * identity ([]).  u is m x n, v is (m*mb/nb) x (n*ma/na).  Factors up to
 * 32 x 32 are passed in the kernel parameters; larger ones are copied to
 * stream-ordered device buffers and applied as strided GEMMs. */
int sem_abu(const double* As, int ma, int na, const double* Br, int mb, int nb,
            const double* u, int m, int n, double* v, sem_stream_t stream);

/* ---- local operators on the handle's geometry; flags compose QQ' and mask.
 * lapl(u,msh) (src/lapl.jl:26-36) */
int sem_lapl(sem_mesh_t* mesh, const double* u, double* out, unsigned flags,
             sem_stream_t stream);
/* lapl(u,nu,msh) = nu .* lapl(u,msh) (src/lapl.jl:38-45); nu a device field */
int sem_lapl_nu(sem_mesh_t* mesh, const double* nu, const double* u, double* out,
                unsigned flags, sem_stream_t stream);
/* hlmz(u,nu,k,msh) = nu .* lapl(u) + k .* mass(u) (src/hlmz.jl:12-19);
 * nu_field (device) overrides the scalar nu when not NULL */
int sem_hlmz(sem_mesh_t* mesh, const double* nu_field, double nu, double k,
             const double* u, double* out, unsigned flags, sem_stream_t stream);
/* hlmz with mask(QQ') on HOST buffers (the end-to-end call): u_host and
 * out_host are column-major host arrays of the local layout.
 *  - slabs >= 1 (0: 8): the field moves in and out in that many slabs of
 *    element-tile rows by the copy engines, overlapping the kernels; pinned
 *    host memory is needed for that overlap, pageable memory works with
 *    serialised copies.
 *  - slabs = SEM_HOST_DIRECT: the operator kernels read u_host and write
 *    out_host in place over the CPU-GPU link; the buffers must be addressable
 *    by the device (cudaHostAlloc / cudaHostRegister memory, or any host
 *    memory on a system whose device reads pageable memory through the host
 *    page tables, as Grace-Blackwell does), else SEM_ERR_UNSUPPORTED.
 * The result is bit-identical to sem_hlmz on device buffers.  nu_field, when
 * given, is a DEVICE field: nu .* lapl(u) as in sem_hlmz, or folded into G as
 * in sem_varcoef when flags has SEM_NU_IN_G.  Asynchronous on `stream`:
 * out_host is complete when the stream is.  The slab pipeline keeps two
 * device buffers of the field's size and two streams in the handle. */
#define SEM_HOST_DIRECT (-1)
int sem_hlmz_host(sem_mesh_t* mesh, const double* nu_field, double nu, double k, const double* u_host,
                  double* out_host, unsigned flags, int slabs, sem_stream_t stream);
/* variable-coefficient operator D'(nu G)D u + k B u with nu (device field)
 * folded into G11/G12/G22 at every node, as examples/semPS.jl:163-165 and
 * examples/p2d_explicit.jl:105-107 build G from visc */
int sem_varcoef(sem_mesh_t* mesh, const double* nu_field, double k, const double* u,
                double* out, unsigned flags, sem_stream_t stream);
/* mass(u,msh) = B .* u (src/mass.jl:12-22) */
int sem_mass(sem_mesh_t* mesh, const double* u, double* out, unsigned flags,
             sem_stream_t stream);
/* gatherScatter(u,msh) = QQ' u (src/gatherScatter.jl:8-21) */
int sem_gather_scatter(sem_mesh_t* mesh, const double* u, double* out,
                       sem_stream_t stream);
/* functional gatherScatter(u,QQtx,QQty) (src/gatherScatter.jl:8-16) without a
 * handle: QQtx/QQty are those of semq(Ex,nr,periodic_x) and semq(Ey,ns,
 * periodic_y) (src/semq.jl:6-25); nr may differ from ns.  Bit-identical to
 * sem_gather_scatter on a handle of the same grid. */
int sem_gather_scatter_grid(int nr, int ns, int Ex, int Ey, int periodic_x, int periodic_y,
                            const double* u, double* out, sem_stream_t stream);
/* mask(u,M) = M .* u (src/mask.jl:10-18); M a device array or NULL (copy) */
int sem_mask(const double* M, const double* u, double* out, int64_t len,
             sem_stream_t stream);
/* mask with the handle's generateMask(bc,msh) pattern, no mask array read */
int sem_mask_bc(sem_mesh_t* mesh, const double* u, double* out, sem_stream_t stream);

/* functional lapl(u,M,[],[],QQtx,QQty,Dr,Ds,G11,G12,G22,mult) (src/lapl.jl:54-68):
 * geometry per call (device G11/G12/G22), host Dr/Ds; QQ' and mask from flags,
 * the mask from bc (NULL = no mask). */
int sem_lapl_geom(int nr, int ns, int Ex, int Ey, int periodic_x, int periodic_y,
                  const char* bc, const double* Dr, const double* Ds,
                  const double* G11, const double* G12, const double* G22,
                  const double* u, double* out, unsigned flags, int precision,
                  sem_stream_t stream);

/* ---- operators beside the fused path (tensor-product kernel + pointwise
 * kernels on the device, following the reference's ABu sequences).
 * Host pointers for the small matrices (column-major), device pointers for
 * the fields (reference local layout). */
/* dealiased laplace(u,Jr,Js,Dr,Ds,G11,G12,G22) (src/lapl.jl:83-103): Jr (mr x n)
 * and Js (ms x n) interpolate an element's n GLL points to mr x ms quadrature
 * points; G11/G12/G22 are fine-grid fields (mr*Ex x ms*Ey); u, out are
 * (n*Ex x n*Ey); no QQ', no mask (the functional lapl adds them) */
int sem_laplace_dealiased(int n, int mr, int ms, int Ex, int Ey, const double* Jr, const double* Js,
                          const double* Dr, const double* Ds, const double* G11, const double* G12,
                          const double* G22, const double* u, double* out, sem_stream_t stream);
/* J'(B .* (J u)) of the functional mass(u,M,B,Jr,Js,QQtx,QQty,mult)
 * (src/mass.jl:32-50) before QQ' and mask; B fine-grid or NULL ([]) */
int sem_mass_dealiased(int n, int mr, int ms, int Ex, int Ey, const double* Jr, const double* Js,
                       const double* B, const double* u, double* out, sem_stream_t stream);
/* grad(u,msh) (src/grad.jl:16-34): ux = rx Dr u + sx u Ds', uy = ry .. + sy .. */
int sem_grad(sem_mesh_t* mesh, const double* u, double* ux, double* uy, sem_stream_t stream);
/* gradᵀ(u,msh) (src/grad.jl:43-63), with the factors as src/grad.jl:55-61
 * passes them to ABu */
int sem_grad_t(sem_mesh_t* mesh, const double* u, double* ux, double* uy, sem_stream_t stream);

/* ---- advection (src/advect.jl:27-64), unassembled (no QQ', no mask, as the
 * reference returns it).  sem_advect: B .* (ux Tx + uy Ty) with
 * (Tx, Ty) = grad(T).  sem_advect_dealiased: grad T and the velocity
 * interpolated to the dealiasing grid with ABu(Js,Jr,.) (Jr mr x n, Js ms x n,
 * host, column-major), multiplied there by the dealiasing mesh's mass Bd
 * (device, (mr Ex) x (ms Ey)), and brought back with ABu(Js',Jr',.). */
int sem_advect(sem_mesh_t* mesh, const double* T, const double* ux, const double* uy, double* out,
               sem_stream_t stream);
int sem_advect_dealiased(sem_mesh_t* mesh, int mr, int ms, const double* Jr, const double* Js,
                         const double* Bd, const double* T, const double* ux, const double* uy,
                         double* out, sem_stream_t stream);

/* ---- solver: pcg(b,opA;opM,mult,ifv,tol,maxiter) (src/pcg.jl:16-60) with
 * opA = mask(QQ'(hlmz(.,nu,k))) (src/diffusion.jl:36-45) */
enum sem_precond { SEM_PRECOND_NONE = 0, SEM_PRECOND_JACOBI = 1 };

typedef struct {
  double nu;             /* scalar viscosity (ignored when nu_field set)    */
  const double* nu_field;/* device nu folded into G (variable coefficient); the
                            mixed precisions run their FP32 CG on nu .* G in FP32 */
  double k;              /* mass coefficient (bdfB[1] / lambda)             */
  int precond;           /* enum sem_precond                                 */
  int precision;         /* SEM_F64, SEM_F64_DF or SEM_MIXED                 */
  double tol;            /* absolute Inf-norm tolerance on the residual      */
  int maxiter;           /* <= 0: length(b), as the reference               */
  double inner_tol;      /* SEM_MIXED: relative inner tolerance (1e-4); SEM_MIXED_RR: residual drop between replacements (0.3) */
  int max_outer;         /* SEM_MIXED: defect-correction sweeps (6); SEM_MIXED_RR: replacements (100).
                            When the sweeps or replacements run out, or an FP32 segment stalls
                            (runs 4 times longer than the longest before it, at least 500
                            iterations), the FP64 CG finishes the solve from the current x */
  int check_every;       /* iterations between convergence reads (0 = auto) */
  int mult_ones;         /* 1: unweighted dots, pcg's default mult=ones(size(b)) */
  int path;              /* enum sem_pcg_path                                */
} sem_pcg_opts;

/* how sem_pcg runs the iterations (no counterpart in the reference):
 * CHUNKED replays chunks of check_every iterations as CUDA graphs over the
 * whole GPU; SMALL runs the whole solve in one launch of one thread-block
 * cluster with one thread per point (meshes of at most SEM_SMALL_MAX_LOCAL
 * local DOF, 2 <= n <= 11, scalar nu, SEM_F64_DF, SEM_MIXED or SEM_MIXED_RR); AUTO takes
 * SMALL where it applies. */
enum sem_pcg_path { SEM_PATH_AUTO = 0, SEM_PATH_CHUNKED = 1, SEM_PATH_SMALL = 2 };
#define SEM_SMALL_MAX_LOCAL 100000

typedef struct {
  int iters;        /* CG iterations (inner iterations summed for MIXED) */
  int outer;        /* defect-correction sweeps (MIXED), else 0          */
  double res_inf;   /* final Inf-norm of the residual                    */
  double res0_inf;  /* Inf-norm of b                                     */
  int converged;
} sem_solve_info;

int sem_pcg(sem_mesh_t* mesh, const sem_pcg_opts* opts, const double* b, double* x,
            sem_solve_info* info, sem_stream_t stream);

/* ---- allocation-free solve (no counterpart in the reference).
 * For callers that may not allocate device memory while they run, such as an
 * application's allocation-free real-time loop, a memory manager that owns
 * every device byte, or a plug-in that may not grow the process's device
 * footprint.  It is the solve of sem_pcg (opA = mask(QQ'(hlmz)), SEM_F64 or
 * SEM_F64_DF, Jacobi or no preconditioner) with the direct operator kernel
 * (variant 0: no pre-split geometry), so it runs slower than a tuned sem_pcg
 * on a mesh handle. The mesh is described by arguments instead of a handle:
 * nr = ns, host Dr/Ds, and DEVICE G11, G12, G22, B in the local layout.  All
 * scratch vectors live in one fixed file-scope device array sized for
 * SEM_NOALLOC_MAX_LOCAL local DOF, about 13.4 MB.  The call allocates
 * nothing: no cudaMalloc, cudaFree, pinned host memory or library allocator.
 * Larger meshes are rejected with SEM_ERR_BAD_ARG.
 *  - Every call looks up the array's device address on the current device
 *    (cudaGetSymbolAddress).  With CUDA's default lazy module loading the
 *    first call on a device loads the array and the kernels there, which
 *    grows that device's memory use once; the array then stays until the
 *    process exits.  Make a warm-up call of the same order and precision on
 *    each device before the allocation-free region, and before any stream
 *    capture.
 *  - Every call reuses the same array and overwrites the part it needs, so
 *    calls whose GPU work overlaps (two streams, two host threads) race and
 *    corrupt each other's results; serialise them.
 *  - Like sem_pcg it synchronises the stream to read the convergence flag. */
#define SEM_NOALLOC_MAX_LOCAL 262144
int sem_pcg_noalloc(int nr, int Ex, int Ey, int periodic_x, int periodic_y, const char* bc,
                    const double* Dr, const double* Ds, const double* G11, const double* G12,
                    const double* G22, const double* B, const sem_pcg_opts* opts,
                    const double* b, double* x, sem_solve_info* info, sem_stream_t stream);

/* ---- batched solves (no counterpart in the reference, which solves one
 * system at a time): many independent pcg solves of opA = mask(QQ'(hlmz))
 * on meshes of different sizes and orders (2 <= n <= 11) in ONE persistent
 * launch of thread-block clusters that pull problems from a device work queue.
 * sem_batch_create takes the mesh handles (their bc sets the mask), one nu and
 * one k per problem and the preconditioner; it allocates the per-problem
 * workspace and the Jacobi diagonals.  sem_batch_pcg solves all problems:
 * b[i], x[i] device fields, tol[i] absolute Inf-norm tolerances, maxiter[i]
 * (NULL or <= 0: length(b)), precision SEM_F64_DF or SEM_MIXED (inner_tol,
 * max_outer as in sem_pcg_opts; <= 0 picks 1e-4 and 6); info[i] per problem.
 * Synchronous; returns SEM_ERR_NOT_CONVERGED if any problem reached maxiter. */
typedef struct sem_batch sem_batch_t;
int sem_batch_create(sem_mesh_t* const* meshes, const double* nu, const double* k, int count,
                     int precond, sem_batch_t** out);
int sem_batch_destroy(sem_batch_t* batch);
int sem_batch_pcg(sem_batch_t* batch, const double* const* b, double* const* x, const double* tol,
                  const int* maxiter, int precision, double inner_tol, int max_outer,
                  sem_solve_info* info, sem_stream_t stream);

/* ---- batch launch configuration and its autotuner (new: no counterpart in
 * the reference).  Problems are grouped by order n (groups in increasing n);
 * each group is one persistent launch whose shape is its configuration:
 * cluster_size CTAs per cluster (2, 4, 8 or 16), ctas_per_sm resident CTAs
 * per SM asked of the register allocator (1: up to 255 registers a thread,
 * 2: up to 128), and clusters persistent clusters (0: the group's share of
 * the estimated work times the clusters of its shape the device holds at
 * once, so that all groups' clusters are resident together; the heaviest
 * group launches first).  The default is 8, 2, 0.
 * n and problems are filled by sem_batch_get_config and checked by
 * sem_batch_set_config.  The queue order (sem_batch_get_order /
 * sem_batch_set_order) lists problem indices slot by slot; a group's slots
 * hold its own problems, largest estimated work first by default.
 *
 * A problem marked wide (sem_batch_set_wide, one flag per problem) is solved
 * before the persistent launches, alone on the whole GPU, by sem_pcg's
 * chunked path in the batch's arithmetic; the launches skip it.
 *
 * sem_batch_timeline returns the last sem_batch_pcg's per-problem timeline:
 * device-clock start and end in ns from the first start, and the cluster that
 * solved it (group index * 65536 + the cluster's index in the group's launch;
 * -2 for a wide problem, whose interval is its whole-GPU solve, before the
 * launches; -1 and zeros for problems the host solved in FP64), plus the
 * solve's device time in ms.
 *
 * sem_batch_autotune solves the batch once per launch shape that fits every
 * group (all groups alike, default cluster counts), builds each group's
 * makespan model from the measured per-problem durations (list scheduling
 * onto k clusters, largest first; a cluster costs the fraction of the device
 * one cluster of its shape takes when the device holds as many as fit),
 * picks per group the shape and cluster count of the smallest makespan whose
 * costs fit the device together and orders each group's queue by measured
 * duration.  It then solves once with the 32 longest problems wide, which
 * times each of them on the whole GPU, and picks how many of them (longest
 * first) to keep wide: the sum of their whole-GPU times plus the modelled
 * makespan of the rest.  Every pick is verified by a solve, and whichever
 * configuration measured fastest is kept.  With cache_path, the choice is appended to that file
 * under the batch's signature (device, arithmetic, every problem's shape,
 * coefficients and tolerance), and a later call with the same signature
 * loads it without solving.  runs receives the solves it made, best_ms the
 * fastest device time measured (0 when loaded).  x receives the last solve. */
typedef struct sem_batch_group_config {
  int n;            /* GLL points per direction of the group's problems */
  int problems;     /* problems in the group */
  int cluster_size; /* CTAs per cluster: 2, 4, 8 or 16 */
  int ctas_per_sm;  /* 1 or 2 */
  int clusters;     /* persistent clusters; 0: work-proportional share */
} sem_batch_group_config;
int sem_batch_group_count(const sem_batch_t* batch);
int sem_batch_get_config(const sem_batch_t* batch, sem_batch_group_config* cfg, int count);
int sem_batch_set_config(sem_batch_t* batch, const sem_batch_group_config* cfg, int count);
int sem_batch_get_order(const sem_batch_t* batch, int* order, int count);
int sem_batch_set_order(sem_batch_t* batch, const int* order, int count);
int sem_batch_timeline(const sem_batch_t* batch, long long* start_ns, long long* end_ns, int* cluster,
                       int count, double* total_ms);
int sem_batch_get_wide(const sem_batch_t* batch, int* wide, int count);
int sem_batch_set_wide(sem_batch_t* batch, const int* wide, int count);
int sem_batch_autotune(sem_batch_t* batch, const double* const* b, double* const* x, const double* tol,
                       const int* maxiter, int precision, double inner_tol, int max_outer, const char* cache_path,
                       int* runs, double* best_ms, sem_stream_t stream);

/* Jacobi diagonal of mask(QQ'(hlmz)) with masked entries set to 1 (new: the
 * reference has no Jacobi preconditioner; derived from src/lapl.jl:70-81) */
int sem_jacobi_diag(sem_mesh_t* mesh, const double* nu_field, double nu, double k,
                    double* diag, sem_stream_t stream);

/* ---- adjoint: per-local-copy derivative of lam' A(nu) u with respect to a
 * G-folded nodal nu, g = -(G11 lr ur + G12 (lr us + ls ur) + G22 ls us); the
 * pullback of resi(u,a) = rhs(a) - lhs(a)(u) at lam (src/adjoint.jl:13-16). */
int sem_adjoint_grad(sem_mesh_t* mesh, const double* lam, const double* u,
                     double* grad, unsigned flags, sem_stream_t stream);

/* ---- time stepping (src/time.jl:31-112, src/diffusion.jl:36-137).
 * sem_bdf_coeffs: bdfExtK(t; k) on the host.  t[0..k] = [t(i+1), t(i), ...,
 * t(i-k+1)]; repeated times are dropped (the reference's unique).  Writes the
 * extrapolation weights a[0..k-1] and the derivative weights b[0..k]; a[0] = 1
 * when every time is equal (the steady branch). */
#define SEM_BDF_MAX_ORDER 6
int sem_bdf_coeffs(int k, const double* t, double* a, double* b);

/* makeRHS! (src/diffusion.jl:51-65):
 * rhs = QQ'(mask(B f - nu lapl(ub) - sum_{i<order} bdfB[1+i] B uh[i])).
 * bdfB is a host array of order+1 entries.  f and ub may be NULL (zero
 * fields).  uh is a host array of `order` device fields.  One gather kernel
 * does it, plus one fused operator launch when ub is given. */
int sem_bdf_rhs(sem_mesh_t* mesh, double nu, int order, const double* bdfB, const double* f,
                const double* ub, const double* const* uh, double* rhs, sem_stream_t stream);

/* sem_bdf_run: nsteps of evolve! (src/diffusion.jl:81-106) on the device.
 * Each step:
 *  - shifts the histories (uh[i] <- uh[i-1], uh[0] <- u);
 *  - advances the host time history time[0..order] (in/out) by dt and
 *    recomputes bdfExtK;
 *  - sets ub and f at the new time from modes: f = sum_j fcoef[s*nf+j] F[j]
 *    and ub = sum_j bcoef[s*nb+j] UB[j], for step s of this call (at most 8
 *    modes each);
 *  - builds the right-hand side as sem_bdf_rhs does;
 *  - solves opLHS u = rhs with pcg from u = 0 and k = bdfB[1];
 *  - adds ub to u.
 * The solve options come from `solve`: precond, precision, tol, maxiter,
 * path, mult_ones.  nu and k are set per step; nu_field must be NULL.
 * The reference's Diffusion passes mult = msh.mult (mult_ones = 0) and the
 * identity preconditioner.
 * Where the single-launch small-mesh solver serves the mesh, steps are queued
 * without waiting for the host, and results are read back once per 128 steps.
 * Otherwise each solve reads its convergence flag as sem_pcg does.
 * info (NULL or nsteps entries) receives each step's solve.  A step that
 * reaches maxiter does not stop the run (the reference warns and goes on);
 * the call then returns SEM_ERR_NOT_CONVERGED at the end.  A NaN stops it. */
typedef struct {
  int order;                /* k of BDFk, 1..SEM_BDF_MAX_ORDER (the reference defaults to 3) */
  double nu;                /* scalar viscosity                                */
  double dt;                /* time step                                       */
  int nsteps;               /* steps of this call                              */
  sem_pcg_opts solve;       /* per-step solve options (nu, nu_field, k unused) */
  int nf;                   /* forcing modes                                   */
  const double* const* F;   /* host array of nf device fields                  */
  const double* fcoef;      /* host, nsteps x nf (row per step)                */
  int nb;                   /* boundary-data modes                             */
  const double* const* UB;  /* host array of nb device fields                  */
  const double* bcoef;      /* host, nsteps x nb                               */
} sem_bdf_desc;
int sem_bdf_run(sem_mesh_t* mesh, const sem_bdf_desc* desc, double* time, double* u,
                double* const* uh, sem_solve_info* info, sem_stream_t stream);

/* ---- single-domain spectral operator algebra (src/Spectral/Operators.jl,
 * src/Spectral/OperatorBasics.jl) on batches of fields.  Fields are DEVICE
 * column-major arrays, `batch` of them back to back; operator matrices are
 * DEVICE column-major; a NULL matrix is the identity (the sparse I of
 * gradOp, src/Spectral/LagrangePolynomialSpace.jl:112-138).  FP64.
 * sem_mode_product: V[a,i,b] = sum_k M[i,k] U[a,k,b] for U of shape
 *   (inner, n, outer) and M m x n: the building block of the others.
 * sem_tp2d: TensorProductOp2D mul! (Operators.jl:150-198): V = A U B' per
 *   field, U na x nb, V ma x mb.
 * sem_tp3d: (C (x) B (x) A) U per field, U na x nb x nc (the 3D
 *   tensor_product!, Operators.jl:133-145, with the B mode applied).
 * sem_axpby: out = alpha x + beta y (AffineOp, OperatorBasics.jl:130-210;
 *   x or y NULL drops its term).
 * sem_diag_apply: v = d .* u, or u ./ d when invert (DiagonalOp mul!/ldiv!,
 *   Operators.jl:37-75). */
int sem_mode_product(const double* M, int m, int n, const double* U, double* V, int64_t inner,
                     int64_t outer, sem_stream_t stream);
int sem_tp2d(const double* A, int ma, int na, const double* B, int mb, int nb, const double* U, double* V,
             int batch, sem_stream_t stream);
int sem_tp3d(const double* A, int ma, int na, const double* B, int mb, int nb, const double* C, int mc,
             int nc, const double* U, double* V, int batch, sem_stream_t stream);
int sem_axpby(double alpha, const double* x, double beta, const double* y, double* out, int64_t len,
              sem_stream_t stream);
int sem_diag_apply(const double* d, const double* u, double* v, int64_t len, int invert,
                   sem_stream_t stream);

/* ---- instrumentation (no counterpart in the reference, which only prints
 * @time): CUDA-event timing of every launch of the fused element-operator
 * kernel while enabled; read returns the summed kernel time and the number of
 * launches since the last read (and resets them). */
int sem_timing_enable(int on);
int sem_timing_read(double* total_ms, int* launches);
/* waits of the TMA operator kernel (variant 6) on this device that gave up
 * after their time bound (about 2 s) since the last reset; each such CTA left
 * its tile unfinished (a double-float call is then recomputed by its native
 * FP64 re-run).  reset != 0 clears the count after reading it.  Synchronous. */
int sem_wait_timeouts(int reset, unsigned* count);

#ifdef __cplusplus
}
#endif
#endif /* SEM_B200_H */
