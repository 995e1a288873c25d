"""Loading and building of the native library libsem_b200.so (ctypes).

The library is built in-tree by ``build()`` (nvcc for sm_103a, one object per
translation unit, compiled in parallel) and loaded from
``spectralelements.jl_gb300/lib/``.  There is no pure-Python fallback: every
operator of this package calls the library, and loading fails loudly when it
is missing.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)                      # spectralelements.jl_gb300/
CSRC = os.path.join(ROOT, "csrc")
LIB_DIR = os.path.join(ROOT, "lib")
BUILD_DIR = os.path.join(ROOT, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libsem_b200.so")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]

SOURCES = ["sem_api.cu", "sem_apply.cu", "sem_apply_f64.cu", "sem_apply_df.cu", "sem_apply_f32.cu",
           "sem_apply_f64_hi.cu", "sem_apply_df_hi.cu", "sem_apply_f32_hi.cu", "sem_vec.cu", "sem_geom.cu", "sem_pcg.cu", "sem_batch.cu", "sem_batch_ka.cu",
           "sem_batch_kb.cu", "sem_batch_kc.cu", "sem_batch_kd.cu", "sem_batch_ke.cu", "sem_batch_kf.cu", "sem_small.cu", "sem_tiny.cu", "sem_ext.cu", "sem_time.cu", "sem_spectral.cu", "sem_host.cu"]


class SemError(RuntimeError):
    """A libsem_b200 call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[sem status {status}] {message}")
        self.status = status


class NotConverged(SemError):
    """pcg reached maxiter (the reference prints a warning and returns x)."""


SEM_OK, SEM_ERR_BAD_ARG, SEM_ERR_NOT_CONVERGED, SEM_ERR_NAN, SEM_ERR_TIMEOUT, SEM_ERR_CUDA, \
    SEM_ERR_UNSUPPORTED, SEM_ERR_NO_MEMORY = range(8)
SEM_GS, SEM_MASK, SEM_NU_IN_G = 1, 2, 4
SEM_HOST_DIRECT = -1  # sem_hlmz_host slabs: kernels read and write the host buffers in place
SEM_F64, SEM_F64_DF, SEM_F32, SEM_MIXED, SEM_MIXED_RR = 0, 1, 2, 3, 4
SEM_PRECOND_NONE, SEM_PRECOND_JACOBI = 0, 1
SEM_PATH_AUTO, SEM_PATH_CHUNKED, SEM_PATH_SMALL = 0, 1, 2
SEM_SMALL_MAX_LOCAL = 100000  # include/sem_b200.h
SEM_VARIANTS = 7  # fused element-operator kernel variants (include/sem_b200.h)
SEM_BDF_MAX_ORDER = 6  # include/sem_b200.h
FIELDS = {"x": 0, "y": 1, "Jac": 2, "Jaci": 3, "rx": 4, "ry": 5, "sx": 6, "sy": 7, "B": 8,
          "Bi": 9, "G11": 10, "G12": 11, "G22": 12, "mult": 13, "mask": 14}


def _sources():
    return [os.path.join(CSRC, s) for s in SOURCES]


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "sem_b200.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile csrc/*.cu for sm_103a and link libsem_b200.so (in-tree)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    deps = _deps()
    if not force and not _stale(LIB_PATH, deps):
        return LIB_PATH
    objs = []
    jobs = []
    for src in _sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src).replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, deps):
            jobs.append(["nvcc", *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            print(" ".join(cmd))
        return r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        list(ex.map(run, jobs))
    run(["nvcc", *ARCH, "-shared", "-o", LIB_PATH, *objs])
    return LIB_PATH


class PcgOpts(ctypes.Structure):
    _fields_ = [("nu", ctypes.c_double), ("nu_field", ctypes.c_void_p), ("k", ctypes.c_double),
                ("precond", ctypes.c_int), ("precision", ctypes.c_int), ("tol", ctypes.c_double),
                ("maxiter", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("max_outer", ctypes.c_int), ("check_every", ctypes.c_int),
                ("mult_ones", ctypes.c_int), ("path", ctypes.c_int)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("outer", ctypes.c_int), ("res_inf", ctypes.c_double),
                ("res0_inf", ctypes.c_double), ("converged", ctypes.c_int)]


class BatchGroupConfig(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("problems", ctypes.c_int), ("cluster_size", ctypes.c_int),
                ("ctas_per_sm", ctypes.c_int), ("clusters", ctypes.c_int)]


class BdfDesc(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("nu", ctypes.c_double), ("dt", ctypes.c_double),
                ("nsteps", ctypes.c_int), ("solve", PcgOpts), ("nf", ctypes.c_int),
                ("F", ctypes.POINTER(ctypes.c_void_p)), ("fcoef", ctypes.POINTER(ctypes.c_double)),
                ("nb", ctypes.c_int), ("UB", ctypes.POINTER(ctypes.c_void_p)),
                ("bcoef", ctypes.POINTER(ctypes.c_double))]


class MeshDesc(ctypes.Structure):
    _fields_ = [("nr", ctypes.c_int), ("ns", ctypes.c_int), ("Ex", ctypes.c_int),
                ("Ey", ctypes.c_int), ("periodic_x", ctypes.c_int), ("periodic_y", ctypes.c_int),
                ("Dr", ctypes.c_void_p), ("Ds", ctypes.c_void_p), ("wr", ctypes.c_void_p),
                ("ws", ctypes.c_void_p), ("x", ctypes.c_void_p), ("y", ctypes.c_void_p),
                ("G11", ctypes.c_void_p), ("G12", ctypes.c_void_p), ("G22", ctypes.c_void_p),
                ("B", ctypes.c_void_p), ("bc", ctypes.c_char_p)]


# exported symbols and their ctypes signatures (mirrors include/sem_b200.h)
_P, _I, _D, _U, _L = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint, ctypes.c_int64
SIGNATURES = {
    "sem_mesh_create": (_I, [ctypes.POINTER(MeshDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "sem_mesh_destroy": (_I, [_P]),
    "sem_mesh_set_bc": (_I, [_P, ctypes.c_char_p]),
    "sem_mesh_set_precision": (_I, [_P, _I]),
    "sem_mesh_autotune": (_I, [_P, _I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]),
    "sem_mesh_set_variant": (_I, [_P, _I, _I]),
    "sem_mesh_field": (_I, [_P, _I, _P, _P]),
    "sem_mesh_dims": (_I, [_P, ctypes.POINTER(_L), ctypes.POINTER(_L)]),
    "sem_last_error": (ctypes.c_char_p, []),
    "sem_abi_version": (_I, []),
    "sem_abu": (_I, [_P, _I, _I, _P, _I, _I, _P, _I, _I, _P, _P]),
    "sem_lapl": (_I, [_P, _P, _P, _U, _P]),
    "sem_lapl_nu": (_I, [_P, _P, _P, _P, _U, _P]),
    "sem_hlmz": (_I, [_P, _P, _D, _D, _P, _P, _U, _P]),
    "sem_varcoef": (_I, [_P, _P, _D, _P, _P, _U, _P]),
    "sem_hlmz_host": (_I, [_P, _P, _D, _D, _P, _P, _U, _I, _P]),
    "sem_mass": (_I, [_P, _P, _P, _U, _P]),
    "sem_gather_scatter": (_I, [_P, _P, _P, _P]),
    "sem_gather_scatter_grid": (_I, [_I, _I, _I, _I, _I, _I, _P, _P, _P]),
    "sem_mask": (_I, [_P, _P, _P, _L, _P]),
    "sem_mask_bc": (_I, [_P, _P, _P, _P]),
    "sem_lapl_geom": (_I, [_I, _I, _I, _I, _I, _I, ctypes.c_char_p, _P, _P, _P, _P, _P, _P, _P,
                           _U, _I, _P]),
    "sem_laplace_dealiased": (_I, [_I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sem_mass_dealiased": (_I, [_I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P]),
    "sem_grad": (_I, [_P, _P, _P, _P, _P]),
    "sem_grad_t": (_I, [_P, _P, _P, _P, _P]),
    "sem_advect": (_I, [_P, _P, _P, _P, _P, _P]),
    "sem_advect_dealiased": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "sem_pcg": (_I, [_P, ctypes.POINTER(PcgOpts), _P, _P, ctypes.POINTER(SolveInfo), _P]),
    "sem_pcg_noalloc": (_I, [_I, _I, _I, _I, _I, ctypes.c_char_p, _P, _P, _P, _P, _P, _P,
                             ctypes.POINTER(PcgOpts), _P, _P, ctypes.POINTER(SolveInfo), _P]),
    "sem_batch_create": (_I, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(_D),
                              ctypes.POINTER(_D), _I, _I, ctypes.POINTER(ctypes.c_void_p)]),
    "sem_batch_destroy": (_I, [_P]),
    "sem_batch_pcg": (_I, [_P, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                           ctypes.POINTER(_D), ctypes.POINTER(_I), _I, _D, _I,
                           ctypes.POINTER(SolveInfo), _P]),
    "sem_batch_group_count": (_I, [_P]),
    "sem_batch_get_config": (_I, [_P, ctypes.POINTER(BatchGroupConfig), _I]),
    "sem_batch_set_config": (_I, [_P, ctypes.POINTER(BatchGroupConfig), _I]),
    "sem_batch_get_order": (_I, [_P, ctypes.POINTER(_I), _I]),
    "sem_batch_set_order": (_I, [_P, ctypes.POINTER(_I), _I]),
    "sem_batch_timeline": (_I, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                                ctypes.POINTER(_I), _I, ctypes.POINTER(_D)]),
    "sem_batch_get_wide": (_I, [_P, ctypes.POINTER(_I), _I]),
    "sem_batch_set_wide": (_I, [_P, ctypes.POINTER(_I), _I]),
    "sem_batch_autotune": (_I, [_P, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                ctypes.POINTER(_D), ctypes.POINTER(_I), _I, _D, _I, ctypes.c_char_p,
                                ctypes.POINTER(_I), ctypes.POINTER(_D), _P]),
    "sem_jacobi_diag": (_I, [_P, _P, _D, _D, _P, _P]),
    "sem_adjoint_grad": (_I, [_P, _P, _P, _P, _U, _P]),
    "sem_bdf_coeffs": (_I, [_I, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    "sem_bdf_rhs": (_I, [_P, _D, _I, ctypes.POINTER(_D), _P, _P, ctypes.POINTER(ctypes.c_void_p), _P, _P]),
    "sem_bdf_run": (_I, [_P, ctypes.POINTER(BdfDesc), ctypes.POINTER(_D), _P,
                         ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(SolveInfo), _P]),
    "sem_mode_product": (_I, [_P, _I, _I, _P, _P, _L, _L, _P]),
    "sem_tp2d": (_I, [_P, _I, _I, _P, _I, _I, _P, _P, _I, _P]),
    "sem_tp3d": (_I, [_P, _I, _I, _P, _I, _I, _P, _I, _I, _P, _P, _I, _P]),
    "sem_axpby": (_I, [_D, _P, _D, _P, _P, _L, _P]),
    "sem_diag_apply": (_I, [_P, _P, _P, _L, _I, _P]),
    "sem_timing_enable": (_I, [_I]),
    "sem_timing_read": (_I, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]),
    "sem_wait_timeouts": (_I, [_I, ctypes.POINTER(ctypes.c_uint)]),
}

_lib = None
_lock = threading.Lock()


def load(path: str | None = None):
    """Load libsem_b200.so; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or os.environ.get("SEM_B200_LIB", LIB_PATH)
        if not os.path.exists(p):
            raise RuntimeError(
                f"libsem_b200.so not found at {p}: run __graft_entry__.build() "
                "(there is no CPU fallback)")
        lib = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int):
    if status == SEM_OK:
        return
    msg = (load().sem_last_error() or b"").decode(errors="replace")
    if status == SEM_ERR_NOT_CONVERGED:
        raise NotConverged(status, msg)
    raise SemError(status, msg)
