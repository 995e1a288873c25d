"""ctypes wrapper of the C oracle (test infrastructure only; see sem_oracle.c)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from build_oracle import build


class _Grid(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in
                ("n", "Ex", "Ey", "perx", "pery", "dxmin", "dxmax", "dymin", "dymax")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        _lib.so_apply.argtypes = [ctypes.POINTER(_Grid), P, P, P, P, P, P, P, P, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_int, P, P, P]
        _lib.so_apply.restype = None
        _lib.so_gather_scatter.argtypes = [ctypes.POINTER(_Grid), P, P]
        _lib.so_gather_scatter.restype = None
        _lib.so_pcg.argtypes = [ctypes.POINTER(_Grid), P, P, P, P, P, P, P, ctypes.c_double,
                                ctypes.c_double, P, P, P, ctypes.c_double, ctypes.c_int,
                                ctypes.POINTER(ctypes.c_double)]
        _lib.so_pcg.restype = ctypes.c_int
    return _lib


def grid(n, Ex, Ey, periodic=(False, False), bc=None):
    g = _Grid()
    g.n, g.Ex, g.Ey = n, Ex, Ey
    g.perx, g.pery = int(periodic[0]), int(periodic[1])
    bc = bc or "NNNN"
    g.dxmin, g.dxmax, g.dymin, g.dymax = (int(c == "D") for c in bc)
    return g


def _f(a):
    return None if a is None else np.asfortranarray(np.asarray(a, dtype=np.float64))


def _p(a):
    return None if a is None else a.ctypes.data


def apply(g, Dr, Ds, G11, G12, G22, B, u, nu=1.0, k=0.0, nu_f=None, nug=None, gs=True, msk=True):
    """mask(QQ'(nu lapl(u) + k B u)) on the CPU (OpenMP threads)."""
    arrs = [_f(a) for a in (Dr, Ds, G11, G12, G22, B, nu_f, nug, u)]
    out = np.empty_like(arrs[-1], order="F")
    work = np.empty_like(out, order="F")
    lib().so_apply(ctypes.byref(g), *(_p(a) for a in arrs[:8]), float(nu), float(k),
                   (1 if gs else 0) | (2 if msk else 0), _p(arrs[8]), _p(out), _p(work))
    return out


def gather_scatter(g, u):
    u = _f(u)
    out = np.empty_like(u, order="F")
    lib().so_gather_scatter(ctypes.byref(g), _p(u), _p(out))
    return out


def pcg(g, Dr, Ds, G11, G12, G22, B, b, nu=1.0, k=0.0, d=None, nug=None, tol=1e-8, maxiter=None):
    arrs = [_f(a) for a in (Dr, Ds, G11, G12, G22, B, nug, d, b)]
    x = np.empty_like(arrs[-1], order="F")
    res = ctypes.c_double()
    it = lib().so_pcg(ctypes.byref(g), *(_p(a) for a in arrs[:7]), float(nu), float(k),
                      _p(arrs[7]), _p(arrs[8]), _p(x), float(tol),
                      int(maxiter if maxiter is not None else x.size), ctypes.byref(res))
    return x, it, res.value


def threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
