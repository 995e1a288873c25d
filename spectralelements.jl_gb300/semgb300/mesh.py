"""Device mesh handle with the field names of the reference ``Mesh``
(src/mesh.jl:25-64) and ``generateMask`` (src/mesh.jl:149-175).

Fields are CUDA float64 tensors of shape (nr*Ex, ns*Ey) with column-major
strides (1, nr*Ex): the reference's local layout, byte for byte.
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np
import torch

from . import _lib
from .host import derivMat, fixU, gausslobatto, ndgrid, semmesh, semq_index


def local_empty(nx: int, ny: int, dtype=torch.float64, device=None) -> torch.Tensor:
    """Uninitialised field in the reference layout (column-major)."""
    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    return torch.empty_strided((nx, ny), (1, nx), dtype=dtype, device=dev)


def as_local(t, dtype=torch.float64) -> torch.Tensor:
    """Return a CUDA tensor of the same values in column-major layout."""
    if isinstance(t, np.ndarray):
        t = torch.from_numpy(np.asfortranarray(t))
    if not isinstance(t, torch.Tensor):
        raise TypeError("expected a torch tensor or NumPy array")
    if t.dim() != 2:
        raise ValueError("fields are 2D (nr*Ex, ns*Ey) arrays")
    if t.device.type != "cuda":
        t = t.to("cuda")
    if t.dtype != dtype:
        t = t.to(dtype)
    if t.stride() != (1, t.shape[0]):
        t = t.t().contiguous().t()
    return t


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def _ptr(a) -> int:
    return 0 if a is None else a.data_ptr()


class QQt:
    """Structured stand-in for the dense QQtx / QQty of the reference
    (src/mesh.jl:44-45, 81-82): Q Q' of ``semq(E, n, periodic)``.  ``dense()``
    materialises the matrix for small meshes."""

    def __init__(self, E: int, n: int, periodic: bool, mesh=None):
        self.E, self.n, self.periodic = E, n, bool(periodic)
        self._mesh = weakref.ref(mesh) if mesh is not None else None

    @property
    def shape(self):
        return (self.E * self.n, self.E * self.n)

    def dense(self) -> np.ndarray:
        g, ng = semq_index(self.E, self.n, self.periodic)
        Q = np.zeros((self.E * self.n, ng))
        Q[np.arange(self.E * self.n), g] = 1.0
        return Q @ Q.T


_MASKS: "weakref.WeakValueDictionary[int, torch.Tensor]" = weakref.WeakValueDictionary()
_MASK_BC: dict = {}


def _register_mask(M: torch.Tensor, bc: str, periodic):
    key = id(M)
    _MASKS[key] = M
    _MASK_BC[key] = (bc, tuple(periodic))
    weakref.finalize(M, _MASK_BC.pop, key, None)


def mask_bc_of(M):
    """bc string of a mask made by generateMask, or None."""
    if M is None:
        return None
    key = id(M)
    if key in _MASK_BC and _MASKS.get(key) is M:
        return _MASK_BC[key][0]
    return None


class Mesh:
    """``Mesh(nr, ns, Ex, Ey, ifperiodic=[false,false], deform=fixU)``.

    Host set-up (GLL points, derivative matrices, grid, user deformation) runs
    on the CPU as in src/mesh.jl:66-108; the Jacobian, mass matrix and metric
    factors are computed on the device (src/jac.jl:24-40,
    src/mesh.jl:111-123).  Deviation from the reference: Qy is built from Ey
    (src/mesh.jl:80 passes Ex, which only works for Ex == Ey).
    """

    def __init__(self, nr, ns, Ex, Ey, ifperiodic=(False, False), deform=fixU, *, bc=None,
                 precision=_lib.SEM_F64_DF, _arrays=None):
        self.nr, self.ns, self.Ex, self.Ey = int(nr), int(ns), int(Ex), int(Ey)
        self.ifperiodic = [bool(ifperiodic[0]), bool(ifperiodic[1])]
        self.deform = deform
        if _arrays is None:
            self.zr, self.wr = gausslobatto(self.nr)
            self.zs, self.ws = gausslobatto(self.ns)
            self.Dr = derivMat(self.zr)
            self.Ds = derivMat(self.zs)
            xe, _ = semmesh(self.Ex, self.nr)
            ye, _ = semmesh(self.Ey, self.ns)
            x, y = ndgrid(xe, ye)
            x, y = deform(x, y)
            geom = None
        else:
            self.zr, self.wr, self.zs, self.ws = (np.asarray(_arrays[k], dtype=np.float64)
                                                  for k in ("zr", "wr", "zs", "ws"))
            self.Dr = np.asarray(_arrays["Dr"], dtype=np.float64)
            self.Ds = np.asarray(_arrays["Ds"], dtype=np.float64)
            x, y = _arrays["x"], _arrays["y"]
            geom = [_arrays.get(k) for k in ("G11", "G12", "G22", "B")]
            if any(g is None for g in geom):
                geom = None
        lib = _lib.load()
        f = lambda a: np.asfortranarray(np.asarray(a, dtype=np.float64))  # noqa: E731
        self._host = {"Dr": f(self.Dr), "Ds": f(self.Ds), "wr": f(self.wr), "ws": f(self.ws),
                      "x": f(x), "y": f(y)}
        d = _lib.MeshDesc()
        d.nr, d.ns, d.Ex, d.Ey = self.nr, self.ns, self.Ex, self.Ey
        d.periodic_x, d.periodic_y = int(self.ifperiodic[0]), int(self.ifperiodic[1])
        for k in ("Dr", "Ds", "wr", "ws", "x", "y"):
            setattr(d, k, self._host[k].ctypes.data)
        if geom is not None:
            for k, g in zip(("G11", "G12", "G22", "B"), geom):
                self._host[k] = f(g)
                setattr(d, k, self._host[k].ctypes.data)
        self._bc = bc
        d.bc = bc.encode() if bc else None
        h = ctypes.c_void_p()
        torch.cuda.current_device()  # make sure the CUDA context of the current device exists
        _lib.check(lib.sem_mesh_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self._fields = {}
        self.QQtx = QQt(self.Ex, self.nr, self.ifperiodic[0], self)
        self.QQty = QQt(self.Ey, self.ns, self.ifperiodic[1], self)
        self.l2gx, self.nxg = semq_index(self.Ex, self.nr, self.ifperiodic[0])
        self.l2gy, self.nyg = semq_index(self.Ey, self.ns, self.ifperiodic[1])
        self.set_precision(precision)

    @classmethod
    def from_arrays(cls, nr, Ex, Ey, ifperiodic, arrays, bc=None, precision=_lib.SEM_F64_DF):
        """Handle from host arrays computed elsewhere (zr, wr, zs, ws, Dr, Ds, x, y and
        optionally G11, G12, G22, B), as a Julia ``Mesh`` hands them over."""
        return cls(nr, nr, Ex, Ey, ifperiodic, _arrays=arrays, bc=bc, precision=precision)

    # -- handle management
    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sem_mesh_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_bc(self, bc):
        _lib.check(self._lib.sem_mesh_set_bc(self._h, bc.encode() if bc else None))
        self._bc = bc
        self._fields.pop("mask", None)

    @property
    def bc(self):
        return self._bc

    def set_precision(self, precision):
        _lib.check(self._lib.sem_mesh_set_precision(self._h, int(precision)))
        self.precision = int(precision)

    def autotune(self, precision=None):
        """Time the fused-kernel variants on this mesh and keep the fastest
        (per precision); returns {variant: ms}."""
        prec = self.precision if precision is None else int(precision)
        ms = (ctypes.c_double * _lib.SEM_VARIANTS)()
        ch = ctypes.c_int()
        _lib.check(self._lib.sem_mesh_autotune(self._h, prec, ms, ctypes.byref(ch)))
        return {"chosen": ch.value, "ms": list(ms)}

    def set_variant(self, variant, precision=None):
        prec = self.precision if precision is None else int(precision)
        _lib.check(self._lib.sem_mesh_set_variant(self._h, prec, int(variant)))

    @property
    def shape(self):
        return (self.nr * self.Ex, self.ns * self.Ey)

    def empty(self, dtype=torch.float64):
        return local_empty(*self.shape, dtype=dtype)

    def field(self, name: str) -> torch.Tensor:
        if name not in self._fields:
            out = self.empty()
            _lib.check(self._lib.sem_mesh_field(self._h, _lib.FIELDS[name], out.data_ptr(),
                                                stream_ptr()))
            self._fields[name] = out
        return self._fields[name]

    def __getattr__(self, name):
        if name in ("x", "y", "Jac", "Jaci", "rx", "ry", "sx", "sy", "B", "Bi", "G11", "G12",
                    "G22", "mult"):
            return self.field(name)
        raise AttributeError(name)


def generateMask(bc, msh: Mesh) -> torch.Tensor:
    """Dirichlet mask R'R (src/mesh.jl:149-175): bc = [xmin, xmax, ymin, ymax],
    'D' zeroes the first/last local row/column; a periodic direction keeps all.
    Returns a CUDA bool tensor in the local layout."""
    bcs = "".join(bc)
    if len(bcs) != 4 or any(c not in "DN" for c in bcs):
        raise ValueError("bc must be 4 of 'D'/'N'")
    nx, ny = msh.shape
    mx = torch.ones(nx, dtype=torch.bool)
    my = torch.ones(ny, dtype=torch.bool)
    if bcs[0] == "D":
        mx[0] = False
    if bcs[1] == "D":
        mx[-1] = False
    if bcs[2] == "D":
        my[0] = False
    if bcs[3] == "D":
        my[-1] = False
    if msh.ifperiodic[0]:
        mx[:] = True
    if msh.ifperiodic[1]:
        my[:] = True
    M = as_local(torch.outer(mx, my).to(torch.float64)).to(torch.bool)
    M = M.t().contiguous().t()
    _register_mask(M, bcs, msh.ifperiodic)
    return M
