"""Operators with the reference's call signatures, on device fields.

Each function allocates and returns a new field (the reference's operators are
functional) and launches libsem_b200 kernels on the current torch stream.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .mesh import Mesh, QQt, as_local, local_empty, mask_bc_of, stream_ptr


def _empty(x) -> bool:
    """Julia's ``[]``: None, an empty list/tuple or a size-0 array."""
    if x is None:
        return True
    if isinstance(x, (list, tuple)):
        return len(x) == 0
    if isinstance(x, torch.Tensor):
        return x.numel() == 0
    if isinstance(x, np.ndarray):
        return x.size == 0
    return False


def _field(u, msh):
    """u as a device field checked against the mesh's local shape."""
    u = as_local(u)
    if tuple(u.shape) != msh.shape:
        raise ValueError(f"field of shape {tuple(u.shape)} on a mesh of local shape {msh.shape}")
    return u


def _host_matrix(A):
    if _empty(A):
        return None
    if isinstance(A, torch.Tensor):
        A = A.detach().cpu().numpy()
    return np.asfortranarray(np.asarray(A, dtype=np.float64))


def ABu(As, Br, u):
    """v = (As (x) Br) u (src/ABu.jl:9-37); ``[]``/None means identity."""
    lib = _lib.load()
    u = as_local(u)
    A = _host_matrix(As)
    B = _host_matrix(Br)
    m, n = u.shape
    mo = m if B is None else m * B.shape[0] // B.shape[1]
    no = n if A is None else (n // A.shape[1]) * A.shape[0]
    v = local_empty(mo, no)
    _lib.check(lib.sem_abu(
        None if A is None else A.ctypes.data, 0 if A is None else A.shape[0],
        0 if A is None else A.shape[1],
        None if B is None else B.ctypes.data, 0 if B is None else B.shape[0],
        0 if B is None else B.shape[1], u.data_ptr(), m, n, v.data_ptr(), stream_ptr()))
    return v


def _block_of(D, n):
    """An n x n derivative matrix, or the diagonal block of kron(I_E, D)
    (examples/p2d_explicit.jl:28 passes the block-diagonal form)."""
    D = _host_matrix(D)
    if D.shape == (n, n):
        return D
    if D.shape[0] == D.shape[1] and D.shape[0] % n == 0:
        E = D.shape[0] // n
        blk = D[:n, :n]
        if np.array_equal(D, np.kron(np.eye(E), blk)):
            return np.asfortranarray(blk)
    raise ValueError("derivative matrix must be n x n or kron(I, D) with an n x n block")


def lapl(u, *args):
    """lapl(u, msh) (src/lapl.jl:26-36); lapl(u, nu, msh) = nu .* lapl (:38-45);
    lapl(u, msh1, msh2) (:47-52, the reference ignores msh2); and the functional
    lapl(u, M, Jr, Js, QQtx, QQty, Dr, Ds, G11, G12, G22, mult) (:54-68)."""
    lib = _lib.load()
    if len(args) == 1 or (len(args) == 2 and isinstance(args[0], Mesh) and isinstance(args[1], Mesh)):
        msh = args[0]
        u = _field(u, msh)
        out = msh.empty()
        _lib.check(lib.sem_lapl(msh.handle, u.data_ptr(), out.data_ptr(), 0, stream_ptr()))
        return out
    if len(args) == 2:
        nu, msh = args
        u = _field(u, msh)
        out = msh.empty()
        if isinstance(nu, (int, float)):
            _lib.check(lib.sem_hlmz(msh.handle, None, float(nu), 0.0, u.data_ptr(), out.data_ptr(),
                                    0, stream_ptr()))
        else:
            nu = as_local(nu)
            _lib.check(lib.sem_lapl_nu(msh.handle, nu.data_ptr(), u.data_ptr(), out.data_ptr(), 0,
                                       stream_ptr()))
        return out
    if len(args) == 11:
        return _lapl_functional(u, *args)
    raise TypeError("lapl: unsupported signature")


def _rect_block_of(J, n, E):
    """An m x n interpolation matrix, or the diagonal block of kron(I_E, J)."""
    J = _host_matrix(J)
    if J.shape[1] == n:
        return J
    if J.shape[1] == n * E and J.shape[0] % E == 0:
        m = J.shape[0] // E
        blk = J[:m, :n]
        if np.array_equal(J, np.kron(np.eye(E), blk)):
            return np.asfortranarray(blk)
    raise ValueError("interpolation matrix must be m x n or kron(I, J) with an m x n block")


def _gs_mask(out, M, QQtx, QQty):
    if not _empty(QQtx):
        out = gatherScatter(out, QQtx, QQty)
    if not _empty(M):
        out = mask(out, M)
    return out


def _lapl_dealiased(u, M, Jr, Js, QQtx, QQty, Dr, Ds, G11, G12, G22):
    """Dealiased functional lapl: laplace(u,Jr,Js,Dr,Ds,G11,G12,G22)
    (src/lapl.jl:83-103) on the device, then QQ' and mask (:54-68)."""
    lib = _lib.load()
    u = as_local(u)
    nx, ny = u.shape
    n = QQtx.n if isinstance(QQtx, QQt) else _infer_n(Dr, nx)
    Ex, Ey = nx // n, ny // n
    Drb, Dsb = _block_of(Dr, n), _block_of(Ds, n)
    Jrb, Jsb = _rect_block_of(Jr, n, Ex), _rect_block_of(Js, n, Ey)
    G11, G12, G22 = as_local(G11), as_local(G12), as_local(G22)
    out = local_empty(nx, ny)
    _lib.check(lib.sem_laplace_dealiased(n, Jrb.shape[0], Jsb.shape[0], Ex, Ey, Jrb.ctypes.data,
                                         Jsb.ctypes.data, Drb.ctypes.data, Dsb.ctypes.data,
                                         G11.data_ptr(), G12.data_ptr(), G22.data_ptr(), u.data_ptr(),
                                         out.data_ptr(), stream_ptr()))
    return _gs_mask(out, M, QQtx, QQty)


def _lapl_functional(u, M, Jr, Js, QQtx, QQty, Dr, Ds, G11, G12, G22, mult):
    lib = _lib.load()
    if not (_empty(Jr) and _empty(Js)):
        return _lapl_dealiased(u, M, Jr, Js, QQtx, QQty, Dr, Ds, G11, G12, G22)
    u = as_local(u)
    nx, ny = u.shape
    gs = not _empty(QQtx)
    if gs and not (isinstance(QQtx, QQt) and isinstance(QQty, QQt)):
        raise TypeError("pass the mesh's structured QQtx/QQty (Mesh.QQtx), not dense matrices")
    if gs:
        n = QQtx.n
        Ex, Ey, perx, pery = QQtx.E, QQty.E, QQtx.periodic, QQty.periodic
    else:
        n = _infer_n(Dr, nx)
        Ex, Ey, perx, pery = nx // n, ny // n, False, False
    Drb, Dsb = _block_of(Dr, n), _block_of(Ds, n)
    bc = None if _empty(M) else mask_bc_of(M)
    flags = (_lib.SEM_GS if gs else 0) | (_lib.SEM_MASK if bc else 0)
    G11, G12, G22 = as_local(G11), as_local(G12), as_local(G22)
    out = local_empty(nx, ny)
    _lib.check(lib.sem_lapl_geom(n, n, Ex, Ey, int(perx), int(pery), bc.encode() if bc else None,
                                 Drb.ctypes.data, Dsb.ctypes.data, G11.data_ptr(), G12.data_ptr(),
                                 G22.data_ptr(), u.data_ptr(), out.data_ptr(), flags,
                                 _lib.SEM_F64_DF, stream_ptr()))
    if not _empty(M) and bc is None:
        out = mask(out, M)
    return out


def _infer_n(D, nx):
    """Smallest n with D == kron(I, D[:n,:n]) (a dense element matrix gives its own size)."""
    D = _host_matrix(D)
    for n in range(2, 18):
        if D.shape[0] % n == 0 and nx % n == 0:
            try:
                _block_of(D, n)
                return n
            except ValueError:
                pass
    raise ValueError("cannot infer the element order from D")


def mass(u, *args):
    """mass(u, msh) = B .* u (src/mass.jl:12-22); mass(u, msh1, msh2) (:25-30);
    functional mass(u, M, B, Jr, Js, QQtx, QQty, mult) (:32-50)."""
    lib = _lib.load()
    if len(args) in (1, 2) and isinstance(args[0], Mesh):
        msh = args[0]
        u = _field(u, msh)
        out = msh.empty()
        _lib.check(lib.sem_mass(msh.handle, u.data_ptr(), out.data_ptr(), 0, stream_ptr()))
        return out
    if len(args) == 7:
        M, B, Jr, Js, QQtx, QQty, mult = args
        if not (_empty(Jr) and _empty(Js)):
            # J'(B .* (J u)) on the device (src/mass.jl:37-42), then QQ' and mask
            u = as_local(u)
            nx, ny = u.shape
            if isinstance(QQtx, QQt):
                n = QQtx.n
            else:
                # without QQ' the element order comes from an m x n block Jr
                n = _host_matrix(Jr).shape[1]
                if n > 32 or nx % n:
                    raise ValueError("pass Jr as an m x n element block or give the mesh's QQtx")
            Ex, Ey = nx // n, ny // n
            Jrb, Jsb = _rect_block_of(Jr, n, Ex), _rect_block_of(Js, n, Ey)
            Bf = None if _empty(B) else as_local(B)
            out = local_empty(nx, ny)
            _lib.check(lib.sem_mass_dealiased(n, Jrb.shape[0], Jsb.shape[0], Ex, Ey, Jrb.ctypes.data,
                                              Jsb.ctypes.data, None if Bf is None else Bf.data_ptr(),
                                              u.data_ptr(), out.data_ptr(), stream_ptr()))
            return _gs_mask(out, M, QQtx, QQty)
        u = as_local(u)
        Bu = u.clone(memory_format=torch.preserve_format) if _empty(B) else mask(u, B)
        if not _empty(QQtx):
            Bu = gatherScatter(Bu, QQtx, QQty)
        return mask(Bu, M)
    raise TypeError("mass: unsupported signature")


def hlmz(u, nu, k, *mshs):
    """hlmz(u, nu, k, msh) = nu .* lapl(u) + k .* mass(u) (src/hlmz.jl:12-19);
    the dealiased hlmz(u, nu, k, msh1, msh2) calls the same (:22-30)."""
    lib = _lib.load()
    msh = mshs[0]
    u = _field(u, msh)
    out = msh.empty()
    if isinstance(nu, (int, float)):
        _lib.check(lib.sem_hlmz(msh.handle, None, float(nu), float(k), u.data_ptr(),
                                out.data_ptr(), 0, stream_ptr()))
    else:
        nu = as_local(nu)
        _lib.check(lib.sem_hlmz(msh.handle, nu.data_ptr(), 1.0, float(k), u.data_ptr(),
                                out.data_ptr(), 0, stream_ptr()))
    return out


def gatherScatter(u, *args):
    """QQ' u: gatherScatter(u, QQtx, QQty) (src/gatherScatter.jl:8-16) or
    gatherScatter(u, msh) (:18-21)."""
    lib = _lib.load()
    if len(args) == 1 and isinstance(args[0], Mesh):
        msh = args[0]
    elif len(args) == 2 and isinstance(args[0], QQt):
        msh = args[0]._mesh() if args[0]._mesh is not None else None
        if msh is None:
            raise ValueError("QQt is not attached to a live mesh")
    elif len(args) == 2:
        # dense (or array-like) QQtx, QQty: the numbering is read from them
        from .host import qq_structure
        nr, Ex, px = qq_structure(_host_matrix(args[0]))
        ns, Ey, py = qq_structure(_host_matrix(args[1]))
        u = as_local(u)
        if tuple(u.shape) != (nr * Ex, ns * Ey):
            raise ValueError("field shape does not match QQtx/QQty")
        out = local_empty(*u.shape)
        _lib.check(lib.sem_gather_scatter_grid(nr, ns, Ex, Ey, int(px), int(py), u.data_ptr(),
                                               out.data_ptr(), stream_ptr()))
        return out
    else:
        raise TypeError("gatherScatter(u, msh) or gatherScatter(u, msh.QQtx, msh.QQty)")
    u = _field(u, msh)
    out = msh.empty()
    _lib.check(lib.sem_gather_scatter(msh.handle, u.data_ptr(), out.data_ptr(), stream_ptr()))
    return out


def mask(u, M):
    """Mu = M .* u (src/mask.jl:10-18); an empty M returns a copy."""
    lib = _lib.load()
    u = as_local(u)
    out = local_empty(*u.shape)
    if _empty(M):
        _lib.check(lib.sem_mask(None, u.data_ptr(), out.data_ptr(), u.numel(), stream_ptr()))
        return out
    Mf = as_local(M if not (isinstance(M, torch.Tensor) and M.dtype == torch.bool) else M.to(torch.float64))
    if Mf.shape != u.shape:
        raise ValueError("mask and field shapes differ")
    _lib.check(lib.sem_mask(Mf.data_ptr(), u.data_ptr(), out.data_ptr(), u.numel(), stream_ptr()))
    return out


def grad(u, msh):
    """grad(u, msh) (src/grad.jl:16-34): (ux, uy) = (rx ur + sx us, ry ur + sy us)
    with ur = ABu([],Dr,u), us = ABu(Ds,[],u); no continuity across elements."""
    lib = _lib.load()
    u = _field(u, msh)
    ux, uy = msh.empty(), msh.empty()
    _lib.check(lib.sem_grad(msh.handle, u.data_ptr(), ux.data_ptr(), uy.data_ptr(), stream_ptr()))
    return ux, uy


def gradT(u, msh):
    """gradᵀ(u, msh) (src/grad.jl:43-63), evaluated as the reference writes it:
    ux = ABu(Dr',[],rx.*u) + ABu([],Ds',sx.*u), uy likewise with ry, sy.
    (Python normalises the identifier gradᵀ to gradT.)"""
    lib = _lib.load()
    u = _field(u, msh)
    ux, uy = msh.empty(), msh.empty()
    _lib.check(lib.sem_grad_t(msh.handle, u.data_ptr(), ux.data_ptr(), uy.data_ptr(), stream_ptr()))
    return ux, uy


def advect(T, ux, uy, mshV, mshD=None, Jr=None, Js=None):
    """advect (src/advect.jl:27-78): B .* (ux Tx + uy Ty) with (Tx, Ty) =
    grad(T), unassembled.  With a dealiasing mesh mshD the velocity and grad T
    are interpolated to its grid (Jr = interpMat(mshD.zr, mshV.zr) and Js
    likewise, unless given), multiplied there by mshD.B and brought back with
    ABu(Js',Jr',.)."""
    from .host import interpMat
    lib = _lib.load()
    T, ux, uy = (_field(v, mshV) for v in (T, ux, uy))
    out = mshV.empty()
    if mshD is None:
        _lib.check(lib.sem_advect(mshV.handle, T.data_ptr(), ux.data_ptr(), uy.data_ptr(),
                                  out.data_ptr(), stream_ptr()))
        return out
    if mshD.Ex != mshV.Ex or mshD.Ey != mshV.Ey:
        raise ValueError("the dealiasing mesh must have the same elements")
    Jr = interpMat(mshD.zr, mshV.zr) if Jr is None else np.asarray(Jr, dtype=np.float64)
    Js = interpMat(mshD.zs, mshV.zs) if Js is None else np.asarray(Js, dtype=np.float64)
    Jrb, Jsb = np.asfortranarray(Jr), np.asfortranarray(Js)
    Bd = as_local(mshD.B)
    _lib.check(lib.sem_advect_dealiased(mshV.handle, Jrb.shape[0], Jsb.shape[0], Jrb.ctypes.data,
                                        Jsb.ctypes.data, Bd.data_ptr(), T.data_ptr(), ux.data_ptr(),
                                        uy.data_ptr(), out.data_ptr(), stream_ptr()))
    return out
