"""Single-domain spectral operator algebra of the reference's Spectral module
(src/Spectral/Operators.jl, src/Spectral/OperatorBasics.jl) on the device.

Fields are CUDA float64 tensors of shape (nr,), (nr, ns) or (nr, ns, nt),
stored column-major as the reference's arrays are; one extra trailing
dimension holds a batch of fields.  Every apply runs in libsem_b200
(``sem_tp2d``, ``sem_tp3d``, ``sem_mode_product``, ``sem_diag_apply``,
``sem_axpby``); operator matrices are uploaded once when an operator is built,
and algebra on operators (adjoint, products of tensor-product factors,
inverses of factors) is done on those small host matrices at construction.

Differences from the reference, where its code cannot run:
* the fusion of two TensorProductOp2D (Operators.jl:200-209) rebinds A before
  reading A.B and fails; here ``*`` of two tensor-product operators is the
  product of their factors, (A1 (x) B1)(A2 (x) B2) = A1A2 (x) B1B2, and ``+``/``-``
  fall back to AffineOp as for any other operators;
* TensorProductOp3D is referenced by gradOp (LagrangePolynomialSpace.jl:126-138)
  but not defined, and the 3D tensor_product! (Operators.jl:133-145) never
  applies B; here it is (C (x) B (x) A) u with all three modes applied.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .mesh import stream_ptr

__all__ = ["NullOp", "IdentityOp", "MatrixOp", "DiagonalOp", "TensorProductOp2D",
           "TensorProductOp3D", "AffineOp", "ComposedOp", "InverseOp", "gradOp", "colmajor"]


def colmajor(t, dtype=torch.float64) -> torch.Tensor:
    """A CUDA tensor with the values of t, stored column-major."""
    if isinstance(t, np.ndarray):
        t = torch.from_numpy(np.ascontiguousarray(t))
    if not isinstance(t, torch.Tensor):
        raise TypeError("expected a torch tensor or NumPy array")
    if t.device.type != "cuda":
        t = t.to("cuda")
    t = t.to(dtype)
    d = t.dim()
    if d <= 1:
        return t.contiguous()
    rev = tuple(range(d - 1, -1, -1))
    return t.permute(rev).contiguous().permute(rev)


def _empty_colmajor(shape):
    rev = tuple(reversed(shape))
    t = torch.empty(rev, dtype=torch.float64, device="cuda")
    return t.permute(tuple(range(len(shape) - 1, -1, -1)))


def _host_mat(M):
    if M is None:
        return None
    if isinstance(M, torch.Tensor):
        M = M.detach().cpu().numpy()
    M = np.asarray(M, dtype=np.float64)
    if M.ndim != 2:
        raise ValueError("operator matrices are 2D")
    return M


def _dev_mat(M):
    return None if M is None else colmajor(torch.from_numpy(np.ascontiguousarray(M)))


def _is_colmajor(t):
    return t.is_cuda and t.dtype == torch.float64 and t.is_contiguous() if t.dim() <= 1 else (
        t.is_cuda and t.dtype == torch.float64 and
        t.permute(tuple(range(t.dim() - 1, -1, -1))).is_contiguous())


def _out(shape, out):
    """The output field: a new column-major tensor, or ``out`` when it is one
    of the right shape (mul! writes into v)."""
    if out is None:
        return _empty_colmajor(tuple(shape))
    if tuple(out.shape) != tuple(shape) or not _is_colmajor(out):
        raise ValueError("the output field must be a column-major CUDA float64 tensor of the result's shape")
    return out


def _ptr(t):
    return None if t is None else t.data_ptr()


class AbstractOperator:
    """Operators act on fields with ``A * u`` (or ``A(u)``) and ``A.mul_(v, u)``
    (mul!); ``A * B`` composes (OperatorBasics.jl:32-35); ``+``, ``-`` and
    scalar ``*``, ``/`` build AffineOp (:183-210)."""

    D = None

    def apply(self, u, out=None):
        raise NotImplementedError

    def mul_(self, v, u):
        """mul!(v, A, u): the result is written into v."""
        self.apply(u, out=v)
        return v

    def __call__(self, u, p=None, t=None):
        return self.apply(u)

    def ldiv(self, u, out=None):
        raise NotImplementedError(f"operator inversion not defined for {type(self).__name__}")

    def __mul__(self, other):
        if isinstance(other, AbstractOperator):
            return ComposedOp(self, other)
        if isinstance(other, (int, float)):
            return AffineOp(self, NullOp(self.D), float(other), 0.0)
        return self.apply(other)

    def __rmul__(self, lam):
        return AffineOp(self, NullOp(self.D), float(lam), 0.0)

    def __truediv__(self, lam):
        return AffineOp(self, NullOp(self.D), 1.0 / float(lam), 0.0)

    def __add__(self, other):
        if isinstance(other, (int, float)):
            return AffineOp(self, IdentityOp(self.D), 1.0, float(other))
        return AffineOp(self, other, 1.0, 1.0)

    def __sub__(self, other):
        if isinstance(other, (int, float)):
            return AffineOp(self, IdentityOp(self.D), 1.0, -float(other))
        return AffineOp(self, other, 1.0, -1.0)

    def __matmul__(self, other):  # lazy composition, the reference's ∘
        return ComposedOp(self, other)

    @property
    def H(self):
        return self.adjoint()

    def adjoint(self):
        raise NotImplementedError


class NullOp(AbstractOperator):
    """Zero operator (OperatorBasics.jl:51-79)."""

    def __init__(self, D):
        self.D = D

    def apply(self, u, out=None):
        out = _out(u.shape, out)
        _lib.check(_lib.load().sem_axpby(0.0, None, 0.0, None, out.data_ptr(), out.numel(), stream_ptr()))
        return out

    def adjoint(self):
        return self


class IdentityOp(AbstractOperator):
    """Identity (OperatorBasics.jl:80-110)."""

    def __init__(self, D):
        self.D = D

    def apply(self, u, out=None):
        u = colmajor(u)
        out = _out(u.shape, out)
        _lib.check(_lib.load().sem_axpby(1.0, u.data_ptr(), 0.0, None, out.data_ptr(), out.numel(),
                                         stream_ptr()))
        return out

    def ldiv(self, u, out=None):
        return self.apply(u, out)

    def adjoint(self):
        return self


class MatrixOp(AbstractOperator):
    """1D mat-vec (Operators.jl:6-35): v = mat * u."""

    D = 1

    def __init__(self, mat):
        self.mat = _host_mat(mat)
        self._d = _dev_mat(self.mat)

    def apply(self, u, out=None):
        u = colmajor(u)
        m, n = self.mat.shape
        if u.shape[0] != n:
            raise ValueError("field length does not match the matrix")
        batch = u.shape[1] if u.dim() == 2 else 1
        out = _out((m,) + tuple(u.shape[1:]), out)
        _lib.check(_lib.load().sem_mode_product(self._d.data_ptr(), m, n, u.data_ptr(), out.data_ptr(), 1,
                                                batch, stream_ptr()))
        return out

    def adjoint(self):
        return MatrixOp(self.mat.T)


class DiagonalOp(AbstractOperator):
    """Diagonal scaling (Operators.jl:37-113): v = diag .* u; ``\\`` divides."""

    def __init__(self, diag):
        self.diag = colmajor(diag)
        self.D = self.diag.dim()

    def _run(self, u, invert, out=None):
        u = colmajor(u)
        if tuple(u.shape[:self.D]) != tuple(self.diag.shape):
            raise ValueError("field shape does not match the diagonal")
        out = _out(u.shape, out)
        lib = _lib.load()
        per = self.diag.numel()
        batch = u.numel() // per if per else 0
        for b in range(batch):
            _lib.check(lib.sem_diag_apply(self.diag.data_ptr(), u.data_ptr() + 8 * b * per,
                                          out.data_ptr() + 8 * b * per, per, int(invert), stream_ptr()))
        return out

    def apply(self, u, out=None):
        return self._run(u, False, out)

    def ldiv(self, u, out=None):
        return self._run(u, True, out)

    def adjoint(self):
        return self

    def inv(self):
        ones = torch.ones_like(self.diag)
        return DiagonalOp(self._run(ones, True))

    def _comb(self, other, a, b):
        out = _empty_colmajor(tuple(self.diag.shape))
        _lib.check(_lib.load().sem_axpby(a, self.diag.data_ptr(), b, _ptr(other), out.data_ptr(),
                                         out.numel(), stream_ptr()))
        return DiagonalOp(out)

    def __add__(self, other):
        if isinstance(other, DiagonalOp):
            return self._comb(other.diag, 1.0, 1.0)
        return super().__add__(other)

    def __sub__(self, other):
        if isinstance(other, DiagonalOp):
            return self._comb(other.diag, 1.0, -1.0)
        return super().__sub__(other)

    def __mul__(self, other):
        if isinstance(other, DiagonalOp):
            return DiagonalOp(other.apply(self.diag))
        if isinstance(other, (int, float)):
            return self._comb(None, float(other), 0.0)
        return super().__mul__(other)

    def __rmul__(self, lam):
        return self._comb(None, float(lam), 0.0)

    def __truediv__(self, other):
        if isinstance(other, DiagonalOp):
            return DiagonalOp(other.ldiv(self.diag))
        return self._comb(None, 1.0 / float(other), 0.0)


class TensorProductOp2D(AbstractOperator):
    """(B (x) A) u = A U B' (Operators.jl:147-198).  A or B None: identity."""

    D = 2

    def __init__(self, A, B):
        self.A, self.B = _host_mat(A), _host_mat(B)
        self._A, self._B = _dev_mat(self.A), _dev_mat(self.B)

    def apply(self, u, out=None):
        u = colmajor(u)
        na, nb = u.shape[0], u.shape[1]
        batch = u.shape[2] if u.dim() == 3 else 1
        ma = self.A.shape[0] if self.A is not None else na
        mb = self.B.shape[0] if self.B is not None else nb
        if (self.A is not None and self.A.shape[1] != na) or (self.B is not None and self.B.shape[1] != nb):
            raise ValueError("field shape does not match the operator")
        out = _out((ma, mb) + tuple(u.shape[2:]), out)
        _lib.check(_lib.load().sem_tp2d(_ptr(self._A), ma, na, _ptr(self._B), mb, nb, u.data_ptr(),
                                        out.data_ptr(), batch, stream_ptr()))
        return out

    def adjoint(self):
        return TensorProductOp2D(None if self.A is None else self.A.T, None if self.B is None else self.B.T)

    def inv(self):
        return TensorProductOp2D(None if self.A is None else np.linalg.inv(self.A),
                                 None if self.B is None else np.linalg.inv(self.B))

    def ldiv(self, u, out=None):
        return self.inv().apply(u, out)

    def __mul__(self, other):
        if isinstance(other, TensorProductOp2D):
            return TensorProductOp2D(_prod(self.A, other.A), _prod(self.B, other.B))
        return super().__mul__(other)


class TensorProductOp3D(AbstractOperator):
    """(C (x) B (x) A) u for u of shape (na, nb, nc)."""

    D = 3

    def __init__(self, A, B, C):
        self.A, self.B, self.C = _host_mat(A), _host_mat(B), _host_mat(C)
        self._A, self._B, self._C = _dev_mat(self.A), _dev_mat(self.B), _dev_mat(self.C)

    def apply(self, u, out=None):
        u = colmajor(u)
        ns_ = tuple(u.shape[:3])
        batch = u.shape[3] if u.dim() == 4 else 1
        mats = (self.A, self.B, self.C)
        ms = tuple(M.shape[0] if M is not None else n for M, n in zip(mats, ns_))
        for M, n in zip(mats, ns_):
            if M is not None and M.shape[1] != n:
                raise ValueError("field shape does not match the operator")
        out = _out(ms + tuple(u.shape[3:]), out)
        _lib.check(_lib.load().sem_tp3d(_ptr(self._A), ms[0], ns_[0], _ptr(self._B), ms[1], ns_[1],
                                        _ptr(self._C), ms[2], ns_[2], u.data_ptr(), out.data_ptr(), batch,
                                        stream_ptr()))
        return out

    def adjoint(self):
        return TensorProductOp3D(*(None if M is None else M.T for M in (self.A, self.B, self.C)))

    def inv(self):
        return TensorProductOp3D(*(None if M is None else np.linalg.inv(M) for M in (self.A, self.B, self.C)))

    def ldiv(self, u, out=None):
        return self.inv().apply(u, out)

    def __mul__(self, other):
        if isinstance(other, TensorProductOp3D):
            return TensorProductOp3D(_prod(self.A, other.A), _prod(self.B, other.B), _prod(self.C, other.C))
        return super().__mul__(other)


def _prod(X, Y):
    if X is None:
        return Y
    if Y is None:
        return X
    return X @ Y


class AffineOp(AbstractOperator):
    """v = alpha A u + beta B u (OperatorBasics.jl:126-210)."""

    def __init__(self, A, B, alpha, beta):
        self.A, self.B, self.alpha, self.beta = A, B, float(alpha), float(beta)
        self.D = A.D if A.D is not None else B.D

    def apply(self, u, out=None):
        a = self.A.apply(u)
        b = None if isinstance(self.B, NullOp) else self.B.apply(u)
        out = _out(a.shape, out)
        _lib.check(_lib.load().sem_axpby(self.alpha, a.data_ptr(), self.beta, _ptr(b), out.data_ptr(),
                                         out.numel(), stream_ptr()))
        return out

    def adjoint(self):
        return AffineOp(self.A.adjoint(), self.B.adjoint(), self.alpha, self.beta)


class ComposedOp(AbstractOperator):
    """Lazy composition outer ∘ inner (OperatorBasics.jl:212-292)."""

    def __init__(self, outer, inner):
        self.outer, self.inner = outer, inner
        self.D = outer.D if outer.D is not None else inner.D

    def apply(self, u, out=None):
        return self.outer.apply(self.inner.apply(u), out)

    def ldiv(self, u, out=None):
        return self.inner.ldiv(self.outer.ldiv(u), out)

    def adjoint(self):
        return ComposedOp(self.inner.adjoint(), self.outer.adjoint())


class InverseOp(AbstractOperator):
    """A⁻¹ applied through A's ldiv (OperatorBasics.jl:294-320)."""

    def __init__(self, A):
        self.A = A
        self.D = A.D

    def apply(self, u, out=None):
        return self.A.ldiv(u, out)

    def ldiv(self, u, out=None):
        return self.A.apply(u, out)


def gradOp(*deriv_mats):
    """gradOp (src/Spectral/LagrangePolynomialSpace.jl:104-138): the gradient
    as one operator per direction from the 1D derivative matrices."""
    D = len(deriv_mats)
    if D == 1:
        return [MatrixOp(deriv_mats[0])]
    if D == 2:
        Dr, Ds = deriv_mats
        return [TensorProductOp2D(Dr, None), TensorProductOp2D(None, Ds)]
    if D == 3:
        Dr, Ds, Dt = deriv_mats
        return [TensorProductOp3D(Dr, None, None), TensorProductOp3D(None, Ds, None),
                TensorProductOp3D(None, None, Dt)]
    raise ValueError("1, 2 or 3 derivative matrices")
