"""The Spectral module's operator algebra on the device (src/Spectral/Operators.jl,
src/Spectral/OperatorBasics.jl), against NumPy: the reference's own checks of
test/Operators.jl (DiagonalOp and TensorProductOp2D mul!, the second call too,
since the reference's cache is set on the first) plus the 3D tensor product,
gradOp exactness, affine combinations, composition, adjoints, inverses and
batches.  Tolerance: relative 1e-13 (FP64, another summation order than BLAS)."""
import numpy as np
import pytest
import torch

from _helpers import host, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _f(a):
    from semgb300.spectral import colmajor
    return colmajor(a)


def test_reference_operator_checks(gpu):
    """test/Operators.jl: nr = 8, ns = 12, u and v random fields."""
    from semgb300 import spectral as SP
    rng = np.random.default_rng(1)
    nr, ns = 8, 12
    u, v = rng.random((nr, ns)), rng.random((nr, ns))
    d = rng.random((nr, ns))
    D = SP.DiagonalOp(_f(d))
    vv = _f(v)
    assert D.mul_(vv, _f(u)) is vv
    assert rel_l2(host(vv), d * u) < TOL
    A, B = rng.random((nr, nr)), rng.random((ns, ns))
    T = SP.TensorProductOp2D(A, B)
    for _ in range(2):
        assert rel_l2(host(T.mul_(vv, _f(u))), A @ u @ B.T) < TOL
    assert rel_l2(host(T * _f(u)), A @ u @ B.T) < TOL


@pytest.mark.parametrize("shape,mshape", [((8, 12), (5, 7)), ((70, 33), (90, 40))])
def test_tensor_product_2d_rectangular_and_batched(gpu, shape, mshape):
    from semgb300 import spectral as SP
    rng = np.random.default_rng(shape[0])
    (na, nb), (ma, mb) = shape, mshape
    A, B = rng.standard_normal((ma, na)), rng.standard_normal((mb, nb))
    U = rng.standard_normal((na, nb, 3))
    got = host(SP.TensorProductOp2D(A, B) * _f(U))
    ref = np.einsum("ia,jb,abz->ijz", A, B, U)
    assert rel_l2(got, ref) < TOL
    # identity factors (gradOp's sparse I) and the adjoint
    assert rel_l2(host(SP.TensorProductOp2D(A, None) * _f(U[..., 0])), A @ U[..., 0]) < TOL
    assert rel_l2(host(SP.TensorProductOp2D(None, B) * _f(U[..., 0])), U[..., 0] @ B.T) < TOL
    W = rng.standard_normal((ma, mb))
    Tt = SP.TensorProductOp2D(A, B).adjoint()
    assert rel_l2(host(Tt * _f(W)), A.T @ W @ B) < TOL


def test_tensor_product_3d_and_grad_op(gpu):
    from semgb300 import spectral as SP
    from semgb300.host import derivMat, gausslobatto
    rng = np.random.default_rng(3)
    na, nb, nc = 6, 7, 5
    A, B, C = (rng.standard_normal((m, n)) for m, n in ((4, na), (9, nb), (5, nc)))
    U = rng.standard_normal((na, nb, nc))
    got = host(SP.TensorProductOp3D(A, B, C) * _f(U))
    assert rel_l2(got, np.einsum("ia,jb,kc,abc->ijk", A, B, C, U)) < TOL
    got = host(SP.TensorProductOp3D(None, B, None) * _f(U))
    assert rel_l2(got, np.einsum("jb,abc->ajc", B, U)) < TOL
    # gradOp on a GLL grid differentiates a polynomial exactly
    zr, _ = gausslobatto(na)
    zs, _ = gausslobatto(nb)
    zt, _ = gausslobatto(nc)
    X, Y, Z = np.meshgrid(zr, zs, zt, indexing="ij")
    u = X ** 3 * Y + Z ** 2 * Y ** 2
    Dx, Dy, Dz = SP.gradOp(derivMat(zr), derivMat(zs), derivMat(zt))
    assert np.abs(host(Dx * _f(u)) - 3 * X ** 2 * Y).max() < 1e-12
    assert np.abs(host(Dy * _f(u)) - (X ** 3 + 2 * Z ** 2 * Y)).max() < 1e-12
    assert np.abs(host(Dz * _f(u)) - 2 * Z * Y ** 2).max() < 1e-12
    Dx2, Dy2 = SP.gradOp(derivMat(zr), derivMat(zs))
    u2 = X[..., 0] ** 2 * Y[..., 0]
    assert np.abs(host(Dx2 * _f(u2)) - 2 * X[..., 0] * Y[..., 0]).max() < 1e-12
    (D1,) = SP.gradOp(derivMat(zr))
    assert np.abs(host(D1 * _f(zr ** 4)) - 4 * zr ** 3).max() < 1e-12


def test_operator_algebra(gpu):
    from semgb300 import spectral as SP
    rng = np.random.default_rng(4)
    nr, ns = 9, 6
    u = rng.standard_normal((nr, ns))
    A, B = rng.standard_normal((nr, nr)) + 4 * np.eye(nr), rng.standard_normal((ns, ns)) + 4 * np.eye(ns)
    d1, d2 = rng.random((nr, ns)) + 0.5, rng.random((nr, ns)) + 0.5
    T = SP.TensorProductOp2D(A, B)
    D1, D2 = SP.DiagonalOp(_f(d1)), SP.DiagonalOp(_f(d2))
    Tu = A @ u @ B.T
    # affine combinations and scalar multiples
    assert rel_l2(host((2.0 * T - D1) * _f(u)), 2 * Tu - d1 * u) < TOL
    assert rel_l2(host((T + 3.0) * _f(u)), Tu + 3 * u) < TOL
    assert rel_l2(host((T / 4.0) * _f(u)), Tu / 4) < TOL
    # fused diagonal algebra
    assert rel_l2(host((D1 + D2).diag), d1 + d2) < TOL
    assert rel_l2(host((D1 * D2).diag), d1 * d2) < TOL
    assert rel_l2(host((D1 / D2).diag), d1 / d2) < TOL
    assert rel_l2(host(D1.inv().diag), 1 / d1) < TOL
    assert rel_l2(host(D1.ldiv(_f(u))), u / d1) < TOL
    # composition: lazy for general operators, factor products for tensor products
    assert rel_l2(host((D1 * T) * _f(u)), d1 * Tu) < TOL
    TT = T * T
    assert isinstance(TT, SP.TensorProductOp2D)
    assert rel_l2(host(TT * _f(u)), A @ A @ u @ B.T @ B.T) < 1e-12
    # inverses
    assert rel_l2(host(SP.InverseOp(T) * _f(Tu)), u) < 1e-12
    assert rel_l2(host(SP.InverseOp(D1 @ T) * _f(d1 * Tu)), u) < 1e-12
    # Null and Identity
    assert np.abs(host(SP.NullOp(2) * _f(u))).max() == 0.0
    assert np.array_equal(host(SP.IdentityOp(2) * _f(u)), u)
    # mul! into a preallocated output; a row-major output is refused
    v = _f(np.zeros((nr, ns)))
    T.mul_(v, _f(u))
    assert rel_l2(host(v), Tu) < TOL
    with pytest.raises(ValueError):
        T.mul_(torch.zeros((nr, ns), dtype=torch.float64, device="cuda"), _f(u))
    # MatrixOp on 1D fields
    M = rng.standard_normal((5, nr))
    assert rel_l2(host(SP.MatrixOp(M) * _f(u[:, 0])), M @ u[:, 0]) < TOL
