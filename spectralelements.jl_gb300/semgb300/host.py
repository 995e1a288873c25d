"""Host-side numerics of mesh set-up (small 1D operators; FP64 NumPy).

These run once per mesh on the CPU and feed the device handle, as the
reference's ``Mesh`` constructor does (src/mesh.jl:66-133).  Fields are kept
in the reference's column-major (nr*Ex, ns*Ey) layout.
"""
from __future__ import annotations

import numpy as np


def gausslobatto(n: int):
    """GLL nodes (ascending) and weights on [-1, 1].

    Counterpart of ``FastGaussQuadrature.gausslobatto`` (src/mesh.jl:70-71):
    Newton iteration on x P_N(x) - P_{N-1}(x), N = n-1, from the
    Chebyshev-Gauss-Lobatto points, in extended precision, then symmetrised
    (end points exactly +-1, an odd middle node exactly 0).
    """
    if n < 2:
        raise ValueError("gausslobatto needs n >= 2")
    N = n - 1
    x = -np.cos(np.pi * np.arange(n, dtype=np.longdouble) / N).astype(np.longdouble)
    one = np.longdouble(1)
    for _ in range(100):
        p0 = np.ones_like(x)
        p1 = x.copy()
        for k in range(2, N + 1):
            p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
        dx = (x * p1 - p0) / (n * p1)
        x = x - dx
        if np.max(np.abs(dx)) < np.finfo(np.longdouble).eps * 4:
            break
    p0 = np.ones_like(x)
    p1 = x.copy()
    for k in range(2, N + 1):
        p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
    w = 2 * one / (N * n * p1 * p1)
    z = x.astype(np.float64)
    w = w.astype(np.float64)
    for i in range(n // 2):
        z[n - 1 - i] = -z[i]
        w[n - 1 - i] = w[i]
    z[0], z[-1] = -1.0, 1.0
    if n % 2 == 1:
        z[n // 2] = 0.0
    return z, w


def derivMat(x):
    """Lagrange derivative matrix on the points x (src/derivMat.jl:9-35): barycentric
    weights a_j, diagonal = negative row sum of the off-diagonal 1/(x_i-x_j) sums,
    off-diagonal a_j / (a_i (x_i - x_j))."""
    x = np.asarray(x, dtype=np.float64).reshape(-1)
    n = len(x)
    diff = x[:, None] - x[None, :]
    np.fill_diagonal(diff, 1.0)
    a = 1.0 / np.prod(diff, axis=1)
    inv = 1.0 / diff
    np.fill_diagonal(inv, 0.0)
    D = (a[None, :] / a[:, None]) * inv
    np.fill_diagonal(D, inv.sum(axis=1))
    return D


def interpMat(xo, xi):
    """Lagrange interpolation matrix from xi to xo (src/interp.jl:10-35)."""
    xo = np.atleast_1d(np.asarray(xo, dtype=np.float64))
    xi = np.atleast_1d(np.asarray(xi, dtype=np.float64))
    ni = len(xi)
    diff = xi[:, None] - xi[None, :]
    np.fill_diagonal(diff, 1.0)
    a = 1.0 / np.prod(diff, axis=1)
    J = np.empty((len(xo), ni))
    for i, x in enumerate(xo):
        d = x - xi
        for j in range(ni):
            J[i, j] = a[j] * np.prod(np.delete(d, j))
    return J


def semq_index(E: int, n: int, periodic: bool):
    """Local -> global numbering of src/semq.jl:6-25 (0-based): local row e*n+i
    maps to e*(n-1)+i; periodic folds the last global point onto 0."""
    l = np.arange(E * n)
    g = (l // n) * (n - 1) + (l % n)
    ng = E * (n - 1) + 1
    if periodic:
        g = np.where(g == ng - 1, 0, g)
        ng -= 1
    return g.astype(np.int64), ng


def semmesh(E: int, n: int):
    """1D SEM grid on [-1,1] with E equal elements (src/semmesh.jl:9-27)."""
    z0, w0 = gausslobatto(n)
    z0 = 0.5 * (z0 + 1.0)
    w0 = 0.5 * w0
    ze = np.linspace(-1.0, 1.0, E + 1)
    dz = np.diff(ze)
    z = (dz[:, None] * z0[None, :] + ze[:-1, None]).reshape(-1)
    w = (dz[:, None] * w0[None, :]).reshape(-1)
    return z, w


def ndgrid(v1, v2):
    """(src/ndgrid.jl:8-13), Fortran-ordered outputs."""
    v1 = np.asarray(v1, dtype=np.float64).reshape(-1)
    v2 = np.asarray(v2, dtype=np.float64).reshape(-1)
    X = np.asfortranarray(np.repeat(v1[:, None], len(v2), axis=1))
    Y = np.asfortranarray(np.repeat(v2[None, :], len(v1), axis=0))
    return X, Y


def bdfExtK(t, k: int = 3):
    """BDFk / EXTk coefficients (src/time.jl:31-53): extrapolation weights a
    (length k) and derivative weights b (length k+1) on the time history t."""
    tu = []
    for v in t:
        if v not in tu:
            tu.append(v)
    kk = len(tu) - 1
    a = interpMat([tu[0]], tu[1:]).reshape(-1) if kk > 0 else np.zeros(0)
    b = derivMat(np.array(tu))[0, :]
    if kk < k:
        a = np.concatenate([a, np.zeros(k - kk)])
        b = np.concatenate([b, np.zeros(k - kk)])
    else:
        a, b = a[:k], b[:k + 1]
    if kk == 0:
        a[0] = 1.0
    return a, b


def fixU(x, y):
    """Identity deformation (src/mesh.jl:6-8)."""
    return x, y


def qq_structure(QQ):
    """(n, E, periodic) of a one-direction gather-scatter matrix QQ = Q Q' with
    Q = semq(E, n, periodic) (src/semq.jl:6-25), read from its couplings: the
    first element interface couples local lines n-1 and n (0-based) and a
    periodic direction couples the first and the last line.  Raises
    ValueError for a matrix without that structure."""
    Q = np.asarray(QQ)
    if Q.ndim != 2 or Q.shape[0] != Q.shape[1] or Q.shape[0] < 1:
        raise ValueError("QQ must be a square matrix")
    NL = Q.shape[0]
    periodic = NL > 1 and Q[0, NL - 1] != 0
    n = NL
    for i in range(1, NL - 1):  # n >= 2: the first interface is at line n - 1 >= 1
        if Q[i, i + 1] != 0:
            n = i + 1
            break
    if n < 1 or NL % n:
        raise ValueError("QQ is not the gather-scatter matrix of a semq numbering")
    E = NL // n
    # the couplings of every interface, and nothing else off the diagonal band
    for e in range(1, E):
        if Q[e * n - 1, e * n] == 0:
            raise ValueError("QQ is not the gather-scatter matrix of a semq numbering")
    return n, E, bool(periodic)
