"""CPU oracle for the SEM operator-apply / PCG hot path of SpectralElements.jl.

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  Nothing in the product library
(``spectralelements.jl_gb300/``) imports it, and the product never falls back
to it.

It is a plain NumPy restatement of the reference algorithms, following the
Julia sources line by line (1-based column-major semantics are kept by using
``order='F'`` reshapes; index maps are written 0-based).  Every function cites
the reference file:line it restates (paths are relative to the reference
project root).

PARITY STATUS: parity unpinned.  The reference is Julia and no Julia
toolchain exists here, so no vector produced by the reference itself is
available, and the reference's own tests (``test/Field.jl``,
``test/Operators.jl``) cover only the unrelated ``Spectral`` submodule.  The
oracle is pinned instead by analytic known answers: closed-form GLL nodes and
weights for small n, exactness of the derivative matrix on polynomials,
integral of the mass matrix = area, multiplicities 1/2/4, spectral
convergence of the manufactured Poisson problem of
``examples/p2d_explicit.jl:86-89`` and symmetry of the assembled operator.
Third-party arithmetic: ``FastGaussQuadrature.gausslobatto`` (unpinned
version; no [compat] entry in Project.toml) is restated from the mathematics
(roots of P'_{n-1} plus the end points, weights 2/(n(n-1)P_{n-1}^2)) in
50-digit decimal arithmetic and rounded to double.
"""
from __future__ import annotations

from decimal import Decimal, getcontext
import math

import numpy as np

# --------------------------------------------------------------------------
# quadrature / 1D operators
# --------------------------------------------------------------------------


def gausslobatto(n: int):
    """GLL nodes (ascending) and weights on [-1, 1].

    Stands in for ``FastGaussQuadrature.gausslobatto`` called at
    ``src/mesh.jl:70-71`` and ``src/semmesh.jl:11``.  Newton iteration on
    x P_N - P_{N-1} (N = n-1) in 50-digit decimals; result symmetrised.
    """
    if n < 2:
        raise ValueError("gausslobatto needs n >= 2")
    getcontext().prec = 60
    N = n - 1
    xs = []
    for i in range(n):
        x = Decimal(-math.cos(math.pi * i / N))
        for _ in range(200):
            p0, p1 = Decimal(1), x
            for k in range(2, N + 1):
                p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
            # p1 = P_N(x), p0 = P_{N-1}(x)
            dx = (x * p1 - p0) / (n * p1)
            x -= dx
            if abs(dx) < Decimal("1e-50"):
                break
        xs.append(x)
    ws = []
    for x in xs:
        p0, p1 = Decimal(1), x
        for k in range(2, N + 1):
            p0, p1 = p1, ((2 * k - 1) * x * p1 - (k - 1) * p0) / k
        ws.append(Decimal(2) / (N * n * p1 * p1))
    z = np.array([float(v) for v in xs])
    w = np.array([float(v) for v in ws])
    # exact symmetry (the end points are exactly +-1, an odd middle node is 0)
    for i in range(n // 2):
        z[n - 1 - i] = -z[i]
        w[n - 1 - i] = w[i]
    z[0], z[-1] = -1.0, 1.0
    if n % 2 == 1:
        z[n // 2] = 0.0
    return z, w


def derivMat(x):
    """Lagrange derivative matrix on points x (``src/derivMat.jl:9-35``)."""
    x = np.asarray(x, dtype=np.float64).reshape(-1)
    n = len(x)
    a = np.ones(n)
    for i in range(n):
        for j in range(i):
            a[i] = a[i] * (x[i] - x[j])
        for j in range(i + 1, n):
            a[i] = a[i] * (x[i] - x[j])
    a = 1.0 / a  # barycentric weights
    D = x[:, None] - x[None, :]
    for i in range(n):
        D[i, i] = 1.0
    D = 1.0 / D
    for i in range(n):
        D[i, i] = 0.0
        D[i, i] = np.sum(D[i, :])
    for j in range(n):
        for i in range(n):
            if i != j:
                D[i, j] = a[j] / (a[i] * (x[i] - x[j]))
    return D


def interpMat(xo, xi):
    """Lagrange interpolation matrix from xi to xo (``src/interp.jl:10-35``)."""
    xo = np.atleast_1d(np.asarray(xo, dtype=np.float64))
    xi = np.atleast_1d(np.asarray(xi, dtype=np.float64))
    no, ni = len(xo), len(xi)
    a = np.ones(ni)
    for i in range(ni):
        for j in range(i):
            a[i] = a[i] * (xi[i] - xi[j])
        for j in range(i + 1, ni):
            a[i] = a[i] * (xi[i] - xi[j])
    a = 1.0 / a
    J = np.zeros((no, ni))
    s = np.ones(ni)
    t = np.ones(ni)
    for i in range(no):
        x = xo[i]
        for j in range(1, ni):  # Julia j = 2:ni
            s[j] = s[j - 1] * (x - xi[j - 1])
            t[ni - 1 - j] = t[ni - j] * (x - xi[ni - j])
        J[i, :] = a * s * t
    return J


# --------------------------------------------------------------------------
# numbering, grid, geometry
# --------------------------------------------------------------------------


def semq_index(E: int, n: int, periodic: bool):
    """Local -> global index map of ``semq`` (``src/semq.jl:6-25``).

    Local row l = e*n + i (0-based) maps to global (e*(n-1) + i); a periodic
    direction folds the last global point onto global 0 (``semq.jl:19-22``).
    Returns (l2g, number_of_global_points).
    """
    l = np.arange(E * n)
    g = (l // n) * (n - 1) + (l % n)
    ng = E * (n - 1) + 1
    if periodic:
        g = np.where(g == ng - 1, 0, g)
        ng -= 1
    return g.astype(np.int64), ng


def semq(E: int, n: int, periodic: bool):
    """Dense Q (local x global) of ``src/semq.jl:6-25`` (small sizes only)."""
    g, ng = semq_index(E, n, periodic)
    Q = np.zeros((E * n, ng))
    Q[np.arange(E * n), g] = 1.0
    return Q


def semmesh(E: int, n: int):
    """1D SEM grid and weights on [-1, 1] (``src/semmesh.jl:9-27``)."""
    z0, w0 = gausslobatto(n)
    z0 = 0.5 * (z0 + 1.0)
    w0 = 0.5 * w0
    ze = np.linspace(-1.0, 1.0, E + 1)
    dz = np.diff(ze)
    z = np.kron(dz, z0) + np.kron(ze[:-1], np.ones(n))
    w = np.kron(dz, w0)
    return z.reshape(E * n), w.reshape(E * n)


def ndgrid(v1, v2):
    """``src/ndgrid.jl:8-13``."""
    v1 = np.asarray(v1).reshape(-1, 1)
    v2 = np.asarray(v2).reshape(1, -1)
    return np.repeat(v1, v2.shape[1], axis=1), np.repeat(v2, v1.shape[0], axis=0)


def ABu(As, Br, u):
    """Tensor-product apply (As (x) Br) u (``src/ABu.jl:9-37``).

    ``None`` or a size-0 array stands for Julia's ``[]`` (identity).
    """
    u = np.asarray(u)
    m, n = u.shape
    Bu = u
    if Br is not None and np.size(Br) != 0:
        mb, nb = Br.shape
        m = int(m * mb / nb)
        Bu = Bu.reshape(nb, -1, order="F")
        Bu = Br @ Bu
        Bu = Bu.reshape(m, n, order="F")
    out = Bu
    if As is not None and np.size(As) != 0:
        ma, na = As.shape
        Ey = n / na
        n = int(Ey * ma)
        tmp = np.zeros((m, n), dtype=u.dtype)
        for i in range(int(Ey)):
            tmp[:, i * ma:(i + 1) * ma] = out[:, i * na:(i + 1) * na] @ As.T
        out = tmp
    return out


def jac(x, y, Dr, Ds):
    """Jacobian and inverse metrics (``src/jac.jl:24-40``)."""
    xr = ABu(None, Dr, x)
    xs = ABu(Ds, None, x)
    yr = ABu(None, Dr, y)
    ys = ABu(Ds, None, y)
    J = xr * ys - xs * yr
    Ji = 1.0 / J
    rx = Ji * ys
    ry = -Ji * xs
    sx = -Ji * yr
    sy = Ji * xr
    return J, Ji, rx, ry, sx, sy


def sin_deform(amp: float):
    """Unit-square map used by the benchmark cases.

    x_hat in [-1,1]^2 -> r = (x_hat+1)/2, then x = r + amp sin(pi r) sin(pi s),
    y = s + amp sin(pi r) sin(pi s).  (A user ``deform`` closure of the kind
    ``src/mesh.jl:108`` calls.)
    """
    def deform(x, y):
        r = 0.5 * (x + 1.0)
        s = 0.5 * (y + 1.0)
        b = amp * np.sin(np.pi * r) * np.sin(np.pi * s)
        return r + b, s + b
    return deform


def identity_deform(x, y):
    """``fixU`` of ``src/mesh.jl:6-8``."""
    return x, y


class Mesh:
    """``Mesh`` constructor (``src/mesh.jl:66-133``).

    Deviation: the reference builds Qy with ``semq(Ex, ...)`` (``mesh.jl:80``),
    which only works for Ex == Ey; the oracle uses ``semq(Ey, ...)``.
    ``dense_qq`` keeps the reference's dense QQtx/QQty (``mesh.jl:81-82``)
    for small meshes; large meshes use the structured sum instead.
    """

    def __init__(self, nr, ns, Ex, Ey, ifperiodic=(False, False), deform=identity_deform,
                 dense_qq=None):
        self.nr, self.ns, self.Ex, self.Ey = nr, ns, Ex, Ey
        self.ifperiodic = [bool(ifperiodic[0]), bool(ifperiodic[1])]
        self.zr, self.wr = gausslobatto(nr)
        self.zs, self.ws = gausslobatto(ns)
        self.Dr = derivMat(self.zr)
        self.Ds = derivMat(self.zs)
        self.l2gx, self.nxg = semq_index(Ex, nr, self.ifperiodic[0])
        self.l2gy, self.nyg = semq_index(Ey, ns, self.ifperiodic[1])
        if dense_qq is None:
            dense_qq = (nr * Ex) * (ns * Ey) <= 200_000
        self.dense_qq = dense_qq
        if dense_qq:
            Qx = semq(Ex, nr, self.ifperiodic[0])
            Qy = semq(Ey, ns, self.ifperiodic[1])
            self.QQtx = Qx @ Qx.T
            self.QQty = Qy @ Qy.T
        else:
            self.QQtx = self.QQty = None
        # inner product weights (mesh.jl:94-96)
        self.mult = 1.0 / gatherScatter(np.ones((nr * Ex, ns * Ey)), self)
        xe, _ = semmesh(Ex, nr)
        ye, _ = semmesh(Ey, ns)
        x, y = ndgrid(xe, ye)
        self.x, self.y = deform(x, y)
        self.Jac, self.Jaci, self.rx, self.ry, self.sx, self.sy = jac(self.x, self.y, self.Dr, self.Ds)
        wx = np.kron(np.ones(Ex), self.wr)
        wy = np.kron(np.ones(Ey), self.ws)
        self.B = self.Jac * np.outer(wx, wy)
        self.Bi = 1.0 / self.B
        rx, ry, sx, sy, B = self.rx, self.ry, self.sx, self.sy, self.B
        self.G11 = B * (rx * rx + ry * ry)
        self.G12 = B * (rx * sx + ry * sy)
        self.G22 = B * (sx * sx + sy * sy)

    @property
    def shape(self):
        return (self.nr * self.Ex, self.ns * self.Ey)


def generateMask(bc, msh: Mesh):
    """Dirichlet mask R'R (``src/mesh.jl:149-175``); bc = [xmin,xmax,ymin,ymax]."""
    nx, ny = msh.nr * msh.Ex, msh.ns * msh.Ey
    mx = np.ones(nx, dtype=bool)
    my = np.ones(ny, dtype=bool)
    if bc[0] == "D":
        mx[0] = False
    if bc[1] == "D":
        mx[-1] = False
    if bc[2] == "D":
        my[0] = False
    if bc[3] == "D":
        my[-1] = False
    if msh.ifperiodic[0]:
        mx[:] = True
    if msh.ifperiodic[1]:
        my[:] = True
    return np.outer(mx, my)


# --------------------------------------------------------------------------
# operators
# --------------------------------------------------------------------------


def gatherScatter(u, msh_or_qqtx, QQty=None):
    """QQ' u (``src/gatherScatter.jl:8-21``).

    With dense QQtx/QQty this is literally ``ABu(QQty, QQtx, u)``; for a mesh
    built without dense matrices the same sum is done through the index maps
    (Q' gathers = sums copies onto global nodes, Q scatters back).
    """
    if QQty is not None:
        return ABu(QQty, msh_or_qqtx, u)
    msh = msh_or_qqtx
    if msh.dense_qq and msh.QQtx is not None:
        return ABu(msh.QQty, msh.QQtx, u)
    return gatherScatter_index(u, msh.l2gx, msh.nxg, msh.l2gy, msh.nyg)


def gatherScatter_index(u, l2gx, nxg, l2gy, nyg):
    """QQ' u through the separable local->global maps."""
    u = np.asarray(u)
    g = np.zeros((nxg, nyg), dtype=u.dtype)
    # sum along x, then along y (QQ' = QQty (x) QQtx is separable)
    gx = np.zeros((nxg, u.shape[1]), dtype=u.dtype)
    np.add.at(gx, l2gx, u)
    np.add.at(g.T, l2gy, gx.T)
    return g[np.ix_(l2gx, l2gy)]


def mask(u, M):
    """``src/mask.jl:10-18``."""
    if M is None or np.size(M) == 0:
        return np.array(u, copy=True)
    return np.asarray(M, dtype=np.float64) * u


def laplace(u, Dr, Ds, G11, G12, G22):
    """Weak deformed Laplacian D' G D (``src/lapl.jl:70-81``)."""
    ur = ABu(None, Dr, u)
    us = ABu(Ds, None, u)
    wr = G11 * ur + G12 * us
    ws = G12 * ur + G22 * us
    return ABu(None, Dr.T, wr) + ABu(Ds.T, None, ws)


def laplace_dealias(u, Jr, Js, Dr, Ds, G11, G12, G22):
    """Dealiased Laplacian (``src/lapl.jl:83-103``)."""
    ur = ABu(None, Dr, u)
    us = ABu(Ds, None, u)
    Jur = ABu(Js, Jr, ur)
    Jus = ABu(Js, Jr, us)
    vr = G11 * Jur + G12 * Jus
    vs = G12 * Jur + G22 * Jus
    wr = ABu(_t(Js), _t(Jr), vr)
    ws = ABu(_t(Js), _t(Jr), vs)
    return ABu(None, Dr.T, wr) + ABu(Ds.T, None, ws)


def _t(A):
    return None if A is None or np.size(A) == 0 else A.T


def lapl(u, msh: Mesh, nu=None):
    """``lapl(u,msh)`` (``src/lapl.jl:26-36``); ``lapl(u,nu,msh)`` = nu .* lapl (``:38-45``)."""
    Au = laplace(u, msh.Dr, msh.Ds, msh.G11, msh.G12, msh.G22)
    if nu is not None:
        Au = nu * Au
    return Au


def lapl_functional(u, M, Jr, Js, QQtx, QQty, Dr, Ds, G11, G12, G22, mult):
    """Functional lapl (``src/lapl.jl:54-68``); the Zygote hook is a no-op forward."""
    if (Jr is None or np.size(Jr) == 0) and (Js is None or np.size(Js) == 0):
        Au = laplace(u, Dr, Ds, G11, G12, G22)
    else:
        Au = laplace_dealias(u, Jr, Js, Dr, Ds, G11, G12, G22)
    if QQtx is not None and np.size(QQtx) != 0:
        Au = gatherScatter(Au, QQtx, QQty)
    return mask(Au, M)


def mass(u, msh: Mesh):
    """``src/mass.jl:12-22``."""
    return msh.B * u


def mass_functional(u, M, B, Jr, Js, QQtx, QQty, mult):
    """Functional mass (``src/mass.jl:32-50``)."""
    Ju = ABu(Js, Jr, u)
    BJu = Ju if (B is None or np.size(B) == 0) else B * Ju
    Bu = ABu(_t(Js), _t(Jr), BJu)
    if QQtx is not None and np.size(QQtx) != 0:
        Bu = gatherScatter(Bu, QQtx, QQty)
    return mask(Bu, M)


def hlmz(u, nu, k, msh: Mesh):
    """``src/hlmz.jl:12-19``: nu .* lapl(u) + k .* mass(u)."""
    Hu = nu * lapl(u, msh)
    Hu = Hu + k * mass(u, msh)
    return Hu


def jacobi_diag(msh: Mesh, nu=1.0, k=0.0, M=None, G=None):
    """Diagonal of mask(QQ'(hlmz(.))) (new; derived from ``src/lapl.jl:70-81``).

    d(i,j) = sum_k Dr[k,i]^2 G11(k,j) + sum_l Ds[l,j]^2 G22(i,l)
             + 2 Dr[i,i] Ds[j,j] G12(i,j), times nu, plus k B(i,j); then QQ';
    masked entries are set to 1.
    """
    G11, G12, G22 = G if G is not None else (msh.G11, msh.G12, msh.G22)
    nr, ns, Ex, Ey = msh.nr, msh.ns, msh.Ex, msh.Ey
    Dr2 = msh.Dr ** 2
    Ds2 = msh.Ds ** 2
    d = ABu(None, Dr2.T, G11) + ABu(Ds2.T, None, G22)
    drd = np.kron(np.ones(Ex), np.diag(msh.Dr))
    dsd = np.kron(np.ones(Ey), np.diag(msh.Ds))
    d = d + 2.0 * np.outer(drd, dsd) * G12
    d = nu * d + k * msh.B
    d = gatherScatter(d, msh)
    if M is not None:
        d = np.where(np.asarray(M, dtype=bool), d, 1.0)
    return d


# --------------------------------------------------------------------------
# solver
# --------------------------------------------------------------------------


def pcg(b, opA, opM=None, mult=None, ifv=False, tol=1e-8, maxiter=None, info=None):
    """Left-preconditioned CG with mult-weighted dots (``src/pcg.jl:16-60``).

    ``info`` (a dict, optional) receives the iteration count and final
    Inf-norm residual; the reference itself returns only x.
    """
    if opM is None:
        opM = lambda v: v  # noqa: E731
    if mult is None:
        mult = np.ones(np.shape(b))
    if maxiter is None:
        maxiter = np.size(b)
    x = np.zeros_like(b)
    Ax = np.zeros_like(b)
    ra = b - Ax
    hp = np.zeros_like(b)
    rp = np.zeros_like(b)
    u = np.zeros_like(b)
    k = 0
    converged = True
    while np.max(np.abs(ra)) > tol:
        ha = opM(ra)
        if k == maxiter:
            converged = False
            break
        k += 1
        hpp, rpp = hp, rp
        hp, rp = ha, ra
        t = np.sum(rp * hp * mult)
        if k == 1:
            u = np.array(hp, copy=True)
        else:
            u = hp + (t / np.sum(rpp * hpp * mult)) * u
        Au = opA(u)
        a = t / np.sum(u * Au * mult)
        x = x + a * u
        ra = rp - a * Au
    if info is not None:
        info["iters"] = k
        info["res_inf"] = float(np.max(np.abs(ra)))
        info["converged"] = converged
    return x


# --------------------------------------------------------------------------
# gradient and advection
# --------------------------------------------------------------------------


def grad(u, msh: Mesh):
    """``src/grad.jl:16-34``: ux = rx ur + sx us, uy = ry ur + sy us with
    ur = ABu([],Dr,u), us = ABu(Ds,[],u); no continuity across elements."""
    ur = ABu(None, msh.Dr, u)
    us = ABu(msh.Ds, None, u)
    return msh.rx * ur + msh.sx * us, msh.ry * ur + msh.sy * us


def advect(T, ux, uy, msh: Mesh):
    """``src/advect.jl:27-43``: B .* (ux Tx + uy Ty), unassembled."""
    Tx, Ty = grad(T, msh)
    return (ux * Tx + uy * Ty) * msh.B


def advect_dealiased(T, ux, uy, mshV: Mesh, Bd, Jr, Js):
    """``src/advect.jl:45-64``: the velocity and grad T interpolated to the
    dealiasing grid (ABu(Js,Jr,.)), multiplied there by its mass Bd, and
    brought back with ABu(Js',Jr',.)."""
    Tx, Ty = grad(T, mshV)
    JTx = ABu(Js, Jr, Tx)
    JTy = ABu(Js, Jr, Ty)
    Jux = ABu(Js, Jr, ux)
    Juy = ABu(Js, Jr, uy)
    JCu = (Jux * JTx + Juy * JTy) * Bd
    return ABu(Js.T, Jr.T, JCu)


# --------------------------------------------------------------------------
# time stepping and the Diffusion driver
# --------------------------------------------------------------------------


def bdfExtK(t, k=3):
    """BDFk / EXTk coefficients (``src/time.jl:31-53``)."""
    tu = []
    for v in t:  # Julia unique keeps first occurrences in order
        if v not in tu:
            tu.append(v)
    kk = len(tu) - 1
    t1 = tu[0]
    t0 = tu[1:]
    a = interpMat([t1], t0).reshape(-1) if kk > 0 else np.zeros(0)
    b = derivMat(np.array(tu))[0, :]
    if kk < k:
        a = np.concatenate([a, np.zeros(k - kk)])
        b = np.concatenate([b, np.zeros(k - kk)])
    else:
        a = a[:k]
        b = b[:k + 1]
    if kk == 0:
        a[0] = 1.0
    return a, b


def diffusion_opLHS(u, msh, nu, bdfB1, M):
    """``src/diffusion.jl:36-45``."""
    lhs = hlmz(u, nu, bdfB1, msh)
    lhs = gatherScatter(lhs, msh)
    return mask(lhs, M)


def diffusion_makeRHS(msh, nu, f, ub, uh, bdfB, M):
    """``src/diffusion.jl:51-65``."""
    rhs = mass(f, msh)
    rhs = rhs - nu * lapl(ub, msh)
    for i in range(len(uh)):
        rhs = rhs - bdfB[1 + i] * mass(uh[i], msh)
    rhs = mask(rhs, M)
    return gatherScatter(rhs, msh)


# --------------------------------------------------------------------------
# adjoint (variable-coefficient, G-folded nu)
# --------------------------------------------------------------------------


def grad_dot(lam, u, msh: Mesh):
    """Per-local-copy -B grad(lam).grad(u) with the metric folded into G.

    The derivative of lam' D'(nu G)D u with respect to the nodal nu at one
    local node; with the sign of the residual pullback of
    ``src/adjoint.jl:13-16`` (resi = rhs - lhs(u)).
    """
    lr = ABu(None, msh.Dr, lam)
    ls = ABu(msh.Ds, None, lam)
    ur = ABu(None, msh.Dr, u)
    us = ABu(msh.Ds, None, u)
    return -(msh.G11 * lr * ur + msh.G12 * (lr * us + ls * ur) + msh.G22 * ls * us)
