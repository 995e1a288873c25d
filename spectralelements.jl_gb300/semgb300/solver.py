"""pcg with the reference's keyword interface (src/pcg.jl:16-79), the
operator objects it accepts, the Diffusion driver (src/diffusion.jl) and the
adjoint linsolve (src/adjoint.jl).

``pcg`` runs entirely on the device (libsem_b200 ``sem_pcg``).  It recognises
the operator objects of this module (callables, so ``opA(u)`` works as in the
reference's ``opA * u``) and rejects arbitrary Python closures: there is no
host or eager fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .host import bdfExtK, fixU
from .mesh import Mesh, as_local, generateMask, local_empty, mask_bc_of, stream_ptr


class HelmholtzOp:
    """opA(u) = mask(QQ'(hlmz(u, nu, k))) — ``opLHS`` of src/diffusion.jl:36-45.

    ``nu`` is a scalar; ``nu_field`` (a device field) is folded into the metric
    (variable-coefficient -div(nu grad u), as examples/semPS.jl:163-165 builds
    G11/G12/G22).  The mask is the mesh's bc (``Mesh.set_bc``)."""

    def __init__(self, msh: Mesh, nu=1.0, k=0.0, nu_field=None, precision=None):
        self.msh = msh
        self.nu = float(nu)
        self.k = float(k)
        self.nu_field = None if nu_field is None else as_local(nu_field)
        self.precision = precision

    def __call__(self, u):
        lib = _lib.load()
        msh = self.msh
        u = as_local(u)
        out = msh.empty()
        flags = _lib.SEM_GS | (_lib.SEM_MASK if msh.bc else 0)
        if self.nu_field is not None:
            # D'(nu G)D + k B: the variable coefficient enters the metric factors
            _lib.check(lib.sem_varcoef(msh.handle, self.nu_field.data_ptr(), self.k,
                                       u.data_ptr(), out.data_ptr(), flags, stream_ptr()))
            return out
        _lib.check(lib.sem_hlmz(msh.handle, None, self.nu, self.k, u.data_ptr(), out.data_ptr(),
                                flags, stream_ptr()))
        return out


class Jacobi:
    """opM(r) = r ./ diag(opA) (not in the reference; derived from
    src/lapl.jl:70-81)."""

    def __init__(self, opA: HelmholtzOp):
        self.opA = opA
        self._d = None

    def diag(self):
        if self._d is None:
            lib = _lib.load()
            o = self.opA
            d = o.msh.empty()
            _lib.check(lib.sem_jacobi_diag(o.msh.handle, None if o.nu_field is None else
                                           o.nu_field.data_ptr(), o.nu, o.k, d.data_ptr(),
                                           stream_ptr()))
            self._d = d
        return self._d

    def __call__(self, r):
        return as_local(r) / self.diag()


def _is_identity(opM):
    return opM is None or opM is identity


def identity(x):
    """opM = x -> x, the reference's default preconditioner."""
    return x


def pcg(b, opA, opM=None, mult=None, ifv=False, tol=1e-8, maxiter=None, *, precision=None,
        inner_tol=1e-4, max_outer=6, info=None, x=None):
    """Left-preconditioned CG with mult-weighted dots (src/pcg.jl:16-60).

    tol is the absolute Inf-norm of the residual and maxiter defaults to
    length(b), as in the reference.  On reaching maxiter the reference's
    warning is printed and x is returned.  ``precision``: SEM_F64,
    SEM_F64_DF (default: the mesh's) or SEM_MIXED.  ``info`` (dict) receives
    iterations, outer sweeps and residuals.
    """
    if not isinstance(opA, HelmholtzOp):
        raise TypeError("pcg on the device takes an operator built by this package "
                        "(HelmholtzOp); arbitrary closures are not run on the host")
    msh = opA.msh
    lib = _lib.load()
    b = as_local(b)
    if x is None:
        x = msh.empty()
    o = _lib.PcgOpts()
    o.nu = opA.nu
    o.nu_field = None if opA.nu_field is None else opA.nu_field.data_ptr()
    o.k = opA.k
    if _is_identity(opM):
        o.precond = _lib.SEM_PRECOND_NONE
    elif isinstance(opM, Jacobi) and opM.opA is opA:
        o.precond = _lib.SEM_PRECOND_JACOBI
    else:
        raise TypeError("opM must be identity or Jacobi(opA)")
    prec = precision if precision is not None else (opA.precision if opA.precision is not None
                                                    else msh.precision)
    o.precision = int(prec)
    o.tol = float(tol)
    o.maxiter = 0 if maxiter is None else int(maxiter)
    o.inner_tol = float(inner_tol)
    o.max_outer = int(max_outer)
    o.check_every = 0
    if mult is None:
        o.mult_ones = 1
    else:
        if mult is not msh.mult and not torch.equal(as_local(mult), msh.mult):
            raise ValueError("mult must be the mesh's inner-product weights (Mesh.mult)")
        o.mult_ones = 0
    inf = _lib.SolveInfo()
    st = lib.sem_pcg(msh.handle, ctypes.byref(o), b.data_ptr(), x.data_ptr(), ctypes.byref(inf),
                     stream_ptr())
    if info is not None:
        info.update(iters=inf.iters, outer=inf.outer, res_inf=inf.res_inf, res0_inf=inf.res0_inf,
                    converged=bool(inf.converged), status=st)
    if st == _lib.SEM_ERR_NOT_CONVERGED:
        print("warning: res:", inf.res_inf)
        return x
    _lib.check(st)
    if ifv:
        print("PCG iter: ", inf.iters, ", res: ", inf.res_inf)
    return x


def pcg_(x, b, opA, **kw):
    """pcg!(x, b, opA; ...) (src/pcg.jl:64-79): x .= pcg(b, opA; ...)."""
    y = pcg(b, opA, **kw)
    x.copy_(y)
    return None


# ---------------------------------------------------------------------------
# adjoint: linsolve with a custom backward (src/adjoint.jl:5-24)
# ---------------------------------------------------------------------------
class _VarCoefSolve(torch.autograd.Function):
    """u = A(nu)^{-1} b with A(nu) = mask(QQ'(D'(nu G)D)); backward returns the
    per-local-copy gradient  -G:(grad lam)(grad u)  at lam = A^{-1} mask(QQ'(u_bar)),
    i.e. the pullback of resi(u, nu) = rhs - lhs(nu)(u) (src/adjoint.jl:13-16)."""

    @staticmethod
    def forward(ctx, nu, b, msh, kw):
        op = HelmholtzOp(msh, 1.0, 0.0, nu_field=nu.detach())
        u = pcg(b, op, opM=Jacobi(op), mult=msh.mult, **kw)
        ctx.save_for_backward(nu.detach(), u)
        ctx.msh, ctx.kw = msh, kw
        return u

    @staticmethod
    def backward(ctx, ubar):
        nu, u = ctx.saved_tensors
        msh = ctx.msh
        from .ops import gatherScatter, mask
        rhs = gatherScatter(mask(as_local(ubar), generateMask(msh.bc, msh)), msh)
        op = HelmholtzOp(msh, 1.0, 0.0, nu_field=nu)
        lam = pcg(rhs, op, opM=Jacobi(op), mult=msh.mult, **ctx.kw)
        g = msh.empty()
        _lib.check(_lib.load().sem_adjoint_grad(msh.handle, lam.data_ptr(), u.data_ptr(),
                                                g.data_ptr(), 0, stream_ptr()))
        return g, None, None, None


def linsolve_varcoef(nu, b, msh: Mesh, **kw):
    """Differentiable solve of -div(nu grad u) = f (b = mask(QQ'(B f))) w.r.t.
    the nodal nu, the pattern of ``linsolve`` + ``@adjoint`` (src/adjoint.jl)."""
    return _VarCoefSolve.apply(nu, b, msh, kw)


# ---------------------------------------------------------------------------
# time stepping driver (src/time.jl, src/diffusion.jl)
# ---------------------------------------------------------------------------
class TimeStepper:
    """src/time.jl:70-112.  Coefficients are sized by k (the reference sizes the
    initial arrays with its default k=3, which breaks k != 3)."""

    def __init__(self, Ti, Tf, dt, k=3):
        self.k = k
        self.time = [float(Ti)] * (k + 1)
        self.bdfA, self.bdfB = bdfExtK(self.time, k)
        self.istep = 0
        self.fstep = int(np.ceil(Tf / dt)) if dt != 0 else 0
        self.dt, self.Ti, self.Tf = float(dt), float(Ti), float(Tf)

    def advance(self):
        self.time = [self.time[0]] + self.time[:-1]
        self.istep += 1
        self.time[0] += self.dt
        self.bdfA, self.bdfB = bdfExtK(self.time, self.k)


class Diffusion:
    """``Diffusion(bc, msh; Ti, Tf, dt, k)`` (src/diffusion.jl:7-34) with
    device fields u, uh (histories), ub, nu, f.  ``checkpoint_every`` keeps
    copies of u every that many steps (for adjoint recomputation)."""

    def __init__(self, bc, msh: Mesh, Ti=0.0, Tf=0.0, dt=0.0, k=3, nu=1.0,
                 precision=None, checkpoint_every=0):
        self.msh = msh
        self.bc = "".join(bc)
        msh.set_bc(self.bc)
        self.M = generateMask(self.bc, msh)
        z = lambda: torch.zeros_like(msh.x)  # noqa: E731
        self.u, self.ub, self.f = z(), z(), z()
        self.uh = [z() for _ in range(k)]
        self.nu = float(nu)
        self.tstep = TimeStepper(Ti, Tf, dt, k)
        self.precision = precision
        self.checkpoint_every = checkpoint_every
        self.checkpoints = {}
        self.last_info = {}

    def opLHS(self):
        return HelmholtzOp(self.msh, self.nu, self.tstep.bdfB[0], precision=self.precision)

    def makeRHS(self):
        """src/diffusion.jl:51-65."""
        from .ops import gatherScatter, lapl, mass, mask
        msh, bdfB = self.msh, self.tstep.bdfB
        rhs = mass(self.f, msh)
        if torch.count_nonzero(self.ub):
            rhs = rhs - self.nu * lapl(self.ub, msh)
        for i, uh in enumerate(self.uh):
            if bdfB[1 + i] != 0.0:
                rhs = rhs - bdfB[1 + i] * mass(uh, msh)
        rhs = mask(rhs, self.M)
        return gatherScatter(rhs, msh)

    def solve(self, tol=1e-8):
        op = self.opLHS()
        info = {}
        self.u = pcg(self.makeRHS(), op, opM=Jacobi(op), mult=self.msh.mult, tol=tol, info=info)
        self.last_info = info
        self.u = self.u + self.ub

    def evolve(self, setBC=None, setForcing=None, tol=1e-8):
        """src/diffusion.jl:81-106."""
        for i in range(len(self.uh) - 1, 0, -1):
            self.uh[i].copy_(self.uh[i - 1])
        self.uh[0].copy_(self.u)
        self.tstep.advance()
        t = self.tstep.time[0]
        if setBC is not None:
            setBC(self.ub, self.msh.x, self.msh.y, t)
        if setForcing is not None:
            setForcing(self.f, self.msh.x, self.msh.y, t)
        self.solve(tol)
        if self.checkpoint_every and self.tstep.istep % self.checkpoint_every == 0:
            self.checkpoints[self.tstep.istep] = self.u.clone(memory_format=torch.preserve_format)

    def simulate(self, callback=None, setIC=None, setBC=None, setForcing=None, tol=1e-8):
        """src/diffusion.jl:110-137."""
        if setIC is not None:
            setIC(self.u, self.msh.x, self.msh.y, self.tstep.time[0])
        if callback is not None:
            callback(self)
        while self.tstep.time[0] <= self.tstep.Tf:
            self.evolve(setBC, setForcing, tol)
            if callback is not None:
                callback(self)
            if self.tstep.time[0] < 1e-12:
                break
