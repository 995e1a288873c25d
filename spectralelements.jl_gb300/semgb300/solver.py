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

    def apply_host(self, u_host, out=None, slabs=0):
        """opA on HOST buffers (``sem_hlmz_host``): u_host is a CPU float64
        tensor in the column-major local layout; the result goes to ``out`` (a
        CPU tensor of the same layout, pinned if None) and is complete once the
        current stream has synchronised.  ``slabs``: k >= 1 (0: 8) stages the
        field in k slabs through the copy engines, overlapped with the
        kernels; ``_lib.SEM_HOST_DIRECT`` has the kernels read and write the
        host buffers in place over the CPU-GPU link.  A ``nu_field`` (a device
        field) is folded into G as in ``__call__``."""
        lib = _lib.load()
        msh = self.msh
        nx, ny = msh.shape
        if (u_host.device.type != "cpu" or u_host.dtype != torch.float64 or tuple(u_host.shape) != (nx, ny)
                or u_host.stride() != (1, nx)):
            raise ValueError("u_host must be a CPU float64 tensor of the local shape, column-major")
        if out is None:
            out = torch.empty_strided((nx, ny), (1, nx), dtype=torch.float64, pin_memory=True)
        elif out.device.type != "cpu" or out.dtype != torch.float64 or out.stride() != (1, nx):
            raise ValueError("out must be a CPU float64 tensor of the local shape, column-major")
        flags = _lib.SEM_GS | (_lib.SEM_MASK if msh.bc else 0)
        nu_ptr = None
        if self.nu_field is not None:
            flags |= _lib.SEM_NU_IN_G
            nu_ptr = self.nu_field.data_ptr()
        _lib.check(lib.sem_hlmz_host(msh.handle, nu_ptr, self.nu, self.k, u_host.data_ptr(), out.data_ptr(),
                                     flags, int(slabs), stream_ptr()))
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
        inner_tol=None, max_outer=None, info=None, x=None, path=0):
    """Left-preconditioned CG with mult-weighted dots (src/pcg.jl:16-60).

    tol is the absolute Inf-norm of the residual and maxiter defaults to
    length(b), as in the reference.  On reaching maxiter the reference's
    warning is printed and x is returned.  ``precision``: SEM_F64,
    SEM_F64_DF (default: the mesh's), SEM_MIXED or SEM_MIXED_RR.  ``info`` (dict) receives
    iterations, outer sweeps and residuals.  ``path``: SEM_PATH_AUTO (0),
    SEM_PATH_CHUNKED (graph-replayed chunks over the GPU) or SEM_PATH_SMALL
    (the whole solve in one cluster launch, small meshes).
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
    # None: the library's default for the precision (SEM_MIXED: 1e-4 and 6
    # sweeps; SEM_MIXED_RR: 0.3 and 100 replacements)
    o.inner_tol = 0.0 if inner_tol is None else float(inner_tol)
    o.max_outer = 0 if max_outer is None else int(max_outer)
    o.check_every = 0
    o.path = int(path)
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


class BatchSolver:
    """Many independent pcg solves of mask(QQ'(hlmz(., nu_i, k_i))) on meshes of
    different sizes and orders (n <= 11), run by persistent cluster launches
    (``sem_batch_create`` / ``sem_batch_pcg``)."""

    def __init__(self, meshes, nus, ks, jacobi=True):
        lib = _lib.load()
        self.meshes = list(meshes)
        n = len(self.meshes)
        H = (ctypes.c_void_p * n)(*[m.handle.value for m in self.meshes])
        nu = (ctypes.c_double * n)(*[float(v) for v in nus])
        k = (ctypes.c_double * n)(*[float(v) for v in ks])
        h = ctypes.c_void_p()
        _lib.check(lib.sem_batch_create(H, nu, k, n,
                                        _lib.SEM_PRECOND_JACOBI if jacobi else _lib.SEM_PRECOND_NONE,
                                        ctypes.byref(h)))
        self._h = h
        self._lib = lib

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.sem_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, bs, tols, precision=_lib.SEM_F64_DF, maxiter=None, xs=None, inner_tol=None,
              max_outer=None, infos=None):
        """Solve every problem; returns the list of solutions.  ``infos`` (a list)
        receives one dict per problem.  Raises NotConverged (after filling
        ``infos``) if any problem reached maxiter.  ``precision``: SEM_F64_DF,
        SEM_MIXED or SEM_MIXED_RR (inner_tol/max_outer None: the library's
        defaults for the precision)."""
        n = len(self.meshes)
        bs = [as_local(b) for b in bs]
        if xs is None:
            xs = [m.empty() for m in self.meshes]
        B = (ctypes.c_void_p * n)(*[b.data_ptr() for b in bs])
        X = (ctypes.c_void_p * n)(*[x.data_ptr() for x in xs])
        T = (ctypes.c_double * n)(*[float(t) for t in tols])
        M = None if maxiter is None else (ctypes.c_int * n)(*[int(v) for v in maxiter])
        info = (_lib.SolveInfo * n)()
        st = self._lib.sem_batch_pcg(self._h, B, X, T, M, int(precision),
                                     0.0 if inner_tol is None else float(inner_tol),
                                     0 if max_outer is None else int(max_outer), info, stream_ptr())
        if infos is not None:
            infos[:] = [dict(iters=i.iters, outer=i.outer, res_inf=i.res_inf, converged=bool(i.converged))
                        for i in info]
        _lib.check(st)
        return xs

    def config(self):
        """The launch configuration of every order group (a list of dicts: n,
        problems, cluster_size, ctas_per_sm, clusters; clusters 0 is the
        work-proportional share)."""
        g = self._lib.sem_batch_group_count(self._h)
        cfg = (_lib.BatchGroupConfig * g)()
        _lib.check(self._lib.sem_batch_get_config(self._h, cfg, g))
        return [dict(n=c.n, problems=c.problems, cluster_size=c.cluster_size, ctas_per_sm=c.ctas_per_sm,
                     clusters=c.clusters) for c in cfg]

    def set_config(self, groups):
        """Set every order group's launch configuration (dicts as config())."""
        g = len(groups)
        cfg = (_lib.BatchGroupConfig * g)()
        for c, d in zip(cfg, groups):
            c.n, c.problems = int(d["n"]), int(d.get("problems", 0))
            c.cluster_size, c.ctas_per_sm, c.clusters = int(d["cluster_size"]), int(d["ctas_per_sm"]), int(d["clusters"])
        _lib.check(self._lib.sem_batch_set_config(self._h, cfg, g))

    def order(self):
        """Queue order: problem indices slot by slot (groups in order of n)."""
        n = len(self.meshes)
        o = (ctypes.c_int * n)()
        _lib.check(self._lib.sem_batch_get_order(self._h, o, n))
        return list(o)

    def set_order(self, order):
        """Set the queue order (as order(): every group's slots must hold its
        own problems)."""
        n = len(self.meshes)
        o = (ctypes.c_int * n)(*[int(i) for i in order])
        _lib.check(self._lib.sem_batch_set_order(self._h, o, n))

    def wide(self):
        """Per problem: 1 if it is solved alone on the whole GPU before the
        persistent launches (sem_pcg's chunked path), else 0."""
        n = len(self.meshes)
        w = (ctypes.c_int * n)()
        _lib.check(self._lib.sem_batch_get_wide(self._h, w, n))
        return list(w)

    def set_wide(self, flags):
        n = len(self.meshes)
        w = (ctypes.c_int * n)(*[1 if f else 0 for f in flags])
        _lib.check(self._lib.sem_batch_set_wide(self._h, w, n))

    def timeline(self):
        """Per-problem timeline of the last solve: start and end (ns from the
        first start, device clock), the cluster that solved it (unique over the
        solve's launches; -1 for problems the host solved in FP64), and the
        solve's total device time in ms."""
        import numpy as np
        n = len(self.meshes)
        t0 = (ctypes.c_longlong * n)()
        t1 = (ctypes.c_longlong * n)()
        cl = (ctypes.c_int * n)()
        ms = ctypes.c_double()
        _lib.check(self._lib.sem_batch_timeline(self._h, t0, t1, cl, n, ctypes.byref(ms)))
        return dict(start_ns=np.array(t0[:], dtype=np.int64), end_ns=np.array(t1[:], dtype=np.int64),
                    cluster=np.array(cl[:], dtype=np.int32), total_ms=ms.value)

    def autotune(self, bs, tols, precision=_lib.SEM_F64_DF, maxiter=None, xs=None, inner_tol=None,
                 max_outer=None, cache=None):
        """Choose every group's launch shape (cluster size, CTAs per SM), its
        cluster count and the queue order from measured per-problem
        timelines (``sem_batch_autotune``); the choice is kept on the batch
        and, with ``cache`` (a file path), stored under the batch's signature
        and reused by later calls; it also decides which of the longest
        problems to solve alone on the whole GPU (wide()).  Returns
        dict(runs, best_ms, config, wide)."""
        n = len(self.meshes)
        bs = [as_local(b) for b in bs]
        if xs is None:
            xs = [m.empty() for m in self.meshes]
        B = (ctypes.c_void_p * n)(*[b.data_ptr() for b in bs])
        X = (ctypes.c_void_p * n)(*[x.data_ptr() for x in xs])
        T = (ctypes.c_double * n)(*[float(t) for t in tols])
        M = None if maxiter is None else (ctypes.c_int * n)(*[int(v) for v in maxiter])
        runs, best = ctypes.c_int(), ctypes.c_double()
        _lib.check(self._lib.sem_batch_autotune(self._h, B, X, T, M, int(precision),
                                                0.0 if inner_tol is None else float(inner_tol),
                                                0 if max_outer is None else int(max_outer),
                                                None if cache is None else str(cache).encode(),
                                                ctypes.byref(runs), ctypes.byref(best), stream_ptr()))
        return dict(runs=runs.value, best_ms=best.value, config=self.config(), wide=self.wide())


def pcg_(x, b, opA, **kw):
    """pcg!(x, b, opA; ...) (src/pcg.jl:64-79): x .= pcg(b, opA; ...)."""
    y = pcg(b, opA, **kw)
    x.copy_(y)
    return None


# ---------------------------------------------------------------------------
# adjoint: linsolve with a custom backward (src/adjoint.jl:5-24)
# ---------------------------------------------------------------------------
class _VarCoefSolve(torch.autograd.Function):
    """u = A(nu)^{-1} b with A(nu) = mask(QQ'(D'(nu G)D + k B)); the pullback of
    resi(u, nu, b) = b - A(nu) u (src/adjoint.jl:13-16) at the adjoint state
    lam = A^{-1} mask(QQ'(u_bar)):

    * nu: the per-local-copy gradient -G:(grad lam)(grad u) (``sem_adjoint_grad``);
    * b: mult .* lam.  Fields are local (every global node stored once per
      element that holds it) and autograd sums cotangents over the local
      entries, so the cotangent of an assembled field is the global adjoint
      spread over the copies: for a continuous, masked b = Q b_g the change of
      the loss is lam_g' db_g = sum(mult .* lam .* db).  A right-hand side
      built as mask(QQ'(B f)) then pulls back to B .* lam at f, the gradient
      that finite differences in f give."""

    @staticmethod
    def forward(ctx, nu, b, msh, k, kw):
        op = HelmholtzOp(msh, 1.0, k, nu_field=nu.detach())
        u = pcg(b.detach(), op, opM=Jacobi(op), mult=msh.mult, **kw)
        ctx.save_for_backward(nu.detach(), u)
        ctx.msh, ctx.k, ctx.kw = msh, k, kw
        return u

    @staticmethod
    def backward(ctx, ubar):
        nu, u = ctx.saved_tensors
        msh = ctx.msh
        from .ops import gatherScatter, mask
        rhs = gatherScatter(mask(as_local(ubar), generateMask(msh.bc, msh)), msh)
        op = HelmholtzOp(msh, 1.0, ctx.k, nu_field=nu)
        lam = pcg(rhs, op, opM=Jacobi(op), mult=msh.mult, **ctx.kw)
        g_nu = None
        if ctx.needs_input_grad[0]:
            g_nu = msh.empty()
            _lib.check(_lib.load().sem_adjoint_grad(msh.handle, lam.data_ptr(), u.data_ptr(),
                                                    g_nu.data_ptr(), 0, stream_ptr()))
        g_b = msh.mult * lam if ctx.needs_input_grad[1] else None
        return g_nu, g_b, None, None, None


def linsolve_varcoef(nu, b, msh: Mesh, k=0.0, **kw):
    """Differentiable solve of -div(nu grad u) + k u = f (b = mask(QQ'(B f)))
    in both the nodal nu and the right-hand side b, the pattern of
    ``linsolve`` + ``@adjoint`` (src/adjoint.jl:5-24)."""
    return _VarCoefSolve.apply(nu, b, msh, float(k), kw)


class VarCoefProblem:
    """``problem`` of ``linsolve(a, problem, solver)`` (src/adjoint.jl:5-8) for
    the G-folded diffusion problem: ``problem(a)`` returns
    (lhs, rhs) with lhs = mask(QQ'(D'(a G)D + k B)) (a ``HelmholtzOp``) and
    rhs = ``rhs_fn(a)``, a local field built by differentiable torch
    operations of a (or a fixed field when ``rhs_fn`` is a tensor)."""

    def __init__(self, msh: Mesh, rhs_fn, k=0.0):
        self.msh, self.rhs_fn, self.k = msh, rhs_fn, float(k)

    def __call__(self, a):
        rhs = self.rhs_fn(a) if callable(self.rhs_fn) else self.rhs_fn
        return HelmholtzOp(self.msh, 1.0, self.k, nu_field=a.detach()), rhs


class PcgSolver:
    """``solver(lhs, rhs, adjoint)`` of src/adjoint.jl:5-16: Jacobi PCG on
    the device with the SEM multiplicity dots; ``kw`` are ``pcg`` keywords
    (tol, maxiter, precision, ...).  The operator is symmetric, so the
    adjoint solve is the same solve."""

    def __init__(self, **kw):
        self.kw = kw

    def __call__(self, lhs, rhs, adjoint=False):
        return pcg(as_local(rhs), lhs, opM=Jacobi(lhs), mult=lhs.msh.mult, **self.kw)


def linsolve(a, problem, solver):
    """linsolve(a, problem, solver) (src/adjoint.jl:5-24) on the device:
    u = solver(lhs, rhs) with (lhs, rhs) = problem(a), differentiable in a
    through the whole residual rhs(a) - lhs(a)(u) (the nu gradient of the
    operator plus the pullback of rhs(a) at mult .* lam).  Serves the
    G-folded diffusion problem (``VarCoefProblem``) with ``PcgSolver``;
    anything else raises TypeError rather than running a host loop."""
    if not isinstance(problem, VarCoefProblem) or not isinstance(solver, PcgSolver):
        raise TypeError("linsolve on the device takes a VarCoefProblem and a PcgSolver")
    _, rhs = problem(a)
    return _VarCoefSolve.apply(a, as_local(rhs), problem.msh, problem.k, solver.kw)


def _mass_gs_mask(msh, v, scale):
    """mask(QQ'(scale * B v)) on the device."""
    lib = _lib.load()
    out = msh.empty()
    _lib.check(lib.sem_mass(msh.handle, as_local(v).data_ptr(), out.data_ptr(),
                            _lib.SEM_GS | (_lib.SEM_MASK if msh.bc else 0), stream_ptr()))
    return out if scale == 1.0 else out * scale


def _step_solve(msh, nu, dt, rhs, kw):
    op = HelmholtzOp(msh, 1.0, 1.0 / dt, nu_field=nu)
    return pcg(rhs, op, opM=Jacobi(op), mult=msh.mult, **kw)


class _TransientVarCoef(torch.autograd.Function):
    """Implicit Euler for du/dt = div(nu grad u) + f with nu folded into G:
    (K(nu) + B/dt) u_n = B u_{n-1}/dt + B f, assembled as mask(QQ'(.)), for
    n = 1..nsteps; returns u_nsteps.  Forward states are kept every
    ``checkpoint_every`` steps; backward recomputes each segment from its
    checkpoint and runs the discrete adjoint backwards in time:
    (K + B/dt) lam_T = mask(QQ'(u_bar)), (K + B/dt) lam_n = mask(QQ'(B lam_{n+1}/dt)),
    dJ/dnu = sum_n -G:(grad lam_n)(grad u_n) per local copy.  The initial
    state and the forcing enter every step's right-hand side through
    mask(QQ'(B .)), so their cotangents (summed over local entries, see
    ``_VarCoefSolve``) are B .* lam_1 / dt for u0 and B .* sum_n lam_n for f."""

    @staticmethod
    def forward(ctx, nu, u0, f, msh, dt, nsteps, every, kw):
        nu = nu.detach()
        bf = _mass_gs_mask(msh, f, 1.0)
        u = as_local(u0).clone(memory_format=torch.preserve_format)
        ckpt = {0: u}
        for n in range(1, nsteps + 1):
            rhs = _mass_gs_mask(msh, u, 1.0 / dt) + bf
            u = _step_solve(msh, nu, dt, rhs, kw)
            if every and n % every == 0 and n < nsteps:
                ckpt[n] = u
        ctx.save_for_backward(nu)
        ctx.msh, ctx.dt, ctx.nsteps, ctx.every, ctx.kw = msh, dt, nsteps, every, kw
        ctx.ckpt, ctx.bf, ctx.uT = ckpt, bf, u
        ctx.recomputed_steps = 0
        return u

    @staticmethod
    def backward(ctx, ubar):
        (nu,) = ctx.saved_tensors
        msh, dt, T, every, kw = ctx.msh, ctx.dt, ctx.nsteps, ctx.every, ctx.kw
        lib = _lib.load()
        from .ops import gatherScatter, mask
        M = generateMask(msh.bc, msh) if msh.bc else []
        grad = torch.zeros_like(nu)
        lam_sum = torch.zeros_like(nu) if ctx.needs_input_grad[2] else None
        starts = sorted(ctx.ckpt)
        lam = None
        n = T
        for s in reversed(starts):
            # recompute u_{s+1} .. u_{min(next checkpoint, T)} from the checkpoint at s
            stop = min(T, s + every) if every else T
            seg = {}
            u = ctx.ckpt[s]
            for m in range(s + 1, stop + 1):
                if m == T:
                    u = ctx.uT
                else:
                    rhs = _mass_gs_mask(msh, u, 1.0 / dt) + ctx.bf
                    u = _step_solve(msh, nu, dt, rhs, kw)
                    ctx.recomputed_steps += 1
                seg[m] = u
            for m in range(stop, s, -1):
                if m == T:
                    rhs = gatherScatter(mask(as_local(ubar), M), msh)
                else:
                    rhs = _mass_gs_mask(msh, lam, 1.0 / dt)
                lam = _step_solve(msh, nu, dt, rhs, kw)
                if lam_sum is not None:
                    lam_sum += lam
                g = msh.empty()
                _lib.check(lib.sem_adjoint_grad(msh.handle, lam.data_ptr(), seg[m].data_ptr(),
                                                g.data_ptr(), 0, stream_ptr()))
                grad += g
                n = m
        assert n == 1
        B = msh.B
        g_u0 = B * lam / dt if ctx.needs_input_grad[1] else None
        g_f = B * lam_sum if lam_sum is not None else None
        return grad, g_u0, g_f, None, None, None, None, None


def transient_varcoef(nu, u0, f, msh: Mesh, dt, nsteps, checkpoint_every=20, **kw):
    """Differentiable implicit-Euler run of the variable-coefficient diffusion
    (``Diffusion`` with k=1 and nu folded into G), checkpointing every
    ``checkpoint_every`` steps; returns the final state."""
    return _TransientVarCoef.apply(nu, u0, f, msh, dt, nsteps, checkpoint_every, kw)


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


def simulate_steps(t0, dt, Tf):
    """The number of evolve! calls of the loop of src/diffusion.jl:130-137
    (``while time <= Tf``, leaving after a step that ends below 1e-12), with
    the time advanced by the same floating-point additions."""
    n, t = 0, float(t0)
    while t <= Tf:
        if dt == 0.0 and t >= 1e-12:
            raise ValueError("dt = 0 with Ti > 0 never leaves the loop of src/diffusion.jl:130")
        t += dt
        n += 1
        if t < 1e-12:
            break
    return n


class Diffusion:
    """``Diffusion(bc, msh; Ti, Tf, dt, k)`` (src/diffusion.jl:7-34) with
    device fields u, uh (histories), ub, nu, f.  ``checkpoint_every`` keeps
    copies of u every that many steps (for adjoint recomputation).

    The solve is the reference's: pcg on opLHS with mult = msh.mult and the
    identity preconditioner (src/diffusion.jl:67-77); ``jacobi=True`` uses
    the Jacobi preconditioner instead.  ``path`` picks the solver path
    (SEM_PATH_AUTO, SEM_PATH_CHUNKED, SEM_PATH_SMALL)."""

    def __init__(self, bc, msh: Mesh, Ti=0.0, Tf=0.0, dt=0.0, k=3, nu=1.0,
                 precision=None, checkpoint_every=0, jacobi=False, path=0):
        if not 1 <= k <= _lib.SEM_BDF_MAX_ORDER:
            raise ValueError(f"order k must be in 1..{_lib.SEM_BDF_MAX_ORDER}")
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
        self.jacobi = bool(jacobi)
        self.path = int(path)
        self.checkpoint_every = checkpoint_every
        self.checkpoints = {}
        self.last_info = {}

    def opLHS(self):
        return HelmholtzOp(self.msh, self.nu, self.tstep.bdfB[0], precision=self.precision)

    def makeRHS(self):
        """src/diffusion.jl:51-65 as one gather kernel plus one fused lapl
        launch for the boundary data (``sem_bdf_rhs``)."""
        lib = _lib.load()
        msh, k = self.msh, len(self.uh)
        rhs = msh.empty()
        bdfB = (ctypes.c_double * (k + 1))(*[float(v) for v in self.tstep.bdfB])
        uh = (ctypes.c_void_p * k)(*[as_local(u).data_ptr() for u in self.uh])
        _lib.check(lib.sem_bdf_rhs(msh.handle, self.nu, k, bdfB, as_local(self.f).data_ptr(),
                                   as_local(self.ub).data_ptr(), uh, rhs.data_ptr(), stream_ptr()))
        return rhs

    def _opts(self, tol, maxiter=None):
        o = _lib.PcgOpts()
        o.nu = self.nu
        o.precond = _lib.SEM_PRECOND_JACOBI if self.jacobi else _lib.SEM_PRECOND_NONE
        o.precision = int(self.precision if self.precision is not None else self.msh.precision)
        o.tol = float(tol)
        o.maxiter = 0 if maxiter is None else int(maxiter)
        o.path = self.path
        o.mult_ones = 0
        return o

    def solve(self, tol=1e-8):
        op = self.opLHS()
        info = {}
        opM = Jacobi(op) if self.jacobi else None
        self.u = pcg(self.makeRHS(), op, opM=opM, mult=self.msh.mult, tol=tol, info=info,
                     path=self.path)
        self.last_info = info
        self.u = self.u + self.ub

    def run(self, nsteps, forcing=(), boundary=(), tol=1e-8, maxiter=None):
        """``nsteps`` calls of evolve! in one ``sem_bdf_run`` call: the
        histories, the right-hand side and the solves stay on the device, and
        where the single-launch small-mesh solver serves the mesh no step
        waits for the host.

        ``forcing`` and ``boundary`` are lists of ``(field, fn)`` pairs: at the
        time t of a step, f = sum fn(t) * field and ub = sum fn(t) * field (the
        reference's setForcing!/setBC! closures, restricted to separable
        forms; at most 8 each).  Returns the per-step solve records."""
        lib = _lib.load()
        msh, ts, k = self.msh, self.tstep, len(self.uh)
        nsteps = int(nsteps)
        if nsteps <= 0:
            return []
        forcing, boundary = list(forcing), list(boundary)
        times, t = [], ts.time[0]
        for _ in range(nsteps):  # the additions the library makes
            t += ts.dt
            times.append(t)

        def table(modes):
            vals = [float(fn(tt)) for tt in times for (_, fn) in modes]
            return (ctypes.c_double * max(1, len(vals)))(*vals)

        keep = []  # the device fields the call reads

        def fields(modes):
            keep.extend(as_local(f) for f, _ in modes)
            return (ctypes.c_void_p * max(1, len(modes)))(*[t.data_ptr() for t in keep[-len(modes):]]
                                                            if modes else [])

        d = _lib.BdfDesc()
        d.order, d.nu, d.dt, d.nsteps = k, self.nu, ts.dt, nsteps
        d.solve = self._opts(tol, maxiter)
        F, fc, UB, bc = fields(forcing), table(forcing), fields(boundary), table(boundary)
        d.nf, d.F, d.fcoef = len(forcing), F, fc
        d.nb, d.UB, d.bcoef = len(boundary), UB, bc
        time_arr = (ctypes.c_double * (k + 1))(*ts.time)
        uh = (ctypes.c_void_p * k)(*[as_local(u).data_ptr() for u in self.uh])
        infos = (_lib.SolveInfo * nsteps)()
        self.u = as_local(self.u)
        st = lib.sem_bdf_run(msh.handle, ctypes.byref(d), time_arr, self.u.data_ptr(), uh, infos,
                             stream_ptr())
        if st not in (_lib.SEM_OK, _lib.SEM_ERR_NOT_CONVERGED):
            _lib.check(st)
        ts.time = [float(v) for v in time_arr]
        ts.istep += nsteps
        ts.bdfA, ts.bdfB = bdfExtK(ts.time, k)
        last = times[-1]
        if forcing:
            self.f = sum(float(fn(last)) * as_local(f) for f, fn in forcing)
        if boundary:
            self.ub = sum(float(fn(last)) * as_local(f) for f, fn in boundary)
        out = [dict(iters=i.iters, outer=i.outer, res_inf=i.res_inf, res0_inf=i.res0_inf,
                    converged=bool(i.converged)) for i in infos]
        for i in out:
            if not i["converged"]:
                print("warning: res:", i["res_inf"])
        self.last_info = out[-1]
        return out

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
        """src/diffusion.jl:110-137.  Without a callback or setBC/setForcing
        closures (f and ub then stay as they are) the whole loop runs as one
        ``run`` on the device."""
        if setIC is not None:
            setIC(self.u, self.msh.x, self.msh.y, self.tstep.time[0])
        if callback is not None:
            callback(self)
        if callback is None and setBC is None and setForcing is None and not self.checkpoint_every:
            n = simulate_steps(self.tstep.time[0], self.tstep.dt, self.tstep.Tf)
            forcing = [(self.f.clone(), lambda _t: 1.0)] if torch.count_nonzero(self.f) else []
            boundary = [(self.ub.clone(), lambda _t: 1.0)] if torch.count_nonzero(self.ub) else []
            self.run(n, forcing, boundary, tol=tol)
            return
        while self.tstep.time[0] <= self.tstep.Tf:
            self.evolve(setBC, setForcing, tol)
            if callback is not None:
                callback(self)
            if self.tstep.time[0] < 1e-12:
                break
