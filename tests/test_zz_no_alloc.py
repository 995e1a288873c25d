"""The allocation-free solve, sem_pcg_noalloc, checked against sem_pcg.

sem_pcg_noalloc is for callers that may not allocate device memory while they
run: an application's allocation-free real-time loop, a memory manager that
owns every device byte, or a plug-in that may not grow the process's device
footprint.  It keeps its scratch vectors in one fixed device array of the
library instead of calling cudaMalloc, and takes the geometry from the caller.
These tests call it through the C ABI, twice in a row on the same scratch
array, and compare both results with the solve of sem_pcg on a mesh handle
built from the same arrays, within the solver tests' tolerance.  This file
sorts last, so a run that stops at its first failure has already run every
other test.
"""
import ctypes

import numpy as np
import pytest

import sem_oracle as O
from _helpers import host, meshes, rel_l2

pytestmark = pytest.mark.gpu


def _opts(S, tol, precond, precision):
    o = S._lib.PcgOpts()
    o.nu, o.nu_field, o.k = 1.0, None, 0.0
    o.precond, o.precision, o.tol, o.maxiter = precond, precision, tol, 0
    o.inner_tol, o.max_outer, o.check_every, o.mult_ones, o.path = 1e-4, 6, 0, 0, 0
    return o


@pytest.mark.parametrize("precision", ["DF", "F64"])
def test_noalloc_solve_matches_pcg_on_two_calls(gpu, precision):
    import torch

    import semgb300 as S
    lib = S.load()
    prec = S.SEM_F64_DF if precision == "DF" else S.SEM_F64
    mo, md = meshes(9, 8, 8, (False, False), "DDDD", 0.1, precision=prec)
    M = O.generateMask(["D"] * 4, mo)
    f = 2 * np.pi ** 2 * np.sin(np.pi * mo.x) * np.sin(np.pi * mo.y)
    b = S.as_local(O.gatherScatter(O.mask(O.mass(f, mo), M), mo))
    tol = 1e-10 * b.abs().max().item()

    # the existing entry point on a mesh handle, on the same (chunked) path
    op = S.HelmholtzOp(md, 1.0, 0.0)
    ref_info = {}
    x_ref = host(S.pcg(b, op, opM=S.Jacobi(op), mult=md.mult, tol=tol, precision=prec,
                       info=ref_info, path=S.SEM_PATH_CHUNKED))

    # the allocation-free entry point on caller-owned geometry
    G11, G12, G22, B = (S.as_local(getattr(mo, k)) for k in ("G11", "G12", "G22", "B"))
    Dr = np.asfortranarray(mo.Dr)
    Ds = np.asfortranarray(mo.Ds)
    o = _opts(S, tol, S._lib.SEM_PRECOND_JACOBI, prec)
    stream = S.mesh.stream_ptr()
    for call in range(2):
        x = md.empty()
        x.fill_(float("nan"))  # the solve must overwrite every entry
        info = S._lib.SolveInfo()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]  # driver-level free bytes of the device
        st = lib.sem_pcg_noalloc(9, 8, 8, 0, 0, b"DDDD", Dr.ctypes.data, Ds.ctypes.data,
                                 G11.data_ptr(), G12.data_ptr(), G22.data_ptr(), B.data_ptr(),
                                 ctypes.byref(o), b.data_ptr(), x.data_ptr(), ctypes.byref(info),
                                 stream)
        assert st == 0, lib.sem_last_error()
        torch.cuda.synchronize()
        if call == 1:  # after the warm-up call the solve grows the device's memory use by nothing
            assert torch.cuda.mem_get_info()[0] == free0
        assert info.converged and info.res_inf <= tol, call
        assert info.iters == ref_info["iters"], (call, info.iters, ref_info["iters"])
        assert rel_l2(host(x), x_ref) < 1e-12, call


def test_noalloc_rejects_meshes_beyond_its_scratch(gpu):
    import semgb300 as S
    lib = S.load()
    o = _opts(S, 1e-8, S._lib.SEM_PRECOND_NONE, S.SEM_F64_DF)
    Dr = np.asfortranarray(O.derivMat(O.gausslobatto(9)[0]))
    dummy = S.local_empty(9, 9)  # never read: the size check comes first
    p = dummy.data_ptr()
    st = lib.sem_pcg_noalloc(9, 64, 64, 0, 0, b"DDDD", Dr.ctypes.data, Dr.ctypes.data, p, p, p,
                             p, ctypes.byref(o), p, S.local_empty(9, 9).data_ptr(), None, None)
    assert st == S._lib.SEM_ERR_BAD_ARG
    assert b"at most 262144 local DOF" in lib.sem_last_error()
