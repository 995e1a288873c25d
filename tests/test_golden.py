"""Committed golden fixtures (tests/golden/*.npz, made by gen_golden.py from the
oracle on seeded inputs): the oracle must keep reproducing them (CPU), and the
device path must match them (GPU, through the C ABI)."""
import glob
import os

import numpy as np
import pytest

import sem_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _case(path):
    z = np.load(path)
    n, Ex, Ey, px, py = (int(v) for v in z["params"][:5])
    amp, nu, k = (float(v) for v in z["params"][5:])
    return z, n, Ex, Ey, (bool(px), bool(py)), bytes(z["bc"]).decode(), amp, nu, k


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
def test_oracle_reproduces_golden(path):
    z, n, Ex, Ey, per, bc, amp, nu, k = _case(path)
    mo = O.Mesh(n, n, Ex, Ey, per, O.sin_deform(amp))
    M = O.generateMask(list(bc), mo)
    np.testing.assert_array_equal(mo.zr, z["zr"])
    np.testing.assert_array_equal(M.astype(np.uint8), z["mask"])
    np.testing.assert_array_equal(mo.mult, z["mult"])
    np.testing.assert_array_equal(mo.l2gx, z["l2gx"])
    np.testing.assert_array_equal(mo.l2gy, z["l2gy"])
    for key in ("Dr", "x", "y", "B", "G11", "G12", "G22"):
        np.testing.assert_allclose(getattr(mo, key), z[key], rtol=1e-14, atol=1e-14 * np.abs(z[key]).max())
    u = z["u"]
    np.testing.assert_allclose(O.lapl(u, mo), z["lapl"], rtol=1e-13, atol=1e-13 * np.abs(z["lapl"]).max())
    np.testing.assert_array_equal(O.gatherScatter(u, mo), z["gatherScatter"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f) for f in FILES])
@pytest.mark.parametrize("prec", ["F64", "DF"])
def test_device_matches_golden(gpu, path, prec):
    import semgb300 as S
    from _helpers import host, rel_l2
    z, n, Ex, Ey, per, bc, amp, nu, k = _case(path)
    arrays = {"zr": z["zr"], "wr": z["wr"], "zs": z["zr"], "ws": z["wr"], "Dr": z["Dr"],
              "Ds": z["Dr"], "x": z["x"], "y": z["y"], "G11": z["G11"], "G12": z["G12"],
              "G22": z["G22"], "B": z["B"]}
    md = S.Mesh.from_arrays(n, Ex, Ey, per, arrays, bc=bc,
                            precision=S.SEM_F64 if prec == "F64" else S.SEM_F64_DF)
    u = S.as_local(z["u"])
    assert rel_l2(host(S.lapl(u, md)), z["lapl"]) < 1e-12
    assert rel_l2(host(S.hlmz(u, nu, k, md)), z["hlmz"]) < 1e-12
    assert rel_l2(host(S.HelmholtzOp(md, nu, k)(u)), z["opLHS"]) < 1e-12
    np.testing.assert_array_equal(host(S.gatherScatter(u, md)), z["gatherScatter"])
    np.testing.assert_array_equal(host(md.mult), z["mult"])
    np.testing.assert_array_equal(host(S.generateMask(bc, md)).astype(np.uint8), z["mask"])
    op = S.HelmholtzOp(md, nu, k)
    jac = S.Jacobi(op)
    assert rel_l2(host(jac.diag()), z["jacobi"]) < 1e-13
    info = {}
    x = host(S.pcg(S.as_local(z["b"]), op, opM=jac, mult=md.mult, tol=1e-11, info=info))
    assert abs(info["iters"] - int(z["iters"][0])) <= 2
    assert np.abs(x - z["xsol"]).max() < 1e-9 * max(1.0, np.abs(z["xsol"]).max())
