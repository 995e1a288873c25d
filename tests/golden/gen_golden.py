"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

No vector produced by the Julia reference exists (Julia is not available), so
these fixtures are oracle outputs on seeded inputs (NumPy PCG64), committed so
that parity never depends on regenerating them or on cross-language RNG
equality.  Run:  python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import sem_oracle as O  # noqa: E402

CASES = {
    # name: (n, Ex, Ey, periodic, bc, deform amplitude, nu, k)
    "n5_4x3_DDDD": (5, 4, 3, (False, False), "DDDD", 0.1, 1e-2, 1.0),
    "n9_3x3_perx_DNDD": (9, 3, 3, (True, False), "DNDD", 0.05, 0.5, 2.0),
    "n4_2x5_pery_NNDD": (4, 2, 5, (False, True), "NNDD", 0.05, 1.0, 0.5),
    "n17_2x2_DDDD": (17, 2, 2, (False, False), "DDDD", 0.1, 1.0, 3.0),
}


def case_arrays(n, Ex, Ey, per, bc, amp, nu, k, seed):
    mo = O.Mesh(n, n, Ex, Ey, per, O.sin_deform(amp))
    M = O.generateMask(list(bc), mo)
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1, 1, mo.shape)
    out = {
        "zr": mo.zr, "wr": mo.wr, "Dr": mo.Dr, "x": mo.x, "y": mo.y, "B": mo.B, "G11": mo.G11,
        "G12": mo.G12, "G22": mo.G22, "mult": mo.mult, "mask": M.astype(np.uint8),
        "l2gx": mo.l2gx, "l2gy": mo.l2gy, "u": u,
        "lapl": O.lapl(u, mo),
        "hlmz": O.hlmz(u, nu, k, mo),
        "opLHS": O.mask(O.gatherScatter(O.hlmz(u, nu, k, mo), mo), M),
        "gatherScatter": O.gatherScatter(u, mo),
        "jacobi": O.jacobi_diag(mo, nu, k, M),
        "params": np.array([n, Ex, Ey, int(per[0]), int(per[1]), amp, nu, k]),
        "bc": np.frombuffer(bc.encode(), dtype=np.uint8),
    }
    # a Jacobi-PCG solve of opLHS x = mask(QQ'(B f)) with f = 1 (tol 1e-11 abs)
    b = O.gatherScatter(O.mask(O.mass(np.ones(mo.shape), mo), M), mo)
    d = out["jacobi"]
    info = {}
    x = O.pcg(b, lambda v: O.mask(O.gatherScatter(O.hlmz(v, nu, k, mo), mo), M),
              opM=lambda r: r / d, mult=mo.mult, tol=1e-11, info=info)
    out.update(b=b, xsol=x, iters=np.array([info["iters"]]))
    return out


def main():
    for i, (name, c) in enumerate(CASES.items()):
        arrs = case_arrays(*c, seed=100 + i)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        print(name, sum(a.nbytes for a in arrs.values()))


if __name__ == "__main__":
    main()
