"""Shared set-up of the GPU parity tests: the same mesh in the oracle and on the
device (geometry uploaded verbatim, so operator parity is isolated from
geometry parity, which has its own test)."""
import numpy as np

import sem_oracle as O

GEOM_KEYS = ("zr", "wr", "zs", "ws", "Dr", "Ds", "x", "y", "G11", "G12", "G22", "B")


def meshes(n, Ex, Ey, periodic=(False, False), bc="DDDD", amp=0.05, precision=None):
    import semgb300 as S
    deform = O.sin_deform(amp) if amp else O.identity_deform
    mo = O.Mesh(n, n, Ex, Ey, periodic, deform)
    arrays = {k: getattr(mo, k) for k in GEOM_KEYS}
    kw = {} if precision is None else {"precision": precision}
    md = S.Mesh.from_arrays(n, Ex, Ey, periodic, arrays, bc=bc, **kw)
    return mo, md


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb else 1.0)


def host(t):
    return t.detach().cpu().numpy()


def continuous(mo, rng, M=None):
    """A random continuous (copies equal) field, masked if M is given."""
    u = mo.mult * O.gatherScatter(rng.uniform(-1, 1, mo.shape), mo)
    return u if M is None else O.mask(u, M)
