"""Write the golden fixtures of tests/test_oracle.py::test_golden_fixtures.

Each fixture holds a ghost-filled primitive state Q, the coordinates x, y, z (with ghosts),
the nine metrics and J, and the inviscid RHS computed by the NumPy restatement
(oracle/np_oracle.py), which is written independently of the C++ oracle and evaluates in a
different operation order. The inputs are stored, not regenerated, so the check does not
depend on libm differences between machines.

  python tests/golden/make_golden.py
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from flame3d_mhd_gb300.abi import BC_DIRICHLET, BC_PERIODIC, BC_WALL_ADIABATIC, BC_ZERO_GRADIENT, make_params  # noqa
from oracle import np_oracle as npo  # noqa
from oracle import oracle as orc  # noqa

NG = 4
PER = [dict(kind=BC_PERIODIC)] * 6
REF_BCS = None  # make_params defaults: inlet, outlet, wall, far field, periodic

CASES = {
    "tgv6_weno5_comp_sw": dict(n=(6, 6, 6), params=dict(character=0, viscous=0, phi1=0.0, phi2=0.0,
                                                         phi3=float("inf"), bc=PER), tgv=True),
    "curvi_hybrid_char_sw": dict(n=(7, 6, 6), params=dict(character=1, viscous=0, phi1=0.02, phi2=0.1, phi3=0.4,
                                                           bc=PER), seed=31, spikes=8),
    "curvi_hybrid_comp_ausm_refbc": dict(n=(7, 6, 5), params=dict(character=0, viscous=0, split_method=3,
                                                                   phi1=0.02, phi2=0.1, phi3=0.4), seed=32,
                                         spikes=8),
    "curvi_hybrid_char_lf_mixedbc": dict(n=(6, 6, 6), params=dict(
        character=1, viscous=0, split_method=1, phi1=0.02, phi2=0.1, phi3=0.4,
        bc=[dict(kind=BC_ZERO_GRADIENT), dict(kind=BC_DIRICHLET, rho=1.1, u=0.3, v=0.0, w=0.1, p=0.8),
            dict(kind=BC_WALL_ADIABATIC), dict(kind=BC_ZERO_GRADIENT), dict(kind=BC_PERIODIC),
            dict(kind=BC_PERIODIC)]), seed=33, spikes=6),
    "curvi_hybrid_comp_vl": dict(n=(6, 6, 6), params=dict(character=0, viscous=0, split_method=2, phi1=0.02,
                                                           phi2=0.1, phi3=0.4, bc=PER), seed=34, spikes=6),
}


def coords(n, amp=0.04, tgv=False):
    s = (n[2] + 8, n[1] + 8, n[0] + 8)
    if tgv:
        h = 2 * np.pi / n[0]
        ax = [(np.arange(k) - NG + 0.5) * h for k in s]
        Z, Y, X = np.meshgrid(*ax, indexing="ij")
        return X, Y, Z
    ax = [(np.arange(k) - NG + 0.5) / (k - 8) for k in s]
    Z, E, X = np.meshgrid(*ax, indexing="ij")
    tp = 2 * np.pi
    return (X + amp * np.sin(tp * E) * np.sin(tp * Z), E + amp * np.sin(tp * Z) * np.sin(tp * X),
            Z + amp * np.sin(tp * X) * np.sin(tp * E))


def initial(P, n, seed=0, spikes=0, tgv=False, x=None, y=None, z=None):
    s = (n[2] + 8, n[1] + 8, n[0] + 8)
    Q = np.zeros((6, *s))
    if tgv:
        Q[0] = 1.0
        Q[1] = 0.1 * np.sin(x) * np.cos(y) * np.cos(z)
        Q[2] = -0.1 * np.cos(x) * np.sin(y) * np.cos(z)
        Q[4] = 1 / 1.4 + 0.01 / 16 * (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2)
    else:
        rng = np.random.default_rng(seed)
        Q[0] = 1.0 + 0.1 * rng.uniform(-1, 1, s)
        Q[1:4] = 0.2 * rng.uniform(-1, 1, (3, *s))
        Q[4] = (1.0 + 0.1 * rng.uniform(-1, 1, s)) / 1.4
        for _ in range(spikes):
            a, b, c = [int(rng.integers(NG, k - NG)) for k in s]
            Q[4, a, b, c] *= float(rng.uniform(5, 100))
    Q[5] = Q[4] / (Q[0] * P.rg)
    return Q


def main():
    for name, spec in CASES.items():
        n = spec["n"]
        params = dict(spec["params"])
        P = make_params(*n, **params)
        x, y, z = coords(n, tgv=spec.get("tgv", False))
        Q0 = initial(P, n, spec.get("seed", 0), spec.get("spikes", 0), spec.get("tgv", False), x, y, z)
        # ghost fill with the oracle's restatement of boundary.jl; the fill is compared
        # bitwise with the GPU elsewhere, the fixture pins the RHS
        U = orc.prim2c(P, Q0)
        Q = Q0.copy()
        orc.fill_ghosts(P, Q, U)
        m, J = npo.metrics(x, y, z)
        r = npo.rhs(P, Q, x, y, z)
        meta = dict(n=list(n), params={k: v for k, v in params.items()}, tol=1e-12,
                    source="oracle/np_oracle.py (NumPy restatement)")
        np.savez_compressed(HERE / f"{name}.npz", Q=Q, x=x, y=y, z=z, metrics=np.stack(m), J=J, rhs=r,
                            meta=json.dumps(meta))
        print(name, np.abs(r).max())


if __name__ == "__main__":
    main()
