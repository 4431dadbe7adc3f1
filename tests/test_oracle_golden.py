"""The oracle against golden vectors from the reference's own Python tools.

tests/golden/gen_golden.py ran tools/verify_gather.py (the gather-form
adjoint written like src/adjoint.jl) and tools/verify_adjoint.py (PyTorch
autograd ground truth) and stored inputs and outputs. Those tools use the
explicit Brinkman drag, so the oracle runs its explicit-drag switch here;
all-pairs sums there vs neighbour-list sums here differ in order only.
"""
import os

import numpy as np
import pytest

import oracle as O
from cases import relerr

GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden_verify.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _params(pr):
    return O.params(h=pr[0], m=pr[1], rho0=pr[2], c=pr[3], mu=pr[4], gx=pr[5], gy=pr[6],
                    dt=pr[7], Lx=pr[8], Ly=pr[9], kw=pr[10], ngx=int(pr[11]), ngy=int(pr[12]))


@pytest.mark.parametrize("case", ["gather", "wall"])
def test_oracle_matches_reference_tools(gold, case):
    g = {k.split("/", 1)[1]: gold[k] for k in gold.files if k.startswith(case + "/")}
    p = _params(g["params"])
    o = O.Oracle("f64")
    N = g["X0"].shape[0]
    ns = int(g["nsteps"])
    st = o.state(p, g["X0"], g["V0"], interval=1)
    tp = o.tape(N, ns)
    th = o.theta(g["theta"])
    assert o.simulate(st, th, p, ns, tp, explicit_drag=True) == 0
    X, V = st.get()
    assert relerr(X, g["XT"]) < 1e-13
    assert relerr(V, g["VT"]) < 1e-13
    J = np.sum(X * g["cX"]) + np.sum(V * g["cV"])
    assert abs(J - g["J_torch"]) <= 1e-12 * abs(g["J_torch"])
    ws = o.workspace(N, p)
    o.backward(ws, tp, th, p, g["cX"], g["cV"], interval=1, explicit_drag=True)
    gX, gV, gt = ws.get()
    # against the reference's gather-form adjoint and against autograd
    for got, a, b in ((gX, g["gX"], g["gX_ad"]), (gV, g["gV"], g["gV_ad"]),
                      (gt, g["gtheta"], g["gtheta_ad"])):
        assert relerr(got, a) < 1e-13
        assert relerr(got, b) < 1e-13
    assert np.max(np.abs(gt)) > 0


def test_golden_tools_agree_with_autograd(gold):
    # the fixture itself reproduces the reference README's accuracy table
    for case in ("gather", "wall"):
        for k in ("gX", "gV", "gtheta"):
            assert relerr(gold[f"{case}/{k}"], gold[f"{case}/{k}_ad"]) < 1e-14
