"""Tait equation of state and Monaghan artificial viscosity (model variants
with no counterpart in the reference, which uses the linear EOS and Morris
viscosity, README.md:505-519). Their parity is unpinned: these tests check the
oracle's restatement against its own central differences and limits."""
import numpy as np
import pytest

import cases as K
import oracle as O

VARIANTS = [dict(eos=1, gamma=7), dict(visc=1, alpha=0.5), dict(eos=1, gamma=7, visc=1, alpha=0.5)]


def _run(o, p, X0, V0, theta, n, cX, cV, tape=False):
    st = o.state(p, X0, V0, interval=1)
    th = o.theta(theta)
    tp = o.tape(st.N, n) if tape else None
    o.simulate(st, th, p, n, tp)
    X, V = st.get()
    return np.sum(X * cX.T) + np.sum(V * cV.T), st, th, tp


@pytest.mark.parametrize("model", VARIANTS, ids=["tait", "artvisc", "tait+artvisc"])
def test_variant_adjoint_vs_central_differences(model):
    case = K.adjoint_case(seed=4)
    p = O.params(**case["p"], **model)
    o = O.Oracle("f64")
    X0, V0, theta = case["X0"], case["V0"], case["theta"]
    cX, cV, n = case["cX"], case["cV"], case["nsteps"]
    J, st, th, tp = _run(o, p, X0, V0, theta, n, cX, cV, tape=True)
    ws = o.workspace(st.N, p)
    o.backward(ws, tp, th, p, cX, cV, interval=1)
    gX, gV, gth = ws.get()
    hfd = 1e-6

    def fd(which, idx):
        arrs = {"X": X0, "V": V0, "t": theta}
        vals = []
        for sgn in (1, -1):
            a = {k: v.copy() for k, v in arrs.items()}
            a[which][idx] += sgn * hfd
            vals.append(_run(o, p, a["X"], a["V"], a["t"], n, cX, cV)[0])
        return (vals[0] - vals[1]) / (2 * hfd)

    for j, i in ((0, 0), (3, 2), (4, 5)):
        assert gth[j, i] == pytest.approx(fd("t", (j, i)), rel=1e-5, abs=1e-9)
    for c, k in ((0, 0), (1, 8), (0, 19), (1, 12)):
        assert gX[k, c] == pytest.approx(fd("X", (c, k)), rel=1e-5, abs=1e-8)
    for c, k in ((0, 3), (1, 14), (0, 12)):
        assert gV[k, c] == pytest.approx(fd("V", (c, k)), rel=1e-5, abs=1e-8)


def test_variants_change_the_flow_and_reduce_to_limits():
    case = K.adjoint_case(seed=4)
    o = O.Oracle("f64")
    args = (case["X0"], case["V0"], case["theta"], case["nsteps"], case["cX"], case["cV"])
    base = _run(o, O.params(**case["p"]), *args)[1].get()
    for model in VARIANTS:
        X, V = _run(o, O.params(**case["p"], **model), *args)[1].get()
        assert not np.array_equal(V, base[1]), model
    # Tait with gamma = 1 is the linear EOS up to rounding
    X, V = _run(o, O.params(**case["p"], eos=1, gamma=1), *args)[1].get()
    np.testing.assert_allclose(V, base[1], rtol=1e-9, atol=1e-12)
    # artificial viscosity with alpha = 0 adds exact zeros: Morris with mu = 0
    q = dict(case["p"], mu=0.0)
    a = _run(o, O.params(**q), *args)[1].get()
    b = _run(o, O.params(**q, visc=1, alpha=0.0), *args)[1].get()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_artificial_viscosity_dissipates_approach_only():
    # two particles approaching head-on: AV decelerates them; receding: no force
    o = O.Oracle("f64")
    p = dict(h=0.1, m=0.01, rho0=1.0, c=8.0, mu=0.0, dt=1e-4, Lx=1.0, Ly=1.0, kw=0.0,
             ngx=3, ngy=3)
    X0 = np.array([[0.45, 0.55], [0.5, 0.5]])
    th = np.zeros((3, 3))
    for sign in (1, -1):
        V0 = np.array([[0.2 * sign, -0.2 * sign], [0.0, 0.0]])
        outs = []
        for visc in (0, 1):
            st = o.state(O.params(**p, gy=0.0, visc=visc, alpha=1.0), X0, V0, interval=1)
            o.simulate(st, o.theta(th), O.params(**p, gy=0.0, visc=visc, alpha=1.0), 1)
            outs.append(st.get()[1])
        dv = np.abs(outs[1][0, 0]) - np.abs(outs[0][0, 0])
        if sign == 1:
            assert dv < 0   # approaching: slowed down
        else:
            assert dv == 0  # receding: untouched
