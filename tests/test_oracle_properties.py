"""The reference's own test suite (test/runtests.jl), restated against the
oracle on seeded numpy inputs of the same shapes and parameters."""
import numpy as np
import pytest

import cases as K
import oracle as O


def test_kernel_functions_consistent():
    # test/runtests.jl:13-36: F = (dW/dr)/r and G = dF/dq by central differences
    o = O.Oracle("f64")
    h = 0.1
    A = 7.0 / (4.0 * np.pi * h * h)
    for r in (0.01, 0.05, 0.1, 0.15, 0.19):
        d = 1e-7
        dWdr = (o.w_kern((r + d) / h, A) - o.w_kern((r - d) / h, A)) / (2 * d)
        assert o.f_kern(r / h, A, h) == pytest.approx(dWdr / r, rel=1e-6)
    for q in (0.1, 0.5, 1.0, 1.5, 1.9):
        d = 1e-7
        dFdq = (o.f_kern(q + d, A, h) - o.f_kern(q - d, A, h)) / (2 * d)
        assert o.g_kern(q, A, h) == pytest.approx(dFdq, rel=1e-6)
    assert o.w_kern(2.0, A) == 0 and o.f_kern(2.0, A, h) == 0 and o.g_kern(2.0, A, h) == 0
    assert abs(o.f_kern(1.999, A, h)) < 1e-6 * abs(o.f_kern(1.0, A, h))


def test_cell_and_neighbor_list_vs_brute_force():
    # test/runtests.jl:44-104
    case = K.random_points_case()
    p = O.params(**case["p"])
    o = O.Oracle("f64")
    st = o.state(p, case["X0"], case["V0"])
    N = st.N
    st.build_cells()
    c = st.cells()
    assert np.array_equal(np.sort(c["order"]), np.arange(1, N + 1))
    assert c["counts"].sum() == N
    st.build_neighbors(case["p"]["h"])
    idx, nbc = st.neighbors()
    X = case["X0"].T
    rc = 2 * case["p"]["h"] * 1.2
    r2min = np.finfo(float).eps * case["p"]["h"] ** 2
    d2 = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    for i in range(N):
        want = np.nonzero((d2[i] > r2min) & (d2[i] < rc * rc))[0] + 1
        assert np.array_equal(np.sort(idx[i, : nbc[i]]), want)
    assert np.all(nbc <= 64)
    c = st.cells()
    for s, n in zip(c["starts"], c["counts"]):
        seg = c["order"][s:s + n]
        assert np.all(np.diff(seg) > 0)
    assert st.take_flags() == 0
    st.density(p)
    rho = st.fields()["rho"]
    h = case["p"]["h"]
    A = 7.0 / (4 * np.pi * h * h)
    q = np.sqrt(d2) / h
    u = np.clip(1 - q / 2, 0, None)
    rho_ref = case["p"]["m"] * (A * u ** 4 * (2 * q + 1) * (q < 2)).sum(1)
    np.testing.assert_allclose(rho, rho_ref, rtol=1e-12)


def test_neighbor_list_reuse_does_not_change_results():
    # test/runtests.jl:111-157: interval 1 vs 8, 40 steps
    case = K.reuse_case()
    p = O.params(**case["p"])
    o = O.Oracle("f64")
    th = o.theta(case["theta"])
    a = o.state(p, case["X0"], case["V0"], interval=1)
    b = o.state(p, case["X0"], case["V0"], interval=8)
    o.simulate(a, th, p, 40)
    fb = o.simulate(b, th, p, 40)
    Xa, Va = a.get()
    Xb, Vb = b.get()
    np.testing.assert_allclose(Xa, Xb, rtol=1e-14)
    np.testing.assert_allclose(Va, Vb, rtol=1e-14)
    assert fb == 0
    # effective interaction sets (r < 2h) are identical
    h2 = (2 * case["p"]["h"]) ** 2

    def eff(st, X):
        idx, nbc = st.neighbors()
        out = []
        for i in range(st.N):
            js = idx[i, : nbc[i]] - 1
            out.append(set(js[((X[i] - X[js]) ** 2).sum(1) < h2].tolist()))
        return out

    assert eff(a, Xa) == eff(b, Xb)


def _run_linear(o, p, X0, V0, theta, nsteps, cX, cV, tape=False):
    st = o.state(p, X0, V0, interval=1)
    th = o.theta(theta)
    tp = o.tape(st.N, nsteps) if tape else None
    o.simulate(st, th, p, nsteps, tp)
    X, V = st.get()
    J = np.sum(X * cX.T) + np.sum(V * cV.T)
    return J, st, th, tp


def test_adjoint_vs_central_differences():
    # test/runtests.jl:163-228 (implicit drag)
    case = K.adjoint_case()
    p = O.params(**case["p"])
    o = O.Oracle("f64")
    X0, V0, theta = case["X0"], case["V0"], case["theta"]
    cX, cV, n = case["cX"], case["cV"], case["nsteps"]
    J, st, th, tp = _run_linear(o, p, X0, V0, theta, n, cX, cV, tape=True)
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
            vals.append(_run_linear(o, p, a["X"], a["V"], a["t"], n, cX, cV)[0])
        return (vals[0] - vals[1]) / (2 * hfd)

    for j, i in ((0, 0), (3, 2), (4, 5)):
        assert gth[j, i] == pytest.approx(fd("t", (j, i)), rel=1e-5, abs=1e-9)
    for c, k in ((0, 0), (1, 8), (0, 19)):
        assert gX[k, c] == pytest.approx(fd("X", (c, k)), rel=1e-5, abs=1e-8)
    for c, k in ((0, 3), (1, 14)):
        assert gV[k, c] == pytest.approx(fd("V", (c, k)), rel=1e-5, abs=1e-8)


def test_brinkman_drag_lowers_kinetic_energy():
    # test/runtests.jl:233-255
    p = O.params(h=0.06, m=0.004, rho0=1.0, c=10.0, mu=0.02, dt=1e-4, Lx=1.0, Ly=0.6,
                 kw=1e4, ngx=9, ngy=7)
    X0 = np.array([[0.2 + 0.02 * (k % 8) for k in range(64)],
                   [0.3 + 0.02 * (k // 8) for k in range(64)]])
    V0 = np.ones((2, 64))
    o = O.Oracle("f64")

    def ke(a):
        st = o.state(p, X0, V0, interval=1)
        o.simulate(st, o.theta(np.full((7, 9), a)), p, 200)
        return float(np.sum(st.get()[1] ** 2))

    assert ke(500.0) < ke(0.0)


def test_implicit_drag_stable_beyond_explicit_limit():
    # test/runtests.jl:263-293
    dp = 0.02
    p = O.params(h=1.3 * dp, m=dp * dp, rho0=1.0, c=15.0, mu=0.05, dt=2e-4, Lx=1.0, Ly=0.5,
                 kw=5e4, ngx=33, ngy=17)
    X0 = K.lattice_block(12, 10, dp, dp, dp)
    o = O.Oracle("f64")
    lim = 2 / p.dt

    def run(amax):
        st = o.state(p, X0, np.zeros_like(X0), interval=2)
        o.simulate(st, o.theta(np.full((17, 33), amax)), p, 300)
        X, V = st.get()
        return np.max(np.abs(V)), np.all(np.isfinite(X))

    v_soft, ok_soft = run(lim / 10)
    v_hard, ok_hard = run(lim * 10)
    assert ok_soft and ok_hard and v_hard < v_soft


def test_fp32_oracle_close_to_fp64():
    case = K.adjoint_case(seed=1)
    p = O.params(**case["p"])
    out = {}
    for dt in ("f64", "f32"):
        o = O.Oracle(dt)
        J, st, th, tp = _run_linear(o, p, case["X0"], case["V0"], case["theta"], 12,
                                    case["cX"], case["cV"], tape=True)
        ws = o.workspace(st.N, p)
        o.backward(ws, tp, th, p, case["cX"], case["cV"], interval=1)
        out[dt] = (st.get()[0],) + ws.get()
    for a, b in zip(out["f32"], out["f64"]):
        assert K.relerr(a, b) < 1e-5
