"""Edge cases of the hot path on the GPU: an empty state, a batch with an
empty member, and heavy neighbour-row truncation (small maxnb) in both the
thread-per-particle and the lane-group forms, against the oracle."""
import numpy as np
import pytest

import cases as K
from runners import linear_seeds, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_empty_state(dtype):
    case = K.adjoint_case(seed=1)
    p = S.SPHParams(**case["p"], dtype=dtype)
    X0 = np.zeros((2, 0))
    st = S.State(X0, X0, p, interval=2)
    th = S.DesignField(case["theta"], dtype)
    tp = S.Tape(0, 5, p)
    S.simulate(st, th, p, 5, tp)
    assert st.last_flags == 0
    ws = S.AdjointWorkspace(0, p)
    assert ws.objective(st, "ke_right") == 0.0
    S.backward(ws, tp, th, p, X0, X0, interval=2)
    gX, gV, gt = ws.get()
    assert gX.shape == (2, 0) and gV.shape == (2, 0)
    assert not np.any(np.asarray(gt))


def test_batch_with_an_empty_member():
    cases = [K.adjoint_case(seed=11), None, K.gradcheck_case(seed=12)]
    base = cases[0]
    empty = dict(p=dict(base["p"]), X0=np.zeros((2, 0)), V0=np.zeros((2, 0)),
                 theta=np.ones((7, 7)), cX=np.zeros((2, 0)), cV=np.zeros((2, 0)))
    cases[1] = empty
    n = 8
    ps = [S.SPHParams(**c["p"]) for c in cases]
    bt = S.Batch([c["X0"] for c in cases], [c["V0"] for c in cases], ps, interval=2)
    th = S.BatchField([c["theta"] for c in cases])
    tp = S.Tape(bt.N, n, ps[0])
    S.simulate(bt, th, None, n, tp)
    states = bt.get()
    ws = S.BatchWorkspace(bt)
    S.batch_backward(ws, tp, th, [c["cX"] for c in cases], [c["cV"] for c in cases], interval=2)
    grads = ws.get()
    for b, c in enumerate(cases):
        if c is empty:
            assert np.asarray(states[b][0]).shape == (2, 0)
            assert not np.any(np.asarray(grads[b][2]))
            continue
        solo = run_gpu(c, n, seeds=linear_seeds(c), interval=2)
        assert np.array_equal(np.asarray(states[b][0]), solo["X"])
        assert np.array_equal(np.asarray(grads[b][0]), solo["gX"])


@pytest.mark.parametrize("lanes", [1, 32])
def test_small_maxnb_truncation_matches_oracle(lanes):
    S.set_group_lanes(lanes)
    try:
        case = K.dambreak_case(nx=20, ny=14, theta_seed=2, jitter=0.05)
        case["cX"] = np.random.default_rng(1).standard_normal(case["X0"].shape)
        case["cV"] = np.random.default_rng(2).standard_normal(case["X0"].shape)
        seeds = linear_seeds(case)
        g = run_gpu(case, 12, seeds=seeds, interval=2, maxnb=8)
        r = run_oracle(case, 12, seeds=seeds, interval=2, maxnb=8)
        assert r["flags"] & 1 and g["flags"] == r["flags"] and g["bflags"] == r["bflags"]
        for k in ("X", "V", "gX", "gV"):
            assert np.array_equal(g[k], r[k]), k
        assert K.relerr(g["gtheta"], r["gtheta"]) <= 1e-12
    finally:
        S.set_group_lanes(0)


@pytest.mark.parametrize("lanes", [1, 32])
def test_non_finite_particle_is_flagged_and_isolated(lanes):
    """A particle with a NaN position raises the non-finite flag, never enters
    another particle's neighbour rows (its r^2 fails every test), and leaves
    the other particles exactly as a run without it."""
    S.set_group_lanes(lanes)
    try:
        case = K.adjoint_case(seed=13)
        p = S.SPHParams(**case["p"])
        X0 = case["X0"].copy()
        X0[:, 0] = np.nan
        st = S.State(X0, case["V0"], p, interval=2)
        with pytest.warns(RuntimeWarning, match="non-finite"):
            S.simulate(st, case["theta"], p, 4)
        assert st.last_flags & 4
        ref = S.State(case["X0"][:, 1:], case["V0"][:, 1:], p, interval=2)
        S.simulate(ref, case["theta"], p, 4)
        X, V = (np.asarray(a) for a in st.get())
        Xr, Vr = (np.asarray(a) for a in ref.get())
        assert np.array_equal(X[:, 1:], Xr) and np.array_equal(V[:, 1:], Vr)
    finally:
        S.set_group_lanes(0)
