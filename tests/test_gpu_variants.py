"""Tait equation of state and Monaghan artificial viscosity on the GPU
against the oracle's restatement (model variants with no counterpart in the
reference; parity is unpinned against the reference, pinned against the
oracle, whose adjoint passes central differences in test_oracle_variants.py).

FP64: bit-identical positions, velocities, dJ/dX0, dJ/dV0 (dJ/dtheta within
1e-12) with one thread or lane groups per particle; FP32 within 1e-5; batch
members equal solo runs; server requests carry the model."""
import numpy as np
import pytest

import cases as K
from runners import linear_seeds, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")

MODELS = {
    "tait": dict(eos=1, gamma=7),
    "artvisc": dict(visc=1, alpha=0.5),
    "both": dict(eos=1, gamma=7, visc=1, alpha=0.5),
}


def with_model(case, model):
    case = dict(case)
    case["p"] = dict(case["p"], **model)
    return case


@pytest.fixture
def lanes():
    yield S.set_group_lanes
    S.set_group_lanes(0)


@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("g", [1, 32])
def test_variant_fp64_matches_oracle(lanes, name, g):
    lanes(g)
    case = with_model(K.adjoint_case(seed=6), MODELS[name])
    seeds = linear_seeds(case)
    r = run_oracle(case, case["nsteps"], seeds=seeds)
    o = run_gpu(case, case["nsteps"], seeds=seeds)
    for k in ("X", "V", "gX", "gV"):
        assert np.array_equal(o[k], r[k]), (name, g, k)
    assert K.relerr(o["gtheta"], r["gtheta"]) <= 1e-12


def test_variant_dambreak_fp64():
    # Tait (gamma 7) + artificial viscosity 0.02 on a jittered dam break, as
    # the configuration text of the small benchmark case describes the physics
    case = with_model(K.dambreak_case(nx=30, ny=20, theta_seed=3, jitter=0.05),
                      dict(eos=1, gamma=7, visc=1, alpha=0.02))
    p = case["p"]
    seeds = lambda X, V: K.ke_seeds(X, V, p)[1:]  # noqa: E731
    r = run_oracle(case, 60, seeds=seeds)
    o = run_gpu(case, 60, seeds=seeds)
    for k in ("X", "V", "gX", "gV"):
        assert np.array_equal(o[k], r[k]), k
    assert K.relerr(o["gtheta"], r["gtheta"]) <= 1e-12


@pytest.mark.parametrize("name", sorted(MODELS))
def test_variant_fp32_close_to_fp64_oracle(name):
    case = with_model(K.adjoint_case(seed=2), MODELS[name])
    seeds = linear_seeds(case)
    r = run_oracle(case, case["nsteps"], seeds=seeds)
    f = run_gpu(case, case["nsteps"], dtype="f32", seeds=seeds)
    for k in ("X", "V", "gX", "gV", "gtheta"):
        assert K.relerr(f[k], r[k]) <= 1e-5, (name, k)


def test_batch_of_mixed_models_equals_solo_runs():
    """FP64: every member equals its solo run bit for bit. FP32: a batch that
    mixes viscosity models runs the artificial-viscosity kernel variant for
    all members, whose contraction of multiply-adds differs from the Morris-
    only variant, so Morris members agree with their solo runs to FP32
    rounding; members of the same variant still match exactly."""
    cases = [K.adjoint_case(seed=11), with_model(K.adjoint_case(seed=12), MODELS["both"]),
             with_model(K.gradcheck_case(seed=13), MODELS["tait"])]
    n = 10
    for dtype in ("f64", "f32"):
        ps = [S.SPHParams(**c["p"], dtype=dtype) for c in cases]
        bt = S.Batch([c["X0"] for c in cases], [c["V0"] for c in cases], ps, interval=2)
        th = S.BatchField([c["theta"] for c in cases], dtype)
        tp = S.Tape(bt.N, n, ps[0])
        S.simulate(bt, th, None, n, tp)
        states = bt.get()
        ws = S.BatchWorkspace(bt)
        S.batch_backward(ws, tp, th, [c["cX"] for c in cases], [c["cV"] for c in cases],
                         interval=2)
        S.set_group_lanes(1)  # solo runs in the batch's form (one thread per particle)
        try:
            for c, (X, V), (gX, gV, gt) in zip(cases, states, ws.get()):
                solo = run_gpu(c, n, dtype=dtype, seeds=linear_seeds(c), interval=2)
                got = dict(X=X, gX=gX, gV=gV, gtheta=gt)
                exact = dtype == "f64" or c["p"].get("visc", 0) == 1
                for k, a in got.items():
                    a = np.asarray(a, np.float64)
                    if exact:
                        assert np.array_equal(a, solo[k]), (dtype, k)
                    else:
                        assert K.relerr(a, solo[k]) <= 1e-5, (dtype, k)
        finally:
            S.set_group_lanes(0)


def test_server_request_carries_the_model():
    from sphadjoint_gb300.serve import Server
    case = with_model(K.adjoint_case(seed=21), MODELS["both"])
    p = S.SPHParams(**case["p"])
    n = case["nsteps"]
    st = S.State(case["X0"], case["V0"], p, interval=1)
    th = S.DesignField(case["theta"])
    tp = S.Tape(st.N, n, p)
    S.simulate(st, th, p, n, tp)
    X, V = st.get()
    J, sX, sV = S.kinetic_energy_right_half(X, V, p)
    ws = S.AdjointWorkspace(st.N, p)
    S.backward(ws, tp, th, p, sX, sV, interval=1)
    with Server(workers=2, hbm_budget_bytes=2 << 30, dtype="f64") as srv:
        r = srv.submit(p, case["X0"], case["V0"], case["theta"], n, interval=1).wait()
    assert r["J"] == pytest.approx(J, rel=1e-12)
    assert np.array_equal(np.asarray(r["gtheta"]), np.asarray(ws.get()[2]))


def test_invalid_model_parameters_are_rejected():
    case = K.adjoint_case(seed=1)
    for bad in (dict(eos=1, gamma=0), dict(eos=1, gamma=16), dict(eos=2), dict(visc=3),
                dict(visc=1, alpha=-1.0)):
        p = S.SPHParams(**dict(case["p"], **bad))
        with pytest.raises(S.ArgumentError):
            S.State(case["X0"], case["V0"], p)
