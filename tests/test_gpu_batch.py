"""Batches: B instances with uneven particle counts, their own parameters,
cell grids and design fields, packed into one State. Every instance must give
exactly what it gives when run alone (same kernels, same per-particle
summation order, per-instance exact dJ/dtheta scale)."""
import numpy as np
import pytest

import cases as K
from runners import linear_seeds, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")


def three_instances():
    a = K.adjoint_case(seed=11)
    b = K.gradcheck_case(seed=12, theta_scale=5.0)
    c = K.dambreak_case(nx=20, ny=14, theta_seed=6, jitter=0.05, seed=3)
    rng = np.random.default_rng(5)
    c["cX"] = rng.standard_normal(c["X0"].shape)
    c["cV"] = rng.standard_normal(c["X0"].shape)
    return [a, b, c]


def run_batch(cases, nsteps, dtype, snapshots=0, interval=2):
    ps = [S.SPHParams(**c["p"], dtype=dtype) for c in cases]
    bt = S.Batch([c["X0"] for c in cases], [c["V0"] for c in cases], ps, interval=interval)
    th = S.BatchField([c["theta"] for c in cases], dtype)
    tp = S.Tape(bt.N, nsteps, ps[0], snapshots=snapshots)
    S.simulate(bt, th, None, nsteps, tp)
    states = bt.get()
    ws = S.BatchWorkspace(bt)
    S.batch_backward(ws, tp, th, [c["cX"] for c in cases], [c["cV"] for c in cases],
                     interval=interval)
    return states, ws.get(), bt, tp


@pytest.mark.parametrize("dtype,snapshots", [("f64", 0), ("f32", 0), ("f64", 3)])
def test_batch_members_equal_solo_runs(dtype, snapshots):
    cases = three_instances()
    n = 16
    states, grads, bt, tp = run_batch(cases, n, dtype, snapshots=snapshots)
    # batches run one thread per particle; small solo FP32 states default to
    # lane groups, whose multiply-add contraction differs, so compare with the
    # same form (FP64 is bit-identical in either form)
    S.set_group_lanes(1)
    try:
        solos = [run_gpu(c, n, dtype=dtype, seeds=linear_seeds(c), interval=2,
                         snapshots=snapshots) for c in cases]
    finally:
        S.set_group_lanes(0)
    for c, (X, V), (gX, gV, gt), solo in zip(cases, states, grads, solos):
        assert np.array_equal(np.asarray(X, np.float64), solo["X"])
        assert np.array_equal(np.asarray(V, np.float64), solo["V"])
        assert np.array_equal(np.asarray(gX, np.float64), solo["gX"])
        assert np.array_equal(np.asarray(gV, np.float64), solo["gV"])
        assert np.array_equal(np.asarray(gt, np.float64), solo["gtheta"])


def test_batch_fp64_matches_oracle():
    cases = three_instances()
    n = 12
    states, grads, _, _ = run_batch(cases, n, "f64")
    for c, (X, V), (gX, gV, gt) in zip(cases, states, grads):
        r = run_oracle(c, n, seeds=linear_seeds(c), interval=2)
        assert np.array_equal(X, r["X"]) and np.array_equal(V, r["V"])
        assert np.array_equal(gX, r["gX"]) and np.array_equal(gV, r["gV"])
        assert K.relerr(gt, r["gtheta"]) <= 1e-12


def test_batch_objective_and_flags():
    cases = three_instances()
    ps = [S.SPHParams(**c["p"]) for c in cases]
    bt = S.Batch([c["X0"] for c in cases], [c["V0"] for c in cases], ps, interval=2)
    th = S.BatchField([c["theta"] for c in cases])
    S.simulate(bt, th, None, 6)
    ws = S.BatchWorkspace(bt)
    J = ws.objective(bt, "target", [[0.3, 0.3, 0.1]] * 3)
    for b, (X, V) in enumerate(bt.get()):
        Jref, _ = S.target_objective(np.asarray(X), 0.3, 0.3, 0.1)
        assert J[b] == pytest.approx(float(Jref), rel=1e-12)
    assert len(bt.take_flags()) == 3
