"""Captured sequences: one whole forward + adjoint solve recorded as a CUDA
graph and replayed gives bit-identical results to running it call by call,
picks up new inputs written into the same device arrays (design field,
initial state), and refuses to capture allocations."""
import numpy as np
import pytest

import cases as K

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")


class Solve:
    """The bench's solve: reset the state from a pristine copy, reset the
    tape, simulate, on-device objective, seeded backward."""

    def __init__(self, case, dtype="f64", snapshots=3, nsteps=16, interval=2):
        self.p = S.SPHParams(**case["p"], dtype=dtype)
        self.st0 = S.State(case["X0"], case["V0"], self.p, interval=interval)
        self.st = S.State(case["X0"], case["V0"], self.p, interval=interval)
        self.th = S.DesignField(case["theta"], dtype)
        self.tp = S.Tape(self.st.N, nsteps, self.p, snapshots=snapshots)
        self.ws = S.AdjointWorkspace(self.st.N, self.p)
        self.n, self.interval = nsteps, interval

    def __call__(self):
        self.st.assign(self.st0)
        S.reset(self.tp)
        S.simulate(self.st, self.th, self.p, self.n, self.tp)
        self.ws.objective(self.st, "target", (0.5, 0.3, 0.2))
        S.backward_seeded(self.ws, self.tp, self.th, self.p, interval=self.interval)

    def results(self):
        X, V = self.st.get()
        gX, gV, gt = self.ws.get()
        return dict(J=self.ws.objective_value(), X=np.array(X), V=np.array(V), gX=np.array(gX),
                    gV=np.array(gV), gt=np.array(gt))


@pytest.mark.parametrize("dtype,lanes", [("f64", 0), ("f64", 1), ("f32", 0)])
def test_replayed_solve_is_bit_identical(dtype, lanes):
    S.set_group_lanes(lanes)
    try:
        case = K.dambreak_case(nx=24, ny=16, theta_seed=5, jitter=0.05)
        sv = Solve(case, dtype=dtype)
        sv()
        ref = sv.results()
        g = S.capture(sv)
        assert g.nodes > 50
        for _ in range(2):
            g.launch()
            S.synchronize()
            out = sv.results()
            for k in ref:
                assert np.array_equal(out[k], ref[k]), k
    finally:
        S.set_group_lanes(0)


def test_replay_reads_new_inputs_in_place():
    case = K.dambreak_case(nx=24, ny=16, theta_seed=5, jitter=0.05)
    sv = Solve(case)
    sv()
    g = S.capture(sv)
    rng = np.random.default_rng(3)
    theta2 = case["theta"] + 0.5 * rng.random(case["theta"].shape)
    X2 = case["X0"] + 1e-4 * rng.standard_normal(case["X0"].shape)
    # eager reference with the new inputs
    case2 = dict(case, theta=theta2, X0=X2)
    ref = Solve(case2)
    ref()
    want = ref.results()
    # same graph, new values written into the captured arrays
    sv.th.upload(theta2)
    sv.st0.set(X=X2)
    g.launch()
    S.synchronize()
    out = sv.results()
    for k in want:
        assert np.array_equal(out[k], want[k]), k


def test_capture_refuses_first_use_allocations():
    case = K.adjoint_case(seed=3)
    sv = Solve(case, snapshots=2, nsteps=8)
    with pytest.raises(S.SPHError):
        S.capture(sv)  # never run: the workspace and snapshots would allocate
    sv()  # the thread and its stream still work eagerly
    assert np.isfinite(sv.results()["J"])
