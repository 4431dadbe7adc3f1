"""The packed request server: every request in flight advances one time step
per tick and each pass of a tick is one launch over all of them. A request's
result must not depend on what shares its launches: the same request alone
and in a mix of others (different sizes, horizons, tape modes, designs, some
forward-only) gives bit-identical results, equal to the solo API's (FP64 bit
for bit; FP32 within its tolerance of the solo run with one thread per
particle, the packed kernels' form). Admission follows the HBM budget."""
import numpy as np
import pytest

import cases as K

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")
from sphadjoint_gb300.serve import Server  # noqa: E402


def requests(dtype):
    """Five dam breaks of different sizes and designs; snapshots 0 (full
    tape), 3, 0, 3 (binomial checkpoints), auto."""
    out = []
    for k, (nx, ny, steps) in enumerate([(12, 9, 30), (20, 14, 24), (8, 8, 40), (25, 16, 18),
                                          (15, 15, 33)]):
        c = K.dambreak_case(nx=nx, ny=ny, theta_seed=10 + k, jitter=0.05, seed=k)
        c["p"] = dict(c["p"], ngx=9 + k, ngy=7 + k)
        c["theta"] = 40.0 * np.random.default_rng(k).random((7 + k, 9 + k))
        snap = "auto" if k == 4 else 3 * (k % 2)
        out.append((S.SPHParams(**c["p"], dtype=dtype), c, steps, snap))
    return out


def solo(p, c, steps, snapshots):
    S.set_group_lanes(1)
    try:
        st = S.State(c["X0"], c["V0"], p)
        tp = S.Tape(st.N, steps, p, snapshots=0 if snapshots == "auto" else snapshots)
        th = S.DesignField(c["theta"], p.dtype)
        S.simulate(st, th, p, steps, tp)
        ws = S.AdjointWorkspace(st.N, p)
        J = ws.objective(st, "ke_right")
        S.backward_seeded(ws, tp, th, p)
        return J, ws.get()
    finally:
        S.set_group_lanes(0)


def serve(reqs, dtype, budget=8 << 30, forward_only=()):
    with Server(hbm_budget_bytes=budget, dtype=dtype, packed=True) as srv:
        ts = [srv.submit(p, c["X0"], c["V0"], c["theta"], steps, snapshots=snap,
                         adjoint=k not in forward_only)
              for k, (p, c, steps, snap) in enumerate(reqs)]
        res = [t.wait() for t in ts]
        return res, srv.stats()


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_packed_results_same_alone_and_in_the_mix(dtype):
    reqs = requests(dtype)
    mix, st = serve(reqs, dtype)
    assert st["completed"] == len(reqs) and st["peak_inflight"] >= 2
    for k, (p, c, steps, snap) in enumerate(reqs):
        alone, _ = serve([reqs[k]], dtype)
        for key in ("gX", "gV", "gtheta"):
            assert np.array_equal(mix[k][key], alone[0][key]), (k, key)
        assert mix[k]["J"] == alone[0]["J"]
        J, (gX, gV, gt) = solo(p, c, steps, snap)
        if dtype == "f64":
            assert np.array_equal(mix[k]["gX"], gX) and np.array_equal(mix[k]["gV"], gV), k
            assert np.array_equal(mix[k]["gtheta"], gt), k
            assert mix[k]["J"] == J
        else:
            for a, b in ((mix[k]["gX"], gX), (mix[k]["gV"], gV), (mix[k]["gtheta"], gt)):
                assert K.relerr(a, b) <= 1e-5, k
            assert mix[k]["J"] == pytest.approx(J, rel=1e-5)


def test_packed_forward_only_requests_share_the_ticks():
    reqs = requests("f64")
    res, st = serve(reqs, "f64", forward_only=(1, 3))
    full, _ = serve(reqs, "f64")
    for k in range(len(reqs)):
        assert res[k]["J"] == full[k]["J"]
        assert ("gX" in res[k]) == (k not in (1, 3))


def test_packed_admission_follows_the_budget():
    """With a budget of 2.5x the largest request's bytes (read back as the
    peak admitted bytes of that request alone), not all five requests can be
    in flight at once; all complete, admitted bytes never exceed the budget,
    and a request larger than the whole budget is refused at submission."""
    reqs = requests("f32")
    one = max(serve([r], "f32")[1]["peak_bytes"] for r in reqs)
    budget = int(one * 2.5)
    res, st = serve(reqs, "f32", budget=budget)
    assert st["completed"] == len(reqs)
    assert 0 < st["peak_bytes"] <= budget
    assert st["peak_inflight"] < len(reqs)
    with Server(hbm_budget_bytes=budget, dtype="f32", packed=True) as srv:
        p, c, steps, _ = reqs[0]
        with pytest.raises(S.SPHError):
            srv.submit(p, np.tile(c["X0"], 200), np.tile(c["V0"], 200), c["theta"], 5000)
