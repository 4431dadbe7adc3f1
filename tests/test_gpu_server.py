"""The request server: requests that run concurrently (continuous batching on
several streams) give exactly the result of the same request solved alone;
admission respects the HBM budget."""
import numpy as np
import pytest

import cases as K

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")
from sphadjoint_gb300.serve import Server  # noqa: E402


def requests(dtype):
    out = []
    for k, (nx, ny, steps) in enumerate([(12, 9, 30), (20, 14, 24), (8, 8, 40), (25, 16, 18),
                                          (15, 15, 33)]):
        c = K.dambreak_case(nx=nx, ny=ny, theta_seed=10 + k, jitter=0.05, seed=k)
        c["p"] = dict(c["p"], ngx=9 + k, ngy=7 + k)
        c["theta"] = 40.0 * np.random.default_rng(k).random((7 + k, 9 + k))
        out.append((S.SPHParams(**c["p"], dtype=dtype), c, steps, k % 2))
    return out


def solo(p, c, steps, snapshots):
    st = S.State(c["X0"], c["V0"], p)
    tp = S.Tape(st.N, steps, p, snapshots=snapshots * 3)
    th = S.DesignField(c["theta"], p.dtype)
    S.simulate(st, th, p, steps, tp)
    X, V = st.get()
    J, sX, sV = S.kinetic_energy_right_half(np.asarray(X), np.asarray(V), p)
    ws = S.AdjointWorkspace(st.N, p)
    S.backward(ws, tp, th, p, sX, sV)
    return J, ws.get()


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_results_same_alone_and_in_the_mix(dtype):
    reqs = requests(dtype)
    with Server(workers=3, hbm_budget_bytes=8 << 30, dtype=dtype) as srv:
        tickets = [srv.submit(p, c["X0"], c["V0"], c["theta"], steps, snapshots=snap * 3)
                   for p, c, steps, snap in reqs]
        res = [t.wait() for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["peak_inflight"] >= 2  # requests overlapped
    for (p, c, steps, snap), r in zip(reqs, res):
        J, (gX, gV, gt) = solo(p, c, steps, snap)
        assert np.array_equal(r["gX"], gX)
        assert np.array_equal(r["gV"], gV)
        assert np.array_equal(r["gtheta"], gt)
        assert r["J"] == pytest.approx(J, rel=1e-5 if dtype == "f32" else 1e-12)


def test_admission_respects_hbm_budget():
    reqs = requests("f32")
    one = max(S.load().sph_request_bytes(
        __import__("ctypes").byref(_req_struct(p, c, steps)), 1) for p, c, steps, _ in reqs)
    with Server(workers=4, hbm_budget_bytes=int(one * 1.2), dtype="f32") as srv:
        ts = [srv.submit(p, c["X0"], c["V0"], c["theta"], steps) for p, c, steps, _ in reqs]
        for t in ts:
            t.wait()
        st = srv.stats()
        assert st["peak_bytes"] <= int(one * 1.2)
        assert st["completed"] == len(reqs)
        with pytest.raises(S.SPHError):
            p, c, steps, _ = reqs[0]
            srv.submit(p, np.tile(c["X0"], 60), np.tile(c["V0"], 60), c["theta"], 5000)


def _req_struct(p, c, steps):
    from sphadjoint_gb300 import _lib as LB
    r = LB.sph_request()
    r.p = p.c_struct()
    r.N = c["X0"].shape[1]
    r.nsteps = steps
    r.skin, r.interval, r.maxnb = 0.2, 4, 64
    return r
