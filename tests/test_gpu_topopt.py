"""The topology-optimisation caller on the GPU: the design gradient
(filter -> alpha(rho) -> solve -> adjoint -> chain rule) against central
differences, as the reference's scripts/10_design_gradcheck.jl does, and a
few line-search iterations with the server giving the sequential trajectory."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")
from sphadjoint_gb300 import topopt as T  # noqa: E402
from sphadjoint_gb300.serve import Server  # noqa: E402


def test_design_gradient_vs_central_differences():
    # 10_design_gradcheck.jl: qp = 10, alpha_max = 100, interior design near 0.9
    prob = T.reference_problem(alpha_max=100.0, qp=10.0)
    rng = np.random.default_rng(7)
    rd = 0.90 + 0.10 * (rng.random((prob.p.ngy, prob.p.ngx)) - 0.5)
    J, g = prob.objective_and_grad(rd)
    assert abs(J) > 1e-3  # the water reaches the target: J carries signal
    idx = np.argsort(-np.abs(g).ravel())[:3]
    h = 1e-5
    for li in idx:
        k = np.unravel_index(li, g.shape)
        xp = rd.copy(); xp[k] += h
        xm = rd.copy(); xm[k] -= h
        fd = (prob.objective_only(xp) - prob.objective_only(xm)) / (2 * h)
        assert abs(g[k] - fd) <= 1e-5 * abs(fd), (k, g[k], fd)


def test_optimisation_reaches_published_objective():
    """The reference's published run of this set-up (float64, 240 particles,
    4000 steps, alpha_max 2000): J -48.816 -> -49.685, converged after 2
    iterations (README.md:600-602)."""
    prob = T.reference_problem(dtype="f64")
    rd_dev, h_dev = T.optimize(prob, maxit=40)  # design side on the device
    assert len(h_dev) == 3
    assert round(h_dev[0], 3) == -48.816 and round(h_dev[-1], 3) == -49.685
    assert all(b < a for a, b in zip(h_dev, h_dev[1:]))
    # the host restatement of the design side takes the same steps
    host = T.reference_problem(dtype="f64")
    host.device = False
    rd_seq, h_seq = T.optimize(host, maxit=40)
    assert np.max(np.abs(rd_dev - rd_seq)) <= 1e-12
    assert h_dev == pytest.approx(h_seq, rel=1e-12)
    # concurrent line-search candidates on a request server: the sequential
    # host trajectory exactly
    with Server(workers=6, hbm_budget_bytes=16 << 30, dtype="f64") as srv:
        rd_par, h_par = T.optimize(host, maxit=40, server=srv)
    assert np.array_equal(rd_seq, rd_par)
    assert h_seq == pytest.approx(h_par, rel=1e-12)


def test_forward_only_request_matches_simulate():
    prob = T.reference_problem(t_end=0.2)
    rd = np.full((prob.p.ngy, prob.p.ngx), 0.95)
    J_host = prob.objective_only(rd)
    with Server(workers=2, hbm_budget_bytes=4 << 30, dtype="f64") as srv:
        t = srv.submit(prob.p, prob.X0, prob.V0, prob.theta_of(rd), prob.nsteps,
                       objective="target", args=(0.85, 0.10, 0.10), interval=2, adjoint=False)
        r = t.wait()
    assert "gtheta" not in r
    assert r["J"] == pytest.approx(J_host, rel=1e-13)
