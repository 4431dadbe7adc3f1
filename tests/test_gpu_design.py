"""The design side of the topology-optimisation caller on the device
(sph_design_*) against its host restatement (sphadjoint_gb300.topopt, which
follows scripts/03_optimize.jl:142-219): alpha(rho), its derivative, the
density filter and its adjoint bit for bit (same operations in the same
order, FP64 without contraction); the volume projection and the line-search
candidate within 1e-12 (their means are summed in another order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")
from sphadjoint_gb300 import topopt as T  # noqa: E402

SHAPES = [(17, 33, 2), (9, 13, 1), (64, 48, 3), (128, 128, 2)]


@pytest.mark.parametrize("ngy,ngx,r", SHAPES)
def test_filter_adjoint_alpha_bit_identical(ngy, ngx, r):
    rng = np.random.default_rng(ngy * ngx)
    dd = T.DeviceDesign(ngy, ngx, r, 2.0e3, 0.1, 0.75)
    f = T.DensityFilter(ngy, ngx, r)
    x = rng.random((ngy, ngx)) * 1.2 - 0.1  # some outside [0, 1]: the clamp acts
    g = rng.standard_normal((ngy, ngx))
    assert np.array_equal(dd.apply(dd.FILTER, x), f.apply(x))
    assert np.array_equal(dd.apply(dd.FILTER_ADJOINT, g), f.adjoint(g))
    rd = rng.random((ngy, ngx))
    assert np.array_equal(dd.apply(dd.ALPHA, rd), T.alpha_of(rd, 2.0e3, 0.1))
    assert np.array_equal(dd.apply(dd.DALPHA, rd), T.dalpha_of(rd, 2.0e3, 0.1))


@pytest.mark.parametrize("ngy,ngx,r", SHAPES)
def test_projection(ngy, ngx, r):
    rng = np.random.default_rng(7 + ngx)
    dd = T.DeviceDesign(ngy, ngx, r, 2.0e3, 0.1, 0.75)
    for x in (rng.random((ngy, ngx)) * 0.9, 0.8 + 0.2 * rng.random((ngy, ngx)),
              rng.random((ngy, ngx)) * 1.4 - 0.2):
        assert np.max(np.abs(dd.apply(dd.PROJECT, x) - T.project_volume(x, 0.75))) <= 1e-12


def test_design_gradient_chain_on_the_device():
    """grad = filter_adjoint(dJ/dtheta * dalpha(filter(rd))) from a real
    backward, device vs host restatement (bit for bit; J equal, so the theta
    the device wrote into the field is the host's alpha(filter(rd))), and the
    line-search candidate within 1e-12."""
    prob = T.reference_problem(t_end=0.1)
    rng = np.random.default_rng(3)
    rd = 0.85 + 0.15 * rng.random((prob.p.ngy, prob.p.ngx))
    J_host, g_host = prob.objective_and_grad(rd)
    dd, sv = prob.dev(), prob.solver()
    dd.set(rd)
    dd.to_theta(sv.th)
    J = sv.solve(True)
    gmax = dd.gradient(sv.ws)
    rd_d, rdf_d, g_d = dd.get()
    assert np.array_equal(rd_d, rd)
    assert np.array_equal(rdf_d, prob.filt.apply(rd))
    assert J == J_host
    assert np.array_equal(g_d, g_host)
    assert gmax == np.max(np.abs(g_host))
    # the line-search candidate project(rd - s g / max|g|), accepted
    for step in (0.05, 0.3):
        dd.set(rd)
        dd.candidate(step)
        dd.accept()
        host = T.project_volume(rd - step * g_host / np.max(np.abs(g_host)), prob.volfrac)
        assert np.max(np.abs(dd.get()[0] - host)) <= 1e-12
