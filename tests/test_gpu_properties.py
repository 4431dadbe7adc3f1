"""The reference's own property tests (test/runtests.jl), run through the
CUDA library: neighbour-list reuse does not change results, Brinkman drag
lowers the kinetic energy, and the implicit drag stays stable far beyond the
explicit limit."""
import numpy as np
import pytest

import cases as K

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")


def test_neighbor_list_reuse_does_not_change_results():
    # test/runtests.jl:111-157: interval 1 vs 8, 40 steps
    case = K.reuse_case()
    p = S.SPHParams(**case["p"])
    a = S.State(case["X0"], case["V0"], p, interval=1)
    b = S.State(case["X0"], case["V0"], p, interval=8)
    S.simulate(a, case["theta"], p, 40)
    S.simulate(b, case["theta"], p, 40)
    Xa, Va = a.get()
    Xb, Vb = b.get()
    np.testing.assert_allclose(Xa, Xb, rtol=1e-14)
    np.testing.assert_allclose(Va, Vb, rtol=1e-14)
    assert b.last_flags == 0


def test_brinkman_drag_lowers_kinetic_energy():
    # test/runtests.jl:233-255
    p = S.SPHParams(h=0.06, m=0.004, rho0=1.0, c=10.0, mu=0.02, dt=1e-4, Lx=1.0, Ly=0.6,
                    kw=1e4, ngx=9, ngy=7)
    X0 = np.array([[0.2 + 0.02 * (k % 8) for k in range(64)],
                   [0.3 + 0.02 * (k // 8) for k in range(64)]])
    V0 = np.ones((2, 64))

    def ke(a):
        st = S.State(X0, V0, p, interval=1)
        S.simulate(st, np.full((7, 9), a), p, 200)
        return float(np.sum(np.asarray(st.get()[1]) ** 2))

    assert ke(500.0) < ke(0.0)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_implicit_drag_stable_beyond_explicit_limit(dtype):
    # test/runtests.jl:263-293: alpha_max at 10x the explicit limit 2/dt
    dp = 0.02
    p = S.SPHParams(h=1.3 * dp, m=dp * dp, rho0=1.0, c=15.0, mu=0.05, dt=2e-4, Lx=1.0, Ly=0.5,
                    kw=5e4, ngx=33, ngy=17, dtype=dtype)
    X0 = K.lattice_block(12, 10, dp, dp, dp)
    lim = 2 / p.dt

    def run(amax):
        st = S.State(X0, np.zeros_like(X0), p, interval=2)
        S.simulate(st, np.full((17, 33), amax), p, 300)
        X, V = st.get()
        return np.max(np.abs(V)), np.all(np.isfinite(X))

    v_soft, ok_soft = run(lim / 10)
    v_hard, ok_hard = run(lim * 10)
    assert ok_soft and ok_hard and v_hard < v_soft
