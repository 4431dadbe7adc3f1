"""CUDA library vs CPU oracle on the same seeded inputs, through the C ABI.

FP64: cell lists and neighbour rows are compared exactly; positions,
velocities, dJ/dX0 and dJ/dV0 bit for bit (same summation order, no FMA);
dJ/dtheta within 1e-12 relative (the oracle sums it serially in particle
order, the library with an exact fixed-point reduction).
FP32: within 1e-5 relative of the FP64 oracle on short horizons.
"""
import numpy as np
import pytest

import cases as K
from runners import linear_seeds, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")
import oracle as O  # noqa: E402


def _states(case, dtype="f64", **kw):
    p = S.SPHParams(**case["p"], dtype=dtype)
    st = S.State(case["X0"], case["V0"], p, **kw)
    o = O.Oracle(dtype)
    ost = o.state(O.params(**case["p"]), case["X0"], case["V0"], **kw)
    return p, st, o, ost


@pytest.mark.parametrize("maker", [K.random_points_case, K.dambreak_case])
def test_celllist_bit_exact(maker):
    case = maker()
    p, st, o, ost = _states(case)
    S.build(st)
    ost.build_cells()
    g = st.celllist()
    c = ost.cells()
    assert np.array_equal(g["counts"], c["counts"])
    assert np.array_equal(g["starts"], c["starts"])
    assert np.array_equal(g["order"], c["order"])
    # build_neighbors! gives the same cell list, and the same rows in order
    S.build_neighbors(st)
    ost.build_neighbors(case["p"]["h"])
    g = st.celllist()
    assert np.array_equal(g["order"], c["order"])
    gi, gn = st.neighbors()
    oi, on = ost.neighbors()
    assert np.array_equal(gn, on)
    for i in range(st.N):
        assert np.array_equal(gi[i, : gn[i]], oi[i, : on[i]]), i
    assert st.take_flags() == ost.take_flags() == 0


def test_density_bit_exact():
    case = K.random_points_case()
    p, st, o, ost = _states(case)
    S.build_neighbors(st)
    ost.build_neighbors(case["p"]["h"])
    ost.density(O.params(**case["p"]))
    S.step(st, np.zeros((7, 9)), p)  # density is the first pass of a step
    # the step rebuilt nothing (age 0 < interval) and computed rho at X0
    g = st.fields()
    r = ost.fields()
    assert np.array_equal(g["rho"], r["rho"])
    assert np.array_equal(g["pterm"], r["pterm"])
    assert np.array_equal(g["invrho"], r["invrho"])


@pytest.mark.parametrize("interval", [1, 4])
def test_forward_bit_exact_dambreak(interval):
    case = K.dambreak_case()
    g = run_gpu(case, 300, interval=interval, tape=False)
    r = run_oracle(case, 300, interval=interval, tape=False)
    assert g["flags"] == r["flags"]
    assert np.array_equal(g["X"], r["X"])
    assert np.array_equal(g["V"], r["V"])


@pytest.mark.parametrize("maker", [K.adjoint_case, K.gradcheck_case])
def test_adjoint_bit_exact(maker):
    case = maker()
    seeds = linear_seeds(case)
    g = run_gpu(case, case["nsteps"], seeds=seeds)
    r = run_oracle(case, case["nsteps"], seeds=seeds)
    assert np.array_equal(g["X"], r["X"]) and np.array_equal(g["V"], r["V"])
    assert np.array_equal(g["gX"], r["gX"])
    assert np.array_equal(g["gV"], r["gV"])
    assert K.relerr(g["gtheta"], r["gtheta"]) <= 1e-12
    assert np.max(np.abs(r["gtheta"])) > 0


def test_adjoint_dambreak_ke_interval4():
    case = K.dambreak_case(theta_seed=3)
    p = case["p"]
    seeds = lambda X, V: K.ke_seeds(X, V, p)[1:]  # noqa: E731
    n = 120
    g = run_gpu(case, n, seeds=seeds)
    r = run_oracle(case, n, seeds=seeds)
    assert np.array_equal(g["X"], r["X"]) and np.array_equal(g["V"], r["V"])
    assert np.array_equal(g["gX"], r["gX"])
    assert np.array_equal(g["gV"], r["gV"])
    assert K.relerr(g["gtheta"], r["gtheta"]) <= 1e-12


def test_checkpointed_tape_matches_full_tape():
    case = K.adjoint_case(seed=5)
    seeds = linear_seeds(case)
    n = 40
    full = run_gpu(case, n, seeds=seeds, interval=3)
    for c in (1, 2, 3, 6):
        ck = run_gpu(case, n, seeds=seeds, interval=3, snapshots=c)
        assert np.array_equal(ck["gX"], full["gX"]), c
        assert np.array_equal(ck["gV"], full["gV"]), c
        assert np.array_equal(ck["gtheta"], full["gtheta"]), c
        # backward recomputes everything the optimal schedule needs except the
        # advances of its first descent, which simulate! already made
        lib = S.load()
        pos, left, slots = 0, n, c
        while left > 1 and slots >= 2:
            m = lib.sph_plan_split(left, slots)
            pos, left, slots = pos + m, left - m, slots - 1
        assert ck["tape"].recomputed_steps() == lib.sph_plan_cost(n, c) - pos, c


def test_fp32_close_to_fp64_oracle():
    case = K.adjoint_case(seed=2)
    seeds = linear_seeds(case)
    g = run_gpu(case, case["nsteps"], dtype="f32", seeds=seeds)
    r = run_oracle(case, case["nsteps"], seeds=seeds)
    assert K.relerr(g["X"], r["X"]) <= 1e-5
    assert K.relerr(g["V"], r["V"]) <= 1e-5
    assert K.relerr(g["gX"], r["gX"]) <= 1e-5
    assert K.relerr(g["gV"], r["gV"]) <= 1e-5
    assert K.relerr(g["gtheta"], r["gtheta"]) <= 1e-5


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_repeat_runs_bit_identical(dtype):
    case = K.dambreak_case(theta_seed=4, jitter=0.05)
    p = case["p"]
    seeds = lambda X, V: K.ke_seeds(X, V, p)[1:]  # noqa: E731
    a = run_gpu(case, 80, dtype=dtype, seeds=seeds)
    b = run_gpu(case, 80, dtype=dtype, seeds=seeds)
    for k in ("X", "V", "gX", "gV", "gtheta"):
        assert np.array_equal(a[k], b[k]), k


def test_dense_cells_spill_and_overflow_match_oracle():
    # h = 3 dp: ~160 neighbours within the skin radius, rows of ~150 slots
    # (beyond the 64-slot masks) and maxnb = 64 truncation, like the reference.
    rng = np.random.default_rng(9)
    dp = 0.02
    p = dict(h=3 * dp, m=dp ** 2, rho0=1.0, c=10.0, mu=0.02, dt=1e-4, Lx=1.0, Ly=0.6,
             kw=1e4, ngx=9, ngy=7)
    X0 = K.lattice_block(14, 12, dp, dp, dp, 0.1 * dp, rng)
    case = dict(p=p, X0=X0, V0=0.05 * rng.standard_normal(X0.shape), theta=np.ones((7, 9)),
                cX=rng.standard_normal(X0.shape), cV=rng.standard_normal(X0.shape))
    seeds = linear_seeds(case)
    g = run_gpu(case, 10, seeds=seeds, interval=2)
    r = run_oracle(case, 10, seeds=seeds, interval=2)
    assert r["flags"] & 1 and g["flags"] == r["flags"]
    assert g["bflags"] == r["bflags"]
    assert np.array_equal(g["X"], r["X"]) and np.array_equal(g["V"], r["V"])
    assert np.array_equal(g["gX"], r["gX"]) and np.array_equal(g["gV"], r["gV"])
    assert K.relerr(g["gtheta"], r["gtheta"]) <= 1e-12


def test_particles_outside_tank_and_single_particle():
    case = K.adjoint_case(seed=3)
    case["X0"][:, :3] = [[-0.05, 1.07, 0.5], [0.5, -0.02, 1.1]]  # beyond the walls
    seeds = linear_seeds(case)
    g = run_gpu(case, 8, seeds=seeds)
    r = run_oracle(case, 8, seeds=seeds)
    assert np.array_equal(g["X"], r["X"]) and np.array_equal(g["gX"], r["gX"])
    one = dict(p=case["p"], X0=np.array([[0.5], [0.5]]), V0=np.array([[0.1], [0.0]]),
               theta=case["theta"], cX=np.ones((2, 1)), cV=np.ones((2, 1)))
    g = run_gpu(one, 5, seeds=linear_seeds(one))
    r = run_oracle(one, 5, seeds=linear_seeds(one))
    assert np.array_equal(g["X"], r["X"]) and np.array_equal(g["gV"], r["gV"])


def test_autotuned_block_sizes_do_not_change_results():
    case = K.adjoint_case(seed=7)
    seeds = linear_seeds(case)
    ref = run_gpu(case, 10, seeds=seeds)
    p = S.SPHParams(**case["p"])
    st = S.State(case["X0"], case["V0"], p, interval=1)
    import ctypes as C
    b6 = (C.c_int32 * 6)()
    lib = S.load()
    assert lib.sph_autotune(st.h, S.DesignField(case["theta"]).h, 2, b6) == 0
    assert all(b in (64, 128, 256) for b in b6)
    again = run_gpu(case, 10, seeds=seeds)
    for k in ("X", "V", "gX", "gV", "gtheta"):
        assert np.array_equal(ref[k], again[k]), k


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_block_sizes_set_directly_or_in_solve_do_not_change_results(dtype):
    # one thread per particle (the tuned kernels); every block size runs the
    # same per-particle code, so results are bit-identical in both precisions
    case = K.jittered_block_case(side=40, ntheta=16, seed=8)
    rng = np.random.default_rng(4)
    case["cX"] = rng.standard_normal(case["X0"].shape)
    case["cV"] = rng.standard_normal(case["X0"].shape)
    seeds = linear_seeds(case)
    p = S.SPHParams(**case["p"], dtype=dtype)
    st = S.State(case["X0"], case["V0"], p)
    S.set_group_lanes(1)
    try:
        outs = []
        for b in (64, 256, 128):
            st.set_block_sizes([b] * 6)
            assert st.block_sizes() == [b] * 6
            outs.append(run_gpu(case, 12, dtype=dtype, seeds=seeds))
        for o in outs[1:]:
            for k in ("X", "V", "gX", "gV", "gtheta"):
                assert np.array_equal(outs[0][k], o[k]), k
        with pytest.raises(S.ArgumentError):
            st.set_block_sizes([96] * 6)
        th = S.DesignField(case["theta"], dtype)
        tp = S.Tape(st.N, 8, p)
        ws = S.AdjointWorkspace(st.N, p)
        st0 = S.State(case["X0"], case["V0"], p)

        def solve():
            st.assign(st0)
            tp.reset()
            S.simulate(st, th, p, 8, tp)
            ws.objective(st, "ke_right")
            S.backward_seeded(ws, tp, th, p)

        solve()
        chosen = S.autotune_in_solve(st, solve)
        assert st.block_sizes() == chosen and all(b in (64, 128, 256) for b in chosen)
        again = run_gpu(case, 12, dtype=dtype, seeds=seeds)
        for k in ("X", "V", "gX", "gV", "gtheta"):
            assert np.array_equal(outs[0][k], again[k]), k
    finally:
        S.set_group_lanes(0)
        st.set_block_sizes([256] * 6)


def test_small_dambreak_full_horizon_bit_exact():
    """The reference's CPU case: 2072 particles, 5333 steps in FP64, KE of the
    right half. J, the final state and dJ/dX0, dJ/dV0 stay bit-identical to the
    oracle over the whole horizon (same summation order, no FMA); repeated
    runs give the same J (the reference's determinism claim)."""
    case = K.dambreak_case(theta_seed=21)
    case["theta"] = case["theta"] * 0.1
    p = case["p"]
    seeds = lambda X, V: K.ke_seeds(X, V, p)[1:]  # noqa: E731
    n = 5333
    g = run_gpu(case, n, seeds=seeds)
    r = run_oracle(case, n, seeds=seeds)
    assert g["flags"] == r["flags"] and g["bflags"] == r["bflags"]
    assert np.array_equal(g["X"], r["X"]) and np.array_equal(g["V"], r["V"])
    Jg = K.ke_seeds(g["X"], g["V"], p)[0]
    Jr = K.ke_seeds(r["X"], r["V"], p)[0]
    assert Jg == Jr and Jg > 0
    assert np.array_equal(g["gX"], r["gX"]) and np.array_equal(g["gV"], r["gV"])
    assert K.relerr(g["gtheta"], r["gtheta"]) <= 1e-12
    g2 = run_gpu(case, n, seeds=seeds)
    assert np.array_equal(g2["X"], g["X"]) and np.array_equal(g2["gtheta"], g["gtheta"])


def test_fp32_error_on_the_benchmark_workload_is_ieee_fp32_error():
    """The benchmark's jittered block (64 x 64 here) starts with a violent
    acoustic transient: by step 20 velocities reach ~3 m/s and the
    displacement flag is set, and rounding differences grow quickly (the
    oracle's own FP32 build differs from its FP64 build by ~2e-4 in V at
    step 20). The GPU's FP32 (fast reciprocal square root, multiply-add
    contraction) must stay within a small factor of that IEEE FP32 error."""
    case = K.jittered_block_case(64)
    p = case["p"]
    seeds = lambda X, V: K.ke_seeds(X, V, p)[1:]  # noqa: E731
    n = 20
    r64 = run_oracle(case, n, seeds=seeds)
    r32 = run_oracle(case, n, dtype="f32", seeds=seeds)
    g32 = run_gpu(case, n, dtype="f32", seeds=seeds)
    for k in ("X", "V", "gX", "gV", "gtheta"):
        ieee = K.relerr(r32[k], r64[k])
        assert K.relerr(g32[k], r64[k]) <= 4 * ieee + 1e-6, (k, ieee)


def test_standalone_celllist_and_neighborlist_match_oracle():
    # CellList(backend, N, p; cs = support(p)) + build!, NeighborList + build_neighbors!
    case = K.random_points_case()
    p = S.SPHParams(**case["p"])
    X = case["X0"]
    cl = S.CellList(X.shape[1], p)
    S.build(cl, X)
    o = O.Oracle("f64")
    ost = o.state(O.params(**case["p"]), X, case["V0"], skin=0.0)
    ost.build_cells()
    c = ost.cells()
    for k in ("counts", "starts", "order"):
        assert np.array_equal(getattr(cl, k), c[k]), k
    nl = S.NeighborList(X.shape[1], p, skin=0.2, layout="slot")
    cl2 = S.CellList(X.shape[1], p, cs=nl.rc)
    S.build_neighbors(nl, cl2, X)
    ost2 = o.state(O.params(**case["p"]), X, case["V0"], skin=0.2)
    ost2.build_neighbors(case["p"]["h"])
    oi, on = ost2.neighbors()
    assert nl.age == 0 and np.array_equal(nl.counts, on)
    for i in range(X.shape[1]):
        assert np.array_equal(nl.indices[i, : nl.counts[i]], oi[i, : on[i]]), i
    assert np.array_equal(cl2.order, ost2.cells()["order"])


@pytest.mark.parametrize("lanes", [1, 32])
def test_step_by_step_fields_match_oracle(lanes):
    """step! one step at a time, reading every step's density, pterm, 1/rho,
    acceleration a_rest and Brinkman alpha (keep_accel), against the oracle's
    arrays after each step (FP64, bit for bit)."""
    S.set_group_lanes(lanes)
    try:
        case = K.adjoint_case(seed=9)
        p, st, o, ost = _states(case, interval=2)
        st.keep_accel(True)
        th = S.DesignField(case["theta"])
        oth = o.theta(case["theta"])
        op = O.params(**case["p"])
        for n in range(6):
            S.step(st, th, p)
            o.step(ost, oth, op)
            g = st.fields(accel=True)
            r = ost.fields()
            for k in ("rho", "pterm", "invrho", "alpha"):
                assert np.array_equal(g[k], r[k]), (n, k)
            assert np.array_equal(np.asarray(g["a"]).T, r["a"]), n
            X, V = st.get()
            oX, oV = ost.get()
            assert np.array_equal(np.asarray(X).T, oX) and np.array_equal(np.asarray(V).T, oV)
    finally:
        S.set_group_lanes(0)
