"""Alternative kernel forms against the default ones on the same inputs.

The cell-tile density (a warp stages its 32 particles' neighbouring cell rows
in shared memory, every lane scans all staged candidates) and the two-
candidate mask walk (packed f32x2 arithmetic) keep exactly the mask walk's
interaction set and summation order, so they must agree with it to FP32
rounding (multiply-add contraction may differ between kernels); on states
where tiles span two cell rows or hold spilled particles, those warps take the
mask walk."""
import numpy as np
import pytest

import cases as K
from runners import linear_seeds, run_gpu

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")


@pytest.fixture
def one_thread():
    S.set_group_lanes(1)
    yield
    S.set_group_lanes(0)
    S.set_density_form("pairs")


def dense_case():
    # rows beyond 64 slots (spilled particles) and cells of ~25 particles
    rng = np.random.default_rng(9)
    dp = 0.02
    p = dict(h=3 * dp, m=dp ** 2, rho0=1.0, c=10.0, mu=0.02, dt=1e-4, Lx=1.0, Ly=0.6,
             kw=1e4, ngx=9, ngy=7)
    X0 = K.lattice_block(14, 12, dp, dp, dp, 0.1 * dp, rng)
    return dict(p=p, X0=X0, V0=0.05 * rng.standard_normal(X0.shape), theta=np.ones((7, 9)))


CASES = {
    "jittered-128": (lambda: K.jittered_block_case(128, ntheta=32), 20),
    "dambreak": (lambda: K.dambreak_case(theta_seed=4, jitter=0.05), 40),
    "dense": (dense_case, 8),
}


@pytest.mark.parametrize("form", ["tiles", "pairs"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_density_forms_match_the_mask_walk(one_thread, name, form):
    make, n = CASES[name]
    case = make()
    rng = np.random.default_rng(3)
    case["cX"] = rng.standard_normal(case["X0"].shape)
    case["cV"] = rng.standard_normal(case["X0"].shape)
    out = {}
    for f in ("mask", form):
        S.set_density_form(f)
        assert S.density_form() == f
        out[f] = run_gpu(case, n, dtype="f32", seeds=linear_seeds(case))
    for k in ("X", "V", "gX", "gV", "gtheta"):
        if form == "pairs":  # the same operations in the same order: same bits
            assert np.array_equal(out[form][k], out["mask"][k]), k
        else:
            assert K.relerr(out[form][k], out["mask"][k]) <= 1e-5, k


@pytest.mark.parametrize("dtype,lanes", [("f64", 0), ("f32", 0), ("f32", 1)])
def test_launch_overlap_does_not_change_results(dtype, lanes):
    """Programmatic dependent launch only moves when a kernel is scheduled;
    every kernel waits for its predecessor's results, so the results are the
    same bits with and without it (small states: lane-group kernels, or one
    thread per particle; the cell list is rebuilt every other step)."""
    case = K.dambreak_case(theta_seed=4, jitter=0.05)
    rng = np.random.default_rng(5)
    case["cX"] = rng.standard_normal(case["X0"].shape)
    case["cV"] = rng.standard_normal(case["X0"].shape)
    S.set_group_lanes(lanes)
    out = {}
    try:
        for on in (False, True):
            S.set_launch_overlap(on)
            out[on] = run_gpu(case, 30, dtype=dtype, seeds=linear_seeds(case), interval=2)
    finally:
        S.set_launch_overlap(True)
        S.set_group_lanes(0)
    for k in ("X", "V", "gX", "gV", "gtheta"):
        assert np.array_equal(out[True][k], out[False][k]), k


@pytest.mark.parametrize("dtype,lanes,snapshots", [("f64", 0, 0), ("f64", 0, 4), ("f32", 1, 3),
                                                   ("f32", 0, 0)])
def test_step_graphs_do_not_change_results(dtype, lanes, snapshots):
    """simulate and backward replay their steps in recorded groups (CUDA
    graphs); the groups hold the same launches in the same order as direct
    launches, so results are the same bits and the launch count is the same,
    for group sizes that do and do not divide the rebuild interval, with a
    full tape and with checkpoints (restores, recomputed steps and snapshot
    copies inside the groups)."""
    case = K.dambreak_case(theta_seed=4, jitter=0.05)
    rng = np.random.default_rng(6)
    case["cX"] = rng.standard_normal(case["X0"].shape)
    case["cV"] = rng.standard_normal(case["X0"].shape)
    S.set_group_lanes(lanes)
    out, launches = {}, {}
    try:
        for steps in (0, 1, 3, 32):
            S.set_step_graphs(steps)
            assert S.step_graphs() == steps
            n0, (r0, _) = S.launch_count(), S.step_graph_counts()
            out[steps] = run_gpu(case, 37, dtype=dtype, seeds=linear_seeds(case), interval=2,
                                 snapshots=snapshots)
            launches[steps] = S.launch_count() - n0
            replays = S.step_graph_counts()[0] - r0
            # forward steps and at least as many reverse steps, in groups
            assert (replays == 0) == (steps == 0), (steps, replays)
            if steps:
                assert replays >= 2 * -(-37 // steps), (steps, replays)
    finally:
        S.set_step_graphs(32)
        S.set_group_lanes(0)
    for steps in (1, 3, 32):
        assert launches[steps] == launches[0], steps
        for k in ("X", "V", "gX", "gV", "gtheta"):
            assert np.array_equal(out[steps][k], out[0][k]), (steps, k)
    with pytest.raises(Exception):
        S.set_step_graphs(-1)


def test_step_graphs_fall_back_on_the_legacy_default_stream():
    """The legacy default stream cannot be recorded: a library stream set to it
    runs simulate and backward launch by launch, with the same results."""
    from sphadjoint_gb300 import _lib as LB
    import ctypes as C
    case = K.dambreak_case(theta_seed=4, jitter=0.05)
    rng = np.random.default_rng(7)
    case["cX"] = rng.standard_normal(case["X0"].shape)
    case["cV"] = rng.standard_normal(case["X0"].shape)
    L = S.load()
    ref = run_gpu(case, 20, dtype="f64", seeds=linear_seeds(case), snapshots=3)
    LB.check(L.sph_set_stream(C.c_void_p(1)))  # cudaStreamLegacy
    try:
        r0 = S.step_graph_counts()[0]
        out = run_gpu(case, 20, dtype="f64", seeds=linear_seeds(case), snapshots=3)
        assert S.step_graph_counts()[0] == r0
    finally:
        LB.check(L.sph_set_stream(None))
    for k in ("X", "V", "gX", "gV", "gtheta"):
        assert np.array_equal(out[k], ref[k]), k
