"""Lane groups per particle (16 or 32 lanes) against one thread per particle.

Each setting adds a particle's pair terms in the same slot order with the same
operations, so FP64 results are bit-identical across settings and to the
oracle: neighbour lists (including spilled rows and maxnb truncation), the
forward state and every gradient. FP32 with lane groups stays within the FP32
tolerance of the FP64 oracle."""
import numpy as np
import pytest

import cases as K
from runners import linear_seeds, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")


@pytest.fixture
def lanes():
    def set_(n):
        S.set_group_lanes(n)
        assert S.group_lanes() == n
    yield set_
    S.set_group_lanes(0)


def dense_case():
    # rows beyond 64 slots (spilled particles) and maxnb truncation
    rng = np.random.default_rng(9)
    dp = 0.02
    p = dict(h=3 * dp, m=dp ** 2, rho0=1.0, c=10.0, mu=0.02, dt=1e-4, Lx=1.0, Ly=0.6,
             kw=1e4, ngx=9, ngy=7)
    X0 = K.lattice_block(14, 12, dp, dp, dp, 0.1 * dp, rng)
    return dict(p=p, X0=X0, V0=0.05 * rng.standard_normal(X0.shape), theta=np.ones((7, 9)),
                cX=rng.standard_normal(X0.shape), cV=rng.standard_normal(X0.shape))


# name: (case, steps, rebuild interval, maxnb). "dense": spilled particles,
# whose groups list their rows in shared memory, and maxnb truncation;
# "dense-maxnb96": a row limit above the shared list, where spilled particles
# take the serial walk on one lane.
CASES = {
    "adjoint": (lambda: K.adjoint_case(seed=5), 12, 4, 64),
    "dambreak": (lambda: K.dambreak_case(theta_seed=4, jitter=0.05), 40, 4, 64),
    "dense": (dense_case, 8, 2, 64),
    "dense-maxnb96": (dense_case, 6, 2, 96),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_bit_identical_across_lane_settings(lanes, name):
    make, n, interval, maxnb = CASES[name]
    case = make()
    if "cX" not in case:
        rng = np.random.default_rng(3)
        case["cX"] = rng.standard_normal(case["X0"].shape)
        case["cV"] = rng.standard_normal(case["X0"].shape)
    seeds = linear_seeds(case)
    out = {}
    for g in (1, 16, 32):
        lanes(g)
        out[g] = run_gpu(case, n, seeds=seeds, interval=interval, maxnb=maxnb)
        nb, cnt = out[g]["state"].neighbors()
        out[g]["nb"], out[g]["cnt"] = nb, cnt
    r = run_oracle(case, n, seeds=seeds, interval=interval, maxnb=maxnb)
    for g in (16, 32):
        for k in ("X", "V", "gX", "gV", "gtheta", "nb", "cnt"):
            assert np.array_equal(out[g][k], out[1][k]), (g, k)
        assert out[g]["flags"] == out[1]["flags"] and out[g]["bflags"] == out[1]["bflags"]
    assert np.array_equal(out[32]["X"], r["X"]) and np.array_equal(out[32]["gX"], r["gX"])
    assert np.array_equal(out[32]["gV"], r["gV"])
    assert K.relerr(out[32]["gtheta"], r["gtheta"]) <= 1e-12
    assert out[32]["flags"] == r["flags"]


def test_fp32_lane_groups_within_tolerance(lanes):
    case = K.adjoint_case(seed=2)
    seeds = linear_seeds(case)
    r = run_oracle(case, case["nsteps"], seeds=seeds)
    for g in (16, 32):
        lanes(g)
        o = run_gpu(case, case["nsteps"], dtype="f32", seeds=seeds)
        for k in ("X", "V", "gX", "gV", "gtheta"):
            assert K.relerr(o[k], r[k]) <= 1e-5, (g, k)


def test_fp32_lane_groups_with_spilled_rows_within_tolerance(lanes):
    # FP32 lane groups on the dense case: spilled particles' rows listed in
    # shared memory, maxnb truncation; against the FP64 oracle and the
    # one-thread FP32 form
    case = dense_case()
    seeds = linear_seeds(case)
    r = run_oracle(case, 6, seeds=seeds, interval=2)
    lanes(1)
    one = run_gpu(case, 6, dtype="f32", seeds=seeds, interval=2)
    for g in (16, 32):
        lanes(g)
        o = run_gpu(case, 6, dtype="f32", seeds=seeds, interval=2)
        assert o["flags"] == r["flags"]
        for k in ("X", "V", "gX", "gV", "gtheta"):
            assert K.relerr(o[k], r[k]) <= 1e-5, (g, k)
            assert K.relerr(o[k], one[k]) <= 1e-5, (g, k)


def test_lane_setting_rejects_other_values():
    with pytest.raises(S.ArgumentError):
        S.set_group_lanes(8)
    assert S.group_lanes() == 0
