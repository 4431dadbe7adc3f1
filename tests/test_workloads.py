"""The benchmark's seeded workloads on CPU: sizes and distributions of each
configuration (the single instance, the small dam break, the dense case,
the 64 batched instances, the served request stream)."""
import math
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_single_instance():
    p, X0, V0, theta, cfg = bench.workload(n_side=64, nsteps=10, snapshots=4, ntheta=32)
    assert X0.shape == (2, 64 * 64) and not V0.any() and theta.shape == (32, 32)
    dx = 1e-3
    lattice = dx + dx * np.arange(64)
    jitter = X0[0].reshape(64, 64) - lattice[None, :]
    assert np.abs(jitter).max() <= 0.05 * dx + 1e-15          # U(+-0.05 dx)
    assert 0.0 <= theta.min() and theta.max() <= 1.0          # smoothed U[0, 1]
    assert math.isclose(p["h"], 1.3 * dx) and math.isclose(p["dt"], 0.25 * p["h"] / p["c"])


def test_small_dambreak():
    p, X0, V0, theta, cfg = bench.small_workload()
    assert X0.shape == (2, 56 * 37) and not theta.any() and theta.shape == (32, 32)
    assert math.isclose(X0[0].min(), 0.01) and math.isclose(X0[1].min(), 0.01)
    assert (p["Lx"], p["Ly"]) == (1.6, 1.0) and math.isclose(p["m"], 0.1)


def test_dense_case_is_compressed():
    p, X0, V0, theta, cfg = bench.dense_workload(side=128, ntheta=64)
    spacing = np.diff(np.unique(np.round(X0[1].reshape(128, 128)[:, 0], 9))).mean()
    assert math.isclose(spacing, 1e-3 / 1.15, rel_tol=0.05)
    solid = (theta > 0).mean()
    assert 0.4 <= solid <= 0.6                                  # ~50% solid blobs


def test_batched_instances():
    inst, cfg = bench.batched_workload(B=64, nsteps=2000)
    ns = [x[1].shape[1] for x in inst]
    assert len(inst) == 64 and cfg["particles"] == sum(ns)
    assert 900 <= min(ns) and max(ns) <= 66000                 # log-uniform in [1k, 64k]
    for p, X0, V0, theta in inst:
        assert theta.shape == (64, 64)


def test_served_stream():
    reqs = bench.served_requests(40, rate=100.0)
    t = np.array([r["t"] for r in reqs])
    assert np.all(np.diff(t) > 0)                               # Poisson arrivals
    assert 0.1 < t[-1] < 1.0                                    # mean gap 1/rate
    ns = [r["X0"].shape[1] for r in reqs]
    steps = [r["steps"] for r in reqs]
    assert 1900 <= min(ns) and max(ns) <= 201000
    assert 500 <= min(steps) and max(steps) <= 5000
    for r in reqs:
        assert r["theta"].shape == (128, 128) and r["snapshots"] == 32
        assert 0.0 <= r["theta"].min() and r["theta"].max() <= 1.0
