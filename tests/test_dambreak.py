"""scripts/02_dambreak.jl restated (sphadjoint_gb300.dambreak): its set-up and
CSV frames on CPU; its frames against the oracle on the GPU (FP64, bit-exact:
the script's forward loop is step! only)."""
import csv

import numpy as np
import pytest

import oracle as O
from sphadjoint_gb300 import dambreak as D
from sphadjoint_gb300.topopt import write_frames_csv


def test_script_setup_matches_the_script():
    p, X0, V0, theta = D.script_setup()
    # 0.012:0.012:0.30 x 0.012:0.012:0.45 -> 25 x 37, x varying fastest
    assert X0.shape == (2, 925) and V0.shape == (2, 925) and not V0.any()
    assert np.allclose(X0[:, 0], [0.012, 0.012]) and np.allclose(X0[:, 1], [0.024, 0.012])
    assert np.isclose(X0[0].max(), 0.30) and np.isclose(X0[1].max(), 0.444)
    assert (p.ngx, p.ngy) == (33, 21) and theta.shape == (21, 33) and not theta.any()
    assert np.isclose(p.h, 1.3 * 0.012) and np.isclose(p.m, 0.012 ** 2)


def test_frames_csv_format(tmp_path):
    frames = [np.array([[0.1, 0.2], [0.3, 0.4]]), np.array([[0.5, 0.6], [0.7, 0.8]])]
    path = tmp_path / "dambreak_frames.csv"
    write_frames_csv(path, frames)
    rows = list(csv.reader(open(path)))
    assert rows[0] == ["frame", "id", "x", "y"]
    assert rows[1] == ["1", "1", "0.1", "0.3"] and rows[4] == ["2", "2", "0.6", "0.8"]
    assert len(rows) == 5


@pytest.mark.gpu
def test_frames_equal_the_oracle():
    frames, sps = D.run("f64", nsteps=120, save_every=50, log=None)
    assert len(frames) == 2 and sps > 0
    p, X0, V0, theta = D.script_setup()
    op = O.params(h=p.h, m=p.m, rho0=p.rho0, c=p.c, mu=p.mu, dt=p.dt, Lx=p.Lx, Ly=p.Ly,
                  kw=p.kw, ngx=p.ngx, ngy=p.ngy)
    o = O.Oracle("f64")
    st = o.state(op, X0, V0)
    th = o.theta(theta)
    for F in frames:
        o.simulate(st, th, op, 50, None)
        X, _ = st.get()
        assert np.array_equal(F, np.asarray(X).T if np.asarray(X).shape[0] != 2 else X)
