"""Design-side maths of the topology-optimisation caller (CPU only)."""
import csv

import numpy as np
import pytest

from sphadjoint_gb300 import topopt as T


def test_alpha_derivative_and_endpoints():
    rd = np.linspace(0.05, 0.95, 7)
    for qp in (0.01, 0.1, 10.0):
        h = 1e-6
        fd = (T.alpha_of(rd + h, 2e3, qp) - T.alpha_of(rd - h, 2e3, qp)) / (2 * h)
        np.testing.assert_allclose(T.dalpha_of(rd, 2e3, qp), fd, rtol=1e-6)
        assert T.alpha_of(1.0, 2e3, qp) == 0.0 and T.alpha_of(0.0, 2e3, qp) == pytest.approx(2e3)


def test_filter_is_normalised_and_adjoint_is_transpose():
    f = T.DensityFilter(9, 13, 2)
    rng = np.random.default_rng(0)
    x = 0.2 + 0.6 * rng.random((9, 13))  # interior: no clamp
    y = rng.standard_normal((9, 13))
    np.testing.assert_allclose(f.apply(np.ones((9, 13))), 1.0, rtol=1e-14)
    assert np.sum(f.apply(x) * y) == pytest.approx(np.sum(x * f.adjoint(y)), rel=1e-12)
    # weights (r+1) - dist, e.g. the centre row of an interior node
    row = f.rows[4 * 13 + 6]
    ws = {(jj, ii): w for jj, ii, w in row}
    assert ws[(4, 6)] / ws[(4, 7)] == pytest.approx(3.0 / 2.0)


def test_project_volume_lower_bound():
    rng = np.random.default_rng(1)
    x = rng.random((17, 33)) * 0.9
    y = T.project_volume(x, 0.75)
    assert y.mean() == pytest.approx(0.75, abs=1e-12) and y.min() >= 0 and y.max() <= 1
    z = T.project_volume(np.full((4, 4), 0.9), 0.75)
    assert np.all(z == 0.9)  # already feasible: unchanged


def test_csv_writers(tmp_path):
    T.write_frames_csv(tmp_path / "f.csv", [np.array([[0.1, 0.2], [0.3, 0.4]])])
    rows = list(csv.reader(open(tmp_path / "f.csv")))
    assert rows[0] == ["frame", "id", "x", "y"] and rows[2][:2] == ["1", "2"]
    T.write_history_csv(tmp_path / "h.csv", [-1.0, -2.0])
    assert list(csv.reader(open(tmp_path / "h.csv")))[2] == ["2", "-2.0"]
    assert T.mnd(np.array([0.0, 1.0])) == 0.0 and T.mnd(np.array([0.5])) == 100.0
