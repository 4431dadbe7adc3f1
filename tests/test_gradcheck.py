"""scripts/01_gradcheck.jl restated (sphadjoint_gb300.gradcheck): set-up on
CPU; on the GPU the adjoint gradients at the script's entries against central
differences, at the script's THETA_SCALE and at one where the implicit drag
factor D = 1/(1 + dt alpha) is far from 1."""
import numpy as np
import pytest

from sphadjoint_gb300 import gradcheck as G


def test_script_setup():
    p, X0, V0, theta0, cX, cV, nsteps = G.script_setup()
    assert X0.shape == (2, 49) and V0.shape == (2, 49) and theta0.shape == (9, 9)
    assert nsteps == 25 and (p.ngx, p.ngy) == (9, 9)
    # 7 x 7 block from (0.12, 0.12), spacing 0.05, ix innermost, jitter 0.004
    assert abs(X0[0, 1] - X0[0, 0] - 0.05) < 0.03 and abs(X0[1, 7] - X0[1, 0] - 0.05) < 0.03
    assert theta0.min() >= 0 and theta0.max() < 3
    assert all(1 <= a <= 2 and 1 <= b <= 49 for a, b in G.X0_ENTRIES + G.V0_ENTRIES)


@pytest.mark.gpu
@pytest.mark.parametrize("scale", [3.0, 300.0])
def test_adjoint_matches_central_differences(scale):
    res = G.check(theta_scale=scale, log=None)
    assert len(res) == 8
    for name, adj, fd, rel in res:
        assert rel <= 1e-5 or abs(adj - fd) <= 1e-9, (name, adj, fd, rel)
