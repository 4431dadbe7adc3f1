"""Gradient check of the hand-written adjoint against central differences:
the body of scripts/01_gradcheck.jl over this library.

The script's set-up (01_gradcheck.jl:24-77): 49 particles on a 7 x 7 block
(spacing 0.05 from (0.12, 0.12), jitter 0.004 N(0, 1)), velocities
0.05 N(0, 1), h = 0.10, m = 0.010, rho0 = 1, c = 8, mu = 0.02, dt = 1e-3,
1 x 1 tank, kw = 2e4, a 9 x 9 design field THETA_SCALE * U[0, 1)
(THETA_SCALE = 3), 25 steps, the neighbour list rebuilt every step, and the
objective J = sum(cX .* X_T) + sum(cV .* V_T) with cX, cV ~ N(0, 1). One
backward! gives dJ/dtheta, dJ/dX0, dJ/dV0; each is compared at the script's
entries with a central difference of step 1e-6 (theta: 1e-6 max(1,
THETA_SCALE)), 01_gradcheck.jl:97-140. The random numbers come from a
seeded numpy generator (Julia's MersenneTwister stream is not reproducible
here), so the values differ from the script's while the check is the same.

    python -m sphadjoint_gb300.gradcheck [--theta-scale 3] [--dtype f64]
"""
from __future__ import annotations

import argparse

import numpy as np

from . import api as S

# the script's checked entries, 1-based (row, column) as in CartesianIndex
THETA_ENTRIES = [(1, 1), (4, 5), (6, 3)]
X0_ENTRIES = [(1, 1), (2, 18), (1, 41)]
V0_ENTRIES = [(1, 5), (2, 30)]


def script_setup(theta_scale=3.0, dtype="f64", seed=0):
    """(params, X0, V0, theta0, cX, cV, nsteps) of 01_gradcheck.jl."""
    p = S.SPHParams(h=0.10, m=0.010, rho0=1.0, c=8.0, mu=0.02, dt=1.0e-3, Lx=1.0, Ly=1.0,
                    kw=2.0e4, ngx=9, ngy=9, dtype=dtype)
    rng = np.random.default_rng(seed)
    nx = ny = 7
    X0 = np.zeros((2, nx * ny))
    k = 0
    for jy in range(ny):          # `for jy in 0:ny-1, ix in 0:nx-1`: ix innermost
        for ix in range(nx):
            X0[0, k] = 0.12 + 0.05 * ix + 0.004 * rng.standard_normal()
            X0[1, k] = 0.12 + 0.05 * jy + 0.004 * rng.standard_normal()
            k += 1
    V0 = 0.05 * rng.standard_normal(X0.shape)
    theta0 = theta_scale * rng.random((p.ngy, p.ngx))
    cX = rng.standard_normal(X0.shape)
    cV = rng.standard_normal(X0.shape)
    return p, X0, V0, theta0, cX, cV, 25


def check(theta_scale=3.0, dtype="f64", hfd=1e-6, log=print):
    """Adjoint vs central differences at the script's entries. Returns a list
    of (name, adjoint, fd, relative error)."""
    p, X0, V0, theta0, cX, cV, nsteps = script_setup(theta_scale, dtype)
    N = X0.shape[1]

    def forward(X, V, theta, tape=None):
        st = S.State(X, V, p, interval=1)
        S.simulate(st, S.DesignField(theta, dtype), p, nsteps, tape)
        XT, VT = st.get()
        return float(np.sum(np.asarray(XT, np.float64) * cX) +
                     np.sum(np.asarray(VT, np.float64) * cV))

    tape = S.Tape(N, nsteps, p)
    th = S.DesignField(theta0, dtype)
    st = S.State(X0, V0, p, interval=1)
    S.simulate(st, th, p, nsteps, tape)
    ws = S.AdjointWorkspace(N, p)
    S.backward(ws, tape, th, p, cX, cV, interval=1)
    gX, gV, gth = (np.asarray(a, np.float64) for a in ws.get())

    def fd(f, x, idx, h):
        xp, xm = x.copy(), x.copy()
        xp[idx] += h
        xm[idx] -= h
        return (f(xp) - f(xm)) / (2 * h)

    out = []
    ht = hfd * max(1.0, theta_scale)
    rows = [("theta", e, gth, lambda t: forward(X0, V0, t), theta0, ht) for e in THETA_ENTRIES]
    rows += [("X0", e, gX, lambda x: forward(x, V0, theta0), X0, hfd) for e in X0_ENTRIES]
    rows += [("V0", e, gV, lambda v: forward(X0, v, theta0), V0, hfd) for e in V0_ENTRIES]
    for name, (a, b), g, f, x, h in rows:
        idx = (a - 1, b - 1)
        d = fd(f, x, idx, h)
        rel = abs(g[idx] - d) / max(abs(d), 1e-30)
        out.append((f"{name}[{a},{b}]", float(g[idx]), d, rel))
        if log:
            log(f"  {name}[{a},{b}]: adjoint {g[idx]: .9e}   FD {d: .9e}   rel {rel:.2e}")
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--theta-scale", type=float, default=3.0)
    ap.add_argument("--dtype", default="f64", choices=["f64", "f32"])
    a = ap.parse_args(argv)
    print(f"N = 49 particles, 25 steps, 81 design variables, THETA_SCALE = {a.theta_scale}")
    res = check(a.theta_scale, a.dtype)
    print(f"largest relative error {max(r[3] for r in res):.2e}")


if __name__ == "__main__":
    main()
