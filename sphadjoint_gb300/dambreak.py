"""Forward-only dam break: the body of scripts/02_dambreak.jl over this
library.

The script's set-up (02_dambreak.jl:30-60): a water column 0.30 wide and
0.45 high on a square lattice of spacing dp = 0.012 starting at (dp, dp)
(25 x 37 = 925 particles, x varying fastest), in a 1.0 x 0.6 tank;
h = 1.3 dp, m = dp^2, rho0 = 1, c = 20, mu = 0.05, dt = 1.5e-4, kw = 5e4, a
33 x 21 design grid of zeros (no obstacle), the State's default neighbour
list (skin 0.2, interval 4, maxnb 64). Its loop (02_dambreak.jl:66-79) calls
step! 6000 times and keeps the positions every 50 steps; the frames are
written as dambreak_frames.csv with rows frame,id,x,y (1-based,
02_dambreak.jl:82-88). The script's steps/second line is printed too.

    python -m sphadjoint_gb300.dambreak [--out DIR] [--dtype f64|f32]
        [--nsteps 6000] [--save-every 50]
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np

from . import api as S
from .topopt import write_frames_csv


def script_setup(dtype="f64", dp=0.012, col_w=0.30, col_h=0.45):
    """(params, X0, V0, theta) of 02_dambreak.jl."""
    p = S.SPHParams(h=1.3 * dp, m=dp * dp, rho0=1.0, c=20.0, mu=0.05, dt=1.5e-4, Lx=1.0,
                    Ly=0.6, kw=5.0e4, ngx=33, ngy=21, dtype=dtype)
    # dp:dp:col_w and dp:dp:col_h; `for y in ys, x in xs` puts x innermost
    xs = np.arange(1, int(np.floor(col_w / dp + 1e-9)) + 1) * dp
    ys = np.arange(1, int(np.floor(col_h / dp + 1e-9)) + 1) * dp
    X, Y = np.meshgrid(xs, ys)
    X0 = np.vstack([X.ravel(), Y.ravel()])
    return p, X0, np.zeros_like(X0), np.zeros((p.ngy, p.ngx))


def run(dtype="f64", nsteps=6000, save_every=50, log=print):
    """The script's time loop: returns the saved frames ((2, N) arrays) and
    the steps per second."""
    p, X0, V0, theta = script_setup(dtype)
    st = S.State(X0, V0, p)
    th = S.DesignField(theta, dtype)
    if log:
        log(f"N = {st.N} particles")
    frames = []
    t0 = time.perf_counter()
    done = 0
    while done < nsteps:
        # step! save_every times, then keep the positions (the script's
        # n % save_every == 0 test)
        n = min(save_every - done % save_every, nsteps - done)
        S.simulate(st, th, p, n)
        done += n
        if done % save_every == 0:
            frames.append(np.array(st.get()[0]))
    S.synchronize()
    sec = time.perf_counter() - t0
    if log:
        log(f"{nsteps} steps / {sec:.2f} s  ({nsteps / sec:.1f} steps/s)")
    return frames, nsteps / sec


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--out", default=".")
    ap.add_argument("--dtype", default="f64", choices=["f64", "f32"])
    ap.add_argument("--nsteps", type=int, default=6000)
    ap.add_argument("--save-every", type=int, default=50)
    a = ap.parse_args(argv)
    frames, _ = run(a.dtype, a.nsteps, a.save_every)
    os.makedirs(a.out, exist_ok=True)
    path = os.path.join(a.out, "dambreak_frames.csv")
    write_frames_csv(path, frames)
    print(f"wrote {path} ({len(frames)} frames)")


if __name__ == "__main__":
    main()
