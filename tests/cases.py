"""Seeded inputs shared by the tests (shapes and parameters of the reference's
own tests and scripts; the Julia MersenneTwister streams cannot be reproduced
without Julia, so numpy generators with fixed seeds stand in for them)."""
from __future__ import annotations

import math

import numpy as np

P_FIELDS = ("h", "m", "rho0", "c", "mu", "dt", "Lx", "Ly", "kw", "ngx", "ngy")


def adjoint_case(seed=0):
    """test/runtests.jl:163-180: 5 x 5 jittered block, theta = 3 rand on 7 x 7, 12 steps."""
    rng = np.random.default_rng(seed)
    p = dict(h=0.10, m=0.010, rho0=1.0, c=8.0, mu=0.02, dt=1.0e-3, Lx=1.0, Ly=1.0,
             kw=2.0e4, ngx=7, ngy=7)
    nx, ny = 5, 5
    X0 = np.zeros((2, nx * ny))
    k = 0
    for jy in range(ny):
        for ix in range(nx):
            X0[0, k] = 0.20 + 0.06 * ix + 0.004 * rng.standard_normal()
            X0[1, k] = 0.20 + 0.06 * jy + 0.004 * rng.standard_normal()
            k += 1
    V0 = 0.05 * rng.standard_normal((2, nx * ny))
    theta = 3 * rng.random((7, 7))
    cX = rng.standard_normal((2, nx * ny))
    cV = rng.standard_normal((2, nx * ny))
    return dict(p=p, X0=X0, V0=V0, theta=theta, nsteps=12, cX=cX, cV=cV, interval=1)


def gradcheck_case(seed=0, theta_scale=3.0):
    """scripts/01_gradcheck.jl:26-66: 7 x 7 block, 25 steps, 9 x 9 theta."""
    rng = np.random.default_rng(seed)
    p = dict(h=0.10, m=0.010, rho0=1.0, c=8.0, mu=0.02, dt=1.0e-3, Lx=1.0, Ly=1.0,
             kw=2.0e4, ngx=9, ngy=9)
    n = 7
    X0 = np.zeros((2, n * n))
    k = 0
    for jy in range(n):
        for ix in range(n):
            X0[0, k] = 0.12 + 0.05 * ix + 0.004 * rng.standard_normal()
            X0[1, k] = 0.12 + 0.05 * jy + 0.004 * rng.standard_normal()
            k += 1
    V0 = 0.05 * rng.standard_normal((2, n * n))
    theta = theta_scale * rng.random((9, 9))
    cX = rng.standard_normal((2, n * n))
    cV = rng.standard_normal((2, n * n))
    return dict(p=p, X0=X0, V0=V0, theta=theta, nsteps=25, cX=cX, cV=cV, interval=1)


def random_points_case(seed=42, N=400):
    """test/runtests.jl:44-50: N random points in a 1 x 0.6 tank, h = 0.06."""
    rng = np.random.default_rng(seed)
    p = dict(h=0.06, m=0.004, rho0=1.0, c=10.0, mu=0.02, dt=1e-4, Lx=1.0, Ly=0.6,
             kw=1e4, ngx=9, ngy=7)
    X0 = np.vstack([rng.random(N) * p["Lx"], rng.random(N) * p["Ly"]])
    return dict(p=p, X0=X0, V0=np.zeros((2, N)), theta=np.zeros((7, 9)))


def lattice_block(nx, ny, dx, x0, y0, jitter=0.0, rng=None):
    xs = x0 + dx * np.arange(nx)
    ys = y0 + dx * np.arange(ny)
    X, Y = np.meshgrid(xs, ys)  # row-major over y, x fastest: like `for y in ys, x in xs`
    P = np.vstack([X.ravel(), Y.ravel()])
    if jitter:
        P = P + rng.uniform(-jitter, jitter, P.shape)
    return P


def reuse_case(seed=7):
    """test/runtests.jl:111-130: 12 x 10 jittered lattice at dp = 0.02, h = 1.3 dp."""
    rng = np.random.default_rng(seed)
    dp = 0.02
    p = dict(h=1.3 * dp, m=dp ** 2, rho0=1.0, c=10.0, mu=0.02, dt=1e-4, Lx=1.0, Ly=0.6,
             kw=1e4, ngx=9, ngy=7)
    nx, ny = 12, 10
    X0 = np.zeros((2, nx * ny))
    k = 0
    for jy in range(ny):
        for ix in range(nx):
            X0[0, k] = dp * (ix + 1) + 0.1 * dp * rng.standard_normal()
            X0[1, k] = dp * (jy + 1) + 0.1 * dp * rng.standard_normal()
            k += 1
    V0 = 0.05 * rng.standard_normal((2, nx * ny))
    return dict(p=p, X0=X0, V0=V0, theta=np.zeros((7, 9)))


def dambreak_params(dx=0.01, col_h=0.37, Lx=1.6, Ly=1.0, ngx=32, ngy=32, rho0=1000.0):
    """Small dam break: h = 1.3 dx, m = rho0 dx^2, c0 = 10 sqrt(2 g H),
    mu = 0.02, kw = 5e4, dt = 0.25 h / c0."""
    h = 1.3 * dx
    c0 = 10.0 * math.sqrt(2 * 9.81 * col_h)
    return dict(h=h, m=rho0 * dx * dx, rho0=rho0, c=c0, mu=0.02, dt=0.25 * h / c0, Lx=Lx,
                Ly=Ly, kw=5e4, ngx=ngx, ngy=ngy)


def dambreak_case(nx=56, ny=37, dx=0.01, theta_seed=None, jitter=0.0, seed=1):
    """56 x 37 = 2072 particles, dx = 0.01, origin (dx, dx), 1.6 x 1.0 tank,
    theta 32 x 32 (zeros unless theta_seed is given)."""
    rng = np.random.default_rng(seed)
    p = dambreak_params(dx=dx, col_h=ny * dx)
    X0 = lattice_block(nx, ny, dx, dx, dx, jitter * dx, rng)
    th = np.zeros((p["ngy"], p["ngx"]))
    if theta_seed is not None:
        th = 50.0 * np.random.default_rng(theta_seed).random(th.shape)
    return dict(p=p, X0=X0, V0=np.zeros_like(X0), theta=th)


def ke_seeds(X, V, p):
    """Kinetic energy of the right half of the tank and its terminal seeds."""
    right = X[0] > p["Lx"] / 2
    J = 0.5 * p["m"] * float(np.sum((V[0] ** 2 + V[1] ** 2)[right]))
    return J, np.zeros_like(X), np.where(right, p["m"] * V, 0.0)


def relerr(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def jittered_block_case(side=64, ntheta=32, seed=1):
    """The benchmark's single-instance workload at a smaller side: a side x side
    lattice, dx = 1e-3, jitter U(+-0.05 dx), h = 1.3 dx, rho0 = 1000,
    c0 = 10 sqrt(2 g H), dt = 0.25 h / c0, tank 2H x 1.25H, smoothed theta."""
    dx = 1e-3
    H = side * dx
    h = 1.3 * dx
    c0 = 10.0 * math.sqrt(2 * 9.81 * H)
    p = dict(h=h, m=1000.0 * dx * dx, rho0=1000.0, c=c0, mu=0.02, dt=0.25 * h / c0,
             Lx=2.0 * H, Ly=1.25 * H, kw=5e4, ngx=ntheta, ngy=ntheta)
    rng = np.random.default_rng(seed)
    xs = dx + dx * np.arange(side)
    X, Y = np.meshgrid(xs, xs)
    X0 = np.vstack([X.ravel(), Y.ravel()]) + rng.uniform(-0.05 * dx, 0.05 * dx, (2, side * side))
    t = np.random.default_rng(seed + 1).random((ntheta, ntheta))
    pad = np.pad(t, 2, mode="edge")
    theta = sum(pad[i:i + ntheta, j:j + ntheta] for i in range(5) for j in range(5)) / 25.0
    return dict(p=p, X0=X0, V0=np.zeros_like(X0), theta=theta)


def dense_block_case(side=2896, ntheta=512, seed=5):
    """The benchmark's dense stress workload: a side x side block compressed
    1.15x (spacing dx / 1.15, mass of the uncompressed lattice), theta with
    50% solid blobs (1000 vs 0)."""
    dx = 1e-3
    sp = dx / 1.15
    H = side * sp
    h = 1.3 * dx
    c0 = 10.0 * math.sqrt(2 * 9.81 * H)
    p = dict(h=h, m=1000.0 * dx * dx, rho0=1000.0, c=c0, mu=0.02, dt=0.25 * h / c0,
             Lx=2.0 * H, Ly=1.25 * H, kw=5e4, ngx=ntheta, ngy=ntheta)
    rng = np.random.default_rng(seed)
    xs = sp + sp * np.arange(side)
    X, Y = np.meshgrid(xs, xs)
    X0 = np.vstack([X.ravel(), Y.ravel()]) + rng.uniform(-0.05 * sp, 0.05 * sp, (2, side * side))
    f = rng.standard_normal((ntheta, ntheta))
    for _ in range(6):
        pad = np.pad(f, 2, mode="wrap")
        f = sum(pad[i:i + ntheta, j:j + ntheta] for i in range(5) for j in range(5)) / 25.0
    theta = np.where(f > np.median(f), 1000.0, 0.0)
    return dict(p=p, X0=X0, V0=np.zeros_like(X0), theta=theta)
