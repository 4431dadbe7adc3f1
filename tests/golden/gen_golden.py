"""Generate golden vectors from the reference's own Python verification tools.

The reference package ships two NumPy/PyTorch harnesses next to its Julia
source: ``tools/verify_adjoint.py`` (all-pairs forward, PyTorch autograd
ground truth) and ``tools/verify_gather.py`` (the gather-form adjoint written
line by line like src/adjoint.jl). Both use the older *explicit* Brinkman drag
(``a -= alpha * v``); the Julia kernels use the implicit form. The oracle has
an explicit-drag switch so that these vectors pin its pair formulas, wall,
design-field interpolation and time-loop adjoint.

This script imports those tools from a checkout of the reference, whose path
is the first argument or the ``SPHADJOINT_REF`` environment variable (one of
them is required), and writes
``golden_verify.npz`` beside itself. It needs numpy and torch; the tests only
read the committed ``.npz``.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_tools():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPHADJOINT_REF")
    if not ref:
        sys.exit("usage: gen_golden.py <reference checkout> (or set SPHADJOINT_REF)")
    sys.path.insert(0, os.path.join(ref, "tools"))
    import verify_adjoint as va  # noqa: E402
    import verify_gather as vg  # noqa: E402
    return va, vg


def _case(va, vg, name, X0, V0, theta, cX, cV, nsteps, P):
    import torch

    XT, VT, tape = vg.simulate_gather(X0, V0, theta, P, nsteps)
    gX, gV, gth = vg.backward_gather(tape, theta, P, cX, cV)
    tX0 = torch.tensor(X0, dtype=torch.float64, requires_grad=True)
    tV0 = torch.tensor(V0, dtype=torch.float64, requires_grad=True)
    tth = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    J = va.torch_simulate(tX0, tV0, tth, P, nsteps,
                          torch.tensor(cX, dtype=torch.float64),
                          torch.tensor(cV, dtype=torch.float64))
    J.backward()
    out = {
        "X0": X0, "V0": V0, "theta": theta, "cX": cX, "cV": cV,
        "nsteps": np.int64(nsteps),
        "XT": XT, "VT": VT, "J": np.float64(np.sum(XT * cX) + np.sum(VT * cV)),
        "J_torch": np.float64(J.item()),
        "gX": gX, "gV": gV, "gtheta": gth,
        "gX_ad": tX0.grad.numpy().copy(), "gV_ad": tV0.grad.numpy().copy(),
        "gtheta_ad": tth.grad.numpy().copy(),
        "params": np.array([P.h, P.m, P.rho0, P.c, P.mu, P.g[0], P.g[1], P.dt,
                            P.Lx, P.Ly, P.kw, P.ngx, P.ngy], dtype=np.float64),
    }
    return {f"{name}/{k}": v for k, v in out.items()}


def main():
    va, vg = _import_tools()
    data = {}

    # case "gather": the harness's own main() inputs (tools/verify_gather.py:154-170)
    rng = np.random.default_rng(0)
    P = va.Params()
    nx, ny = 7, 7
    xs = np.linspace(0.12, 0.12 + (nx - 1) * 0.05, nx)
    ys = np.linspace(0.12, 0.12 + (ny - 1) * 0.05, ny)
    XX, YY = np.meshgrid(xs, ys)
    X0 = np.stack([XX.ravel(), YY.ravel()], axis=1) + 0.004 * rng.standard_normal((nx * ny, 2))
    V0 = 0.05 * rng.standard_normal(X0.shape)
    N = X0.shape[0]
    theta = 3.0 * rng.random((P.ngy, P.ngx))
    cX = rng.standard_normal((N, 2))
    cV = rng.standard_normal((N, 2))
    data.update(_case(va, vg, "gather", X0, V0, theta, cX, cV, 25, P))

    # case "wall": a block pushed into the lower-left corner so the relu^2
    # wall penalty and its derivative are active; larger theta (drag).
    rng = np.random.default_rng(11)
    P2 = va.Params()
    P2.ngx, P2.ngy = 7, 5
    nx, ny = 6, 6
    xs = np.linspace(0.01, 0.01 + (nx - 1) * 0.05, nx)
    ys = np.linspace(0.01, 0.01 + (ny - 1) * 0.05, ny)
    XX, YY = np.meshgrid(xs, ys)
    X0 = np.stack([XX.ravel(), YY.ravel()], axis=1) + 0.003 * rng.standard_normal((nx * ny, 2))
    V0 = np.array([-0.6, -0.4]) + 0.05 * rng.standard_normal((nx * ny, 2))
    N = X0.shape[0]
    theta = 20.0 * rng.random((P2.ngy, P2.ngx))
    cX = rng.standard_normal((N, 2))
    cV = rng.standard_normal((N, 2))
    data.update(_case(va, vg, "wall", X0, V0, theta, cX, cV, 20, P2))

    path = os.path.join(HERE, "golden_verify.npz")
    np.savez_compressed(path, **data)
    for case in ("gather", "wall"):
        def rel(a, b):
            return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30)
        print(case, "gather vs autograd:",
              f"X0 {rel(data[case + '/gX'], data[case + '/gX_ad']):.2e}",
              f"V0 {rel(data[case + '/gV'], data[case + '/gV_ad']):.2e}",
              f"theta {rel(data[case + '/gtheta'], data[case + '/gtheta_ad']):.2e}")
    print("wrote", path)


if __name__ == "__main__":
    main()
