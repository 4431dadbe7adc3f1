"""Run one case through the CUDA library (C ABI) and through the CPU oracle."""
from __future__ import annotations

import warnings

import numpy as np

import oracle as O


def run_oracle(case, nsteps, dtype="f64", seeds=None, skin=0.2, interval=None, maxnb=64,
               tape=True, explicit_drag=False):
    p = case["p"]
    op = O.params(**p)
    o = O.Oracle(dtype)
    itv = interval if interval is not None else case.get("interval", 4)
    st = o.state(op, case["X0"], case["V0"], skin=skin, interval=itv, maxnb=maxnb)
    th = o.theta(case["theta"])
    N = st.N
    tp = o.tape(N, nsteps) if tape else None
    flags = o.simulate(st, th, op, nsteps, tp, explicit_drag=explicit_drag)
    X, V = st.get()
    out = dict(X=X.T, V=V.T, flags=flags, state=st)
    if seeds is not None:
        sX, sV = seeds(out["X"], out["V"])
        ws = o.workspace(N, op)
        bflags = o.backward(ws, tp, th, op, sX.T, sV.T, skin=skin, interval=itv, maxnb=maxnb,
                            explicit_drag=explicit_drag)
        gX, gV, gt = ws.get()
        out.update(gX=gX.T, gV=gV.T, gtheta=gt, bflags=bflags)
    return out


def run_gpu(case, nsteps, dtype="f64", seeds=None, skin=0.2, interval=None, maxnb=64,
            snapshots=0, tape=True, quiet=True):
    import sphadjoint_gb300 as S

    p = S.SPHParams(**case["p"], dtype=dtype)
    itv = interval if interval is not None else case.get("interval", 4)
    st = S.State(case["X0"], case["V0"], p, skin=skin, interval=itv, maxnb=maxnb)
    N = st.N
    th = S.DesignField(case["theta"], dtype)
    tp = S.Tape(N, nsteps, p, snapshots=snapshots) if tape else None
    with warnings.catch_warnings():
        warnings.simplefilter("ignore" if quiet else "default")
        S.simulate(st, th, p, nsteps, tp)
    X, V = st.get()
    out = dict(X=np.array(X, np.float64), V=np.array(V, np.float64), state=st, tape=tp,
               flags=st.last_flags)
    if seeds is not None:
        sX, sV = seeds(out["X"], out["V"])
        ws = S.AdjointWorkspace(N, p)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore" if quiet else "default")
            S.backward(ws, tp, th, p, sX, sV, skin=skin, interval=itv, maxnb=maxnb)
        out["bflags"] = ws.last_flags
        gX, gV, gt = ws.get()
        out.update(gX=np.array(gX, np.float64), gV=np.array(gV, np.float64),
                   gtheta=np.array(gt, np.float64), ws=ws)
    return out


def linear_seeds(case):
    cX, cV = case["cX"], case["cV"]
    return lambda X, V: (cX, cV)
