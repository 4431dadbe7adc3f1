"""Topology-optimisation caller of the forward + adjoint step.

Restates the design-side maths of the reference's scripts/03_optimize.jl
(the caller that runs simulate!/backward! twice per iteration) over this
library's API:

- Borrvall-Petersson interpolation alpha(rho) = alpha_max q (1 - rho) / (q + rho)
  and its derivative (03_optimize.jl:142-143)
- linear-weight density filter, its clamp and its adjoint (:151-191)
- volume projection by bisection on a lower bound (:200-219)
- objective_and_grad / objective_only on target_objective (:228-254)
- projected-gradient iterations with a backtracking line search (:299-341)
- the non-discreteness measure Mnd and the CSV outputs (:360-393)

Design variables stay in float64 whatever the particle precision, as in the
reference (`TW = Float64`). By default the design side runs on the device
(``DeviceDesign``, the library's sph_design_* kernels): the design, its
filtered field, theta and the gradient never leave the GPU between solves,
and the line search writes each candidate's theta straight into the solver's
field. The numpy functions below are the host restatement the device kernels
are checked against, and the path a request Server takes (it uploads theta per
request): the line search may run its candidate steps concurrently there and
still picks exactly the candidate the sequential search would (the first
improving one).
"""
from __future__ import annotations

import ctypes as C
import csv
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from . import api as S


def alpha_of(rd, alpha_max, qp):
    """alpha(rho) = alpha_max * qp * (1 - rho) / (qp + rho)."""
    return alpha_max * qp * (1 - rd) / (qp + rd)


def dalpha_of(rd, alpha_max, qp):
    """d alpha / d rho = -alpha_max * qp * (qp + 1) / (qp + rho)^2."""
    return -alpha_max * qp * (qp + 1) / (qp + rd) ** 2


class DensityFilter:
    """Linear-weight filter of radius r (grid points): weight (r + 1) - dist,
    normalised per node, neighbours in the reference's order (rows outer,
    columns inner)."""

    def __init__(self, ngy, ngx, r):
        self.shape = (ngy, ngx)
        self.rows = []
        for j in range(ngy):
            for i in range(ngx):
                lst, s = [], 0.0
                for jj in range(max(0, j - r), min(ngy - 1, j + r) + 1):
                    for ii in range(max(0, i - r), min(ngx - 1, i + r) + 1):
                        w = float(r + 1) - np.sqrt(float((ii - i) ** 2 + (jj - j) ** 2))
                        if w > 0:
                            lst.append((jj, ii, w))
                            s += w
                self.rows.append([(jj, ii, w / s) for jj, ii, w in lst])
        # the same weights as a dense-index sparse structure for the adjoint
        self._src = np.array([jj * ngx + ii for row in self.rows for jj, ii, _ in row])
        self._dst = np.array([k for k, row in enumerate(self.rows) for _ in row])
        self._w = np.array([w for row in self.rows for _, _, w in row])

    def apply(self, x):
        """apply_filter: weighted average in the listed order, clamped to [0, 1]."""
        x = np.asarray(x, dtype=np.float64)
        flat = x.ravel()
        ngx = self.shape[1]
        y = np.empty(len(self.rows))
        for k, row in enumerate(self.rows):
            acc = 0.0
            for jj, ii, w in row:
                acc += w * flat[jj * ngx + ii]
            y[k] = min(max(acc, 0.0), 1.0)
        return y.reshape(self.shape)

    def adjoint(self, g):
        """filter_adjoint: out[jj, ii] += w * g[j, i] over every (j, i) row."""
        g = np.asarray(g, dtype=np.float64).ravel()
        out = np.zeros(g.size)
        np.add.at(out, self._src, self._w * g[self._dst])
        return out.reshape(self.shape)


class DeviceDesign:
    """The design side of 03_optimize.jl on the device (sph_design_* in the C
    ABI): alpha(rho), the density filter and its adjoint, the volume
    projection and the line-search candidate, on a design kept on the GPU.
    Host arrays are numpy (ngy, ngx)."""

    FILTER, FILTER_ADJOINT, PROJECT, ALPHA, DALPHA = range(5)

    def __init__(self, ngy, ngx, r, alpha_max, qp, volfrac):
        self._L = L.load()
        self.shape = (ngy, ngx)
        h = C.c_void_p()
        L.check(self._L.sph_design_create(int(ngx), int(ngy), int(r), float(alpha_max),
                                          float(qp), float(volfrac), C.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self._L.sph_design_destroy(self.h)
            self.h = None

    def _in(self, x):
        a = np.asfortranarray(np.asarray(x, dtype=np.float64))
        if a.shape != self.shape:
            raise ValueError("design shape differs")
        return a

    def set(self, rd):
        a = self._in(rd)
        L.check(self._L.sph_design_set(self.h, a.ctypes.data_as(C.c_void_p)))

    def get(self):
        """(rd, filtered rd, gradient) from the device."""
        out = [np.empty(self.shape, order="F") for _ in range(3)]
        L.check(self._L.sph_design_get(self.h, *(o.ctypes.data_as(C.c_void_p) for o in out)))
        return tuple(np.ascontiguousarray(o) for o in out)

    def apply(self, op, x):
        a = self._in(x)
        out = np.empty(self.shape, order="F")
        L.check(self._L.sph_design_apply(self.h, int(op), a.ctypes.data_as(C.c_void_p),
                                         out.ctypes.data_as(C.c_void_p)))
        return np.ascontiguousarray(out)

    def to_theta(self, field):
        L.check(self._L.sph_design_to_theta(self.h, field.h))

    def gradient(self, ws):
        """grad = filter_adjoint(dJ/dtheta * dalpha(filter(rd))) from the
        workspace's last backward; returns max |grad|."""
        g = C.c_double()
        L.check(self._L.sph_design_gradient(self.h, ws.h, C.byref(g)))
        return g.value

    def candidate(self, step, field=None):
        L.check(self._L.sph_design_candidate(self.h, float(step),
                                             field.h if field is not None else None))

    def accept(self):
        L.check(self._L.sph_design_accept(self.h))


def project_volume(rd, volfrac):
    """Clamp to [0, 1]; if mean < volfrac, shift up by bisection (60 halvings)."""
    x = np.clip(rd, 0.0, 1.0)
    if x.mean() >= volfrac:
        return x
    lo, hi = 0.0, 1.0
    for _ in range(60):
        mid = (lo + hi) / 2
        if np.clip(x + mid, 0.0, 1.0).mean() < volfrac:
            lo = mid
        else:
            hi = mid
    return np.clip(x + (lo + hi) / 2, 0.0, 1.0)


def mnd(x):
    """Sigmund's non-discreteness measure, in percent."""
    x = np.asarray(x)
    return 100.0 * np.sum(4 * x * (1 - x)) / x.size


@dataclass
class Problem:
    """One topology-optimisation set-up (03_optimize.jl's globals)."""

    p: S.SPHParams
    X0: np.ndarray
    V0: np.ndarray
    nsteps: int
    target: tuple = (0.85, 0.10)
    sigma: float = 0.10
    alpha_max: float = 2.0e3
    qp: float = 0.1
    volfrac: float = 0.75
    filt_r: int = 2
    interval: int = 2
    snapshots: int = 0

    use_graphs: bool = True
    device: bool = True
    filt: DensityFilter = field(init=False)

    def __post_init__(self):
        self.filt = DensityFilter(self.p.ngy, self.p.ngx, self.filt_r)
        self.N = int(np.asarray(self.X0).size // 2)
        self._solver = None
        self._dev = None

    def dev(self) -> DeviceDesign:
        if self._dev is None:
            self._dev = DeviceDesign(self.p.ngy, self.p.ngx, self.filt_r, self.alpha_max,
                                     self.qp, self.volfrac)
        return self._dev

    def solver(self):
        if self._solver is None:
            self._solver = _Solver(self)
        return self._solver

    def theta_of(self, rd):
        return alpha_of(self.filt.apply(rd), self.alpha_max, self.qp)

    def _solve(self, theta, grad):
        """J (and dJ/dtheta) of one design: objects made once per problem, the
        two solve sequences captured as CUDA graphs on first use and replayed
        with the new design written into the same device field."""
        return self.solver().run(theta, grad)

    def objective_and_grad(self, rd):
        """J and dJ/drd: filter -> alpha -> simulate -> target_objective ->
        backward -> d alpha/d rho -> filter adjoint."""
        rdf = self.filt.apply(rd)
        theta = alpha_of(rdf, self.alpha_max, self.qp)
        J, gtheta = self._solve(theta, grad=True)
        grdf = gtheta * dalpha_of(rdf, self.alpha_max, self.qp)
        return J, self.filt.adjoint(grdf)

    def objective_only(self, rd):
        return self._solve(self.theta_of(rd), grad=False)[0]

    def objectives_concurrent(self, server, rds):
        """objective_only for several designs at once: forward-only requests on
        a Server, run concurrently; J is reduced on the device."""
        tickets = [server.submit(self.p, self.X0, self.V0, self.theta_of(rd), self.nsteps,
                                 objective="target",
                                 args=(self.target[0], self.target[1], self.sigma),
                                 interval=self.interval, adjoint=False) for rd in rds]
        return [t.wait()["J"] for t in tickets]


class _Solver:
    """Device objects of one Problem and its two captured solves: forward +
    target objective, and forward (taped) + target objective + seeded
    backward. Each starts from a pristine copy of the initial state, so a
    replay repeats the whole solve for whatever design the field holds."""

    def __init__(self, prob: Problem):
        self.prob = prob
        p, n = prob.p, prob.nsteps
        self.st0 = S.State(prob.X0, prob.V0, p, interval=prob.interval)
        self.st = S.State(prob.X0, prob.V0, p, interval=prob.interval)
        self.th = S.DesignField(np.zeros((p.ngy, p.ngx)), p.dtype)
        self.tp = S.Tape(prob.N, n, p, snapshots=prob.snapshots)
        self.ws = S.AdjointWorkspace(prob.N, p)
        self.args = (prob.target[0], prob.target[1], prob.sigma)
        self.graphs = {}

    def _forward(self, tape):
        pr = self.prob
        self.st.assign(self.st0)
        if tape is not None:
            S.reset(tape)
        S.simulate(self.st, self.th, pr.p, pr.nsteps, tape)
        self.ws.objective(self.st, "target", self.args)

    def _grad(self):
        self._forward(self.tp)
        S.backward_seeded(self.ws, self.tp, self.th, self.prob.p, interval=self.prob.interval)

    def run(self, theta, grad):
        """J (and dJ/dtheta on the host) for a host theta."""
        self.th.upload(theta)
        J = self.solve(grad)
        gt = np.asarray(self.ws.get()[2], np.float64) if grad else None
        return J, gt

    def solve(self, grad):
        """One solve of the design the device field holds; returns J (the
        gradient stays in the workspace)."""
        fn = self._grad if grad else (lambda: self._forward(None))
        if not self.prob.use_graphs:
            fn()
        elif grad in self.graphs:
            self.graphs[grad].launch()
            S.synchronize()
        else:
            fn()  # first run allocates; then record it
            self.graphs[grad] = S.capture(fn)
        return self.ws.objective_value()


def optimize(prob: Problem, rd0=None, maxit=40, step0=0.05, server=None, log=None):
    """Projected gradient descent with backtracking (03_optimize.jl:299-341):
    up to 6 candidates per iteration, step halved until J improves, grown by
    1.3 (capped at 0.3) after an accepted step. With a Server the 6 candidates
    are evaluated concurrently and the first improving one is taken."""
    rd = np.ones((prob.p.ngy, prob.p.ngx)) if rd0 is None else np.array(rd0, np.float64)
    if prob.device and server is None:
        return _optimize_device(prob, rd, maxit, step0, log)
    step = float(step0)
    J, g = prob.objective_and_grad(rd)
    hist = [J]
    for it in range(1, maxit + 1):
        gn = np.max(np.abs(g))
        if gn < 1e-30:
            break
        steps = [step * 0.5 ** k for k in range(6)]
        cands = [project_volume(rd - s * g / gn, prob.volfrac) for s in steps]
        if server is not None:
            Js = prob.objectives_concurrent(server, cands)
        else:
            Js = []
            for c in cands:
                Js.append(prob.objective_only(c))
                if Js[-1] < J:
                    break
        accepted = None
        for k, Jc in enumerate(Js):
            if Jc < J:
                accepted = k
                break
        if accepted is None:
            break
        rd, J = cands[accepted], Js[accepted]
        step = min(steps[accepted] * 1.3, 0.30)
        hist.append(J)
        _, g = prob.objective_and_grad(rd)
        if log:
            log(it, J, float(np.max(np.abs(g))), step, accepted + 1)
    return rd, hist


def _optimize_device(prob: Problem, rd, maxit, step0, log):
    """optimize() with the design on the device: theta of the design and of
    each candidate is written straight into the solver's field, the gradient
    is chained from the workspace's dJ/dtheta on the device; only J and
    max |grad| come back per solve. Same steps, same acceptance rule, same
    arithmetic as the host path (the filter, its adjoint and alpha(rho) are
    bit-identical; the projection's means are summed in another order)."""
    dd, sv = prob.dev(), prob.solver()
    dd.set(rd)
    step = float(step0)
    dd.to_theta(sv.th)
    J = sv.solve(True)
    gn = dd.gradient(sv.ws)
    hist = [J]
    for it in range(1, maxit + 1):
        if gn < 1e-30:
            break
        steps = [step * 0.5 ** k for k in range(6)]
        accepted = None
        for k, s_ in enumerate(steps):
            dd.candidate(s_, sv.th)
            Jc = sv.solve(False)
            if Jc < J:
                accepted, J = k, Jc
                break
        if accepted is None:
            break
        dd.accept()
        step = min(steps[accepted] * 1.3, 0.30)
        hist.append(J)
        dd.to_theta(sv.th)
        sv.solve(True)
        gn = dd.gradient(sv.ws)
        if log:
            log(it, J, gn, step, accepted + 1)
    return dd.get()[0], hist


# ---- outputs (the reference's CSV formats) ---------------------------------

def write_frames_csv(path, frames):
    """frame,id,x,y rows (02_dambreak.jl:82-88); frames: list of (2, N) arrays."""
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["frame", "id", "x", "y"])
        for fi, F in enumerate(frames, start=1):
            F = np.asarray(F)
            for i in range(F.shape[1]):
                w.writerow([fi, i + 1, repr(float(F[0, i])), repr(float(F[1, i]))])


def write_design_csv(path, prob: Problem, rd):
    """j,i,rho_design,rho_filtered,alpha rows (03_optimize.jl:381-388), 1-based."""
    rdf = prob.filt.apply(rd)
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["j", "i", "rho_design", "rho_filtered", "alpha"])
        for j in range(prob.p.ngy):
            for i in range(prob.p.ngx):
                w.writerow([j + 1, i + 1, repr(float(rd[j, i])), repr(float(rdf[j, i])),
                            repr(float(alpha_of(rdf[j, i], prob.alpha_max, prob.qp)))])


def write_history_csv(path, hist):
    """iter,J rows (03_optimize.jl:389-393)."""
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["iter", "J"])
        for k, J in enumerate(hist, start=1):
            w.writerow([k, repr(float(J))])


def reference_problem(dtype="f64", alpha_max=2.0e3, qp=0.1, t_end=0.8, dp=0.020, dt=2.0e-4):
    """03_optimize.jl's CPU set-up: a 12 x 20 water column (dp = 0.02),
    1.0 x 0.5 tank, 33 x 17 design grid, target (0.85, 0.10), sigma 0.1,
    t_end = 0.8 s, neighbour list rebuilt every 2 steps. The script's GPU
    set-up is dp = 0.008, dt = 1.5e-4 in float32 (a 30 x 50 column, 5333
    steps): reference_problem("f32", dp=0.008, dt=1.5e-4)."""
    p = S.SPHParams(h=1.3 * dp, m=dp * dp, rho0=1.0, c=15.0, mu=0.05, dt=dt, Lx=1.0, Ly=0.5,
                    kw=5.0e4, ngx=33, ngy=17, dtype=dtype)
    xs = np.arange(1, int(round(0.24 / dp)) + 1) * dp
    ys = np.arange(1, int(round(0.40 / dp)) + 1) * dp
    X, Y = np.meshgrid(xs, ys)
    X0 = np.vstack([X.ravel(), Y.ravel()])
    return Problem(p=p, X0=X0, V0=np.zeros_like(X0), nsteps=int(round(t_end / dt)),
                   alpha_max=alpha_max, qp=qp)


def main(argv=None):
    """Command-line run of the optimisation (03_optimize.jl's script body):
    python -m sphadjoint_gb300.topopt --out DIR [--maxit 40] [--alpha-max 2e3]
    [--qp 0.1] [--volfrac 0.75] [--step0 0.05] [--dtype f64] [--workers 6]."""
    import argparse
    import os
    import time

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--out", default="topopt_out")
    ap.add_argument("--maxit", type=int, default=40)
    ap.add_argument("--alpha-max", type=float, default=2.0e3)
    ap.add_argument("--qp", type=float, default=0.1)
    ap.add_argument("--volfrac", type=float, default=0.75)
    ap.add_argument("--step0", type=float, default=0.05)
    ap.add_argument("--t-end", type=float, default=0.8)
    ap.add_argument("--dtype", choices=("f64", "f32"), default="f64")
    ap.add_argument("--dp", type=float, default=0.020, help="0.008 with --dt 1.5e-4: the GPU set-up")
    ap.add_argument("--dt", type=float, default=2.0e-4)
    ap.add_argument("--workers", type=int, default=0,
                    help="evaluate the line-search candidates on a Server with this many workers")
    a = ap.parse_args(argv)
    prob = reference_problem(dtype=a.dtype, alpha_max=a.alpha_max, qp=a.qp, t_end=a.t_end,
                             dp=a.dp, dt=a.dt)
    prob.volfrac = a.volfrac
    os.makedirs(a.out, exist_ok=True)
    print(f"N = {prob.N} particles, {prob.nsteps} steps, {prob.filt.shape[0] * prob.filt.shape[1]}"
          " design variables")

    def log(it, J, gmax, step, ntry):
        print(f"{it:4d}  {J:+.6e}  {gmax:.3e}  {step:.4f}  {ntry}")

    t0 = time.time()
    if a.workers > 0:
        from .serve import Server
        with Server(workers=a.workers, hbm_budget_bytes=16 << 30, dtype=a.dtype) as srv:
            rd, hist = optimize(prob, maxit=a.maxit, step0=a.step0, server=srv, log=log)
    else:
        rd, hist = optimize(prob, maxit=a.maxit, step0=a.step0, log=log)
    print(f"{len(hist) - 1} iterations in {time.time() - t0:.1f} s, J {hist[0]:+.6e} -> "
          f"{hist[-1]:+.6e}, Mnd {mnd(prob.filt.apply(rd)):.1f} %")
    write_design_csv(os.path.join(a.out, "design_field.csv"), prob, rd)
    write_history_csv(os.path.join(a.out, "objective_history.csv"), hist)
    return rd, hist


if __name__ == "__main__":
    main()
