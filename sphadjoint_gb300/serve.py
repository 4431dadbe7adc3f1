"""Python side of the request servers (sph_server_* in the C ABI).

A topology-optimisation caller (the reference's scripts/03_optimize.jl runs
one simulate!/backward! pair per candidate design) submits forward + adjoint
solves as its line search produces them. The packed server (``packed=True``)
advances every request in flight one time step per tick and runs each pass of
a tick as one launch over all of them, admitting requests FIFO while their
device memory fits in the HBM budget (and fewer than ``max_inflight`` run).
The stream server (``packed=False``) runs up to ``workers`` whole solves
concurrently, each on its own CUDA stream.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .api import SPHParams, _ptr, _xy

OBJECTIVES = {"ke_right": 0, "target": 1}


class Ticket:
    """One submitted request: keeps its host inputs alive and owns its outputs."""

    def __init__(self, server, p, X0, V0, theta, nsteps, snapshots, objective, args, skin,
                 interval, maxnb, adjoint=True):
        self.server = server
        N = int(np.asarray(X0).size // 2)
        self.N, self.p, self.nsteps = N, p, int(nsteps)
        self._x = _xy(X0, N, p.np)
        self._v = _xy(V0, N, p.np)
        self._th = np.asfortranarray(np.asarray(theta, dtype=p.np))
        self.adjoint = bool(adjoint)
        if self.adjoint:
            self.gX = np.empty((N, 2), p.np)
            self.gV = np.empty((N, 2), p.np)
            self.gt = np.empty((p.ngx, p.ngy), p.np)
        else:  # forward only: J alone, no tape and no reverse sweep
            self.gX = self.gV = self.gt = None
        r = L.sph_request()
        r.p = p.c_struct()
        r.N = N
        r.X0, r.V0, r.theta = _ptr(self._x), _ptr(self._v), _ptr(self._th)
        r.nsteps = self.nsteps
        r.snapshots = int(snapshots)
        r.objective = OBJECTIVES[objective]
        for k, a in enumerate(args if args is not None else (0.0, 0.0, 1.0)):
            r.obj_args[k] = float(a)
        r.skin, r.interval, r.maxnb = float(skin), int(interval), int(maxnb)
        r.gX, r.gV, r.gtheta = _ptr(self.gX), _ptr(self.gV), _ptr(self.gt)
        self.req = r
        self.bytes = int(server._L.sph_request_bytes(C.byref(r), p.code))
        t = C.c_int64()
        L.check(server._L.sph_server_submit(server.h, C.byref(r), C.byref(t)))
        self.ticket = t.value
        self.result = None

    def wait(self):
        if self.result is None:
            J, lat, f = C.c_double(), C.c_double(), C.c_uint32()
            L.check(self.server._L.sph_server_wait(self.server.h, self.ticket, C.byref(J),
                                                   C.byref(lat), C.byref(f)))
            self.result = dict(J=J.value, latency_ms=lat.value, flags=f.value)
            if self.adjoint:
                self.result.update(gX=self.gX.T, gV=self.gV.T, gtheta=self.gt.T)
        return self.result

    def done(self) -> bool:
        d = C.c_int32()
        L.check(self.server._L.sph_server_poll(self.server.h, self.ticket, C.byref(d)))
        return bool(d.value)


class Server:
    def __init__(self, workers: int = 4, hbm_budget_bytes: int = 64 << 30, dtype: str = "f32",
                 packed: bool = False, max_inflight: int = 256):
        self._L = L.load()
        self.dtype = dtype
        self.packed = bool(packed)
        h = C.c_void_p()
        code = {"f64": L.SPH_F64, "f32": L.SPH_F32}[dtype]
        if self.packed:
            L.check(self._L.sph_server_create_packed(int(max_inflight), int(hbm_budget_bytes),
                                                     code, C.byref(h)))
        else:
            L.check(self._L.sph_server_create(int(workers), int(hbm_budget_bytes), code,
                                              C.byref(h)))
        self.h = h
        self.tickets = []

    def submit(self, p: SPHParams, X0, V0, theta, nsteps, snapshots=0, objective="ke_right",
               args=None, skin=0.2, interval=4, maxnb=64, adjoint=True) -> Ticket:
        """Queue one solve. adjoint=False: forward only, the result holds J alone.
        snapshots: 0 full tape, c > 0 checkpoints, "auto" (or -1) chosen by the
        server from its budget."""
        if snapshots == "auto":
            snapshots = -1
        if p.dtype != self.dtype:
            raise ValueError("request dtype differs from the server's")
        t = Ticket(self, p, X0, V0, theta, nsteps, snapshots, objective, args, skin, interval,
                   maxnb, adjoint)
        self.tickets.append(t)
        return t

    def stats(self):
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        n, pb, pi = C.c_int64(), C.c_int64(), C.c_int32()
        L.check(self._L.sph_server_stats(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(n),
                                         C.byref(pb), C.byref(pi)))
        return dict(p50_ms=a.value, p99_ms=b.value, particle_steps_per_s=c.value,
                    completed=n.value, peak_bytes=pb.value, peak_inflight=pi.value)

    def reset_stats(self):
        L.check(self._L.sph_server_reset_stats(self.h))

    def close(self):
        if getattr(self, "h", None):
            for t in self.tickets:
                try:
                    t.wait()
                except L.SPHError:
                    pass
            self._L.sph_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()
