"""Python mirror of SPHAdjoint's public API over the C ABI.

Names follow the reference module's exports (src/SPHAdjoint.jl:39-40):
``SPHParams, State, Tape, AdjointWorkspace, simulate, step, build,
build_neighbors, backward, target_objective, reset`` (Julia's ``simulate!``
is ``simulate`` here, etc.). Arrays use the reference's shapes: positions,
velocities, seeds and gradients are (2, N); theta is (ngy, ngx). All compute
runs in the CUDA library; nothing here falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

_DT = {"f64": (L.SPH_F64, np.float64), "f32": (L.SPH_F32, np.float32)}


@dataclass
class SPHParams:
    """SPHParams{T} (src/params.jl:14-28); ``dtype`` is T ("f64" or "f32").

    ``eos`` and ``visc`` select model variants that the reference does not
    have (it uses the linear EOS and Morris viscosity): ``eos="tait"`` with
    integer exponent ``gamma``, ``visc="artificial"`` (Monaghan) with
    coefficient ``alpha``; ``mu`` is then unused."""

    h: float
    m: float
    rho0: float
    c: float
    mu: float
    dt: float
    Lx: float
    Ly: float
    kw: float
    ngx: int
    ngy: int
    gx: float = 0.0
    gy: float = -9.81
    dtype: str = "f64"
    eos: str = "linear"
    gamma: int = 7
    visc: str = "morris"
    alpha: float = 0.0

    _EOS = {"linear": 0, "tait": 1}
    _VISC = {"morris": 0, "artificial": 1}

    def c_struct(self) -> L.sph_params:
        p = L.sph_params()
        for k in ("h", "m", "rho0", "c", "mu", "gx", "gy", "dt", "Lx", "Ly", "kw"):
            setattr(p, k, float(getattr(self, k)))
        p.ngx, p.ngy = int(self.ngx), int(self.ngy)
        try:
            p.eos = self._EOS[self.eos] if isinstance(self.eos, str) else int(self.eos)
            p.visc = self._VISC[self.visc] if isinstance(self.visc, str) else int(self.visc)
        except KeyError as e:
            raise L.ArgumentError(1, f"unknown model variant {e}") from None
        p.gamma, p.alpha = int(self.gamma), float(self.alpha)
        return p

    @property
    def code(self) -> int:
        return _DT[self.dtype][0]

    @property
    def np(self):
        return _DT[self.dtype][1]

    # src/params.jl:30-32
    def support(self) -> float:
        return 2 * self.h

    def dxg(self) -> float:
        return self.Lx / (self.ngx - 1)

    def dyg(self) -> float:
        return self.Ly / (self.ngy - 1)


def _check_layout(layout):
    """NeighborList's index layout (src/neighbors.jl:178-184): :auto, :slot or
    :particle. The library keeps its own per-particle row masks in every case
    (results do not depend on the layout); sph_get_neighbors returns rows in
    the particle-major form."""
    if str(layout).lstrip(":") not in ("auto", "slot", "particle"):
        raise L.ArgumentError(1, "layout must be :slot, :particle or :auto")


def _xy(a, N, dt):
    """(2, N) or (N, 2) -> contiguous (N, 2) of T (the interleaved layout)."""
    a = np.asarray(a)
    if a.shape == (2, N):
        a = a.T
    return np.ascontiguousarray(a.reshape(N, 2), dtype=dt)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class DesignField:
    """Device copy of the design field theta, (ngy, ngx) column-major T."""

    def __init__(self, theta, dtype: str = "f64"):
        self._L = L.load()
        code, npdt = _DT[dtype]
        th = np.asarray(theta, dtype=np.float64)
        self.shape = th.shape
        self.dtype = dtype
        ngy, ngx = th.shape
        h = C.c_void_p()
        cm = np.asfortranarray(th.astype(npdt))
        L.check(self._L.sph_field_create(ngx, ngy, code, _ptr(cm), C.byref(h)))
        self.h = h

    def upload(self, theta):
        cm = np.asfortranarray(np.asarray(theta, dtype=_DT[self.dtype][1]))
        if cm.shape != self.shape:
            raise ValueError("theta shape changed")
        L.check(self._L.sph_field_upload(self.h, _ptr(cm)))

    def __del__(self):
        if getattr(self, "h", None):
            self._L.sph_field_destroy(self.h)
            self.h = None


def _field(theta, p: SPHParams) -> DesignField:
    if isinstance(theta, DesignField):
        return theta
    return DesignField(theta, p.dtype)


class State:
    """State(backend, X0, V0, p; skin, interval, maxnb) (src/driver.jl:24-36)."""

    def __init__(self, X0, V0, p: SPHParams, skin=0.2, interval=4, maxnb=64, layout="auto"):
        _check_layout(layout)
        self._L = L.load()
        self.p = p
        self.N = N = int(np.asarray(X0).size // 2)
        self.maxnb = int(maxnb)
        self.skin, self.interval = float(skin), int(interval)
        x = _xy(X0, N, p.np)
        v = _xy(V0, N, p.np)
        h = C.c_void_p()
        L.check(self._L.sph_state_create(C.byref(p.c_struct()), N, _ptr(x), _ptr(v), p.code,
                                         float(skin), int(interval), int(maxnb), C.byref(h)))
        self.h = h
        self.last_flags = 0

    def __del__(self):
        if getattr(self, "h", None):
            self._L.sph_state_destroy(self.h)
            self.h = None

    # Array(st.X) / Array(st.V): (2, N)
    def get(self):
        X = np.empty((self.N, 2), self.p.np)
        V = np.empty((self.N, 2), self.p.np)
        L.check(self._L.sph_state_get(self.h, _ptr(X), _ptr(V)))
        return X.T, V.T

    @property
    def X(self):
        return self.get()[0]

    @property
    def V(self):
        return self.get()[1]

    def set(self, X=None, V=None):
        x = _xy(X, self.N, self.p.np) if X is not None else None
        v = _xy(V, self.N, self.p.np) if V is not None else None
        L.check(self._L.sph_state_set(self.h, _ptr(x), _ptr(v)))

    def keep_accel(self, on=True):
        L.check(self._L.sph_state_keep_accel(self.h, int(bool(on))))

    def fields(self, accel=False):
        N, dt = self.N, self.p.np
        rho, pt, ir = (np.empty(N, dt) for _ in range(3))
        a = np.empty((N, 2), dt) if accel else None
        al = np.empty(N, dt) if accel else None
        L.check(self._L.sph_state_fields(self.h, _ptr(rho), _ptr(pt), _ptr(ir), _ptr(a), _ptr(al)))
        out = dict(rho=rho, pterm=pt, invrho=ir)
        if accel:
            out.update(a=a.T, alpha=al)
        return out

    def grid(self):
        nx, ny, cs, age = C.c_int32(), C.c_int32(), C.c_double(), C.c_int64()
        L.check(self._L.sph_state_grid(self.h, C.byref(nx), C.byref(ny), C.byref(cs), C.byref(age)))
        return nx.value, ny.value, cs.value, age.value

    def celllist(self):
        """CellList counts, starts (0-based), order (1-based ids)."""
        nx, ny, _, _ = self.grid()
        counts = np.empty(nx * ny, np.int32)
        starts = np.empty(nx * ny, np.int32)
        order = np.empty(max(self.N, 1), np.int32)[: self.N]
        L.check(self._L.sph_get_celllist(self.h, _ptr(counts), _ptr(starts), _ptr(order)))
        return dict(counts=counts, starts=starts, order=order)

    def neighbors(self):
        """NeighborList rows (particle-major, 1-based ids) and counts."""
        idx = np.zeros((self.N, self.maxnb), np.int32)
        nbc = np.zeros(self.N, np.int32)
        L.check(self._L.sph_get_neighbors(self.h, _ptr(idx), _ptr(nbc)))
        return idx, nbc

    def take_flags(self) -> int:
        f = C.c_uint32()
        L.check(self._L.sph_state_take_flags(self.h, C.byref(f)))
        return f.value

    def set_block_sizes(self, blocks) -> None:
        """Threads per block of the six tuned kernels (neighbour-list build,
        density, accel, drag, pass 1, pass 2), each 64, 128 or 256, for every
        object of this precision and kind (no counterpart in the reference)."""
        b = (C.c_int32 * 6)(*[int(x) for x in blocks])
        L.check(self._L.sph_set_block_sizes(self.h, b))

    def block_sizes(self):
        b = (C.c_int32 * 6)()
        L.check(self._L.sph_get_block_sizes(self.h, b))
        return list(b)

    def assign(self, src: "State") -> "State":
        """Make this state a device copy of src (same configuration): particles,
        order, neighbour structure and the neighbour-list age."""
        L.check(self._L.sph_state_assign(self.h, src.h))
        return self


def _warn_flags(f: int, maxnb: int):
    # check_neighbor_flags (src/neighbors.jl:282-290)
    if f & L.FLAG_NL_OVERFLOW:
        warnings.warn(f"neighbour-list row overflowed (maxnb={maxnb}); neighbours are missing. "
                      "Increase maxnb.", RuntimeWarning, stacklevel=3)
    if f & L.FLAG_DISPLACEMENT:
        warnings.warn("neighbour-list rebuild interval too long (displacement exceeded skin*h); "
                      "neighbours may be missing. Lower interval or raise skin.",
                      RuntimeWarning, stacklevel=3)
    if f & L.FLAG_NONFINITE:
        warnings.warn("non-finite positions or velocities were produced", RuntimeWarning,
                      stacklevel=3)


class Tape:
    """Tape(backend, N, nsteps, p) (src/driver.jl:62-65).

    ``snapshots=0`` keeps every step's (X, V) like the reference. ``snapshots=c``
    keeps c device snapshots and recomputes the rest during ``backward``
    (binomial checkpointing), for horizons whose full history would not fit.
    ``snapshots="auto"`` picks the full tape when it fits in ``budget_bytes``
    (default: 90% of the device's free memory) and otherwise as many snapshots
    as fit; ``self.snapshots`` holds the choice.
    """

    def __init__(self, N: int, nsteps: int, p: SPHParams, snapshots=0, budget_bytes=None,
                 skin=0.2):
        self._L = L.load()
        self.N, self.cap, self.p = int(N), int(nsteps), p
        h = C.c_void_p()
        if snapshots == "auto":
            budget = -1 if budget_bytes is None else int(budget_bytes)
            L.check(self._L.sph_tape_create_auto(C.byref(p.c_struct()), self.N, self.cap, p.code,
                                                 float(skin), budget, C.byref(h)))
            c = C.c_int32()
            L.check(self._L.sph_tape_snapshots(h, C.byref(c)))
            snapshots = c.value
        elif snapshots:
            L.check(self._L.sph_tape_create_checkpointed(self.N, self.cap, int(snapshots), p.code,
                                                         C.byref(h)))
        else:
            L.check(self._L.sph_tape_create(self.N, self.cap, p.code, C.byref(h)))
        self.snapshots = int(snapshots)
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self._L.sph_tape_destroy(self.h)
            self.h = None

    def __len__(self):
        n = C.c_int64()
        L.check(self._L.sph_tape_length(self.h, C.byref(n)))
        return n.value

    def capacity(self):
        return self.cap

    def reset(self):
        L.check(self._L.sph_tape_reset(self.h))
        return self

    def get(self, n):
        X = np.empty((self.N, 2), self.p.np)
        V = np.empty((self.N, 2), self.p.np)
        L.check(self._L.sph_tape_get(self.h, int(n), _ptr(X), _ptr(V)))
        return X.T, V.T

    def recomputed_steps(self):
        n = C.c_int64()
        L.check(self._L.sph_tape_recomputed_steps(self.h, C.byref(n)))
        return n.value


def tape_plan(N: int, nsteps: int, p: SPHParams, budget_bytes: int, skin=0.2):
    """(snapshots, device bytes) of the tape ``Tape(..., snapshots="auto")``
    would create under ``budget_bytes``: 0 snapshots = the full tape."""
    lib = L.load()
    c, b = C.c_int32(), C.c_int64()
    L.check(lib.sph_tape_plan(C.byref(p.c_struct()), int(N), int(nsteps), p.code, float(skin),
                              int(budget_bytes), C.byref(c), C.byref(b)))
    return c.value, b.value


class AdjointWorkspace:
    """AdjointWorkspace(backend, N, p) (src/driver.jl:128-133)."""

    def __init__(self, N: int, p: SPHParams):
        self._L = L.load()
        self.N, self.p = int(N), p
        h = C.c_void_p()
        L.check(self._L.sph_workspace_create(self.N, C.byref(p.c_struct()), p.code, C.byref(h)))
        self.h = h
        self.last_flags = 0

    def __del__(self):
        if getattr(self, "h", None):
            self._L.sph_workspace_destroy(self.h)
            self.h = None

    def get(self):
        gX = np.empty((self.N, 2), self.p.np)
        gV = np.empty((self.N, 2), self.p.np)
        gt = np.empty((self.p.ngx, self.p.ngy), self.p.np)  # column-major (ngy, ngx)
        L.check(self._L.sph_workspace_get(self.h, _ptr(gX), _ptr(gV), _ptr(gt)))
        return gX.T, gV.T, gt.T

    def objective(self, st: "State", kind="ke_right", args=None, p: SPHParams | None = None):
        """J of the state's current positions/velocities on the device; the
        terminal seeds stay on the device for backward_seeded. kind:
        "ke_right" (kinetic energy of the right half) or "target"
        (target_objective with args = (xc, yc, sigma)). While capturing, the
        returned J is 0: read it after a replay with objective_value()."""
        kinds = {"ke_right": 0, "target": 1}
        a = (C.c_double * 3)(*args) if args is not None else None
        J = C.c_double()
        pc = (p or self.p).c_struct()
        L.check(self._L.sph_objective(self.h, st.h, kinds[kind], a, C.byref(pc), C.byref(J)))
        return J.value

    def objective_value(self) -> float:
        J = C.c_double()
        L.check(self._L.sph_workspace_objective_value(self.h, C.byref(J)))
        return J.value

    def take_flags(self) -> int:
        """Neighbour-list flags of the last backward's reverse sweep."""
        f = C.c_uint32()
        L.check(self._L.sph_workspace_take_flags(self.h, C.byref(f)))
        return f.value

    @property
    def gX(self):
        return self.get()[0]

    @property
    def gV(self):
        return self.get()[1]

    @property
    def gtheta(self):
        return self.get()[2]


class Batch:
    """B independent instances packed into one State (no counterpart in the
    reference, which runs one State per call). Each instance keeps its own
    SPHParams, particle count, cell grid and design field; step/simulate/
    backward run every kernel once for all of them, and each instance's
    results equal those of the same instance run alone.

    ``X0s``/``V0s`` are lists of (2, N_b) arrays; ``params`` a list of
    SPHParams (one dtype for all).
    """

    def __init__(self, X0s, V0s, params, skin=0.2, interval=4, maxnb=64):
        self._L = L.load()
        self.params = list(params)
        p0 = self.params[0]
        if any(p.dtype != p0.dtype for p in self.params):
            raise ValueError("all instances of a batch share one dtype")
        self.p = p0
        self.B = len(self.params)
        self.sizes = [int(np.asarray(x).size // 2) for x in X0s]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        self.N = int(self.offsets[-1])
        self.maxnb = int(maxnb)
        X = np.concatenate([_xy(x, n, p0.np) for x, n in zip(X0s, self.sizes)]) if self.N else \
            np.zeros((0, 2), p0.np)
        V = np.concatenate([_xy(v, n, p0.np) for v, n in zip(V0s, self.sizes)]) if self.N else \
            np.zeros((0, 2), p0.np)
        cps = (L.sph_params * self.B)(*[q.c_struct() for q in self.params])
        ns = (C.c_int64 * self.B)(*self.sizes)
        h = C.c_void_p()
        L.check(self._L.sph_batch_create(self.B, cps, ns, _ptr(np.ascontiguousarray(X)),
                                         _ptr(np.ascontiguousarray(V)), p0.code, float(skin),
                                         int(interval), int(maxnb), C.byref(h)))
        self.h = h
        self.last_flags = 0

    def __del__(self):
        if getattr(self, "h", None):
            self._L.sph_state_destroy(self.h)
            self.h = None

    def get(self):
        """[(X_b, V_b)] with (2, N_b) arrays."""
        X = np.empty((self.N, 2), self.p.np)
        V = np.empty((self.N, 2), self.p.np)
        L.check(self._L.sph_state_get(self.h, _ptr(X), _ptr(V)))
        o = self.offsets
        return [(X[o[b]:o[b + 1]].T, V[o[b]:o[b + 1]].T) for b in range(self.B)]

    def take_flags(self):
        f = (C.c_uint32 * self.B)()
        L.check(self._L.sph_batch_take_flags(self.h, f))
        return list(f)

    def set_block_sizes(self, blocks) -> None:
        """Threads per block of the six tuned kernels (neighbour-list build,
        density, accel, drag, pass 1, pass 2), each 64, 128 or 256, for every
        object of this precision and kind (no counterpart in the reference)."""
        b = (C.c_int32 * 6)(*[int(x) for x in blocks])
        L.check(self._L.sph_set_block_sizes(self.h, b))

    def block_sizes(self):
        b = (C.c_int32 * 6)()
        L.check(self._L.sph_get_block_sizes(self.h, b))
        return list(b)


class BatchField(DesignField):
    """The design fields of a batch, one (ngy_b, ngx_b) array per instance."""

    def __init__(self, thetas, dtype: str = "f64"):
        self._L = L.load()
        code, npdt = _DT[dtype]
        ths = [np.asarray(t, dtype=np.float64) for t in thetas]
        self.dtype = dtype
        self.shapes = [t.shape for t in ths]
        self.shape = self.shapes[0]
        B = len(ths)
        gy = (C.c_int32 * B)(*[t.shape[0] for t in ths])
        gx = (C.c_int32 * B)(*[t.shape[1] for t in ths])
        packed = np.concatenate([np.asfortranarray(t.astype(npdt)).ravel(order="F") for t in ths])
        h = C.c_void_p()
        L.check(self._L.sph_batch_field_create(B, gx, gy, code, _ptr(packed), C.byref(h)))
        self.h = h


class BatchWorkspace:
    """AdjointWorkspace for a Batch."""

    def __init__(self, batch: Batch):
        self._L = L.load()
        self.B, self.N, self.p = batch.B, batch.N, batch.p
        self.params, self.sizes, self.offsets = batch.params, batch.sizes, batch.offsets
        cps = (L.sph_params * self.B)(*[q.c_struct() for q in self.params])
        ns = (C.c_int64 * self.B)(*self.sizes)
        h = C.c_void_p()
        L.check(self._L.sph_batch_workspace_create(self.B, cps, ns, self.p.code, C.byref(h)))
        self.h = h
        self.last_flags = 0

    def __del__(self):
        if getattr(self, "h", None):
            self._L.sph_workspace_destroy(self.h)
            self.h = None

    def get(self):
        """[(gX_b, gV_b, gtheta_b)] per instance."""
        gX = np.empty((self.N, 2), self.p.np)
        gV = np.empty((self.N, 2), self.p.np)
        nn = [q.ngx * q.ngy for q in self.params]
        gt = np.empty(sum(nn), self.p.np)
        L.check(self._L.sph_workspace_get(self.h, _ptr(gX), _ptr(gV), _ptr(gt)))
        o = self.offsets
        out, t0 = [], 0
        for b, q in enumerate(self.params):
            g = gt[t0:t0 + nn[b]].reshape(q.ngx, q.ngy).T
            out.append((gX[o[b]:o[b + 1]].T, gV[o[b]:o[b + 1]].T, g))
            t0 += nn[b]
        return out

    def objective(self, batch: Batch, kind="ke_right", args=None):
        J = (C.c_double * self.B)()
        k = {"ke_right": 0, "target": 1}[kind]
        a = None
        if args is not None:
            arr = np.ascontiguousarray(np.asarray(args, np.float64).reshape(self.B, 3))
            a = arr.ctypes.data_as(C.POINTER(C.c_double))
        L.check(self._L.sph_batch_objective(self.h, batch.h, k, a, J))
        return np.array(J[:])


def batch_backward(ws: BatchWorkspace, tape: Tape, theta: BatchField, seedsX=None, seedsV=None,
                   scratch=None, skin=0.2, interval=4, maxnb=64, seeded=False):
    """backward! over a Batch: seeds are lists of (2, N_b) arrays (or, with
    seeded=True, the seeds left by BatchWorkspace.objective)."""
    f = C.c_uint32()
    if seeded:
        L.check(ws._L.sph_backward_seeded(ws.h, tape.h, theta.h, None,
                                          scratch.h if scratch is not None else None, float(skin),
                                          int(interval), int(maxnb), C.byref(f)))
    else:
        dt = ws.p.np
        sx = np.concatenate([_xy(a, n, dt) for a, n in zip(seedsX, ws.sizes)]) if seedsX else None
        sv = np.concatenate([_xy(a, n, dt) for a, n in zip(seedsV, ws.sizes)]) if seedsV else None
        L.check(ws._L.sph_backward(ws.h, tape.h, theta.h, None, _ptr(sx), _ptr(sv),
                                   scratch.h if scratch is not None else None, float(skin),
                                   int(interval), int(maxnb), C.byref(f)))
    ws.last_flags = f.value
    _warn_flags(f.value, maxnb)
    return ws


def backward_seeded(ws: AdjointWorkspace, tape: Tape, theta, p: SPHParams, scratch=None,
                    skin=0.2, interval=4, maxnb=64) -> AdjointWorkspace:
    """backward! seeded by the workspace's last on-device objective."""
    th = _field(theta, p)
    f = C.c_uint32()
    L.check(ws._L.sph_backward_seeded(ws.h, tape.h, th.h, C.byref(p.c_struct()),
                                      scratch.h if scratch is not None else None, float(skin),
                                      int(interval), int(maxnb), C.byref(f)))
    ws.last_flags = f.value
    _warn_flags(f.value, maxnb)
    return ws


class Graph:
    """A captured sequence of library calls (a CUDA graph, no counterpart in
    the reference). launch() replays its device work on the calling thread's
    library stream without waiting."""

    def __init__(self, h):
        self._L = L.load()
        self.h = h

    def launch(self) -> "Graph":
        L.check(self._L.sph_graph_launch(self.h))
        return self

    @property
    def nodes(self) -> int:
        n = C.c_int64()
        L.check(self._L.sph_graph_nodes(self.h, C.byref(n)))
        return n.value

    def __del__(self):
        if getattr(self, "h", None):
            self._L.sph_graph_destroy(self.h)
            self.h = None


def capture(fn) -> Graph:
    """Record the library calls fn() makes on this thread into a Graph instead
    of running them. Run the same sequence once before capturing it (first uses
    allocate); host results (J, flags) read as 0 during capture."""
    lib = L.load()
    L.check(lib.sph_capture_begin())
    g = C.c_void_p()
    try:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            fn()
    except BaseException:
        lib.sph_capture_end(C.byref(g))
        if g.value:
            lib.sph_graph_destroy(g)
        raise
    L.check(lib.sph_capture_end(C.byref(g)))
    return Graph(g)


def reset(tape: Tape) -> Tape:
    """reset!(tape) (src/driver.jl:71)."""
    return tape.reset()


def _skin_for(cs: float, p: SPHParams) -> float:
    """The neighbour-list skin whose cutoff Float64(support(p)) * (1 + skin)
    equals cs exactly (the library's cell width is that cutoff)."""
    s = float(p.np(2) * p.np(p.h))
    skin = cs / s - 1.0
    for _ in range(64):
        rc = s * (1.0 + skin)
        if rc == cs:
            return skin
        skin = np.nextafter(skin, np.inf if rc < cs else -np.inf)
    raise L.ArgumentError(1, f"cell width {cs!r} is not reachable as 2h(1 + skin)")


class CellList:
    """CellList(backend, N, p; cs = support(p)) (src/neighbors.jl:9-36) as a
    standalone object: after build(cl, X) it holds counts, starts (0-based),
    order (1-based ids) and cellof of the positions X, bit for bit as the
    reference computes them. cs must be at least the support 2h."""

    def __init__(self, N: int, p: SPHParams, cs=None):
        self.N, self.p = int(N), p
        self.cs = float(cs) if cs is not None else float(p.np(2) * p.np(p.h))
        self._skin = _skin_for(self.cs, p)
        self.nx = max(1, int(np.ceil(float(p.np(p.Lx)) / self.cs)) + 2)
        self.ny = max(1, int(np.ceil(float(p.np(p.Ly)) / self.cs)) + 2)
        self.counts = self.starts = self.order = None


class NeighborList:
    """NeighborList(backend, N, p; skin, interval, maxnb, layout)
    (src/neighbors.jl:150-190) as a standalone object: after
    build_neighbors(nl, cl, X) it holds indices (particle-major, 1-based ids,
    shape (N, maxnb)), counts and flags, and age = 0."""

    def __init__(self, N: int, p: SPHParams, skin=0.2, interval=4, maxnb=64, layout="auto"):
        _check_layout(layout)
        self.N, self.p = int(N), p
        self.skin, self.interval, self.maxnb = float(skin), int(interval), int(maxnb)
        self.rc = float(p.np(2) * p.np(p.h)) * (1.0 + self.skin)
        self.age = np.iinfo(np.int64).max
        self.indices = self.counts = None
        self.flags = 0
        self._st = None


def build(st, X=None, p: SPHParams | None = None, backend=None):
    """build!(cl, X, p, backend) (src/neighbors.jl:97-114): the cell list of a
    State's current positions, or of positions X into a standalone CellList."""
    if isinstance(st, CellList):
        cl = st
        if X is None:
            raise L.ArgumentError(1, "build(cl, X): positions are required")
        s = State(X, np.zeros_like(np.asarray(X, np.float64)), p or cl.p, skin=cl._skin)
        L.check(s._L.sph_build_cells(s.h))
        c = s.celllist()
        cl.counts, cl.starts, cl.order = c["counts"], c["starts"], c["order"]
        return cl
    L.check(st._L.sph_build_cells(st.h))
    return st


def build_neighbors(st, cl: CellList | None = None, X=None, p: SPHParams | None = None,
                    backend=None):
    """build_neighbors!(nl, cl, X, p, backend) (src/neighbors.jl:252-263): on
    a State, or into a standalone NeighborList (and its CellList) from
    positions X; the displacement check runs against the previous build."""
    if isinstance(st, NeighborList):
        nl = st
        if X is None:
            raise L.ArgumentError(1, "build_neighbors(nl, cl, X): positions are required")
        pp = p or nl.p
        if nl._st is None:
            nl._st = State(X, np.zeros_like(np.asarray(X, np.float64)), pp, skin=nl.skin,
                           interval=nl.interval, maxnb=nl.maxnb)
        else:
            nl._st.set(X=X)
        L.check(nl._st._L.sph_build_neighbors(nl._st.h))
        nl.indices, nl.counts = nl._st.neighbors()
        nl.flags |= nl._st.take_flags()
        nl.age = 0
        if cl is not None:
            c = nl._st.celllist()
            cl.counts, cl.starts, cl.order = c["counts"], c["starts"], c["order"]
        return nl
    L.check(st._L.sph_build_neighbors(st.h))
    return st


def step(st: State, theta, p: SPHParams | None = None) -> State:
    """step!(st, theta, p, backend) (src/forward.jl:161-173)."""
    th = _field(theta, st.p)
    L.check(st._L.sph_step(st.h, th.h, C.byref(p.c_struct()) if p is not None else None))
    return st


def simulate(st: State, theta, p: SPHParams | None, nsteps: int, tape: Tape | None = None) -> State:
    """simulate!(st, theta, p, backend, nsteps; tape) (src/driver.jl:92-115).
    Also runs a Batch (p = None, theta a BatchField)."""
    th = theta if isinstance(theta, DesignField) else _field(theta, st.p)
    f = C.c_uint32()
    L.check(st._L.sph_simulate(st.h, th.h, C.byref(p.c_struct()) if p is not None else None,
                               int(nsteps), tape.h if tape is not None else None, C.byref(f)))
    st.last_flags = f.value
    _warn_flags(f.value, st.maxnb)
    return st


def backward(ws: AdjointWorkspace, tape: Tape, theta, p: SPHParams, seedX, seedV=None,
             scratch: State | None = None, skin=0.2, interval=4, maxnb=64,
             layout="auto") -> AdjointWorkspace:
    """backward!(ws, tape, theta, p, backend; seedX, seedV, scratch, skin,
    interval, maxnb, layout) (src/driver.jl:141-207)."""
    _check_layout(layout)
    th = _field(theta, p)
    N = ws.N
    sx = _xy(seedX, N, p.np) if seedX is not None else None
    sv = _xy(seedV, N, p.np) if seedV is not None else None
    f = C.c_uint32()
    L.check(ws._L.sph_backward(ws.h, tape.h, th.h, C.byref(p.c_struct()), _ptr(sx), _ptr(sv),
                               scratch.h if scratch is not None else None, float(skin),
                               int(interval), int(maxnb), C.byref(f)))
    ws.last_flags = f.value
    _warn_flags(f.value, maxnb)
    return ws


def target_objective(X, xc, yc, sigma):
    """target_objective(X, xc, yc, sigma) (src/driver.jl:219-234): J and dJ/dX_T."""
    X = np.asarray(X)
    T = X.dtype.type
    dx = X[0] - T(xc)
    dy = X[1] - T(yc)
    s2 = T(sigma) ** 2
    e = np.exp(-(dx * dx + dy * dy) / (2 * s2))
    J = -np.sum(e, dtype=X.dtype)
    seed = np.stack([e * dx / s2, e * dy / s2])
    return J, seed


def kinetic_energy_right_half(X, V, p: SPHParams):
    """J = sum_i 1/2 m |v_i|^2 over particles with x_i > Lx/2, and its seeds
    (dJ/dX_T = 0 almost everywhere, dJ/dV_T = m v_i on the right half)."""
    X, V = np.asarray(X), np.asarray(V)
    right = X[0] > p.Lx / 2
    J = float(0.5 * p.m * np.sum((V[0] ** 2 + V[1] ** 2)[right]))
    seedV = np.where(right, p.m * V, 0.0).astype(V.dtype)
    return J, np.zeros_like(X), seedV


def launch_count() -> int:
    return int(L.load().sph_launch_count())


TUNED_KERNELS = ("nl_build", "density", "accel_integrate", "accel_drag", "pass1", "pass2")


def autotune_in_solve(state, solve, candidates=(64, 128, 256)):
    """Choose the block size of each tuned kernel from its launches inside
    real solves (no counterpart in the reference). solve() runs one short
    forward+adjoint solve with ``state``'s precision and kind; it is called
    once per candidate with every tuned kernel at that size, each kernel's
    launches are timed with CUDA events, and each kernel keeps its fastest
    size. Returns the chosen sizes (TUNED_KERNELS order). It uses the
    library's kernel timers: they are reset, and the six kernels' timers are
    off afterwards.

    Repeated launches of one kernel, as the engine's own autotune times them,
    can favour a size that is slower inside the solve's kernel sequence (on
    1M particles pass 2 runs 8% faster at 64 threads than at the 256 that
    repeated launches pick)."""
    lib = L.load()
    ids = [L.KERNEL_ID[k] for k in TUNED_KERNELS]
    best = [None] * 6
    pick = [int(candidates[0])] * 6
    try:
        for c in candidates:
            state.set_block_sizes([int(c)] * 6)
            L.check(lib.sph_profile_reset())
            for i in ids:
                L.check(lib.sph_profile_enable(i, 1))
            solve()
            synchronize()
            for k, i in enumerate(ids):
                ms, n = C.c_double(), C.c_int64()
                L.check(lib.sph_profile_read(i, C.byref(ms), C.byref(n)))
                if n.value and (best[k] is None or ms.value / n.value < best[k]):
                    best[k] = ms.value / n.value
                    pick[k] = int(c)
    finally:
        for i in ids:
            lib.sph_profile_enable(i, 0)
        L.check(lib.sph_profile_reset())
    state.set_block_sizes(pick)
    return pick


def synchronize():
    L.check(L.load().sph_synchronize())


def set_group_lanes(lanes: int) -> None:
    """Lanes per particle of the pair-sum kernels, process-wide (no counterpart
    in the reference): 0 = by state size (default: lane groups for single
    states of up to 16384 particles), 1 = one thread per particle, 16 or 32 =
    a lane group per particle for single states. FP64 results are
    bit-identical across settings; FP32 results differ in the last bits."""
    L.check(L.load().sph_set_group_lanes(int(lanes)))


DENSITY_FORMS = {"mask": 0, "tiles": 1, "pairs": 2}


def set_density_form(form) -> None:
    """Density kernel form of FP32 states with one thread per particle (no
    counterpart in the reference), process-wide: "mask" walks each particle's
    neighbour masks one candidate at a time, "tiles" uses the cell-tile form
    (a warp stages its 32 particles' neighbouring cell rows in shared memory
    and every lane scans all staged candidates; single states), "pairs" (the
    default) walks the masks two candidates per iteration with packed f32x2
    arithmetic."""
    L.check(L.load().sph_set_density_form(DENSITY_FORMS[form] if isinstance(form, str)
                                          else int(form)))


def set_launch_overlap(on: bool) -> None:
    """Programmatic dependent launch of the engine's kernels (default on): each
    kernel may be scheduled while its predecessor still runs and waits on the
    device for its results. Results do not depend on it."""
    L.check(L.load().sph_set_launch_overlap(1 if on else 0))


def set_step_graphs(steps: int) -> None:
    """Steps per recorded group (no counterpart in the reference),
    process-wide: simulate and backward record the launches of this many
    consecutive steps and replay each group as one CUDA graph (default 32;
    0 launches every kernel on its own). Results do not depend on it."""
    L.check(L.load().sph_set_step_graphs(int(steps)))


def step_graphs() -> int:
    v = C.c_int32()
    L.check(L.load().sph_get_step_graphs(C.byref(v)))
    return v.value


def step_graph_counts() -> tuple:
    """(groups replayed as graphs, graphs instantiated) since the library was
    loaded, process-wide."""
    r, i = C.c_int64(), C.c_int64()
    L.check(L.load().sph_step_graph_counts(C.byref(r), C.byref(i)))
    return r.value, i.value


def density_form() -> str:
    v = C.c_int32()
    L.check(L.load().sph_get_density_form(C.byref(v)))
    return {c: k for k, c in DENSITY_FORMS.items()}[v.value]


def group_lanes() -> int:
    v = C.c_int32()
    L.check(L.load().sph_get_group_lanes(C.byref(v)))
    return v.value
