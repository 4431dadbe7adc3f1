"""ctypes wrapper of the CPU parity oracle (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, and only as the parity reference (or the timed CPU
baseline). The product (``sphadjoint_gb300``) never imports it.

The oracle restates the reference Julia package SPHAdjoint (src/*.jl) in C;
see ``sph_oracle_body.h`` for the line-by-line correspondence. Arrays follow
the reference layout: positions/velocities are (2, N) column-major, exposed
here as numpy arrays of shape (N, 2) (same memory); theta is (ngy, ngx)
column-major, taken here as a numpy (ngy, ngx) array.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsph_oracle.so")
_lib = None


class OrcParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("h", "m", "rho0", "c", "mu", "gx", "gy", "dt", "Lx", "Ly", "kw")] + \
               [("ngx", C.c_int32), ("ngy", C.c_int32), ("eos", C.c_int32),
                ("gamma", C.c_int32), ("visc", C.c_int32), ("pad", C.c_int32),
                ("alpha", C.c_double)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP, -ffp-contract=off)."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < max(
                os.path.getmtime(os.path.join(_HERE, f))
                for f in ("sph_oracle.c", "sph_oracle_body.h")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)


def _declare(L):
    L.orc_set_threads.argtypes = [C.c_int]
    L.orc_get_threads.restype = C.c_int
    for s, r in (("_f64", C.c_double), ("_f32", C.c_float)):
        f = lambda n: getattr(L, n + s)  # noqa: E731
        f("orc_state_new").restype = _P
        f("orc_state_new").argtypes = [C.POINTER(OrcParams), C.c_int64, _D, _D,
                                       C.c_double, C.c_int, C.c_int]
        f("orc_state_free").argtypes = [_P]
        f("orc_tape_new").restype = _P
        f("orc_tape_new").argtypes = [C.c_int64, C.c_int64]
        f("orc_tape_free").argtypes = [_P]
        f("orc_tape_get").argtypes = [_P, C.c_int64, _D, _D]
        f("orc_tape_length").restype = C.c_int64
        f("orc_tape_length").argtypes = [_P]
        f("orc_tape_reset").argtypes = [_P]
        f("orc_work_new").restype = _P
        f("orc_work_new").argtypes = [C.c_int64, C.c_int, C.c_int]
        f("orc_work_free").argtypes = [_P]
        f("orc_work_get").argtypes = [_P, _D, _D, _D]
        f("orc_theta_new").restype = _P
        f("orc_theta_new").argtypes = [_D, C.c_int, C.c_int]
        f("orc_theta_free").argtypes = [_P]
        f("orc_step").argtypes = [_P, _P, C.POINTER(OrcParams), C.c_int]
        f("orc_simulate").restype = C.c_int32
        f("orc_simulate").argtypes = [_P, _P, C.POINTER(OrcParams), C.c_int64, _P, C.c_int]
        f("orc_backward").restype = C.c_int32
        f("orc_backward").argtypes = [_P, _P, _P, C.POINTER(OrcParams), _D, _D, _P,
                                      C.c_double, C.c_int, C.c_int, C.c_int]
        f("orc_build_cells").argtypes = [_P]
        f("orc_build_neighbors").argtypes = [_P, r]
        f("orc_state_get").argtypes = [_P, _D, _D]
        f("orc_state_set").argtypes = [_P, _D, _D]
        f("orc_state_fields").argtypes = [_P, _D, _D, _D, _D, _D]
        f("orc_state_grid").argtypes = [_P, _I, _I, _D, C.POINTER(C.c_int64)]
        f("orc_state_cells").argtypes = [_P, _I, _I, _I, _I]
        f("orc_state_neighbors").argtypes = [_P, _I, _I]
        f("orc_take_flags").restype = C.c_int32
        f("orc_take_flags").argtypes = [_P]
        for k in ("orc_w_kern",):
            f(k).restype = r
            f(k).argtypes = [r, r]
        for k in ("orc_f_kern", "orc_g_kern"):
            f(k).restype = r
            f(k).argtypes = [r, r, r]
        f("orc_density").argtypes = [_P, _P]
        f("orc_eos").argtypes = [_P, _P]


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def params(**kw) -> OrcParams:
    """SPHParams with the reference's defaults gx = 0, gy = -9.81 (linear EOS,
    Morris viscosity). eos=1 selects Tait (gamma, default 7), visc=1 the
    artificial viscosity (alpha)."""
    p = OrcParams()
    p.gx = kw.pop("gx", 0.0)
    p.gy = kw.pop("gy", -9.81)
    p.gamma = kw.pop("gamma", 7)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _xy(a, N):
    a = np.asarray(a, dtype=np.float64)
    if a.shape == (2, N):
        a = a.T
    return np.ascontiguousarray(a.reshape(N, 2))


class Oracle:
    """One precision instantiation of the oracle (``"f64"`` or ``"f32"``)."""

    def __init__(self, dtype: str = "f64"):
        assert dtype in ("f64", "f32")
        self.sfx = "_" + dtype
        self.L = lib()
        self.real = C.c_double if dtype == "f64" else C.c_float

    def fn(self, name):
        return getattr(self.L, name + self.sfx)

    # -- objects -----------------------------------------------------------
    def state(self, p, X0, V0, skin=0.2, interval=4, maxnb=64):
        return OState(self, p, X0, V0, skin, interval, maxnb)

    def tape(self, N, cap):
        return OTape(self, N, cap)

    def workspace(self, N, p):
        return OWork(self, N, p)

    def theta(self, theta):
        return OTheta(self, theta)

    # -- driver ------------------------------------------------------------
    def simulate(self, st, th, p, nsteps, tape=None, explicit_drag=False):
        r = self.fn("orc_simulate")(st.h, th.h, C.byref(p), int(nsteps),
                                    tape.h if tape is not None else None,
                                    int(explicit_drag))
        if r < 0:
            raise ValueError("tape capacity exceeded")
        return r

    def step(self, st, th, p, explicit_drag=False):
        self.fn("orc_step")(st.h, th.h, C.byref(p), int(explicit_drag))

    def backward(self, ws, tape, th, p, seedX, seedV, scratch=None, skin=0.2,
                 interval=4, maxnb=64, explicit_drag=False):
        N = ws.N
        sx = _xy(seedX, N)
        sv = _xy(seedV, N)
        return self.fn("orc_backward")(ws.h, tape.h, th.h, C.byref(p), _dp(sx), _dp(sv),
                                       scratch.h if scratch is not None else None,
                                       float(skin), int(interval), int(maxnb),
                                       int(explicit_drag))

    def w_kern(self, q, A):
        return self.fn("orc_w_kern")(q, A)

    def f_kern(self, q, A, h):
        return self.fn("orc_f_kern")(q, A, h)

    def g_kern(self, q, A, h):
        return self.fn("orc_g_kern")(q, A, h)


class OState:
    def __init__(self, o, p, X0, V0, skin, interval, maxnb):
        self.o = o
        self.N = N = int(np.asarray(X0).size // 2)
        x = _xy(X0, N)
        v = _xy(V0, N)
        self.maxnb = maxnb
        self.h = o.fn("orc_state_new")(C.byref(p), N, _dp(x), _dp(v), float(skin),
                                       int(interval), int(maxnb))

    def __del__(self):
        if getattr(self, "h", None):
            self.o.fn("orc_state_free")(self.h)
            self.h = None

    def get(self):
        X = np.zeros((self.N, 2))
        V = np.zeros((self.N, 2))
        self.o.fn("orc_state_get")(self.h, _dp(X), _dp(V))
        return X, V

    def set(self, X=None, V=None):
        x = _xy(X, self.N) if X is not None else None
        v = _xy(V, self.N) if V is not None else None
        self.o.fn("orc_state_set")(self.h, _dp(x) if x is not None else None,
                                   _dp(v) if v is not None else None)

    def fields(self):
        N = self.N
        rho, pt, ir, al = (np.zeros(N) for _ in range(4))
        a = np.zeros((N, 2))
        self.o.fn("orc_state_fields")(self.h, _dp(rho), _dp(pt), _dp(ir), _dp(a), _dp(al))
        return dict(rho=rho, pterm=pt, invrho=ir, a=a, alpha=al)

    def grid(self):
        nx, ny = C.c_int32(), C.c_int32()
        cs = C.c_double()
        age = C.c_int64()
        self.o.fn("orc_state_grid")(self.h, C.byref(nx), C.byref(ny), C.byref(cs),
                                    C.byref(age))
        return nx.value, ny.value, cs.value, age.value

    def cells(self):
        nx, ny, _, _ = self.grid()
        nc = nx * ny
        counts = np.zeros(nc, np.int32)
        starts = np.zeros(nc, np.int32)
        order = np.zeros(self.N, np.int32)
        cellof = np.zeros(self.N, np.int32)
        self.o.fn("orc_state_cells")(self.h, _ip(counts), _ip(starts), _ip(order), _ip(cellof))
        return dict(counts=counts, starts=starts, order=order, cellof=cellof)

    def neighbors(self):
        idx = np.zeros(self.N * self.maxnb, np.int32)
        nbc = np.zeros(self.N, np.int32)
        self.o.fn("orc_state_neighbors")(self.h, _ip(idx), _ip(nbc))
        return idx.reshape(self.N, self.maxnb), nbc

    def build_cells(self):
        self.o.fn("orc_build_cells")(self.h)

    def build_neighbors(self, h):
        self.o.fn("orc_build_neighbors")(self.h, h)

    def density(self, p):
        self.o.fn("orc_density")(self.h, C.byref(_inner_params(self.o, p)))
        self.o.fn("orc_eos")(self.h, C.byref(_inner_params(self.o, p)))

    def take_flags(self):
        return int(self.o.fn("orc_take_flags")(self.h))


def _inner_params(o, p):
    """The oracle's per-precision parameter struct (every field converted to T)."""
    R = o.real

    class _OP(C.Structure):
        _fields_ = [(n, R) for n in
                    ("h", "m", "rho0", "c", "mu", "gx", "gy", "dt", "Lx", "Ly", "kw")] + \
                   [("ngx", C.c_int), ("ngy", C.c_int), ("eos", C.c_int), ("gamma", C.c_int),
                    ("visc", C.c_int), ("alpha", R)]
    q = _OP()
    for n, _ in _OP._fields_:
        setattr(q, n, getattr(p, n))
    return q


class OTape:
    def __init__(self, o, N, cap):
        self.o, self.N, self.cap = o, int(N), int(cap)
        self.h = o.fn("orc_tape_new")(self.N, self.cap)

    def __del__(self):
        if getattr(self, "h", None):
            self.o.fn("orc_tape_free")(self.h)
            self.h = None

    def __len__(self):
        return int(self.o.fn("orc_tape_length")(self.h))

    def reset(self):
        self.o.fn("orc_tape_reset")(self.h)

    def get(self, n):
        X = np.zeros((self.N, 2))
        V = np.zeros((self.N, 2))
        self.o.fn("orc_tape_get")(self.h, int(n), _dp(X), _dp(V))
        return X, V


class OWork:
    def __init__(self, o, N, p):
        self.o, self.N = o, int(N)
        self.ngx, self.ngy = int(p.ngx), int(p.ngy)
        self.h = o.fn("orc_work_new")(self.N, self.ngx, self.ngy)

    def __del__(self):
        if getattr(self, "h", None):
            self.o.fn("orc_work_free")(self.h)
            self.h = None

    def get(self):
        gX = np.zeros((self.N, 2))
        gV = np.zeros((self.N, 2))
        gt = np.zeros(self.ngx * self.ngy)
        self.o.fn("orc_work_get")(self.h, _dp(gX), _dp(gV), _dp(gt))
        # column-major (ngy, ngx) -> numpy (ngy, ngx)
        return gX, gV, gt.reshape(self.ngx, self.ngy).T.copy()


class OTheta:
    def __init__(self, o, theta):
        self.o = o
        th = np.asarray(theta, dtype=np.float64)
        ngy, ngx = th.shape
        cm = np.ascontiguousarray(th.T)  # column-major (ngy, ngx)
        self.h = o.fn("orc_theta_new")(_dp(cm), ngx, ngy)

    def __del__(self):
        if getattr(self, "h", None):
            self.o.fn("orc_theta_free")(self.h)
            self.h = None
