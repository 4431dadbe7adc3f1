"""Host logic of autotune_in_solve on CPU: one solve per candidate size,
each kernel keeps the size with its lowest per-launch time (a fake kernel
timer stands in for the library's CUDA events)."""
import ctypes as C

import pytest

import sphadjoint_gb300.api as A
import sphadjoint_gb300._lib as LB


class FakeLib:
    """sph_profile_* over a table ms_per_launch[kernel][block size]."""

    def __init__(self, table):
        self.table, self.on, self.size = table, set(), None
        self.resets = 0

    def sph_profile_reset(self):
        self.resets += 1
        return 0

    def sph_profile_enable(self, kid, on):
        (self.on.add if on else self.on.discard)(kid)
        return 0

    def sph_profile_read(self, kid, ms, n):
        name = LB.KERNELS[kid]
        launches = 10
        C.cast(ms, C.POINTER(C.c_double))[0] = self.table[name][self.size] * launches
        C.cast(n, C.POINTER(C.c_int64))[0] = launches
        return 0


class FakeState:
    def __init__(self, lib):
        self.lib, self.sizes = lib, [256] * 6

    def set_block_sizes(self, b):
        self.sizes = list(b)
        if len(set(b)) == 1:
            self.lib.size = b[0]

    def block_sizes(self):
        return self.sizes


def test_each_kernel_keeps_its_fastest_size(monkeypatch):
    table = {
        "nl_build": {64: 1.0, 128: 0.9, 256: 0.95},
        "density": {64: 2.0, 128: 1.9, 256: 1.9},
        "accel_integrate": {64: 2.1, 128: 1.6, 256: 1.7},
        "accel_drag": {64: 0.8, 128: 0.7, 256: 0.75},
        "pass1": {64: 1.05, 128: 0.91, 256: 0.92},
        "pass2": {64: 0.70, 128: 0.72, 256: 0.77},
    }
    lib = FakeLib(table)
    monkeypatch.setattr(LB, "load", lambda: lib)
    monkeypatch.setattr(A, "synchronize", lambda: None)
    st = FakeState(lib)
    solves = []
    chosen = A.autotune_in_solve(st, lambda: solves.append(lib.size))
    assert solves == [64, 128, 256]
    assert chosen == [128, 128, 128, 128, 128, 64]  # ties keep the first (smaller) size
    assert st.block_sizes() == chosen
    assert not lib.on and lib.resets >= 4  # timers off and reset afterwards


def test_timers_are_released_when_the_solve_fails(monkeypatch):
    lib = FakeLib({k: {64: 1.0, 128: 1.0, 256: 1.0} for k in A.TUNED_KERNELS})
    monkeypatch.setattr(LB, "load", lambda: lib)
    monkeypatch.setattr(A, "synchronize", lambda: None)

    def boom():
        raise RuntimeError("solve failed")

    with pytest.raises(RuntimeError):
        A.autotune_in_solve(FakeState(lib), boom)
    assert not lib.on
