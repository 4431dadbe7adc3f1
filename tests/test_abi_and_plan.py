"""CPU checks of the C ABI library: it loads without a GPU, exports every
symbol the header declares, rejects bad arguments before touching the
device, and its binomial checkpoint schedule is optimal (brute-force DP)."""
import ctypes as C
import functools
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sphadjoint_gb300.h")


@pytest.fixture(scope="module")
def lib():
    import sphadjoint_gb300 as S

    return S.load()


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"SPH_API\s+[\w\s\*]+?\b(sph_\w+)\s*\(", txt)))


def test_header_symbols_exported(lib):
    names = declared_symbols()
    assert len(names) > 30
    raw = C.CDLL(lib._name)
    for n in names:
        assert hasattr(raw, n), n


def test_bad_arguments_rejected_without_gpu(lib):
    from sphadjoint_gb300 import _lib as LB

    h = C.c_void_p()
    p = LB.sph_params()
    assert lib.sph_state_create(None, 4, None, None, 0, 0.2, 4, 64, C.byref(h)) == 1
    assert b"params" in lib.sph_last_error()
    assert lib.sph_state_create(C.byref(p), 4, None, None, 7, 0.2, 4, 64, C.byref(h)) == 4
    assert lib.sph_tape_create_checkpointed(4, 10, 0, 0, C.byref(h)) == 1
    assert lib.sph_simulate(None, None, None, 1, None, None) == 1
    assert lib.sph_version() >= 100


@functools.lru_cache(maxsize=None)
def dp_cost(l, c):
    """Brute force: forward steps to reverse l steps with c slots, the state at
    the start held in one of them (recursive split, every m tried)."""
    if l <= 1:
        return 0
    if c <= 1:
        return l * (l - 1) // 2
    return min(m + dp_cost(l - m, c - 1) + dp_cost(m, c) for m in range(1, l))


@pytest.mark.parametrize("c", [1, 2, 3, 4, 6])
def test_checkpoint_schedule_is_optimal(lib, c):
    for l in range(1, 61):
        assert lib.sph_plan_cost(l, c) == dp_cost(l, c), (l, c)
        if l > 1 and c > 1:
            m = lib.sph_plan_split(l, c)
            assert m + dp_cost(l - m, c - 1) + dp_cost(m, c) == dp_cost(l, c)


def test_checkpoint_cost_of_the_benchmark_horizon(lib):
    # 1000 steps, 32 snapshots: repetition number 3, 3*1000 - C(35, 2) = 2405
    assert lib.sph_plan_cost(1000, 32) == 2405


def test_layout_keyword_is_validated_like_the_reference():
    # src/neighbors.jl:178-184: :slot / :particle / :auto, else ArgumentError
    import sphadjoint_gb300.api as A
    import sphadjoint_gb300._lib as LB
    for ok in ("auto", ":slot", "particle"):
        A._check_layout(ok)
    with pytest.raises(LB.ArgumentError):
        A._check_layout("columns")


def test_header_is_plain_c_and_links(lib, tmp_path):
    # the boundary as a C caller (cgo, Julia ccall, JNI) sees it: the header
    # compiles as C99 and a C program links against the library and calls
    # host-only entry points (no device work)
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "abi.c"
    src.write_text(r"""
#include <stdio.h>
#include "sphadjoint_gb300.h"
int main(void) {
    sph_params p = {0};
    int32_t lanes = -1;
    if (sph_version() <= 0) return 1;
    if (sph_plan_cost(1000, 32) != 2405) return 2;
    if (sph_set_group_lanes(8) != SPH_ERR_ARG || sph_last_error()[0] == 0) return 3;
    if (sph_get_group_lanes(&lanes) != SPH_OK || lanes != 0) return 4;
    (void)p;
    printf("ok\n");
    return 0;
}
""")
    exe = tmp_path / "abi"
    libdir = os.path.dirname(lib._name)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", str(exe), "-L", libdir, "-lsphgb300",
                        "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)



def test_tape_mode_follows_the_memory_budget():
    """The automatic tape mode (host only with an explicit budget): the full
    tape whenever its 4 sizeof(T) N L bytes fit, otherwise the most snapshots
    that fit beside the recompute state, capped at L - 1; fewer bytes never
    buy fewer recomputed steps; a budget below one snapshot is refused."""
    import sphadjoint_gb300 as S
    from sphadjoint_gb300 import _lib as LB

    p = S.SPHParams(h=1.3e-3, m=1e-3, rho0=1000.0, c=20.0, mu=0.02, dt=1e-5, Lx=2.048,
                    Ly=1.28, kw=5e4, ngx=256, ngy=256, dtype="f32")
    N, L = 1 << 20, 1000
    full = 4 * 4 * N * L
    assert S.tape_plan(N, L, p, full) == (0, full)
    assert S.tape_plan(N, L, p, 10 * full) == (0, full)
    last_c, last_cost = None, None
    for budget in (full - 1, full // 2, full // 8, full // 32, full // 60):
        c, b = S.tape_plan(N, L, p, budget)
        assert 1 <= c <= L - 1 and b <= budget
        # one more snapshot would not have fitted
        c2, _ = S.tape_plan(N, L, p, b + 1)
        assert c2 == c
        cost = LB.load().sph_plan_cost(L, c)
        if last_c is not None:
            assert c <= last_c and cost >= last_cost
        last_c, last_cost = c, cost
    # 16 GB FP32 full tape of the benchmark workload vs a 4 GB budget
    c, _ = S.tape_plan(N, L, p, 4 << 30)
    assert 32 <= c <= 60
    with pytest.raises(S.SPHError) as e:
        S.tape_plan(N, L, p, 1 << 20)
    assert e.value.code == 5
    # FP64 doubles the full tape
    import dataclasses
    p64 = dataclasses.replace(p, dtype="f64")
    assert S.tape_plan(N, L, p64, 2 * full) == (0, 2 * full)
