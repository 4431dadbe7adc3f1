"""sph_build_cells_noalloc: the cell-list build for callers that cannot let a
library allocate device memory (their device arrays come from their own pool
or budgeted allocator). It must give exactly what the allocating path gives
(sph_build_cells + sph_get_celllist): counts, 0-based starts and 1-based
order are integers, so the comparison is exact. Two calls in a row check that
the shared fixed work array left over from one call does not leak into the
next. This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import cases as K

pytestmark = pytest.mark.gpu

S = pytest.importorskip("sphadjoint_gb300")
torch = pytest.importorskip("torch")


def _reference_celllist(case, dtype):
    """Cell list through the existing (allocating) entry points."""
    p = S.SPHParams(**case["p"], dtype=dtype)
    st = S.State(case["X0"], case["V0"], p)
    S.build(st)
    nx, ny, cs, _ = st.grid()
    return st.celllist(), (nx, ny, cs)


def _noalloc(lib, X0, dtype, grid, stream):
    nx, ny, cs = grid
    npdt = np.float64 if dtype == "f64" else np.float32
    tdt = torch.float64 if dtype == "f64" else torch.float32
    X = torch.tensor(np.ascontiguousarray(X0.T, dtype=npdt), dtype=tdt, device="cuda")
    N = X.shape[0]
    counts = torch.full((nx * ny,), -7, dtype=torch.int32, device="cuda")
    starts = torch.full((nx * ny,), -7, dtype=torch.int32, device="cuda")
    order = torch.full((max(N, 1),), -7, dtype=torch.int32, device="cuda")
    # the inputs and the -7 fills were queued on torch's current stream: the
    # library's stream must wait for them, as any caller's stream would
    stream.wait_stream(torch.cuda.current_stream())
    code = lib.sph_build_cells_noalloc(
        C.c_void_p(X.data_ptr()), N, 0 if dtype == "f64" else 1, C.c_double(cs), nx, ny,
        C.cast(C.c_void_p(counts.data_ptr()), C.POINTER(C.c_int32)),
        C.cast(C.c_void_p(starts.data_ptr()), C.POINTER(C.c_int32)),
        C.cast(C.c_void_p(order.data_ptr()), C.POINTER(C.c_int32)),
        C.c_void_p(stream.cuda_stream))
    assert code == 0, lib.sph_last_error().decode()
    torch.cuda.synchronize()
    return counts.cpu().numpy(), starts.cpu().numpy(), order.cpu().numpy()[:N]


def _lib():
    lib = S.load()
    f = lib.sph_build_cells_noalloc
    f.restype = C.c_int32
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_double, C.c_int32, C.c_int32,
                  C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p]
    return lib


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_noalloc_matches_allocating_build_twice(dtype):
    lib = _lib()
    stream = torch.cuda.Stream()
    # two different inputs back to back on the same shared work array
    for case in (K.dambreak_case(jitter=0.3, seed=4), K.random_points_case(seed=5)):
        ref, grid = _reference_celllist(case, dtype)
        counts, starts, order = _noalloc(lib, case["X0"], dtype, grid, stream)
        assert np.array_equal(counts, ref["counts"])
        assert np.array_equal(starts, ref["starts"])
        assert np.array_equal(order, ref["order"])
    # and the first input again: same answer as before
    case = K.dambreak_case(jitter=0.3, seed=4)
    ref, grid = _reference_celllist(case, dtype)
    counts, starts, order = _noalloc(lib, case["X0"], dtype, grid, stream)
    assert np.array_equal(order, ref["order"]) and np.array_equal(counts, ref["counts"])


def _grid_case(nx, ny, N, seed):
    """N random particles in a tank whose cell grid is exactly nx x ny (the
    reference's nx = ceil(L / cs) + 2 with cs = 2h (1 + skin))."""
    rng = np.random.default_rng(seed)
    h = 1.3e-3
    cs = 2 * h * 1.2
    p = dict(h=h, m=1e-3, rho0=1000.0, c=20.0, mu=0.02, dt=1e-5, Lx=(nx - 2.5) * cs,
             Ly=(ny - 2.5) * cs, kw=5e4, ngx=8, ngy=8)
    X0 = np.vstack([rng.random(N) * p["Lx"], rng.random(N) * p["Ly"]])
    return dict(p=p, X0=X0, V0=np.zeros_like(X0), theta=np.zeros((8, 8)))


@pytest.mark.parametrize("nx,ny,N", [(96, 80, 100_000), (1024, 1024, 1 << 20)])
def test_noalloc_multi_block_scan_and_limits(nx, ny, N):
    """Grids above one scan tile (2048 cells) take the three-launch scan whose
    block sums live in the shared work array; the second case sits exactly at
    both limits (2^20 particles, 2^20 cells)."""
    lib = _lib()
    stream = torch.cuda.Stream()
    case = _grid_case(nx, ny, N, seed=nx)
    ref, grid = _reference_celllist(case, "f32")
    assert grid[:2] == (nx, ny)
    for _ in range(2):
        counts, starts, order = _noalloc(lib, case["X0"], "f32", grid, stream)
        assert np.array_equal(counts, ref["counts"])
        assert np.array_equal(starts, ref["starts"])
        assert np.array_equal(order, ref["order"])


def test_noalloc_rejects_sizes_beyond_its_limit():
    lib = _lib()
    big = (1 << 20) + 1
    code = lib.sph_build_cells_noalloc(None, big, 0, 0.1, 10, 10, None, None, None, None)
    assert code == 1 and b"exceeds" in lib.sph_last_error()
    code = lib.sph_build_cells_noalloc(None, 10, 0, 0.1, 2048, 1024, None, None, None, None)
    assert code == 1 and b"cells" in lib.sph_last_error()
