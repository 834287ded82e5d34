"""kmc_build_neighbors_noalloc: neighbour lists for callers that cannot allocate device memory.

Some callers own all device memory (their own pool or a pre-reserved arena) or may not call
cudaMalloc while they run.  This entry point builds one film's neighbour/rate CSR into buffers
the caller passes, using a fixed device array for its intermediate storage.  The test allocates
the buffers itself (with torch) and checks the result against kmc_build_neighbors +
kmc_get_neighbors bit for bit, on two different films in a row (the second smaller, so stale
contents of the shared array would show), plus the sizing call and the size limits; that a
call after the first leaves the device's free memory unchanged; and that a film crowded into a
few cells (hundreds of sites per cell) keeps every cell's members in site order.
"""
import ctypes as C

import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import tables

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _ptr(t, ctype):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ctype))


def _noalloc(torch, f, tab, r_max):
    lib = L.load()
    n = f.n_sites
    pos = _dev(torch, f.pos_m(), torch.float64)
    ori = _dev(torch, f.orient, torch.float64)
    grids = [_dev(torch, g, torch.float64) for g in tab["grids"]]
    rate = _dev(torch, np.ravel(tab["rate"]), torch.float64)
    t = L.kmc_table()
    t.kind = tab["kind"]
    for d, g in enumerate(grids):
        t.n[d] = g.numel()
        t.grid[d] = _ptr(g, C.c_double)
    t.rate = _ptr(rate, C.c_double)
    rowptr = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    total = torch.zeros(n, dtype=torch.float64, device="cuda")
    nnz = C.c_int64(-1)
    err = C.create_string_buffer(256)
    # sizing call: no room for the entries -> KMC_ERR_ARG with the count
    rc = lib.kmc_build_neighbors_noalloc(_ptr(pos, C.c_double), _ptr(ori, C.c_double), n, C.byref(t), r_max,
                                         _ptr(rowptr, C.c_int64), None, None, _ptr(total, C.c_double), 0,
                                         C.byref(nnz), None, err, 256)
    assert rc == L.KMC_ERR_ARG and nnz.value > 0 and b"capacity" in err.value
    col = torch.zeros(nnz.value, dtype=torch.int32, device="cuda")
    cum = torch.zeros(nnz.value, dtype=torch.float64, device="cuda")
    rc = lib.kmc_build_neighbors_noalloc(_ptr(pos, C.c_double), _ptr(ori, C.c_double), n, C.byref(t), r_max,
                                         _ptr(rowptr, C.c_int64), _ptr(col, C.c_int32), _ptr(cum, C.c_double),
                                         _ptr(total, C.c_double), nnz.value, C.byref(nnz), None, err, 256)
    assert rc == L.KMC_OK, err.value
    torch.cuda.synchronize()
    return {"rowptr": rowptr.cpu().numpy(), "col": col.cpu().numpy(), "cum": cum.cpu().numpy(),
            "total": total.cpu().numpy()}


def _existing(f, tab, r_max):
    e = E.Engine(0)
    e.load_films(f)
    e.set_table(tab)
    st = e.build(r_max)
    out = e.neighbors(f.n_sites, st["nnz"])
    e.close()
    return out


def test_noalloc_matches_build_neighbors_on_two_calls():
    torch = pytest.importorskip("torch")
    cases = [
        (F.straight_tubes(40, 60.0, box_nm=(120.0, 120.0, 8.0), seed=5), tables.forster_2d(1e15), 10e-9),
        (F.straight_tubes(12, 40.0, box_nm=(60.0, 60.0, 6.0), seed=3),
         E.forster_table(1e15, (0, 180, 21), (1.5e-9, 10e-9, 11), (-10e-9, 10e-9, 11), (-10e-9, 10e-9, 11)), 10e-9),
    ]
    for f, tab, r_max in cases:
        got = _noalloc(torch, f, tab, r_max)
        ref = _existing(f, tab, r_max)
        for k in ("rowptr", "col", "cum", "total"):
            assert np.array_equal(got[k], ref[k]), k


def test_noalloc_rejects_sizes_beyond_its_limits():
    torch = pytest.importorskip("torch")
    lib = L.load()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = _ptr(buf, C.c_double)
    t = L.kmc_table()
    t.kind = 2
    nnz = C.c_int64(0)
    err = C.create_string_buffer(256)
    rc = lib.kmc_build_neighbors_noalloc(p, p, L.KMC_NOALLOC_MAX_SITES + 1, C.byref(t), 1e-8, None, None, None, None,
                                         0, C.byref(nnz), None, err, 256)
    assert rc == L.KMC_ERR_ARG
    rc = lib.kmc_build_neighbors_noalloc(p, p, L.KMC_NOALLOC_MAX_SITES + 1, C.byref(t), 1e-8,
                                         C.cast(p, C.POINTER(C.c_int64)), None, None, p, 0, C.byref(nnz), None, err, 256)
    assert rc == L.KMC_ERR_ARG and b"takes 1.." in err.value
    # a film whose cell grid exceeds the limit: two sites far apart with a tiny radius
    pos = _dev(torch, np.array([[0.0, 0.0, 0.0], [1e-3, 1e-3, 1e-3]]), torch.float64)
    tab = tables.forster_2d()
    g = [_dev(torch, x, torch.float64) for x in tab["grids"]]
    r = _dev(torch, np.ravel(tab["rate"]), torch.float64)
    t.n[0], t.n[1] = g[0].numel(), g[1].numel()
    t.grid[0], t.grid[1] = _ptr(g[0], C.c_double), _ptr(g[1], C.c_double)
    t.rate = _ptr(r, C.c_double)
    rowptr = torch.zeros(3, dtype=torch.int64, device="cuda")
    rc = lib.kmc_build_neighbors_noalloc(_ptr(pos, C.c_double), _ptr(pos, C.c_double), 2, C.byref(t), 1e-9,
                                         _ptr(rowptr, C.c_int64), None, None, p, 0, C.byref(nnz), None, err, 256)
    assert rc == L.KMC_ERR_ARG and b"cells" in err.value


def _buffers(torch, f, tab):
    """Device inputs and a kmc_table of device pointers for one film (kept alive by the caller)."""
    keep = {"pos": _dev(torch, f.pos_m(), torch.float64), "ori": _dev(torch, f.orient, torch.float64),
            "grids": [_dev(torch, g, torch.float64) for g in tab["grids"]],
            "rate": _dev(torch, np.ravel(tab["rate"]), torch.float64)}
    t = L.kmc_table()
    t.kind = tab["kind"]
    for d, g in enumerate(keep["grids"]):
        t.n[d] = g.numel()
        t.grid[d] = _ptr(g, C.c_double)
    t.rate = _ptr(keep["rate"], C.c_double)
    return keep, t


def test_noalloc_leaves_device_free_memory_unchanged():
    # everything the call needs is allocated here first; a second call (the first may load the
    # library's kernels) must not change the device's free memory
    torch = pytest.importorskip("torch")
    lib = L.load()
    f = F.straight_tubes(40, 60.0, box_nm=(120.0, 120.0, 8.0), seed=5)
    ref = _existing(f, tables.forster_2d(1e15), 10e-9)
    keep, t = _buffers(torch, f, tables.forster_2d(1e15))
    n, cap = f.n_sites, int(ref["rowptr"][-1])
    rowptr = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    total = torch.zeros(n, dtype=torch.float64, device="cuda")
    col = torch.zeros(cap, dtype=torch.int32, device="cuda")
    cum = torch.zeros(cap, dtype=torch.float64, device="cuda")
    nnz = C.c_int64(-1)
    err = C.create_string_buffer(256)

    def call():
        rc = lib.kmc_build_neighbors_noalloc(_ptr(keep["pos"], C.c_double), _ptr(keep["ori"], C.c_double), n,
                                             C.byref(t), 10e-9, _ptr(rowptr, C.c_int64), _ptr(col, C.c_int32),
                                             _ptr(cum, C.c_double), _ptr(total, C.c_double), cap, C.byref(nnz), None,
                                             err, 256)
        assert rc == L.KMC_OK, err.value

    call()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(col.cpu().numpy(), ref["col"]) and np.array_equal(cum.cpu().numpy(), ref["cum"])


def test_noalloc_crowded_cells_match_build_neighbors():
    # 2,000 sites in about 20 x 20 x 5 nm with a 10 nm radius: 18 cells of ~110 sites each (the
    # per-cell ranking runs over many members, more than one pass of the block's threads in the
    # fullest cells)
    torch = pytest.importorskip("torch")
    f = F.straight_tubes(400, 5.0, box_nm=(15.0, 15.0, 4.0), seed=11)
    tab = tables.forster_2d(1e15)
    got = _noalloc(torch, f, tab, 10e-9)
    ref = _existing(f, tab, 10e-9)
    for k in ("rowptr", "col", "cum", "total"):
        assert np.array_equal(got[k], ref[k]), k
