"""The C-ABI library loads, exports every declared symbol, and its host-side functions match the
oracle (CPU only; no device calls)."""
import os
import re

import numpy as np

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import tables
from helpers import CASES, case_inputs, load_case
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "cntkmc.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(kmc_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = L.load()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(L.SIGNATURES)
    assert lib.kmc_version().decode().startswith("cntkmc")
    chk = L.load(checked=True)  # the KMC_CHECK build: same ABI, loaded beside the normal library
    assert chk is not lib
    for s in syms:
        assert hasattr(chk, s), s


def test_trim_and_forster_table_match_oracle():
    for name in CASES:
        d = load_case(name)
        ci = case_inputs(d)
        a = E.trim_sites(ci["pos"], ci["orient"], ci["left"], ci["right"], ci["lim"])
        b = O.trim(ci["pos"], ci["orient"], ci["left"], ci["right"], ci["lim"])
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
        assert np.array_equal(a[0].ravel(), d["ref_pos"])
        t1 = E.forster_table(ci["gamma"], *ci["grids"])
        assert np.array_equal(t1["rate"].ravel(), d["ref_table_rate"])
        for g1, g2 in zip(t1["grids"], (d["ref_table_theta"], d["ref_table_zsh"], d["ref_table_ash1"],
                                        d["ref_table_ash2"])):
            assert np.array_equal(g1, g2)


def test_trim_edge_cases():
    f = F.straight_tubes(3, 6.0, box_nm=(20, 20, 2), seed=2)
    p = f.pos_m()
    # keep nothing, keep everything, keep a slab that cuts tubes in the middle
    for lim in ([1, 2, 1, 2, 1, 2], [-1, 1, -1, 1, -1, 1], [-1, 1, 5e-9, 12e-9, -1, 1]):
        a = E.trim_sites(p, f.orient, f.left, f.right, lim)
        b = O.trim(p, f.orient, f.left, f.right, lim)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
        lk, rk = a[2], a[3]
        n = len(lk)
        assert np.all(lk < n) and np.all(rk < n)
        for i in range(n):  # links stay symmetric
            if lk[i] >= 0:
                assert rk[lk[i]] == i
            if rk[i] >= 0:
                assert lk[rk[i]] == i


def test_mesh_roundtrip(tmp_path):
    f = F.straight_tubes(5, 12.0, box_nm=(30, 30, 3), seed=4)
    F.write_mesh(f, str(tmp_path))
    pos, ori, lk, rk = E.read_mesh(str(tmp_path))
    assert np.array_equal(pos, f.pos_m()) and np.array_equal(ori, f.orient)
    assert np.array_equal(lk, f.left) and np.array_equal(rk, f.right)
    g = F.read_mesh(str(tmp_path))
    assert np.array_equal(g.pos_nm, f.pos_nm)


def test_generator_axes_are_exact_units():
    f = F.straight_tubes(200, 10.0, seed=9)
    a = f.orient
    assert np.all(((a[:, 0] * a[:, 0] + a[:, 2] * a[:, 2]) + a[:, 1] * a[:, 1]) == 1.0)


def test_tables_2d_shape():
    t = tables.forster_2d()
    assert t["kind"] == 2 and t["rate"].shape == (96, 91)
    assert np.all(t["rate"] >= 0) and t["rate"][0, 0] == 1e15 * (1e-9 / 0.5e-9) ** 6


def test_create_without_device_fails_cleanly():
    import ctypes as C

    try:
        import torch

        if torch.cuda.is_available():
            return
    except Exception:
        pass
    st = C.c_int(0)
    h = L.load().kmc_create(0, C.byref(st))
    assert not h and st.value == L.KMC_ERR_NO_DEVICE


def test_header_compiles_as_c_and_host_calls_work_from_c(tmp_path):
    # include/cntkmc.h is a C ABI: a C99 program includes it, links libcntkmc.so and calls the
    # host entry points
    import shutil
    import subprocess

    if shutil.which("gcc") is None:
        import pytest

        pytest.skip("gcc not available")
    pkg = os.path.join(ROOT, "cnt_film_monte_carlo_gb300")
    exe = str(tmp_path / "abi_from_c")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_from_c.c"), "-L", pkg, "-lcntkmc", "-Wl,-rpath," + pkg, "-lm",
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith("ok cntkmc")


GUARD_CHILD = r"""
import ctypes as C, os, resource, sys
sys.path.insert(0, sys.argv[2])
from cnt_film_monte_carlo_gb300 import _lib as L
lib = L.load()
nt, npnt = C.c_int64(0), C.c_int64(0)
vm = next(int(l.split()[1]) for l in open("/proc/self/status") if l.startswith("VmSize:")) * 1024
resource.setrlimit(resource.RLIMIT_AS, (vm + (int(sys.argv[3]) << 20), resource.RLIM_INFINITY))
rc = lib.kmc_read_mesh(sys.argv[1].encode(), C.byref(nt), C.byref(npnt), None, None, None, None)
os.write(1, b"%d" % rc)
"""


def test_host_allocation_failure_is_a_status_not_an_abort(tmp_path):
    # A C++ exception must not cross the C ABI.  With the child's address space capped a little
    # above what it uses, reading a 16 MB one-line matrix (8 M numbers: a 64 MB vector) cannot
    # allocate: inside getline the stream reports a read error (KMC_ERR_IO), in the vector's
    # growth the exception is caught at the ABI (KMC_ERR_NOMEM).  Either way the call returns
    # a status instead of ending the process in std::terminate, and never reports a mesh.
    import subprocess
    import sys

    row = b"0 " * (8 << 20) + b"\n"
    for name in ("pos.x", "pos.y", "pos.z", "orient.x", "orient.y", "orient.z"):
        (tmp_path / f"single_cnt.{name}.dat").write_bytes(row)
    codes = []
    for headroom_mb in (24, 40, 56, 72, 88):
        r = subprocess.run([sys.executable, "-c", GUARD_CHILD, str(tmp_path), ROOT, str(headroom_mb)],
                           capture_output=True, timeout=120)
        assert r.returncode == 0, (headroom_mb, r.returncode, r.stdout, r.stderr[-2000:])
        codes.append(int(r.stdout))
    assert set(codes) <= {L.KMC_ERR_IO, L.KMC_ERR_NOMEM}, codes
    assert L.KMC_ERR_NOMEM in codes, codes
