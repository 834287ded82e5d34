"""ctypes wrapper of the oracle (oracle/liboracle.so) -- TEST INFRASTRUCTURE.

The oracle is the CPU restatement of the reference's hot path (oracle/kmc_oracle.c).  Only
tests/, __graft_entry__.smoke() and bench.py (CPU baseline / reference leg) import this
module, and only as the test oracle or the timed CPU path -- never inside the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_kubo")
REF_TIMING_BIN = os.path.join(HERE, "_ref", "ref_kubo_timing")
REF_CONTACTS_BIN = os.path.join(HERE, "_ref", "ref_contacts")
# the reference checkout (its sources are compiled into oracle/_ref); unset: no oracle/_ref
REF_ENV = "CNT_REFERENCE_DIR"


def reference_dir():
    """The reference checkout named by $CNT_REFERENCE_DIR, or None when it is unset."""
    d = os.environ.get(REF_ENV, "")
    return d or None

_lib = None

D = C.c_double
I32 = C.c_int32
I64 = C.c_int64
U64 = C.c_uint64
PD = C.POINTER(C.c_double)
PI32 = C.POINTER(C.c_int32)
PI64 = C.POINTER(C.c_int64)
PU64 = C.POINTER(C.c_uint64)
PU32 = C.POINTER(C.c_uint32)


class orc_table(C.Structure):
    _fields_ = [("kind", C.c_int), ("n", C.c_int * 4), ("grid", PD * 4), ("rate", PD),
                ("species", C.POINTER(C.c_int32))]


def build(ref_dir: str | None = None) -> None:
    """Compile liboracle.so and, when ``ref_dir`` names a reference checkout, oracle/_ref from its
    sources."""
    targets = ["lib"]
    env = dict(os.environ)
    if ref_dir:
        if not os.path.isfile(os.path.join(ref_dir, "src", "monte_carlo", "particle.cpp")):
            raise RuntimeError(f"oracle.build: no reference sources under {ref_dir!r}")
        targets.append("ref")
        env["CNT_REFERENCE_DIR"] = ref_dir
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True, env=env)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_linspace.argtypes = [D, D, I64, PD]
        L.orc_forster_table.argtypes = [D, PD, PD, PD, PD, PD, PD, PD, PD, PD]
        L.orc_forster2d_table.argtypes = [D, PD, PD, PD, PD, PD]
        L.orc_trim.argtypes = [I64, PD, PD, PI32, PI32, PD]
        L.orc_trim.restype = I64
        L.orc_sim_create.argtypes = [I64, PD, PD, PI32, PI32, C.POINTER(orc_table), D, D, C.c_int]
        L.orc_sim_create.restype = C.c_void_p
        L.orc_sim_destroy.argtypes = [C.c_void_p]
        L.orc_find_neighbors.argtypes = [C.c_void_p, I64, PD, PI32, C.c_int]
        L.orc_find_neighbors.restype = C.c_int
        L.orc_sim_build_csr.argtypes = [C.c_void_p]
        L.orc_sim_build_csr.restype = I64
        L.orc_sim_get_csr.argtypes = [C.c_void_p, PI64, PI32, PD, PD, PD]
        L.orc_sim_domain.argtypes = [C.c_void_p, PD, PD, PI32]
        L.orc_sim_create_excitons.argtypes = [C.c_void_p, C.c_int, C.c_int, I64, U64, U64, C.c_int]
        L.orc_sim_create_excitons.restype = C.c_int
        L.orc_sim_n_inject.argtypes = [C.c_void_p]
        L.orc_sim_n_inject.restype = I64
        L.orc_sim_set_trace.argtypes = [C.c_void_p, I64, I64]
        L.orc_sim_get_trace.argtypes = [C.c_void_p, I64, PI32, I64]
        L.orc_sim_get_trace.restype = I64
        L.orc_sim_step.argtypes = [C.c_void_p, D, I64, PD]
        L.orc_sim_step.restype = C.c_int
        L.orc_sim_step_batches.argtypes = [C.c_void_p, D, I64, C.c_int, PD]
        L.orc_sim_step_batches.restype = C.c_int
        L.orc_sim_get_excitons.argtypes = [C.c_void_p, PI32, PD, PD, PD, PD, PI32, PU64, PI64]
        L.orc_sim_total_hops.argtypes = [C.c_void_p]
        L.orc_sim_total_hops.restype = I64
        L.orc_sim_total_crossings.argtypes = [C.c_void_p]
        L.orc_sim_total_crossings.restype = I64
        L.orc_contacts_init.argtypes = [C.c_void_p, C.c_int, I64, I64, U64, I64, PD, PI64, PI64]
        L.orc_contacts_init.restype = C.c_int
        L.orc_contacts_step.argtypes = [C.c_void_p, D, I64, PI64, PI64, PI64]
        L.orc_contacts_step.restype = C.c_int
        L.orc_sim_use_csr.argtypes = [C.c_void_p, C.c_int]
        L.orc_contacts_track.argtypes = [C.c_void_p, I64, C.c_int, D, I64, PD, PI64, PI32]
        L.orc_contacts_track.restype = C.c_int
        L.orc_log_export.argtypes = [D]
        L.orc_log_export.restype = D
        L.orc_log_array.argtypes = [PD, PD, I64]
        L.orc_acos_export.argtypes = [D]
        L.orc_acos_export.restype = D
        L.orc_philox_export.argtypes = [PU32, PU32, PU32]
        L.orc_rand_export.argtypes = [U64, U64, U64]
        L.orc_rand_export.restype = C.c_int
        L.orc_select_export.argtypes = [PD, C.c_int, D]
        L.orc_select_export.restype = C.c_int
        L.orc_index_min_export.argtypes = [PD, C.c_int, D]
        L.orc_index_min_export.restype = C.c_int
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def log(x: float) -> float:
    return lib().orc_log_export(float(x))


def log_array(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    lib().orc_log_array(_p(x, D), _p(out, D), len(x))
    return out


def acos(x: float) -> float:
    return lib().orc_acos_export(float(x))


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().orc_philox_export(_p(c, C.c_uint32), _p(k, C.c_uint32), _p(o, C.c_uint32))
    return o


def rand(seed: int, stream: int, n: int) -> int:
    return lib().orc_rand_export(seed, stream, n)


def select(cum, dice: float) -> int:
    c = np.ascontiguousarray(cum, dtype=np.float64)
    return lib().orc_select_export(_p(c, C.c_double), len(c), float(dice))


def index_min(grid, x: float) -> int:
    g = np.ascontiguousarray(grid, dtype=np.float64)
    return lib().orc_index_min_export(_p(g, C.c_double), len(g), float(x))


def linspace(a, b, n):
    out = np.zeros(max(int(n), 1), dtype=np.float64)
    lib().orc_linspace(a, b, int(n), _p(out, C.c_double))
    return out[: int(n)]


def forster2d_table(gamma_0=1e15, distance_m=(0.5e-9, 10e-9, 96), theta_deg=(0.0, 90.0, 91)):
    """The benchmark films' 2-D (distance, folded angle) Förster-form table: dict(kind=2,
    grids=[distance m, theta rad], rate=ndarray[nd, nt])."""
    dd = np.ascontiguousarray(distance_m, dtype=np.float64)
    th = np.ascontiguousarray(theta_deg, dtype=np.float64)
    nd, nt = int(dd[2]), int(th[2])
    g = [np.zeros(nd), np.zeros(nt)]
    rate = np.zeros((nd, nt))
    lib().orc_forster2d_table(float(gamma_0), _p(dd, D), _p(th, D), _p(g[0], D), _p(g[1], D), _p(rate, D))
    return {"kind": 2, "grids": g, "rate": rate}


def forster_table(gamma_0, theta_deg, zsh, ash1, ash2):
    """create_forster_scatt_table: returns dict(kind=4, grids=[...], rate=ndarray[nt, nz, n1, n2])."""
    th = np.asarray(theta_deg, dtype=np.float64)
    z = np.asarray(zsh, dtype=np.float64)
    a1 = np.asarray(ash1, dtype=np.float64)
    a2 = np.asarray(ash2, dtype=np.float64)
    nt, nz, n1, n2 = int(th[2]), int(z[2]), int(a1[2]), int(a2[2])
    g = [np.zeros(nt), np.zeros(nz), np.zeros(n1), np.zeros(n2)]
    rate = np.zeros((nt, nz, n1, n2))
    lib().orc_forster_table(gamma_0, _p(th, D), _p(z, D), _p(a1, D), _p(a2, D), _p(g[0], D), _p(g[1], D),
                            _p(g[2], D), _p(g[3], D), _p(rate, D))
    return {"kind": 4, "grids": g, "rate": rate}


def trim(pos, orient, left, right, lim):
    """trim_scats in place on copies; returns (pos, orient, left, right) of the kept sites."""
    pos = np.ascontiguousarray(pos, dtype=np.float64).copy()
    orient = np.ascontiguousarray(orient, dtype=np.float64).copy()
    left = np.ascontiguousarray(left, dtype=np.int32).copy()
    right = np.ascontiguousarray(right, dtype=np.int32).copy()
    lim = np.asarray(lim, dtype=np.float64)
    n = lib().orc_trim(len(left), _p(pos, D), _p(orient, D), _p(left, C.c_int32), _p(right, C.c_int32), _p(lim, D))
    return pos[:n].copy(), orient[:n].copy(), left[:n].copy(), right[:n].copy()


class Sim:
    """The oracle engine over one film (positions in metres, [n][3])."""

    def __init__(self, pos_m, orient, left, right, table, r_max, velocity, n_threads=1, species=None):
        """``table`` as the engine takes it; kind 3 (one 2-D table per chirality pair, rate
        [S][S][n_dist][n_theta]) also needs ``species`` (each site's chirality)."""
        self.pos = np.ascontiguousarray(pos_m, dtype=np.float64)
        self.orient = np.ascontiguousarray(orient, dtype=np.float64)
        self.left = np.ascontiguousarray(left, dtype=np.int32)
        self.right = np.ascontiguousarray(right, dtype=np.int32)
        self.n = len(self.left)
        self._grids = [np.ascontiguousarray(g, dtype=np.float64) for g in table["grids"]]
        self._rate = np.ascontiguousarray(table["rate"], dtype=np.float64)
        t = orc_table()
        t.kind = table["kind"]
        for d, g in enumerate(self._grids):
            t.n[d] = len(g)
            t.grid[d] = _p(g, D)
        t.rate = _p(self._rate, D)
        if table["kind"] == 3:
            self._species = np.ascontiguousarray(species, dtype=np.int32)
            t.n[2] = self._rate.shape[0]
            t.species = _p(self._species, C.c_int32)
        self._t = t
        self.h = lib().orc_sim_create(self.n, _p(self.pos, D), _p(self.orient, D), _p(self.left, C.c_int32),
                                      _p(self.right, C.c_int32), C.byref(t), r_max, velocity, n_threads)
        if not self.h:
            raise RuntimeError("orc_sim_create failed")
        self.n_exc = 0

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_sim_destroy(h)
            self.h = None

    def neighbors(self, site, cap=4096):
        cum = np.zeros(cap)
        col = np.zeros(cap, dtype=np.int32)
        k = lib().orc_find_neighbors(self.h, site, _p(cum, D), _p(col, C.c_int32), cap)
        return cum[:k].copy(), col[:k].copy()

    def build_csr(self):
        nnz = lib().orc_sim_build_csr(self.h)
        rowptr = np.zeros(self.n + 1, dtype=np.int64)
        col = np.zeros(max(nnz, 1), dtype=np.int32)
        cum = np.zeros(max(nnz, 1))
        total = np.zeros(self.n)
        inv = np.zeros(self.n)
        lib().orc_sim_get_csr(self.h, _p(rowptr, C.c_int64), _p(col, C.c_int32), _p(cum, D), _p(total, D), _p(inv, D))
        return {"rowptr": rowptr, "col": col[:nnz], "cum": cum[:nnz], "total": total, "inv_total": inv}

    def domain(self):
        mn = np.zeros(3)
        mx = np.zeros(3)
        nc = np.zeros(3, dtype=np.int32)
        lib().orc_sim_domain(self.h, _p(mn, D), _p(mx, D), _p(nc, C.c_int32))
        return mn, mx, nc

    def set_trace(self, n_trace, cap):
        lib().orc_sim_set_trace(self.h, n_trace, cap)

    def create_excitons(self, mode, n_sections, n_exc, seed, stream_base=0, use_csr=True):
        rc = lib().orc_sim_create_excitons(self.h, mode, n_sections, n_exc, seed, stream_base, 1 if use_csr else 0)
        if rc != 0:
            raise RuntimeError(f"orc_sim_create_excitons failed ({rc})")
        self.n_exc = n_exc

    def n_inject(self):
        return lib().orc_sim_n_inject(self.h)

    def step(self, dt, n_steps=1):
        msd = np.zeros((max(n_steps, 1), 3))
        lib().orc_sim_step(self.h, dt, n_steps, _p(msd, D))
        return msd[:n_steps]

    def step_batches(self, dt, n_steps, batches):
        out = np.zeros((max(n_steps, 1), batches, 3))
        lib().orc_sim_step_batches(self.h, dt, n_steps, batches, _p(out, D))
        return out[:n_steps]

    def excitons(self):
        n = self.n_exc
        out = {
            "site": np.zeros(n, dtype=np.int32),
            "pos": np.zeros((n, 3)),
            "old": np.zeros((n, 3)),
            "delta": np.zeros((n, 3)),
            "ff": np.zeros(n),
            "heading": np.zeros(n, dtype=np.int32),
            "draws": np.zeros(n, dtype=np.uint64),
            "hops": np.zeros(n, dtype=np.int64),
        }
        lib().orc_sim_get_excitons(self.h, _p(out["site"], C.c_int32), _p(out["pos"], D), _p(out["old"], D),
                                   _p(out["delta"], D), _p(out["ff"], D), _p(out["heading"], C.c_int32),
                                   _p(out["draws"], C.c_uint64), _p(out["hops"], C.c_int64))
        return out

    def contacts_init(self, n_seg, pop1, pop2, seed, capacity):
        """Contacts mode set-up; returns dict(area, stat_pop, n_contact)."""
        area = np.zeros(n_seg)
        stat = np.zeros(n_seg, dtype=np.int64)
        nc = np.zeros(2, dtype=np.int64)
        rc = lib().orc_contacts_init(self.h, n_seg, pop1, pop2, seed, capacity, _p(area, D), _p(stat, C.c_int64),
                                     _p(nc, C.c_int64))
        if rc != 0:
            raise RuntimeError(f"orc_contacts_init failed ({rc})")
        self.n_exc = capacity
        self.n_seg = n_seg
        return {"area": area, "stat_pop": stat, "n_contact": nc}

    def contacts_step(self, dt, n_steps):
        """Returns (pop[n_steps][n_seg], curr[n_steps][n_seg-1], n_live[n_steps])."""
        n = self.n_seg
        pop = np.zeros((max(n_steps, 1), n), dtype=np.int64)
        curr = np.zeros((max(n_steps, 1), n - 1), dtype=np.int64)
        live = np.zeros(max(n_steps, 1), dtype=np.int64)
        rc = lib().orc_contacts_step(self.h, dt, n_steps, _p(pop, C.c_int64), _p(curr, C.c_int64),
                                     _p(live, C.c_int64))
        if rc != 0:
            raise RuntimeError(f"orc_contacts_step failed ({rc})")
        return pop[:n_steps], curr[:n_steps], live[:n_steps]

    def use_csr(self, on):
        """Hops from the CSR (True) or from the reference's per-hop neighbour search (False)."""
        lib().orc_sim_use_csr(self.h, 1 if on else 0)

    def contacts_track(self, first, n_tracks, dt, max_steps):
        """track_particle for tracks first..: a list of (path [steps][3], arrived)."""
        path = np.zeros((max(n_tracks, 1), max(max_steps, 1), 3))
        ln = np.zeros(max(n_tracks, 1), dtype=np.int64)
        arr = np.zeros(max(n_tracks, 1), dtype=np.int32)
        rc = lib().orc_contacts_track(self.h, first, n_tracks, dt, max_steps, _p(path, D), _p(ln, C.c_int64),
                                      _p(arr, C.c_int32))
        if rc != 0:
            raise RuntimeError(f"orc_contacts_track failed ({rc})")
        return [(path[t, :ln[t]].copy(), bool(arr[t])) for t in range(n_tracks)]

    def trace(self, e, cap=1 << 20):
        buf = np.zeros(cap, dtype=np.int32)
        n = lib().orc_sim_get_trace(self.h, e, _p(buf, C.c_int32), cap)
        return buf[: min(n, cap)].copy(), n

    def total_hops(self):
        return lib().orc_sim_total_hops(self.h)

    def total_crossings(self):
        return lib().orc_sim_total_crossings(self.h)


def read_ref_dump(path):
    """Read the record file written by oracle/ref_driver.cpp into a dict of arrays."""
    out = {}
    with open(path, "rb") as f:
        if f.read(8) != b"KMCREF1\n":
            raise ValueError("not a ref_driver dump")
        while True:
            name = f.read(32)
            if len(name) < 32:
                break
            dt = f.read(8).rstrip(b"\0").decode()
            n = int(np.frombuffer(f.read(8), dtype=np.int64)[0])
            dtype = np.dtype("<" + dt)
            out[name.rstrip(b"\0").decode()] = np.frombuffer(f.read(n * dtype.itemsize), dtype=dtype).copy()
    return out


def run_reference(input_json, out_path, n_steps, seed, n_trace=0, trace_cap=0, dump_csr=False, timing=False,
                  threads=1):
    """Run oracle/_ref/ref_kubo (the reference's own code) and return (json line, dump dict)."""
    import json

    exe = REF_TIMING_BIN if timing else REF_BIN
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run([exe, input_json, out_path, str(n_steps), str(seed), str(n_trace), str(trace_cap),
                        "1" if dump_csr else "0"], capture_output=True, text=True, env=env, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1]), read_ref_dump(out_path)


def run_reference_contacts(input_json, out_path, n_steps, seed, n_tracks=0, timeout=600):
    """Run oracle/_ref/ref_contacts (the reference's contacts mode, with n_tracks track_particle
    calls first) and return (json line, dump dict)."""
    import json

    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([REF_CONTACTS_BIN, input_json, out_path, str(n_steps), str(seed), str(n_tracks)],
                       capture_output=True, text=True, env=env, check=True, timeout=timeout)
    return json.loads(r.stdout.strip().splitlines()[-1]), read_ref_dump(out_path)
