"""Python handle on one engine context (a thin layer over the C ABI in include/cntkmc.h)."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from .film import Film


def _need(ok: bool, msg: str) -> None:
    """The C ABI reads as many elements as its counts say; a numpy buffer shorter than that is
    refused here, before its pointer is passed."""
    if not ok:
        raise L.KmcError(L.KMC_ERR_ARG, msg)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Engine:
    """Owns a kmc_ctx on one CUDA device.  Every method maps to one C-ABI call and raises
    ``KmcError`` with the library's message when the call fails."""

    def __init__(self, device: int = 0, checked: bool = False):
        # checked: the KMC_CHECK build, whose kernels bounds-check their indices and counters
        self.lib = L.load(checked)
        st = C.c_int(0)
        self.h = self.lib.kmc_create(device, C.byref(st))
        if not self.h:
            raise L.KmcError(st.value, "kmc_create failed (no sm_10x CUDA device?)")
        self._keep = []
        self.n_films = 0
        self.n_exc = None
        self.n_segments = 2  # contacts mode: set by contacts_init
        self.mlp_species = 1  # rate surrogate: set by mlp_init

    def close(self):
        if getattr(self, "h", None):
            self.lib.kmc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc != L.KMC_OK:
            raise L.KmcError(rc, self.lib.kmc_last_error(self.h).decode())

    # ------------------------------------------------------------------ set-up
    def load_films(self, films, positions_m=None):
        """Load one or more films.  ``films`` is a Film or a list of Films; positions are the
        films' nm coordinates scaled by 1e-9 unless ``positions_m`` gives them in metres."""
        if isinstance(films, Film):
            films = [films]
        pos = [(_f64(positions_m[i]) if positions_m is not None else f.pos_m()) for i, f in enumerate(films)]
        off = np.zeros(len(films) + 1, dtype=np.int64)
        off[1:] = np.cumsum([f.n_sites for f in films])
        P = _f64(np.concatenate(pos))
        O = _f64(np.concatenate([f.orient for f in films]))
        Lk = np.ascontiguousarray(np.concatenate([f.left for f in films]), dtype=np.int32)
        R = np.ascontiguousarray(np.concatenate([f.right for f in films]), dtype=np.int32)
        return self.load_arrays(off, P, O, Lk, R)

    def load_arrays(self, offsets, pos_m, orient, left, right):
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        pos_m = _f64(pos_m)
        orient = _f64(orient)
        left = np.ascontiguousarray(left, dtype=np.int32)
        right = np.ascontiguousarray(right, dtype=np.int32)
        _need(offsets.ndim == 1 and len(offsets) >= 2, "load_arrays: offsets needs n_films + 1 entries")
        n = int(offsets[-1])
        _need(n >= 0 and pos_m.size == 3 * n and orient.size == 3 * n and left.size == n and right.size == n,
              f"load_arrays: {n} sites need pos and orient [n][3] and left, right [n]")
        f = L.kmc_film(len(offsets) - 1, L.ptr(offsets, C.c_int64), L.ptr(pos_m, C.c_double),
                       L.ptr(orient, C.c_double), L.ptr(left, C.c_int32), L.ptr(right, C.c_int32))
        self._check(self.lib.kmc_load_film(self.h, C.byref(f)))
        self.n_films = len(offsets) - 1
        self.offsets = offsets
        return self

    def set_table(self, table: dict):
        """``table = {"kind": 4|2|3, "grids": [...], "rate": ndarray}``; kind 3 (one 2-D table per
        chirality pair) has rate [S][S][n_dist][n_theta]."""
        grids = [_f64(g) for g in table["grids"]]
        rate_nd = _f64(table["rate"])
        rate = rate_nd.ravel()
        t = L.kmc_table()
        t.kind = int(table["kind"])
        _need(len(grids) == (4 if t.kind == L.KMC_TABLE_4D else 2), "set_table: 4 grids for kind 4, 2 otherwise")
        n_rates = math.prod(len(g) for g in grids)  # Python integers: no wrap-around
        if t.kind == L.KMC_TABLE_2D_SPECIES:
            _need(rate_nd.ndim == 4 and rate_nd.shape[0] == rate_nd.shape[1], "set_table: kind 3 rate is [S][S][nd][nt]")
            n_rates *= rate_nd.shape[0] * rate_nd.shape[1]
        _need(rate.size == n_rates, f"set_table: {rate.size} rates for grids of {n_rates} points")
        for d, g in enumerate(grids):
            t.n[d] = len(g)
            t.grid[d] = L.ptr(g, C.c_double)
        if t.kind == L.KMC_TABLE_2D_SPECIES:
            t.n[2] = rate_nd.shape[0]
        t.rate = L.ptr(rate, C.c_double)
        self._check(self.lib.kmc_set_rate_table(self.h, C.byref(t)))
        return self

    def set_species(self, species, n_species: int):
        """Chirality index of every loaded site (read by kind-3 tables)."""
        sp = np.ascontiguousarray(species, dtype=np.int32)
        _need(hasattr(self, "offsets") and sp.size == int(self.offsets[-1]),
              "set_species: one species per loaded site")
        self._check(self.lib.kmc_set_site_species(self.h, L.ptr(sp, C.c_int32), int(n_species)))
        return self

    def build(self, r_max: float) -> dict:
        st = L.kmc_nbr_stats()
        self._check(self.lib.kmc_build_neighbors(self.h, float(r_max), C.byref(st)))
        self._nbr = {k: getattr(st, k) for k, _ in L.kmc_nbr_stats._fields_}
        return dict(self._nbr)

    def set_trace(self, n_trace: int, cap: int):
        self._check(self.lib.kmc_set_trace(self.h, n_trace, cap))

    def set_hop_cap(self, cap: int):
        self._check(self.lib.kmc_set_hop_cap(self.h, cap))

    def set_msd_batches(self, batches: int):
        self._check(self.lib.kmc_set_msd_batches(self.h, batches))
        self.batches = batches

    def msd_batches(self, first: int, count: int) -> np.ndarray:
        b = getattr(self, "batches", 1)
        out = np.zeros((self.n_films, count, b, 3))
        self._check(self.lib.kmc_get_msd_batches(self.h, first, count, L.ptr(out, C.c_double)))
        return out

    def set_launch_config(self, block: int, steps_per_launch: int):
        self._check(self.lib.kmc_set_launch_config(self.h, block, steps_per_launch))

    def set_mixed_variant(self, variant: int):
        self._check(self.lib.kmc_set_mixed_variant(self.h, variant))

    def set_work_order(self, mode: int):
        """KMC_ORDER_AUTO, KMC_ORDER_SLOTS or KMC_ORDER_SPATIAL (order the mixed kernel takes excitons)."""
        self._check(self.lib.kmc_set_work_order(self.h, int(mode)))

    def work_order(self) -> int:
        v = C.c_int32()
        self._check(self.lib.kmc_get_work_order(self.h, C.byref(v)))
        return int(v.value)

    def set_graph(self, on: bool):
        self._check(self.lib.kmc_set_graph(self.h, 1 if on else 0))

    def autotune(self, dt: float, velocity: float, trial_steps: int = 2) -> dict:
        r = L.kmc_tune_result()
        self._check(self.lib.kmc_autotune(self.h, float(dt), float(velocity), int(trial_steps), C.byref(r)))
        return {"variant": r.variant, "steps_per_launch": r.steps_per_launch, "hops_per_s": r.hops_per_s}

    def init_excitons(self, n_excitons, seeds, mode=L.KMC_INJECT_UNIFORM, n_sections=5):
        ne = np.ascontiguousarray(np.broadcast_to(np.asarray(n_excitons, dtype=np.int64), (self.n_films,)))
        sd = np.ascontiguousarray(np.broadcast_to(np.asarray(seeds, dtype=np.uint64), (self.n_films,)))
        inj = L.kmc_inject(int(mode), int(n_sections), L.ptr(ne, C.c_int64), L.ptr(sd, C.c_uint64))
        self._check(self.lib.kmc_init_excitons(self.h, C.byref(inj)))
        self.n_exc = ne
        return self

    def contacts_init(self, n_segments: int, contact_pop=(1100, 0), seed: int = 100, capacity: int = 0) -> dict:
        """Contacts (steady-state flux) mode set-up (replaces init_excitons).  Returns the slab
        geometry: ymin, ymax, dy, n_initial, n_contact, capacity, area[n_segments] and the sites
        per slab stat_pop[n_segments]."""
        cfg = L.kmc_contacts(int(n_segments), (C.c_int64 * 2)(*[int(p) for p in contact_pop]), int(seed), int(capacity))
        info = L.kmc_contacts_info()
        area = np.zeros(int(n_segments))
        stat = np.zeros(int(n_segments), np.int64)
        self._check(self.lib.kmc_contacts_init(self.h, C.byref(cfg), C.byref(info), L.ptr(area, C.c_double),
                                               L.ptr(stat, C.c_int64)))
        self.n_segments = int(n_segments)
        out = {k: getattr(info, k) for k, _ in L.kmc_contacts_info._fields_}
        out["n_contact"] = tuple(info.n_contact)
        out.update(area=area, stat_pop=stat)
        self.n_exc = np.array([info.capacity], np.int64)
        return out

    def contacts_run(self, n_steps: int, dt: float, velocity: float, precision=L.KMC_PREC_MIXED):
        """n_steps of step + save_metrics + repopulate_contacts.  Returns (population
        [n_steps][n_segments], current [n_steps][n_segments - 1], n_live [n_steps]) as counts."""
        n = self.n_segments
        pop = np.zeros((max(n_steps, 1), n), np.int64)
        cur = np.zeros((max(n_steps, 1), n - 1), np.int64)
        live = np.zeros(max(n_steps, 1), np.int64)
        self._check(self.lib.kmc_contacts_run(self.h, int(n_steps), float(dt), float(velocity), int(precision),
                                              L.ptr(pop, C.c_int64), L.ptr(cur, C.c_int64), L.ptr(live, C.c_int64)))
        return pop[:n_steps], cur[:n_steps], live[:n_steps]

    def contacts_track(self, first: int, n_tracks: int, dt: float, velocity: float, max_steps: int):
        """track_particle for tracks first.. (contacts mode): a list of (path [steps][3], arrived)."""
        path = np.zeros((max(n_tracks, 1), max(max_steps, 1), 3))
        ln = np.zeros(max(n_tracks, 1), np.int64)
        arr = np.zeros(max(n_tracks, 1), np.int32)
        self._check(self.lib.kmc_contacts_track(self.h, int(first), int(n_tracks), float(dt), float(velocity),
                                                int(max_steps), L.ptr(path, C.c_double), L.ptr(ln, C.c_int64),
                                                L.ptr(arr, C.c_int32)))
        return [(path[t, :ln[t]].copy(), bool(arr[t])) for t in range(n_tracks)]

    def probe_l2(self, nbytes: int = 32 << 20, reps: int = 20) -> float:
        """L2 read bandwidth (GB/s) over an L2-resident buffer of nbytes."""
        out = C.c_double(0.0)
        self._check(self.lib.kmc_probe_l2(self.h, int(nbytes), int(reps), C.byref(out)))
        return out.value

    # ------------------------------------------------------------------ run and read
    def run(self, n_steps: int, dt: float, velocity: float, precision=L.KMC_PREC_MIXED):
        self._check(self.lib.kmc_run(self.h, int(n_steps), float(dt), float(velocity), int(precision)))

    def msd(self, first: int, count: int) -> np.ndarray:
        out = np.zeros((self.n_films, count, 3))
        self._check(self.lib.kmc_get_msd(self.h, first, count, L.ptr(out, C.c_double)))
        return out

    def stats(self) -> dict:
        st = L.kmc_run_stats()
        self._check(self.lib.kmc_get_run_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in L.kmc_run_stats._fields_}

    def excitons(self) -> dict:
        n = int(self.lib.kmc_num_excitons(self.h))
        out = {"site": np.zeros(n, np.int32), "pos": np.zeros((n, 3)), "delta": np.zeros((n, 3)),
               "ff": np.zeros(n), "heading": np.zeros(n, np.int32), "draws": np.zeros(n, np.uint64),
               "hops": np.zeros(n, np.int64)}
        self._check(self.lib.kmc_get_excitons(self.h, L.ptr(out["site"], C.c_int32), L.ptr(out["pos"], C.c_double),
                                              L.ptr(out["delta"], C.c_double), L.ptr(out["ff"], C.c_double),
                                              L.ptr(out["heading"], C.c_int32), L.ptr(out["draws"], C.c_uint64),
                                              L.ptr(out["hops"], C.c_int64)))
        return out

    def set_excitons(self, state: dict) -> None:
        """Restore a state excitons() returned (checkpoint/resume) into the set init_excitons laid
        out with the same films, counts, seeds and injection mode; MSD bins and stats restart."""
        n = int(self.lib.kmc_num_excitons(self.h))
        conv = {"site": np.int32, "pos": np.float64, "delta": np.float64, "ff": np.float64, "heading": np.int32,
                "draws": np.uint64, "hops": np.int64}
        a = {}
        for k, t in conv.items():
            v = np.ascontiguousarray(state[k], dtype=t)
            if v.shape != ((n, 3) if k in ("pos", "delta") else (n,)):
                raise ValueError(f"set_excitons: {k} has shape {v.shape} for {n} excitons")
            a[k] = v
        self._check(self.lib.kmc_set_excitons(self.h, L.ptr(a["site"], C.c_int32), L.ptr(a["pos"], C.c_double),
                                              L.ptr(a["delta"], C.c_double), L.ptr(a["ff"], C.c_double),
                                              L.ptr(a["heading"], C.c_int32), L.ptr(a["draws"], C.c_uint64),
                                              L.ptr(a["hops"], C.c_int64)))

    def neighbors(self, n_sites: int, nnz: int) -> dict:
        nb = getattr(self, "_nbr", None)
        _need(nb is not None and int(n_sites) == int(nb["n_sites"]) and int(nnz) == int(nb["nnz"]),
              "neighbors: n_sites and nnz must be the last build's")
        rowptr = np.zeros(n_sites + 1, np.int64)
        col = np.zeros(max(nnz, 1), np.int32)
        cum = np.zeros(max(nnz, 1))
        total = np.zeros(n_sites)
        self._check(self.lib.kmc_get_neighbors(self.h, L.ptr(rowptr, C.c_int64), L.ptr(col, C.c_int32),
                                               L.ptr(cum, C.c_double), L.ptr(total, C.c_double)))
        return {"rowptr": rowptr, "col": col[:nnz], "cum": cum[:nnz], "total": total}

    def trace(self, e: int, cap: int = 1 << 20):
        buf = np.zeros(cap, np.int32)
        n = self.lib.kmc_get_trace(self.h, e, L.ptr(buf, C.c_int32), cap)
        if n < 0:
            raise L.KmcError(int(n), "kmc_get_trace failed")
        return buf[: min(n, cap)].copy(), int(n)

    def selftest_uniform(self, r0: int, count: int) -> int:
        m = C.c_uint64(0)
        self._check(self.lib.kmc_selftest_uniform(self.h, r0, count, C.byref(m)))
        return int(m.value)

    def math_probe(self, x):
        x = _f64(x)
        lo = np.zeros_like(x)
        ao = np.zeros_like(x)
        self._check(self.lib.kmc_math_probe(self.h, L.ptr(x, C.c_double), len(x), L.ptr(lo, C.c_double),
                                            L.ptr(ao, C.c_double)))
        return lo, ao


# ---------------------------------------------------------------------- host-side algorithms
    # ------------------------------------------------------------ rate surrogate
    def mlp_init(self, n_species: int, d_min: float, d_max: float, log_mean: float, log_scale: float, seed: int = 0):
        sh = L.kmc_mlp_shape(int(n_species), float(d_min), float(d_max), float(log_mean), float(log_scale))
        self._check(self.lib.kmc_mlp_init(self.h, C.byref(sh), int(seed)))
        self.mlp_species = int(n_species)
        return self

    def mlp_params(self) -> np.ndarray:
        p = np.zeros(L.KMC_MLP_PARAMS(self.mlp_species), np.float32)
        self._check(self.lib.kmc_mlp_get_params(self.h, L.ptr(p, C.c_float), len(p)))
        return p

    def mlp_set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self.lib.kmc_mlp_set_params(self.h, L.ptr(p, C.c_float), len(p)))
        return self

    def mlp_set_samples(self, dist, theta, pair, log_rate):
        d, t, lr = _f64(dist), _f64(theta), _f64(log_rate)
        pr = np.ascontiguousarray(pair, dtype=np.int32)
        _need(t.size == d.size and lr.size == d.size and pr.size == d.size, "mlp_set_samples: arrays of one length")
        self._check(self.lib.kmc_mlp_set_samples(self.h, len(d), L.ptr(d, C.c_double), L.ptr(t, C.c_double),
                                                 L.ptr(pr, C.c_int32), L.ptr(lr, C.c_double)))
        return self

    def mlp_gradient(self, first: int, count: int):
        g = np.zeros(L.KMC_MLP_PARAMS(self.mlp_species), np.float32)
        loss = C.c_double(0)
        self._check(self.lib.kmc_mlp_gradient(self.h, int(first), int(count), L.ptr(g, C.c_float), C.byref(loss)))
        return g, loss.value

    def mlp_train(self, epochs: int, batch: int, lr: float, lr_final: float, beta1=0.9, beta2=0.999, eps=1e-8) -> dict:
        cfg = L.kmc_mlp_train_cfg(int(epochs), int(batch), float(lr), float(lr_final), float(beta1), float(beta2),
                                  float(eps))
        st = L.kmc_mlp_train_stats()
        self._check(self.lib.kmc_mlp_train(self.h, C.byref(cfg), C.byref(st)))
        return {k: getattr(st, k) for k, _ in L.kmc_mlp_train_stats._fields_}

    def mlp_predict(self, dist, theta, pair) -> np.ndarray:
        d, t = _f64(dist), _f64(theta)
        pr = np.ascontiguousarray(pair, dtype=np.int32)
        _need(t.size == d.size and pr.size == d.size, "mlp_predict: arrays of one length")
        out = np.zeros(len(d))
        self._check(self.lib.kmc_mlp_predict(self.h, len(d), L.ptr(d, C.c_double), L.ptr(t, C.c_double),
                                             L.ptr(pr, C.c_int32), L.ptr(out, C.c_double)))
        return out

    def mlp_rate_table(self, dist, theta) -> np.ndarray:
        d, t = _f64(dist), _f64(theta)
        S = self.mlp_species
        _table_size((S, S, len(d), len(t)), "mlp_rate_table")
        out = np.zeros((S, S, len(d), len(t)))
        self._check(self.lib.kmc_mlp_rate_table(self.h, len(d), L.ptr(d, C.c_double), len(t), L.ptr(t, C.c_double),
                                                L.ptr(out, C.c_double)))
        return out


def species_rates(model: dict, dist, theta, donor, acceptor) -> np.ndarray:
    """The chirality-resolved labeller (kmc_species_rates) for pairs donor[i] -> acceptor[i]."""
    lib = L.load()
    e, dia = _f64(model["energy"]), _f64(model["diameter"])
    m = L.kmc_species_model(len(e), float(model["gamma_0"]), L.ptr(e, C.c_double), L.ptr(dia, C.c_double),
                            float(model["diameter_ref"]), float(model["width"]), float(model["kT"]),
                            float(model["floor"]), float(model["near_field"]))
    d, t = _f64(dist), _f64(theta)
    a = np.ascontiguousarray(donor, dtype=np.int32)
    b = np.ascontiguousarray(acceptor, dtype=np.int32)
    _need(t.size == d.size and a.size == d.size and b.size == d.size, "species_rates: arrays of one length")
    _need(e.size == int(model.get("n_species", e.size)) == dia.size, "species_rates: energy and diameter per species")
    out = np.zeros(len(d))
    rc = lib.kmc_species_rates(C.byref(m), len(d), L.ptr(d, C.c_double), L.ptr(t, C.c_double), L.ptr(a, C.c_int32),
                               L.ptr(b, C.c_int32), L.ptr(out, C.c_double))
    if rc != L.KMC_OK:
        raise L.KmcError(rc, "kmc_species_rates failed")
    return out


def _grid_n(spec, what: str) -> int:
    """A grid's point count {start, end, n}[2], checked as the library checks it (a number in
    [1, 2^31 - 1]) before the output arrays are sized from it."""
    x = float(spec[2])
    if not (1.0 <= x <= 2147483647.0):
        raise L.KmcError(L.KMC_ERR_ARG, f"{what}: point count {spec[2]!r} is not in [1, 2^31 - 1]")
    return int(x)


def _table_size(ns, what: str) -> int:
    """Entries of a table with grid sizes ns, refused past 2^34 (128 GiB of rates) before anything
    is allocated, as the C++ driver refuses it."""
    p = 1
    for k in ns:
        p *= int(k)
    if p > 1 << 34:
        raise L.KmcError(L.KMC_ERR_ARG, f"{what}: rate table too large ({p} entries)")
    return p


def trim_sites(pos_m, orient, left, right, lim):
    """trim_scats on copies; returns the kept (pos, orient, left, right)."""
    lib = L.load()
    pos = _f64(pos_m).copy()
    ori = _f64(orient).copy()
    lk = np.ascontiguousarray(left, dtype=np.int32).copy()
    rk = np.ascontiguousarray(right, dtype=np.int32).copy()
    lim = _f64(lim)
    n = lk.size
    _need(pos.size == 3 * n and ori.size == 3 * n and rk.size == n and lim.size == 6,
          "trim_sites: pos and orient [n][3], left and right [n], lim [6]")
    n_out = C.c_int64(0)
    rc = lib.kmc_trim_sites(len(lk), L.ptr(pos, C.c_double), L.ptr(ori, C.c_double), L.ptr(lk, C.c_int32),
                            L.ptr(rk, C.c_int32), L.ptr(lim, C.c_double), C.byref(n_out))
    if rc != L.KMC_OK:
        raise L.KmcError(rc, "kmc_trim_sites failed")
    n = n_out.value
    return pos[:n].copy(), ori[:n].copy(), lk[:n].copy(), rk[:n].copy()


def forster2d_table(gamma_0, distance_m, theta_deg) -> dict:
    """The 2-D (distance, folded angle) Förster-form table, built by the library."""
    lib = L.load()
    dd, th = _f64(distance_m), _f64(theta_deg)
    nd, nt = _grid_n(dd, "forster2d_table"), _grid_n(th, "forster2d_table")
    _table_size((nd, nt), "forster2d_table")
    g = [np.zeros(nd), np.zeros(nt)]
    rate = np.zeros((nd, nt))
    rc = lib.kmc_forster2d_table(float(gamma_0), L.ptr(dd, C.c_double), L.ptr(th, C.c_double), L.ptr(g[0], C.c_double),
                                 L.ptr(g[1], C.c_double), L.ptr(rate, C.c_double))
    if rc != L.KMC_OK:
        raise L.KmcError(rc, "kmc_forster2d_table failed")
    return {"kind": 2, "grids": g, "rate": rate}


def forster_table(gamma_0, theta_deg, zshift, ash1, ash2) -> dict:
    """The reference's Förster table on its 4-D grid (monte_carlo.cpp:156-200)."""
    lib = L.load()
    th, z, a1, a2 = (_f64(v) for v in (theta_deg, zshift, ash1, ash2))
    n = [_grid_n(v, "forster_table") for v in (th, z, a1, a2)]
    _table_size(n, "forster_table")
    g = [np.zeros(k) for k in n]
    rate = np.zeros(n)
    rc = lib.kmc_forster_table(float(gamma_0), L.ptr(th, C.c_double), L.ptr(z, C.c_double), L.ptr(a1, C.c_double),
                               L.ptr(a2, C.c_double), L.ptr(g[0], C.c_double), L.ptr(g[1], C.c_double),
                               L.ptr(g[2], C.c_double), L.ptr(g[3], C.c_double), L.ptr(rate, C.c_double))
    if rc != L.KMC_OK:
        raise L.KmcError(rc, "kmc_forster_table failed")
    return {"kind": 4, "grids": g, "rate": rate}


def read_mesh(directory: str):
    """Mesh directory -> (pos_m, orient, left, right) exactly as create_scatterers reads it."""
    lib = L.load()
    nt, npnt = C.c_int64(0), C.c_int64(0)
    rc = lib.kmc_read_mesh(directory.encode(), C.byref(nt), C.byref(npnt), None, None, None, None)
    if rc != L.KMC_OK:
        raise L.KmcError(rc, f"cannot read mesh in {directory}")
    n = nt.value * npnt.value
    pos = np.zeros((n, 3))
    ori = np.zeros((n, 3))
    lk = np.zeros(n, np.int32)
    rk = np.zeros(n, np.int32)
    rc = lib.kmc_read_mesh(directory.encode(), C.byref(nt), C.byref(npnt), L.ptr(pos, C.c_double),
                           L.ptr(ori, C.c_double), L.ptr(lk, C.c_int32), L.ptr(rk, C.c_int32))
    if rc != L.KMC_OK:
        raise L.KmcError(rc, f"cannot read mesh in {directory}")
    return pos, ori, lk, rk
