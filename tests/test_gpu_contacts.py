"""Contacts (steady-state flux) mode on the GPU through the C ABI.

* golden cases: the per-step slab populations, interface currents and live counts, and every
  exciton slot after the run, equal the reference's own contacts mode (oracle/_ref/ref_contacts
  fixtures), in both precisions, with and without the CUDA graph, in both work orders;
* a second contact that keeps excitons, and a 2.4 M-slot set-up (multi-level scans of the
  empty-slot counts) against the oracle;
* too few slots is reported as KMC_ERR_CAPACITY (no fault), as the oracle reports it;
* track_particle paths equal the reference's (SHA-256 of the FP64 positions);
* the drop-in driver and the Python class write the reference's files verbatim.
"""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import contacts as CF
from cnt_film_monte_carlo_gb300 import build as B
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import monte_carlo as MC
from cnt_film_monte_carlo_gb300 import tables
from helpers import CONTACT_CASES, contacts_inputs, load_case, ref_slots
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def engine_contacts(c, pops, seed, capacity, precision, steps, dt, order=L.KMC_ORDER_AUTO, graph=True):
    e = E.Engine(0)
    e.load_arrays(np.array([0, len(c["left"])], np.int64), c["pos"], c["orient"], c["left"], c["right"])
    e.set_table(c["table"])
    e.build(c["r_max"])
    e.set_work_order(order)
    e.set_graph(graph)
    g = e.contacts_init(c["n_seg"], pops, seed, capacity)
    pop, cur, live = e.contacts_run(steps, dt, c["v"], precision)
    x = e.excitons()
    st = e.stats()
    e.close()
    return g, pop, cur, live, x, st


def assert_slots(x, R):
    """Engine slots (site -1: empty) against reference/oracle slots."""
    ns = len(R["site"])
    assert (x["site"][ns:] == -1).all()
    assert np.array_equal(x["site"][:ns], R["site"])
    m = R["site"] >= 0
    for k in ("heading", "ff", "pos"):
        assert np.array_equal(x[k][:ns][m], R[k][m]), k
    assert np.array_equal(x["draws"][:ns], R["draws"])
    assert np.array_equal(x["hops"][:ns], R["hops"].astype(np.int64))


@pytest.mark.parametrize("name", CONTACT_CASES)
@pytest.mark.parametrize("precision", [L.KMC_PREC_MIXED, L.KMC_PREC_FP64])
def test_golden_contacts(name, precision):
    d = load_case(name)
    c = contacts_inputs(d)
    g, pop, cur, live, x, st = engine_contacts(c, c["pops"], c["seed"], len(d["ref_site"]) + 64, precision,
                                               c["steps"], c["dt"])
    assert np.array_equal(g["area"], d["ref_area"])
    assert g["n_contact"] == (len(d["ref_contact1"]), len(d["ref_contact2"]))
    assert g["n_initial"] == int(d["ref_n_initial"][0])
    assert np.array_equal(pop.ravel(), d["ref_pop"])
    assert np.array_equal(cur.ravel(), d["ref_curr"])
    assert np.array_equal(live, d["ref_n_live"])
    assert_slots(x, ref_slots(d))
    assert st["hops"] == int(d["ref_hops"].sum()) and st["steps_done"] == c["steps"]


@pytest.mark.parametrize("order,graph", [(L.KMC_ORDER_SPATIAL, False), (L.KMC_ORDER_SLOTS, True),
                                         (L.KMC_ORDER_SPATIAL, True)])
def test_golden_contacts_orders_and_graph(order, graph):
    d = load_case(CONTACT_CASES[0])
    c = contacts_inputs(d)
    _, pop, cur, live, x, _ = engine_contacts(c, c["pops"], c["seed"], len(d["ref_site"]) + 64, L.KMC_PREC_MIXED,
                                              c["steps"], c["dt"], order, graph)
    assert np.array_equal(pop.ravel(), d["ref_pop"])
    assert np.array_equal(cur.ravel(), d["ref_curr"])
    assert np.array_equal(live, d["ref_n_live"])
    assert_slots(x, ref_slots(d))


def synthetic_contacts(n_seg):
    f = F.straight_tubes(40, 60.0, box_nm=(120.0, 120.0, 8.0), seed=5)
    tab = tables.forster_4d(tables.FORSTER_GAMMA, (0, 180, 21), (1.5e-9, 10e-9, 11), (-10e-9, 10e-9, 11),
                            (-10e-9, 10e-9, 11))
    return dict(pos=f.pos_m(), orient=f.orient, left=f.left, right=f.right, table=tab, r_max=10e-9, v=2e5,
                n_seg=n_seg)


def oracle_slots(sim, n):
    o = sim.excitons()
    return {k: o[k][:n] for k in ("site", "heading", "ff", "pos", "draws", "hops")}


@pytest.mark.parametrize("precision", [L.KMC_PREC_MIXED, L.KMC_PREC_FP64])
def test_second_contact_population_matches_oracle(precision):
    c = synthetic_contacts(6)
    pops, seed, steps, dt = (700, 300), 42, 10, 2e-14
    g, pop, cur, live, x, _ = engine_contacts(c, pops, seed, 0, precision, steps, dt)
    sim = O.Sim(c["pos"], c["orient"], c["left"], c["right"], c["table"], c["r_max"], c["v"], n_threads=8)
    og = sim.contacts_init(c["n_seg"], pops[0], pops[1], seed, g["capacity"])
    opop, ocur, olive = sim.contacts_step(dt, steps)
    assert np.array_equal(g["area"], og["area"]) and np.array_equal(g["stat_pop"], og["stat_pop"])
    assert np.array_equal(pop, opop) and np.array_equal(cur, ocur) and np.array_equal(live, olive)
    assert (pop[:, -1] > 0).all() and np.abs(cur).sum() > 0
    assert_slots(x, oracle_slots(sim, g["capacity"]))


def test_many_slots_match_oracle():
    # 2.4 M slots: the empty-slot counts of 9375 blocks go through a two-level scan
    f = F.straight_tubes(100, 200.0, box_nm=(500.0, 500.0, 10.0), max_tilt_deg=5.0, seed=1234)
    c = dict(pos=f.pos_m(), orient=f.orient, left=f.left, right=f.right, table=tables.forster_2d(1e15),
             r_max=10e-9, v=2e5, n_seg=4)
    pops, seed, steps, dt = (300_000, 100_000), 3, 3, 2e-15
    g, pop, cur, live, x, _ = engine_contacts(c, pops, seed, 0, L.KMC_PREC_MIXED, steps, dt)
    assert g["capacity"] > 2_000_000
    sim = O.Sim(c["pos"], c["orient"], c["left"], c["right"], c["table"], c["r_max"], c["v"], n_threads=8)
    sim.contacts_init(c["n_seg"], pops[0], pops[1], seed, g["capacity"])
    opop, ocur, olive = sim.contacts_step(dt, steps)
    assert np.array_equal(pop, opop) and np.array_equal(cur, ocur) and np.array_equal(live, olive)
    assert_slots(x, oracle_slots(sim, g["capacity"]))


def test_capacity_exhaustion_is_an_error():
    d = load_case(CONTACT_CASES[0])
    c = contacts_inputs(d)
    c["n_seg"] = 2
    sim = O.Sim(c["pos"], c["orient"], c["left"], c["right"], c["table"], c["r_max"], c["v"])
    sim.contacts_init(2, 1024, 0, 5, 1024)
    with pytest.raises(RuntimeError, match="-4"):
        sim.contacts_step(1e-13, 1)
    with pytest.raises(L.KmcError) as ei:
        engine_contacts(c, (1024, 0), 5, 1024, L.KMC_PREC_MIXED, 1, 1e-13)
    assert ei.value.code == L.KMC_ERR_CAPACITY
    # enough slots: the same set-up runs
    _, pop, _, live, _, _ = engine_contacts(c, (1024, 0), 5, 2048, L.KMC_PREC_MIXED, 1, 1e-13)
    assert live[0] == 1024 and pop.sum() == 1024 and pop[0, 1] > 0  # counted before repopulation


@pytest.mark.parametrize("precision", [L.KMC_PREC_MIXED, L.KMC_PREC_FP64])
def test_golden_tracks(precision):
    # track_particle runs the plain FP64 step whatever the precision of the slots' run
    d = load_case(CONTACT_CASES[0])
    c = contacts_inputs(d)
    e = E.Engine(0)
    e.load_arrays(np.array([0, len(c["left"])], np.int64), c["pos"], c["orient"], c["left"], c["right"])
    e.set_table(c["table"])
    e.build(c["r_max"])
    e.contacts_init(c["n_seg"], c["pops"], c["seed"], 8192)
    e.contacts_run(3, c["dt"], c["v"], precision)  # the slots do not touch the tracks' streams
    n = len(d["ref_track_len"])
    tr = e.contacts_track(0, n, c["dt"], c["v"], 1 << 16)
    tail = e.contacts_track(2, 2, c["dt"], c["v"], 1 << 16)
    short = e.contacts_track(1, 1, c["dt"], c["v"], 100)[0]
    e.close()
    for k, (path, arrived) in enumerate(tr):
        assert arrived and len(path) == d["ref_track_len"][k]
        assert hashlib.sha256(np.ascontiguousarray(path).tobytes()).digest() == bytes(d["ref_track_sha256"][k])
    assert np.array_equal(tr[0][0], d["ref_track0_path"])
    assert all(np.array_equal(a[0], b[0]) for a, b in zip(tail, tr[2:]))
    assert not short[1] and np.array_equal(short[0], tr[1][0][:100])


def _contacts_json(d, tmp):
    mesh = os.path.join(tmp, "mesh")
    left = d["film_left"]
    starts = np.nonzero(left < 0)[0]
    off = np.append(starts, len(left)).astype(np.int64)
    F.write_mesh(F.Film(d["film_pos_nm"], d["film_orient"], left, d["film_right"], off), mesh)
    mc = dict(d["config"])
    mc.update({"mesh input directory": mesh, "output directory": os.path.join(tmp, "out"), "keep old results": False,
               "philox seed": int(d["seed"]), "mode": "contacts",
               "maximum time for contacts simulation [seconds]": mc["monte carlo time step"] * int(d["steps"]),
               "contacts capacity": len(d["ref_site"]) + 64,
               "number of tracked particles": len(d["ref_track_len"]), "maximum steps per tracked particle": 1 << 16})
    path = os.path.join(tmp, "input.json")
    with open(path, "w") as f:
        json.dump({"exciton monte carlo": mc}, f)
    return path


def _check_files(out_dir, d):
    n_tracks = len(d["ref_track_len"])
    assert sorted(f for f in os.listdir(out_dir) if f.startswith("particle_path.")) == sorted(
        f"particle_path.{k}.dat" for k in range(n_tracks))
    if n_tracks:
        with open(os.path.join(out_dir, "particle_path.0.dat")) as f:
            assert f.read() == bytes(d["file_particle_path_0"]).decode()
    for key, fn in (("file_scatterer_statistics", "scatterer_statistics.dat"),
                    ("file_population_profile", "population_profile.dat"),
                    ("file_region_current", "region_current.dat")):
        with open(os.path.join(out_dir, fn)) as f:
            got = f.read().splitlines(keepends=True)
        want = bytes(d[key]).decode().splitlines(keepends=True)
        if key == "file_scatterer_statistics":
            assert got == want, fn
            continue
        # header verbatim; then the rows.  The loop runs while time < max time: rounding of the
        # accumulated time can add one step past the fixture's (the reference's loop would run on)
        k = next(i for i, ln in enumerate(want) if ln.startswith("time,")) + 1
        assert got[:k] == want[:k], fn
        assert len(got) in (len(want), len(want) + 1), fn
        assert got[k:len(want)] == want[k:], fn


def _check_report(out_dir):
    # run_report.json: the flux-gradient D of every interface from the counts equals the reference's
    # post-processing of the written files (7 significant digits)
    with open(os.path.join(out_dir, "run_report.json")) as f:
        rep = json.load(f)
    assert rep["mode"] == "contacts" and rep["hops"] > 0
    with open(os.path.join(out_dir, "population_profile.dat")) as f:
        p = CF.read_population(f.read())
    with open(os.path.join(out_dir, "region_current.dat")) as f:
        c = CF.read_current(f.read())
    want = CF.flux_gradient_diffusion(p, c)
    got = np.array([np.nan if v is None else v for v in rep["flux-gradient D [m^2/s]"]], dtype=float)
    assert got.shape == want.shape
    fin = np.isfinite(want)
    assert np.array_equal(np.isfinite(got), fin)
    np.testing.assert_allclose(got[fin], want[fin], rtol=1e-5)


@pytest.mark.parametrize("name", CONTACT_CASES)
def test_driver_writes_reference_contacts_files(name, tmp_path):
    d = load_case(name)
    cfg = _contacts_json(d, str(tmp_path))
    B.build()
    r = subprocess.run([B.DRIVER, cfg], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    _check_files(os.path.join(str(tmp_path), "out"), d)
    _check_report(os.path.join(str(tmp_path), "out"))


@pytest.mark.parametrize("name", CONTACT_CASES)
def test_python_class_writes_reference_contacts_files(name, tmp_path):
    d = load_case(name)
    cfg = _contacts_json(d, str(tmp_path))
    out = MC.run(cfg)
    _check_files(out, d)
    _check_report(out)


def test_contacts_run_in_pieces_and_reinit():
    # a run split over several calls equals one call; a second set-up with another slab count on
    # the same engine starts afresh
    d = load_case(CONTACT_CASES[0])
    c = contacts_inputs(d)
    e = E.Engine(0)
    e.load_arrays(np.array([0, len(c["left"])], np.int64), c["pos"], c["orient"], c["left"], c["right"])
    e.set_table(c["table"])
    e.build(c["r_max"])
    e.contacts_init(3, (400, 100), 9, 0)
    e.contacts_run(2, c["dt"], c["v"], L.KMC_PREC_MIXED)
    e.contacts_init(c["n_seg"], c["pops"], c["seed"], len(d["ref_site"]) + 64)
    parts = [e.contacts_run(k, c["dt"], c["v"], L.KMC_PREC_MIXED) for k in (1, 1, 3, c["steps"] - 5)]
    x = e.excitons()
    e.close()
    pop = np.concatenate([p[0] for p in parts])
    cur = np.concatenate([p[1] for p in parts])
    live = np.concatenate([p[2] for p in parts])
    assert np.array_equal(pop.ravel(), d["ref_pop"])
    assert np.array_equal(cur.ravel(), d["ref_curr"])
    assert np.array_equal(live, d["ref_n_live"])
    assert_slots(x, ref_slots(d))


def test_contacts_at_scale_orders_and_precisions_agree():
    # the cfg4 film (10.8 M sites), 20 slabs, 6 M initial excitons in 13 M slots: mixed precision
    # in spatial and slot order equals the plain FP64 kernel, slot for slot
    f = F.lognormal_tubes(20000, 500.0, 0.4, (5000.0, 5000.0, 50.0), seed=7)
    c = dict(pos=f.pos_m(), orient=f.orient, left=f.left, right=f.right, table=tables.forster_2d(1e15),
             r_max=10e-9, v=2e5, n_seg=20)
    pops, seed, steps, dt = (500_000, 100_000), 4, 2, 2e-13
    runs = []
    for prec, order in ((L.KMC_PREC_MIXED, L.KMC_ORDER_SPATIAL), (L.KMC_PREC_MIXED, L.KMC_ORDER_SLOTS),
                        (L.KMC_PREC_FP64, L.KMC_ORDER_AUTO)):
        g, pop, cur, live, x, st = engine_contacts(c, pops, seed, 0, prec, steps, dt, order)
        runs.append((g, pop, cur, live, x, st))
    g0, pop0, cur0, live0, x0, st0 = runs[0]
    assert g0["n_initial"] > 5_000_000 and g0["capacity"] > 10_000_000
    assert (pop0.sum(axis=1) > 5_000_000).all() and np.abs(cur0).sum() > 0 and (live0 > 5_000_000).all()
    for g, pop, cur, live, x, st in runs[1:]:
        assert np.array_equal(pop, pop0) and np.array_equal(cur, cur0) and np.array_equal(live, live0)
        for k in ("site", "pos", "ff", "heading", "draws", "hops"):
            assert np.array_equal(x[k], x0[k]), k
        assert st["hops"] == st0["hops"]


def test_contacts_argument_and_state_errors():
    d = load_case(CONTACT_CASES[0])
    c = contacts_inputs(d)
    e = E.Engine(0)
    e.load_arrays(np.array([0, len(c["left"])], np.int64), c["pos"], c["orient"], c["left"], c["right"])
    e.set_table(c["table"])
    e.build(c["r_max"])
    for args in ((1, (10, 0)), (5000, (10, 0)), (4, (-1, 0)), (4, (10, 1 << 40))):
        with pytest.raises(L.KmcError) as ei:
            e.contacts_init(args[0], args[1], 1, 0)
        assert ei.value.code == L.KMC_ERR_ARG
    with pytest.raises(L.KmcError) as ei:  # the contacts calls need the set-up first
        e.contacts_run(1, c["dt"], c["v"], L.KMC_PREC_MIXED)
    assert ei.value.code == L.KMC_ERR_STATE
    with pytest.raises(L.KmcError) as ei:
        e.contacts_track(0, 1, c["dt"], c["v"], 10)
    assert ei.value.code == L.KMC_ERR_STATE
    e.contacts_init(4, (50, 10), 1, 0)
    with pytest.raises(L.KmcError) as ei:  # Green-Kubo steps are refused on the contacts slots
        e.run(1, c["dt"], c["v"], L.KMC_PREC_MIXED)
    assert ei.value.code == L.KMC_ERR_STATE
    pop, _, live = e.contacts_run(2, c["dt"], c["v"], L.KMC_PREC_MIXED)
    assert live[-1] > 0
    e.init_excitons(100, 3, L.KMC_INJECT_UNIFORM)  # back to Green-Kubo: contacts calls refused
    e.run(1, c["dt"], c["v"], L.KMC_PREC_MIXED)
    with pytest.raises(L.KmcError) as ei:
        e.contacts_run(1, c["dt"], c["v"], L.KMC_PREC_MIXED)
    assert ei.value.code == L.KMC_ERR_STATE
    e.close()
    # two films: contacts mode runs one
    f2 = F.straight_tubes(10, 20.0, box_nm=(40, 40, 6), seed=2)
    e = E.Engine(0)
    e.load_films([f2, f2])
    e.set_table(c["table"])
    e.build(c["r_max"])
    with pytest.raises(L.KmcError) as ei:
        e.contacts_init(4, (10, 0), 1, 0)
    assert ei.value.code == L.KMC_ERR_ARG
    e.close()


@pytest.mark.parametrize("change", ["build", "table", "film", "trace", "batches"])
def test_contacts_refused_after_buffers_change(change):
    # every call that reallocates the sites, rows, trace or exciton buffers ends the contacts
    # set-up: the captured contacts step holds the old buffers' addresses, so running it would
    # read freed memory; the library refuses instead, and a fresh set-up runs again
    d = load_case(CONTACT_CASES[0])
    c = contacts_inputs(d)
    off = np.array([0, len(c["left"])], np.int64)
    e = E.Engine(0)
    e.load_arrays(off, c["pos"], c["orient"], c["left"], c["right"])
    e.set_table(c["table"])
    e.build(c["r_max"])
    e.contacts_init(4, (50, 10), 1, 0)
    e.contacts_run(2, c["dt"], c["v"], L.KMC_PREC_MIXED)
    if change == "build":
        e.build(c["r_max"])
    elif change == "table":
        e.set_table(c["table"])
    elif change == "film":
        e.load_arrays(off, c["pos"], c["orient"], c["left"], c["right"])
    elif change == "trace":
        e.set_trace(4, 64)
    else:
        e.set_msd_batches(2)
    for call in (lambda: e.contacts_run(1, c["dt"], c["v"], L.KMC_PREC_MIXED),
                 lambda: e.contacts_track(0, 1, c["dt"], c["v"], 10)):
        with pytest.raises(L.KmcError) as ei:
            call()
        assert ei.value.code == L.KMC_ERR_STATE
    if change in ("table", "film"):
        e.set_table(c["table"])
        e.build(c["r_max"])
    e.contacts_init(4, (50, 10), 1, 0)
    _, _, live = e.contacts_run(2, c["dt"], c["v"], L.KMC_PREC_MIXED)
    assert live[-1] > 0
    e.close()
