"""Contacts (steady-state flux) mode on the CPU: the oracle's restatement against the reference's
own contacts mode (golden fixtures made by oracle/_ref/ref_contacts), and the host-side writers of
the three output files against the reference's files, character for character."""
import hashlib

import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import contacts as CF
from helpers import CONTACT_CASES, contacts_inputs, load_case, ref_slots
from oracle import oracle as O


def oracle_contacts(d, threads=4, capacity=None):
    c = contacts_inputs(d)
    sim = O.Sim(c["pos"], c["orient"], c["left"], c["right"], c["table"], c["r_max"], c["v"], n_threads=threads)
    cap = capacity or len(d["ref_site"]) + 64
    geo = sim.contacts_init(c["n_seg"], c["pops"][0], c["pops"][1], c["seed"], cap)
    pop, cur, live = sim.contacts_step(c["dt"], c["steps"])
    return sim, geo, pop, cur, live, c


@pytest.mark.parametrize("name", CONTACT_CASES)
def test_oracle_contacts_equals_reference(name):
    d = load_case(name)
    sim, geo, pop, cur, live, c = oracle_contacts(d)
    n = c["n_seg"]
    assert np.array_equal(geo["area"], d["ref_area"])
    assert tuple(geo["n_contact"]) == (len(d["ref_contact1"]), len(d["ref_contact2"]))
    assert np.array_equal(pop.ravel(), d["ref_pop"])
    assert np.array_equal(cur.ravel(), d["ref_curr"])
    assert np.array_equal(live, d["ref_n_live"])
    assert pop.shape == (c["steps"], n) and pop.sum(axis=1).min() > 500
    assert np.abs(cur).sum() > 0
    R = ref_slots(d)
    o = sim.excitons()
    ns = len(R["site"])
    assert (o["site"][ns:] == -1).all()
    assert np.array_equal(o["site"][:ns], R["site"])
    m = R["live"]
    for k in ("heading", "ff", "pos"):
        assert np.array_equal(o[k][:ns][m], R[k][m]), k
    assert np.array_equal(o["draws"][:ns], R["draws"])
    assert np.array_equal(o["hops"][:ns], R["hops"])


@pytest.mark.parametrize("name", CONTACT_CASES)
def test_file_writers_reproduce_reference_files(name):
    d = load_case(name)
    c = contacts_inputs(d)
    ymin, ymax = c["pos"][:, 1].min(), c["pos"][:, 1].max()
    n = c["n_seg"]
    dy = (ymax - ymin) / float(n)
    area = d["ref_area"]
    sim = O.Sim(c["pos"], c["orient"], c["left"], c["right"], c["table"], c["r_max"], c["v"])
    geo = sim.contacts_init(n, c["pops"][0], c["pops"][1], c["seed"], len(d["ref_site"]) + 64)
    stats = CF.scatterer_statistics_text(ymin, dy, geo["stat_pop"], len(c["left"]), area)
    assert stats == bytes(d["file_scatterer_statistics"]).decode()
    pop = d["ref_pop"].reshape(-1, n)
    cur = d["ref_curr"].reshape(-1, n - 1)
    t = d["ref_time"]
    ptxt = CF.population_header(area, ymin, dy) + "".join(CF.population_row(t[s], pop[s], area, dy) for s in range(len(t)))
    assert ptxt == bytes(d["file_population_profile"]).decode()
    ctxt = CF.current_header(area, ymin, dy) + "".join(CF.current_row(t[s], cur[s], area, c["dt"]) for s in range(len(t)))
    assert ctxt == bytes(d["file_region_current"]).decode()


def test_oracle_contacts_rejects_empty_contact_and_small_capacity():
    d = load_case(CONTACT_CASES[0])
    c = contacts_inputs(d)
    sim = O.Sim(c["pos"], c["orient"], c["left"], c["right"], c["table"], c["r_max"], c["v"])
    with pytest.raises(RuntimeError, match="-4"):  # fewer slots than initial excitons
        sim.contacts_init(c["n_seg"], 1100, 0, 1, 100)
    with pytest.raises(RuntimeError, match="-1"):
        sim.contacts_init(1, 1100, 0, 1, 10000)
    sim.contacts_init(c["n_seg"], 50, 20, 1, 1000)
    pop, cur, live = sim.contacts_step(c["dt"], 3)
    assert live.min() > 0 and pop.sum(axis=1).min() > 0


def track_digest(path):
    return hashlib.sha256(np.ascontiguousarray(path, dtype=np.float64).tobytes()).digest()


def test_oracle_tracks_equal_reference():
    d = load_case(CONTACT_CASES[0])
    c = contacts_inputs(d)
    sim = O.Sim(c["pos"], c["orient"], c["left"], c["right"], c["table"], c["r_max"], c["v"], n_threads=4)
    sim.contacts_init(c["n_seg"], c["pops"][0], c["pops"][1], c["seed"], 8192)
    n = len(d["ref_track_len"])
    assert n == 4
    tr = sim.contacts_track(0, n, c["dt"], 1 << 16)
    for k, (path, arrived) in enumerate(tr):
        assert arrived and len(path) == d["ref_track_len"][k]
        assert track_digest(path) == bytes(d["ref_track_sha256"][k])
    assert np.array_equal(tr[0][0], d["ref_track0_path"])
    assert CF.track_text(tr[0][0]) == bytes(d["file_particle_path_0"]).decode()
    # a track's draws do not depend on the others
    tail = sim.contacts_track(2, 2, c["dt"], 1 << 16)
    assert all(np.array_equal(a[0], b[0]) for a, b in zip(tail, tr[2:]))
    # a step cap shorter than the walk: the path stops there and the track has not arrived
    short = sim.contacts_track(1, 1, c["dt"], 100)[0]
    assert not short[1] and np.array_equal(short[0], tr[1][0][:100])


def test_oracle_contacts_per_hop_search_equals_csr():
    # the timed CPU baseline searches neighbours on every hop, as the reference does
    d = load_case(CONTACT_CASES[1])
    sim_a, _, pop_a, cur_a, live_a, c = oracle_contacts(d)
    sim_b = O.Sim(c["pos"], c["orient"], c["left"], c["right"], c["table"], c["r_max"], c["v"], n_threads=4)
    sim_b.contacts_init(c["n_seg"], c["pops"][0], c["pops"][1], c["seed"], len(d["ref_site"]) + 64)
    sim_b.use_csr(False)
    pop_b, cur_b, live_b = sim_b.contacts_step(c["dt"], c["steps"])
    assert np.array_equal(pop_a, pop_b) and np.array_equal(cur_a, cur_b) and np.array_equal(live_a, live_b)
    a, b = sim_a.excitons(), sim_b.excitons()
    for k in ("site", "ff", "draws", "hops"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("name", CONTACT_CASES)
def test_flux_gradient_diffusion_from_reference_files(name):
    # the contacts mode's D per interface as the reference's post-processing forms it
    # (visualization/monte_carlo_results.py:428-442) from the reference's own output files, against
    # the same formula on the exact counts (the files hold 7 significant digits)
    d = load_case(name)
    c = contacts_inputs(d)
    n = c["n_seg"]
    ymin, ymax = c["pos"][:, 1].min(), c["pos"][:, 1].max()
    dy = (ymax - ymin) / float(n)
    p = CF.read_population(bytes(d["file_population_profile"]).decode())
    cur = CF.read_current(bytes(d["file_region_current"]).decode())
    assert p["pop"].shape == (len(d["ref_time"]), n) and cur["current"].shape == (len(d["ref_time"]), n - 1)
    np.testing.assert_allclose(p["area"], d["ref_area"], rtol=1e-6)
    np.testing.assert_allclose(p["dy"], dy, rtol=1e-6)
    # the reference's own steps restated: averages over the steps, then steady / (diff(avg) / dy)
    want = cur["current"].mean(axis=0) / (np.diff(p["pop"].mean(axis=0)) / p["dy"][:-1])
    got = CF.flux_gradient_diffusion(p, cur)
    np.testing.assert_array_equal(got, want)
    exact = CF.flux_gradient_diffusion_from_counts(d["ref_pop"].reshape(-1, n), d["ref_curr"].reshape(-1, n - 1),
                                                   d["ref_area"], dy, c["dt"])
    fin = np.isfinite(exact) & np.isfinite(got)
    assert fin.any()
    np.testing.assert_allclose(got[fin], exact[fin], rtol=1e-5)


LIVE_CONTACTS = {
    # film, cutoff, segments, dt, steps, seed, (xlim, ylim)
    "tjunction_3seg": (("tjunction",), 2.5e-9, 3, 2e-14, 12, 17, ([-1, 1], [-1, 1])),
    "random_6seg": (("random", 16, 30.0, (50, 50, 5), 9), 8e-9, 6, 2e-14, 10, 31, ([4e-9, 46e-9], [-1, 1])),
    "grid_5seg": (("grid",), 2e-9, 5, 3e-14, 10, 2, ([-1, 1], [-1, 1])),
}


@pytest.mark.parametrize("name", sorted(LIVE_CONTACTS))
def test_oracle_contacts_equals_the_live_reference(name, tmp_path):
    """More films through the reference's own contacts mode, run right now: slab populations,
    interface currents, live counts and every exciton slot equal the oracle's bit for bit."""
    import json
    import os

    if not os.path.exists(O.REF_CONTACTS_BIN):
        pytest.skip("oracle/_ref not built: build() compiles it where the reference sources are present")
    import importlib.util

    from cnt_film_monte_carlo_gb300 import film as F

    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    film, r_max, n_seg, dt, steps, seed, (xlim, ylim) = LIVE_CONTACTS[name]
    if film[0] == "random":
        f = F.straight_tubes(film[1], film[2], box_nm=film[3], seed=film[4])
    elif film[0] == "tjunction":
        f = mg.tjunction_film()
    else:
        f = mg.grid_film()
    F.write_mesh(f, str(tmp_path / "mesh"))
    mc = {"mesh input directory": str(tmp_path / "mesh"), "output directory": str(tmp_path / "out"),
          "keep old results": False, "rate type": "forster", "zshift [m]": [1.5e-9, 10e-9, 11],
          "axis shift 1 [m]": [-10e-9, 10e-9, 11], "axis shift 2 [m]": [-10e-9, 10e-9, 11],
          "theta [degrees]": [0, 180, 21], "max hopping radius [m]": r_max,
          "trim limits": {"xlim": xlim, "ylim": ylim, "zlim": [-1, 1]}, "exciton velocity [m/s]": 2e5,
          "monte carlo time step": dt, "number of segments": n_seg}
    p = tmp_path / "in.json"
    p.write_text(json.dumps({"exciton monte carlo": mc}))
    _, R = O.run_reference_contacts(str(p), str(tmp_path / "ref.bin"), steps, seed)
    d = {"film_pos_nm": f.pos_nm, "film_orient": f.orient, "film_left": f.left, "film_right": f.right,
         "config": mc, "steps": steps, "seed": seed, **{"ref_" + k: v for k, v in R.items()}}
    sim, geo, pop, cur, live, c = oracle_contacts(d)
    assert np.array_equal(geo["area"], d["ref_area"])
    assert tuple(geo["n_contact"]) == (len(d["ref_contact1"]), len(d["ref_contact2"]))
    assert np.array_equal(pop.ravel(), d["ref_pop"]) and np.array_equal(cur.ravel(), d["ref_curr"])
    assert np.array_equal(live, d["ref_n_live"]) and pop.sum() > 0
    Rs = ref_slots(d)
    o = sim.excitons()
    ns = len(Rs["site"])
    assert (o["site"][ns:] == -1).all() and np.array_equal(o["site"][:ns], Rs["site"])
    m = Rs["live"]
    for k in ("heading", "ff", "pos"):
        assert np.array_equal(o[k][:ns][m], Rs[k][m]), k
    assert np.array_equal(o["draws"][:ns], Rs["draws"]) and np.array_equal(o["hops"][:ns], Rs["hops"])
