"""The drop-in surfaces end to end on the GPU: `cntkmc_run input.json` (the reference's main) and
the Python `monte_carlo` class, each driven by an input.json built from a golden case, must
write the reference's MSD file with the reference's numbers (the golden fixtures are outputs of
the reference's own code under the same Philox streams).
"""
import json
import os
import subprocess

import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import build as B
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import monte_carlo as MC
from helpers import CASES, load_case

pytestmark = pytest.mark.gpu


def _film_from_case(d):
    left = d["film_left"]
    starts = np.nonzero(left < 0)[0]
    offsets = np.append(starts, len(left)).astype(np.int64)
    return F.Film(d["film_pos_nm"], d["film_orient"], left, d["film_right"], offsets)


def _input_json(d, tmp, precision):
    mesh = os.path.join(tmp, "mesh")
    F.write_mesh(_film_from_case(d), mesh)
    mc = dict(d["config"])
    mc.update({"mesh input directory": mesh, "output directory": os.path.join(tmp, "out"),
               "keep old results": False, "philox seed": int(d["seed"]), "precision": precision})
    path = os.path.join(tmp, "input.json")
    with open(path, "w") as f:
        json.dump({"exciton monte carlo": mc}, f)
    return path


def _read_msd_file(out_dir):
    rows = []
    with open(os.path.join(out_dir, "particle_dispalcement.avg.squared.dat")) as f:
        for line in f:
            if line[:1] in ("+", "-"):
                rows.append([float(v) for v in line.split(",")])
    return np.array(rows)


def _header_ok(out_dir, n):
    # the reference's header (monte_carlo.cpp:384-392; showpos leaves the unsigned count bare)
    with open(os.path.join(out_dir, "particle_dispalcement.avg.squared.dat")) as f:
        head = [f.readline() for _ in range(4)]
    assert head == ["# this file contains the average of dx^2, dy^2, and dz^2 of the particle ensemble over time\n",
                    f"# number of particles: {n}\n", "\n", "time,x,y,z\n"]


def _expected(d):
    n = d["config"]["number of particles for kubo simulation"]
    return d["ref_time"], d["ref_msd"].reshape(-1, 3) / n


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_driver_writes_reference_msd(name, precision, tmp_path):
    d = load_case(name)
    cfg = _input_json(d, str(tmp_path), precision)
    B.build()
    r = subprocess.run([B.DRIVER, cfg], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = _read_msd_file(os.path.join(str(tmp_path), "out"))
    _header_ok(os.path.join(str(tmp_path), "out"), d["config"]["number of particles for kubo simulation"])
    t, msd = _expected(d)
    # main's loop runs while time < max time: accumulated rounding can add a step past the
    # fixture's (the reference's main does the same)
    assert got.shape[0] in (len(t), len(t) + 1) and got.shape[1] == 4
    got = got[:len(t)]
    np.testing.assert_allclose(got[:, 0], t, rtol=1e-6)   # the file holds %+e (7 significant digits)
    np.testing.assert_allclose(got[:, 1:], msd, rtol=1e-6, atol=1e-30)
    with open(os.path.join(str(tmp_path), "out", "input.json")) as f:  # save_json_properties
        assert json.load(f)["number of particles for kubo simulation"] == d["config"][
            "number of particles for kubo simulation"]


@pytest.mark.parametrize("name", CASES)
def test_python_class_writes_reference_msd(name, tmp_path):
    d = load_case(name)
    cfg = _input_json(d, str(tmp_path), "mixed")
    out = MC.run(cfg)
    got = _read_msd_file(out)
    _header_ok(out, d["config"]["number of particles for kubo simulation"])
    t, msd = _expected(d)
    assert got.shape[0] in (len(t), len(t) + 1)
    got = got[:len(t)]
    np.testing.assert_allclose(got[:, 0], t, rtol=1e-6)
    np.testing.assert_allclose(got[:, 1:], msd, rtol=1e-6, atol=1e-30)


def test_driver_with_a_table_saved_by_the_reference(tmp_path):
    # rate type "davoody" reads a table the reference saved (scattering_struct::save); the
    # Förster table of the golden case, saved at full precision, gives the case's MSD file
    from oracle import oracle as O
    from test_tables import save_like_reference

    name = "ref_forster_region"
    d = load_case(name)
    mc = d["config"]
    tab = O.forster_table(1e15, mc["theta [degrees]"], mc["zshift [m]"], mc["axis shift 1 [m]"],
                          mc["axis shift 2 [m]"])
    tdir = os.path.join(str(tmp_path), "table")
    os.makedirs(tdir)
    save_like_reference(tab, tdir)
    cfg = _input_json(d, str(tmp_path), "mixed")
    with open(cfg) as f:
        j = json.load(f)
    j["exciton monte carlo"].update({"rate type": "davoody", "rate table directory": tdir})
    with open(cfg, "w") as f:
        json.dump(j, f)
    B.build()
    r = subprocess.run([B.DRIVER, cfg], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = _read_msd_file(os.path.join(str(tmp_path), "out"))
    t, msd = _expected(d)
    got = got[:len(t)]
    np.testing.assert_allclose(got[:, 0], t, rtol=1e-6)
    np.testing.assert_allclose(got[:, 1:], msd, rtol=1e-6, atol=1e-30)


REPORT_KEYS = ("engine", "mode", "precision", "philox seed", "injection", "particles", "steps", "time step [s]",
               "simulated time [s]", "sites", "neighbour entries", "mean neighbours per site", "max neighbours per site",
               "neighbour build [s]", "hops", "crossings", "exact re-resolves", "device seconds",
               "hops per second (device)", "wall seconds", "hops per second (wall)", "msd batches", "fit fraction",
               "diffusion coefficient [m^2/s]", "diffusion 95% interval [m^2/s]")


@pytest.mark.parametrize("name", CASES[:1])
def test_run_reports_of_driver_and_class_agree(name, tmp_path):
    # run_report.json from cntkmc_run and from the Python class: the same counters, and the same
    # D per axis (MSD batch sums of device atomics: equal to rounding)
    d = load_case(name)
    reports = []
    for which in ("driver", "class"):
        tmp = os.path.join(str(tmp_path), which)
        os.makedirs(tmp)
        cfg = _input_json(d, tmp, "mixed")
        if which == "driver":
            B.build()
            r = subprocess.run([B.DRIVER, cfg], capture_output=True, text=True, timeout=300)
            assert r.returncode == 0, r.stderr
            out = os.path.join(tmp, "out")
        else:
            out = MC.run(cfg)
        with open(os.path.join(out, "run_report.json")) as f:
            rep = json.load(f)
        assert set(REPORT_KEYS) <= set(rep), set(REPORT_KEYS) - set(rep)
        rows = _read_msd_file(out)
        assert rep["mode"] == "kubo" and rep["precision"] == "mixed" and rep["philox seed"] == int(d["seed"])
        assert rep["steps"] == rows.shape[0] and rep["simulated time [s]"] == pytest.approx(rows[-1, 0], rel=1e-6)
        assert rep["particles"] == d["config"]["number of particles for kubo simulation"]
        assert rep["hops"] > 0 and rep["device seconds"] > 0 and rep["hops per second (device)"] > 0
        reports.append(rep)
    a, b = reports
    for k in ("particles", "steps", "sites", "neighbour entries", "max neighbours per site", "hops", "crossings",
              "exact re-resolves", "msd batches"):
        assert a[k] == b[k], k
    if a["steps"] >= 2:
        np.testing.assert_allclose(a["diffusion coefficient [m^2/s]"], b["diffusion coefficient [m^2/s]"], rtol=1e-9)
        assert all(v is not None for v in a["diffusion coefficient [m^2/s]"])
        if a["msd batches"] >= 2:
            assert all(v is not None and v > 0 for v in a["diffusion 95% interval [m^2/s]"])


BIG = 2147483647
BAD_GRIDS = [
    ({"zshift [m]": [1.5e-9, 10e-9, 0.5]}, "bad rate-table grids"),
    ({"zshift [m]": [1.5e-9, 10e-9, -3]}, "bad rate-table grids"),
    ({"axis shift 1 [m]": [-1e-9, 1e-9, 1e300]}, "bad rate-table grids"),
    ({k: [0.0, 1.0, BIG] for k in ("theta [degrees]", "zshift [m]", "axis shift 1 [m]", "axis shift 2 [m]")},
     "rate table too large"),
    ({"rate type": "forster2d", "distance [m]": [0.5e-9, 10e-9, 0]}, "bad rate-table grids"),
]


@pytest.mark.parametrize("change,message", BAD_GRIDS, ids=range(len(BAD_GRIDS)))
def test_bad_table_grids_are_refused(change, message, tmp_path):
    # a grid's point count outside [1, 2^31 - 1], or a table past 2^34 entries, is refused
    # before anything is sized from it, by the driver and by the Python class
    d = load_case(CASES[0])
    cfg = _input_json(d, str(tmp_path), "mixed")
    with open(cfg) as f:
        j = json.load(f)
    j["exciton monte carlo"].update(change)
    with open(cfg, "w") as f:
        json.dump(j, f)
    B.build()
    r = subprocess.run([B.DRIVER, cfg], capture_output=True, text=True, timeout=300)
    assert r.returncode != 0 and message in r.stdout + r.stderr, (r.returncode, r.stdout, r.stderr)
    with pytest.raises(Exception) as ei:
        MC.run(cfg)
    assert "point count" in str(ei.value) or "too large" in str(ei.value) or "grid" in str(ei.value)


def test_corrupt_saved_table_is_refused(tmp_path):
    # a saved table (rate type "davoody") whose grid or rates file holds a token that is not a
    # number is refused by the driver and by the Python class, not read short
    from oracle import oracle as O
    from test_tables import save_like_reference

    d = load_case(CASES[0])
    mc = d["config"]
    tab = O.forster_table(1e15, mc["theta [degrees]"], mc["zshift [m]"], mc["axis shift 1 [m]"],
                          mc["axis shift 2 [m]"])
    for target in ("scat_table.z_shift.dat", "scat_table.rates.dat"):
        run_dir = tmp_path / target
        tdir = run_dir / "table"
        os.makedirs(tdir)
        save_like_reference(tab, str(tdir))
        with open(tdir / target, "a") as f:
            f.write("\nnot-a-number\n")
        cfg = _input_json(d, str(run_dir), "mixed")
        with open(cfg) as f:
            j = json.load(f)
        j["exciton monte carlo"].update({"rate type": "davoody", "rate table directory": str(tdir)})
        with open(cfg, "w") as f:
            json.dump(j, f)
        B.build()
        r = subprocess.run([B.DRIVER, cfg], capture_output=True, text=True, timeout=300)
        assert r.returncode != 0 and "not a number" in r.stdout + r.stderr, (target, r.stdout, r.stderr)
        with pytest.raises(ValueError):
            MC.run(cfg)


@pytest.mark.parametrize("dt", [0.0, -1e-15, 1e-40])
def test_time_steps_that_never_reach_the_end_are_refused_by_the_driver(dt, tmp_path):
    # main.cpp's loop `while (time < max time)` would never end with these steps
    d = load_case(CASES[0])
    cfg = _input_json(d, str(tmp_path), "mixed")
    with open(cfg) as f:
        j = json.load(f)
    j["exciton monte carlo"]["monte carlo time step"] = dt
    with open(cfg, "w") as f:
        json.dump(j, f)
    B.build()
    r = subprocess.run([B.DRIVER, cfg], capture_output=True, text=True, timeout=300)
    assert r.returncode != 0 and "time step" in r.stdout + r.stderr, (r.returncode, r.stdout, r.stderr)
