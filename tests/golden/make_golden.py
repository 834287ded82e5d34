"""Regenerate the golden fixtures in tests/golden/ from the reference's own code.

The reference ships no tests or golden vectors, so the fixtures are outputs of the reference's
Green-Kubo engine itself: src/monte_carlo/{particle,scatterer,monte_carlo}.cpp compiled unchanged
against the project's Armadillo shim (oracle/_ref/ref_kubo, built by ``make -C oracle ref``
from the reference sources), with the per-exciton Philox rand() and the project log/acos
interposed.  Each case stores the generated film, the config and everything the reference
produced (trimmed sites, rate table, neighbour lists, per-step MSD sums, exciton states, hop
traces).  The contacts cases come from the reference's contacts (steady-state flux) mode
(oracle/_ref/ref_contacts): per-step segment populations and interface currents, the exciton
slots after the run, and the reference's own three output files.

Needs the reference sources: set CNT_REFERENCE_DIR to the reference checkout (the script stops
with a message when it is unset); the fixtures themselves are self-contained.
Run: CNT_REFERENCE_DIR=<checkout> python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cnt_film_monte_carlo_gb300 import film as F  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES = {
    # reference Green-Kubo set-up: trimmed film, central injection cell, removal slab, Förster table
    "ref_forster_region": dict(tubes=12, length=40.0, box=(60, 60, 6), film_seed=3, rate="forster",
                               trim=([5e-9, 55e-9], [-1e-6, 1e-6], [-1e-6, 1e-6]), r_max=10e-9, sections=3,
                               n_exc=200, dt=1e-14, steps=40, seed=1234, n_trace=16),
    # slower "wong" rates, longer steps (more free-flight crossings), wider cutoff
    "ref_wong_region": dict(tubes=10, length=30.0, box=(40, 40, 8), film_seed=11, rate="wong",
                            trim=([-1e-6, 1e-6], [2e-9, 38e-9], [-1e-6, 1e-6]), r_max=12e-9, sections=5,
                            n_exc=150, dt=2e-13, steps=30, seed=7, n_trace=16),
    # a T-junction and a crossing, with sites at whole nanometres and a 2 nm cutoff: many sites lie
    # exactly on cell boundaries (x - xmin = k r), where create_scatterer_buckets' truncating
    # division and the 27-cell order decide the order of every neighbour row
    "ref_tjunction_cells": dict(film="tjunction", rate="forster", trim=([-1e-6, 1e-6], [-1e-6, 1e-6], [-1e-6, 1e-6]),
                                r_max=2e-9, sections=3, n_exc=120, dt=2e-14, steps=40, seed=21, n_trace=16),
}


def tjunction_film(n_pts=9):
    """Six tubes of n_pts sites 1 nm apart (nm): A along x at y = z = 0; B along y from (4, 1, 0),
    ending 1 nm from A's middle site (a T-junction); C along x at y = 4, z = 1, crossing 1 nm over
    B; D along z at (4, 4.5); E and F along x off the grid, at (y, z) = (2.5, 2.5) and (7.5, 6)
    starting at x = 0.5."""
    tubes = [((0.0, 0.0, 0.0), (1.0, 0.0, 0.0)), ((4.0, 1.0, 0.0), (0.0, 1.0, 0.0)),
             ((0.0, 4.0, 1.0), (1.0, 0.0, 0.0)), ((4.0, 4.5, 0.0), (0.0, 0.0, 1.0)),
             ((0.5, 2.5, 2.5), (1.0, 0.0, 0.0)), ((0.5, 7.5, 6.0), (1.0, 0.0, 0.0))]
    pos, ori, left, right = [], [], [], []
    for t, (p0, u) in enumerate(tubes):
        for k in range(n_pts):
            i = t * n_pts + k
            pos.append(tuple(p0[c] + k * u[c] for c in range(3)))
            ori.append(u)
            left.append(i - 1 if k > 0 else -1)
            right.append(i + 1 if k < n_pts - 1 else -1)
    return F.Film(np.array(pos), np.array(ori), np.array(left, np.int32), np.array(right, np.int32),
                  np.arange(0, len(tubes) * n_pts + 1, n_pts, dtype=np.int64))


def make_case(name, c, tmp):
    if c.get("film") == "tjunction":
        f = tjunction_film()
    else:
        f = F.straight_tubes(c["tubes"], c["length"], box_nm=c["box"], seed=c["film_seed"])
    mesh = os.path.join(tmp, name, "mesh")
    F.write_mesh(f, mesh)
    mc = {
        "mesh input directory": mesh, "output directory": os.path.join(tmp, name, "out"), "keep old results": False,
        "rate type": c["rate"], "zshift [m]": [1.5e-9, 10e-9, 11], "axis shift 1 [m]": [-10e-9, 10e-9, 11],
        "axis shift 2 [m]": [-10e-9, 10e-9, 11], "theta [degrees]": [0, 180, 21], "temperature [kelvin]": 300,
        "max hopping radius [m]": c["r_max"],
        "trim limits": {"xlim": c["trim"][0], "ylim": c["trim"][1], "zlim": c["trim"][2]},
        "exciton velocity [m/s]": 2e5, "monte carlo time step": c["dt"],
        "number of sections for injection region": c["sections"],
        "maximum time for kubo simulation [seconds]": c["dt"] * c["steps"],
        "number of particles for kubo simulation": c["n_exc"],
    }
    cfg_path = os.path.join(tmp, name, "input.json")
    with open(cfg_path, "w") as fh:
        json.dump({"exciton monte carlo": mc}, fh)
    info, R = O.run_reference(cfg_path, os.path.join(tmp, name, "ref.bin"), c["steps"], c["seed"],
                              n_trace=c["n_trace"], trace_cap=1 << 16, dump_csr=True)
    out = {
        "film_pos_nm": f.pos_nm, "film_orient": f.orient, "film_left": f.left, "film_right": f.right,
        "config": np.frombuffer(json.dumps({k: v for k, v in mc.items() if "directory" not in k}).encode(), np.uint8),
        "seed": np.uint64(c["seed"]), "steps": np.int64(c["steps"]),
    }
    for k, v in R.items():
        out["ref_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, info, {k: v.shape for k, v in out.items() if hasattr(v, "shape") and v.size > 1000})


# contacts (steady-state flux) mode: the reference's init / step / save_metrics / repopulate,
# with its hard-coded contact populations (1100, 0)
CONTACT_CASES = {
    "ref_contacts_5seg": dict(tubes=12, length=40.0, box=(60, 60, 6), film_seed=3,
                              trim=([5e-9, 55e-9], [-1e-6, 1e-6], [-1e-6, 1e-6]), r_max=10e-9, n_seg=5, dt=1e-14,
                              steps=20, seed=1234, tracks=4),
    "ref_contacts_8seg": dict(tubes=20, length=30.0, box=(80, 80, 8), film_seed=11,
                              trim=([-1e-6, 1e-6], [2e-9, 78e-9], [-1e-6, 1e-6]), r_max=12e-9, n_seg=8, dt=3e-14,
                              steps=12, seed=99, tracks=0),
    # sites on the slab boundaries: tubes along y with sites at whole nanometres and slabs of 2 nm
    # put sites exactly on every boundary (k * 1e-9 rounds the same way as i * dy), where the
    # reference's half-open segments, inclusive contacts and <, >= interface tests decide
    "ref_contacts_grid": dict(film="grid", r_max=3e-9, n_seg=4, dt=1e-14, steps=15, seed=5,
                              trim=([-1e-6, 1e-6], [-1e-6, 1e-6], [-1e-6, 1e-6]), tracks=2),
    # two slabs: the contacts share the sites at y = ymin + dy, so contact 1's new excitons placed
    # there are removed again by contact 2 in the same repopulation
    "ref_contacts_grid2": dict(film="grid", r_max=3e-9, n_seg=2, dt=1e-14, steps=10, seed=8,
                               trim=([-1e-6, 1e-6], [-1e-6, 1e-6], [-1e-6, 1e-6]), tracks=0),
}
CONTACT_FILES = ("population_profile.dat", "region_current.dat", "scatterer_statistics.dat")


def grid_film(nx=4, nz=3, n_pts=9):
    """Tubes along y, sites at y = 0, 1, ..., n_pts - 1 nm; tube t at x = 1.5 (t mod nx) nm,
    z = 1.25 (t div nx) nm."""
    n_t = nx * nz
    pos, ori, left, right = [], [], [], []
    for t in range(n_t):
        for k in range(n_pts):
            i = t * n_pts + k
            pos.append((1.5 * (t % nx), float(k), 1.25 * (t // nx)))
            ori.append((0.0, 1.0, 0.0))
            left.append(i - 1 if k > 0 else -1)
            right.append(i + 1 if k < n_pts - 1 else -1)
    return F.Film(np.array(pos), np.array(ori), np.array(left, np.int32), np.array(right, np.int32),
                  np.arange(0, n_t * n_pts + 1, n_pts, dtype=np.int64))


def make_contacts_case(name, c, tmp):
    if c.get("film") == "grid":
        f = grid_film()
    else:
        f = F.straight_tubes(c["tubes"], c["length"], box_nm=c["box"], seed=c["film_seed"])
    mesh = os.path.join(tmp, name, "mesh")
    F.write_mesh(f, mesh)
    out_dir = os.path.join(tmp, name, "out")
    mc = {
        "mesh input directory": mesh, "output directory": out_dir, "keep old results": False,
        "rate type": "forster", "zshift [m]": [1.5e-9, 10e-9, 11], "axis shift 1 [m]": [-10e-9, 10e-9, 11],
        "axis shift 2 [m]": [-10e-9, 10e-9, 11], "theta [degrees]": [0, 180, 21], "temperature [kelvin]": 300,
        "max hopping radius [m]": c["r_max"],
        "trim limits": {"xlim": c["trim"][0], "ylim": c["trim"][1], "zlim": c["trim"][2]},
        "exciton velocity [m/s]": 2e5, "monte carlo time step": c["dt"], "number of segments": c["n_seg"],
    }
    cfg_path = os.path.join(tmp, name, "input.json")
    with open(cfg_path, "w") as fh:
        json.dump({"exciton monte carlo": mc}, fh)
    info, R = O.run_reference_contacts(cfg_path, os.path.join(tmp, name, "ref.bin"), c["steps"], c["seed"],
                                       n_tracks=c["tracks"])
    # track_particle paths: per track the SHA-256 of its FP64 positions, track 0 in full, and the
    # reference's own particle_path.0.dat
    tl, tp = R.pop("track_len"), R.pop("track_path").reshape(-1, 3)
    off = np.concatenate([[0], np.cumsum(tl)])
    digests = [hashlib.sha256(np.ascontiguousarray(tp[off[k]:off[k + 1]]).tobytes()).digest() for k in range(len(tl))]
    out_tracks = {"ref_track_len": tl, "ref_track_sha256": np.frombuffer(b"".join(digests), np.uint8).reshape(-1, 32)}
    if len(tl):
        out_tracks["ref_track0_path"] = tp[:tl[0]]
        with open(os.path.join(out_dir, "particle_path.0.dat"), "rb") as fh:
            out_tracks["file_particle_path_0"] = np.frombuffer(fh.read(), np.uint8)
    out = {
        "film_pos_nm": f.pos_nm, "film_orient": f.orient, "film_left": f.left, "film_right": f.right,
        "config": np.frombuffer(json.dumps({k: v for k, v in mc.items() if "directory" not in k}).encode(), np.uint8),
        "seed": np.uint64(c["seed"]), "steps": np.int64(c["steps"]),
    }
    for k, v in R.items():
        out["ref_" + k] = v
    out.update(out_tracks)
    for fn in CONTACT_FILES:  # the reference's own output files, verbatim
        with open(os.path.join(out_dir, fn), "rb") as fh:
            out["file_" + fn.split(".")[0]] = np.frombuffer(fh.read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, info)


def main(names=()):
    """Regenerate the named cases (all when none is named)."""
    ref_dir = O.reference_dir()
    if ref_dir is None:
        sys.exit("make_golden.py: set CNT_REFERENCE_DIR to the reference checkout")
    O.build(ref_dir)
    with tempfile.TemporaryDirectory() as tmp:
        for name, c in CASES.items():
            if not names or name in names:
                make_case(name, c, tmp)
        for name, c in CONTACT_CASES.items():
            if not names or name in names:
                make_contacts_case(name, c, tmp)


if __name__ == "__main__":
    main(sys.argv[1:])
