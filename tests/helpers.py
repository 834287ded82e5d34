"""Shared test helpers: golden cases, oracle engines and GPU engines on the same inputs."""
from __future__ import annotations

import json
import os

import numpy as np

from cnt_film_monte_carlo_gb300 import film as F
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("ref_forster_region", "ref_wong_region", "ref_tjunction_cells")
CONTACT_CASES = ("ref_contacts_5seg", "ref_contacts_8seg", "ref_contacts_grid", "ref_contacts_grid2")


def load_case(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    d["config"] = json.loads(bytes(d["config"]).decode())
    return d


def case_inputs(d):
    """(pos_m, orient, left, right) of the untrimmed film, lim, table dict, r_max, v, dt."""
    mc = d["config"]
    pos_m = d["film_pos_nm"] * 1.0e-9
    tl = mc["trim limits"]
    lim = [*tl["xlim"], *tl["ylim"], *tl["zlim"]]
    gamma = 1e15 if mc["rate type"] == "forster" else 1e13
    return dict(pos=pos_m, orient=d["film_orient"], left=d["film_left"], right=d["film_right"], lim=lim,
                gamma=gamma, grids=(mc["theta [degrees]"], mc["zshift [m]"], mc["axis shift 1 [m]"],
                                    mc["axis shift 2 [m]"]),
                r_max=mc["max hopping radius [m]"], v=mc["exciton velocity [m/s]"], dt=mc["monte carlo time step"],
                sections=mc["number of sections for injection region"],
                n_exc=mc["number of particles for kubo simulation"])


def ref_traces(d):
    """Per-exciton hop traces of the reference (update_state results)."""
    out, off = [], 0
    for n in d["ref_trace_len"]:
        out.append(d["ref_trace"][off:off + n])
        off += n
    return out


def hop_events(trace):
    """Keep only update_state results from an engine/oracle trace (drop crossings and reinjections)."""
    keep, skip = [], False
    for v in trace:
        if skip:
            skip = False
            continue
        if v == np.iinfo(np.int32).min:
            skip = True
            continue
        if v >= 0:
            keep.append(v)
    return np.asarray(keep, dtype=np.int32)


def synthetic_film(n_tubes=40, length=60.0, box=(120.0, 120.0, 8.0), seed=5):
    return F.straight_tubes(n_tubes, length, box_nm=box, seed=seed)


def oracle_sim(pos_m, orient, left, right, table, r_max, v, threads=1):
    return O.Sim(pos_m, orient, left, right, table, r_max, v, n_threads=threads)


def contacts_inputs(d):
    """Trimmed film (pos_m, orient, left, right), 4-D Förster table and run settings of a contacts
    golden case (the reference's own trim_scats and create_forster_scatt_table, restated)."""
    mc = d["config"]
    tl = mc["trim limits"]
    lim = [*tl["xlim"], *tl["ylim"], *tl["zlim"]]
    pos, ori, lk, rk = O.trim(d["film_pos_nm"] * 1.0e-9, d["film_orient"], d["film_left"], d["film_right"], lim)
    tab = O.forster_table(1e15, mc["theta [degrees]"], mc["zshift [m]"], mc["axis shift 1 [m]"],
                          mc["axis shift 2 [m]"])
    return dict(pos=pos, orient=ori, left=lk, right=rk, table=tab, r_max=mc["max hopping radius [m]"],
                v=mc["exciton velocity [m/s]"], dt=mc["monte carlo time step"], n_seg=mc["number of segments"],
                steps=int(d["steps"]), seed=int(d["seed"]), pops=tuple(int(x) for x in d["ref_contact_pop"]))


def ref_slots(d):
    """The reference's exciton slots after the run: live mask and per-slot state."""
    site = d["ref_site"]
    return {"live": site >= 0, "site": site, "heading": d["ref_heading"], "ff": d["ref_ff"],
            "pos": d["ref_xpos"].reshape(-1, 3), "draws": d["ref_draws"], "hops": d["ref_hops"]}
