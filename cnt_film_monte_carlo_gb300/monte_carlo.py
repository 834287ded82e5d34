"""Host-side mirror of the reference's ``mc::monte_carlo`` interface: the Green-Kubo driver
(kubo_*) and the contacts / steady-state flux driver (init, step, save_metrics,
repopulate_contacts).

Same method names, argument meaning, JSON keys and output files as
src/monte_carlo/monte_carlo.{h,cpp} and the driver loops of src/main.cpp:62-105, so a caller of
the reference switches by changing the import.  Every step runs on the GPU engine through the
C ABI (include/cntkmc.h).

Keys read from the "exciton monte carlo" JSON section (input.json:40-68):
  mesh input directory, output directory, keep old results, rate type ("forster", "wong";
  "davoody" needs "rate table directory" with a table saved by the reference),
  zshift [m], axis shift 1 [m], axis shift 2 [m], theta [degrees], max hopping radius [m],
  trim limits, exciton velocity [m/s], monte carlo time step,
  number of sections for injection region, maximum time for kubo simulation [seconds],
  number of particles for kubo simulation.
Extensions: "philox seed" (default 100, the reference's srand(100) of main.cpp:30),
  "injection": "region" (default) | "uniform", "precision": "mixed" (default) | "fp64",
  "rate type": "forster2d" with "distance [m]" and "theta 2d [degrees]" grids.
"""
from __future__ import annotations

import json
import math
import os
import shutil
import time

import numpy as np

from . import _lib as L
from . import contacts, diffusion, tables
from .engine import Engine, read_mesh, trim_sites


def _expand(path: str) -> str:
    """A leading '~' is replaced by $HOME, nothing more (prepare_directory.hpp:12-16, 75-79):
    "~/out" is $HOME/out and "~out" is $HOMEout, not another user's home."""
    return os.environ.get("HOME", "") + path[1:] if path.startswith("~") else path


def prepare_directory(path: str, keep_old_files: bool = True) -> str:
    """prepare_directory (src/helper/prepare_directory.hpp:8-65): create the output directory;
    an existing non-empty one is renamed to <dir>.N (keep) or emptied."""
    path = _expand(path)
    if not os.path.exists(path):
        os.makedirs(path)
        return path
    if not os.path.isdir(path):
        raise ValueError("The input value for output directory is not acceptable.")
    if os.listdir(path):
        if keep_old_files:
            n = 1
            while os.path.exists(f"{path}.{n}"):
                n += 1
            os.rename(path, f"{path}.{n}")
        else:
            shutil.rmtree(path)
        os.makedirs(path)
    return path


def check_directory(path: str, should_be_empty: bool = False) -> str:
    """check_directory (prepare_directory.hpp:68-105)."""
    path = _expand(path)
    if not os.path.exists(path):
        raise ValueError("directory does NOT exists!!!")
    if not os.path.isdir(path):
        raise ValueError("input path is NOT a directory!!!")
    if not os.listdir(path) and not should_be_empty:
        raise ValueError("directory is empty!!!")
    return path


class monte_carlo:  # noqa: N801  (the reference's class name)
    def __init__(self, j: dict, device: int = 0):
        self._json_prop = dict(j)
        keep = bool(j.get("keep old results", True))
        self._output_directory = prepare_directory(j["output directory"], keep)
        self._input_directory = check_directory(j["mesh input directory"], False)
        self._time = 0.0  # the reference leaves _time uninitialised (monte_carlo.h:45)
        self._engine = Engine(device)
        self._max_time = 0.0
        self._msd_file = None
        self._n_particles = 0
        self._device_ms = 0.0
        self._dt = 0.0
        self._step = 0
        self._times = []
        self._batches = 1
        self._contacts = None

    # -- monte_carlo.h:139
    def time(self) -> float:
        return self._time

    def kubo_max_time(self) -> float:
        return self._max_time

    def output_path(self) -> str:
        return self._output_directory

    def number_of_particles(self) -> int:
        return self._n_particles

    def create_scattering_table(self, j: dict) -> dict:
        """monte_carlo.cpp:24-61."""
        rt = j["rate type"]
        grids = (j["theta [degrees]"], j["zshift [m]"], j["axis shift 1 [m]"], j["axis shift 2 [m]"])
        if rt == "forster":
            return tables.forster_4d(tables.FORSTER_GAMMA, *grids)
        if rt == "wong":
            return tables.forster_4d(tables.WONG_GAMMA, *grids)
        if rt == "forster2d":
            return tables.forster_2d(tables.FORSTER_GAMMA, j.get("distance [m]", (0.5e-9, 10e-9, 96)),
                                     j.get("theta 2d [degrees]", (0.0, 90.0, 91)))
        if rt == "davoody":
            if "rate table directory" not in j:
                raise ValueError("rate type davoody needs \"rate table directory\" (a table saved by the reference)")
            return tables.read_reference_table(_expand(j["rate table directory"]))
        raise ValueError('rate type must be one of the following: "davoody", "forster", "wong", "forster2d"')

    def kubo_init(self):
        """monte_carlo.cpp:254-305."""
        self._setup_film()
        j = self._json_prop
        self._n_sections = int(j["number of sections for injection region"])
        self._max_time = float(j["maximum time for kubo simulation [seconds]"])

    def _setup_film(self):
        """The film part of kubo_init / init: table, mesh, trim_scats, buckets, neighbour lists."""
        j = self._json_prop
        self._max_hopping_radius = float(j["max hopping radius [m]"])
        self._particle_velocity = float(j["exciton velocity [m/s]"])
        self._scat_table = self.create_scattering_table(j)
        pos, ori, lk, rk = read_mesh(self._input_directory)
        tl = j["trim limits"]
        lim = [*tl["xlim"], *tl["ylim"], *tl["zlim"]]
        pos, ori, lk, rk = trim_sites(pos, ori, lk, rk, lim)
        self._sites = (pos, ori, lk, rk)
        e = self._engine
        e.load_arrays(np.array([0, len(lk)], np.int64), pos, ori, lk, rk)
        e.set_table(self._scat_table)
        self._nbr_stats = e.build(self._max_hopping_radius)

    # ------------------------------------------------------------------ contacts mode
    def init(self):
        """Contacts (steady-state flux) set-up, monte_carlo.h:157-195: the film, the y slabs
        ("number of segments"), scatterer_statistics.dat, the contact sites and the initial
        linear profile (create_particles :274-316).  Extensions: "contact populations" (default
        [1100, 0], the reference's hard-coded values), "contacts capacity" (exciton slots),
        "maximum time for contacts simulation [seconds]"."""
        self._setup_film()
        j = self._json_prop
        self._n_seg = int(j["number of segments"])
        pops = tuple(int(p) for p in j.get("contact populations", (1100, 0)))
        g = self._engine.contacts_init(self._n_seg, pops, int(j.get("philox seed", 100)),
                                       int(j.get("contacts capacity", 0)))
        self._contacts = g
        self._n_particles = int(g["n_initial"])
        self._max_time = float(j.get("maximum time for contacts simulation [seconds]", 0.0))
        with open(os.path.join(self._output_directory, "scatterer_statistics.dat"), "w") as f:
            f.write(contacts.scatterer_statistics_text(g["ymin"], g["dy"], g["stat_pop"],
                                                       int(self._nbr_stats["n_sites"]), g["area"]))
        self._pop_file = self._cur_file = None
        self._last = None
        self._pop_sum = self._cur_sum = None
        self._metric_rows = 0

    def track_particle(self, dt: float, file_no: int):
        """track_particle (monte_carlo.h:786-818): particle_path.<file_no>.dat."""
        self.track_particles(dt, 1, first=file_no)

    def track_particles(self, dt: float, count: int, first: int = 0):
        """Tracks first .. first + count - 1 in one launch (each has its own stream, so this equals
        count track_particle calls).  At most "maximum steps per tracked particle" (default 2^18)
        steps each; the reference loops until the exciton reaches the last slab."""
        if count <= 0:
            return []
        cap = int(self._json_prop.get("maximum steps per tracked particle", 1 << 18))
        tr = self._engine.contacts_track(first, count, dt, self._particle_velocity, cap)
        for t, (path, arrived) in enumerate(tr):
            with open(os.path.join(self._output_directory, f"particle_path.{first + t}.dat"), "w") as f:
                f.write(contacts.track_text(path))
            if not arrived:
                print(f"track_particle {first + t}: not at the last slab after {cap} steps")
        return tr

    def contacts_max_time(self) -> float:
        return self._max_time

    def step(self, dt: float):
        """step (monte_carlo.h:343-354).  The engine runs the step, the counts behind
        save_metrics and repopulate_contacts as one unit, in the order of src/main.cpp:99-102."""
        pop, cur, live = self._engine.contacts_run(1, dt, self._particle_velocity, self._precision())
        self._device_ms += self._engine.stats()["last_run_ms"]
        self._dt = dt
        self._step += 1
        self._last = (pop[0], cur[0], int(live[0]))
        self._time += dt

    def save_metrics(self, dt: float):
        """save_metrics (monte_carlo.h:519-643): one row of population_profile.dat and of
        region_current.dat for the last step."""
        g = self._contacts
        if self._pop_file is None:
            self._pop_file = open(os.path.join(self._output_directory, "population_profile.dat"), "w")
            self._cur_file = open(os.path.join(self._output_directory, "region_current.dat"), "w")
            self._pop_file.write(contacts.population_header(g["area"], g["ymin"], g["dy"]))
            self._cur_file.write(contacts.current_header(g["area"], g["ymin"], g["dy"]))
        pop, cur, _ = self._last
        self._pop_sum = self._pop_sum + np.asarray(pop, np.int64) if self._pop_sum is not None else np.asarray(pop, np.int64)
        self._cur_sum = self._cur_sum + np.asarray(cur, np.int64) if self._cur_sum is not None else np.asarray(cur, np.int64)
        self._metric_rows += 1
        self._pop_file.write(contacts.population_row(self._time, pop, g["area"], g["dy"]))
        self._cur_file.write(contacts.current_row(self._time, cur, g["area"], dt))
        self._pop_file.flush()
        self._cur_file.flush()

    def repopulate_contacts(self):
        """repopulate_contacts (monte_carlo.h:443-455): done by the engine at the end of step();
        the particle count changes here, as the reference's list does."""
        self._n_particles = self._last[2]

    def save_json_properties(self):
        """monte_carlo.h:319-324."""
        with open(os.path.join(self._output_directory, "input.json"), "w") as f:
            json.dump(self._json_prop, f, indent=4)

    def kubo_create_particles(self):
        """monte_carlo.cpp:308-316 (exciton i draws from Philox stream i of "philox seed").  The
        MSD sums are also kept per exciton batch (exciton i in batch (i // 32) % B, B = min(32,
        n // 32)) for the interval of D in the run report."""
        j = self._json_prop
        n = int(j["number of particles for kubo simulation"])
        mode = L.KMC_INJECT_UNIFORM if j.get("injection", "region") == "uniform" else L.KMC_INJECT_REGION
        self._batches = max(1, min(32, n // 32))
        self._engine.set_msd_batches(self._batches)
        self._engine.init_excitons(n, int(j.get("philox seed", 100)), mode, self._n_sections)
        self._n_particles = n
        self._step = 0
        self._times = []

    def _precision(self) -> int:
        return L.KMC_PREC_FP64 if self._json_prop.get("precision", "mixed") == "fp64" else L.KMC_PREC_MIXED

    def _run(self, n: int, dt: float):
        self._engine.run(n, dt, self._particle_velocity, self._precision())
        self._device_ms += self._engine.stats()["last_run_ms"]
        self._dt = dt

    def kubo_step(self, dt: float):
        """monte_carlo.cpp:319-342."""
        self._run(1, dt)
        self._step += 1
        self._time += dt
        self._times.append(self._time)

    def _open_msd_file(self):
        if self._msd_file is None:
            self._msd_file = open(os.path.join(self._output_directory, "particle_dispalcement.avg.squared.dat"), "w")
            self._msd_file.write("# this file contains the average of dx^2, dy^2, and dz^2 of the particle ensemble "
                                 "over time\n")
            self._msd_file.write(f"# number of particles: {self._n_particles}\n\n")
            self._msd_file.write("time,x,y,z\n")

    def kubo_save_avg_dispalcement_squared(self):
        """monte_carlo.cpp:382-409: one row "time,<dx^2>,<dy^2>,<dz^2>" (showpos, scientific)."""
        self._open_msd_file()
        s = self._engine.msd(self._step - 1, 1)[0, 0] / float(self._n_particles)
        self._msd_file.write(f"{self._time:+.6e},{s[0]:+.6e},{s[1]:+.6e},{s[2]:+.6e}\n")
        self._msd_file.flush()

    def kubo_steps_and_save(self, n: int, dt: float):
        """n calls of kubo_step(dt), each followed by kubo_save_avg_dispalcement_squared, as one
        engine call (the rows and times are those of the n separate calls)."""
        if n <= 0:
            return
        self._run(n, dt)
        sums = self._engine.msd(self._step, n)[0] / float(self._n_particles)
        rows = []
        for k in range(n):
            self._time += dt
            self._step += 1
            self._times.append(self._time)
            rows.append(f"{self._time:+.6e},{sums[k, 0]:+.6e},{sums[k, 1]:+.6e},{sums[k, 2]:+.6e}\n")
        self._open_msd_file()
        self._msd_file.write("".join(rows))
        self._msd_file.flush()

    def contacts_steps_and_save(self, n: int, dt: float):
        """n rounds of step(dt), save_metrics(dt), repopulate_contacts() as one engine call."""
        if n <= 0:
            return
        pop, cur, live = self._engine.contacts_run(n, dt, self._particle_velocity, self._precision())
        self._device_ms += self._engine.stats()["last_run_ms"]
        self._dt = dt
        self._step += n
        for k in range(n):
            self._last = (pop[k], cur[k], int(live[k]))
            self._time += dt
            self.save_metrics(dt)
            self.repopulate_contacts()

    def steps_until(self, t_max: float, dt: float) -> int:
        """The number of steps of main.cpp's `while (time < max time)` loop from the current time,
        with the same floating-point accumulation of the time.  A time step that cannot advance
        the time, or needs more than 1e10 steps, is refused (the loop would not end)."""
        n, t = 0, self._time
        if t < t_max and dt > 0 and (t_max - t) / dt > 1e10:
            raise ValueError("monte carlo time step: more than 1e10 steps to the maximum time")
        while t < t_max:
            if not (0 < dt < math.inf) or t + dt == t:  # the loop would never end
                raise ValueError("monte carlo time step does not advance the time")
            t += dt
            n += 1
        return n

    def run_report(self, wall_seconds: float) -> dict:
        """The run report (no counterpart in the reference, which prints only wall-clock start and
        end, main.cpp:26-27,109-111), with the keys cntkmc_run writes to run_report.json: what ran,
        the neighbour lists, hop counters, device and wall seconds with hops/s, and in Green-Kubo
        mode D per axis with its 95 % interval from the exciton batches (last 80 % of the steps)."""
        st = self._engine.stats()
        nb = self._nbr_stats
        j = self._json_prop
        kubo = self._contacts is None
        fin = (lambda v: float(v) if math.isfinite(v) else None)
        dev_s = self._device_ms / 1e3
        r = {"engine": L.load().kmc_version().decode(), "mode": "kubo" if kubo else "contacts",
             "precision": "fp64" if self._precision() == L.KMC_PREC_FP64 else "mixed",
             "philox seed": int(j.get("philox seed", 100))}
        if kubo:
            r["injection"] = "uniform" if j.get("injection", "region") == "uniform" else "region"
        r.update({"particles": int(self._n_particles), "steps": int(self._step), "time step [s]": fin(self._dt),
                  "simulated time [s]": fin(self._time), "sites": int(nb["n_sites"]), "neighbour entries": int(nb["nnz"]),
                  "mean neighbours per site": fin(nb["k_mean"]), "max neighbours per site": int(nb["k_max"]),
                  "neighbour build [s]": fin(nb["build_ms"] / 1e3), "hops": int(st["hops"]),
                  "crossings": int(st["crossings"]), "exact re-resolves": int(st["exact_resolves"]),
                  "device seconds": fin(dev_s), "hops per second (device)": fin(st["hops"] / dev_s) if dev_s > 0 else None,
                  "wall seconds": fin(wall_seconds),
                  "hops per second (wall)": fin(st["hops"] / wall_seconds) if wall_seconds > 0 else None})
        if kubo:
            D, ci = [None] * 3, [None] * 3
            if self._step >= 2 and len(self._times) == self._step:
                m = self._engine.msd_batches(0, self._step)[0]
                d, c = diffusion.fit_counts(m, diffusion.batch_counts(self._n_particles, self._batches),
                                            np.array(self._times), 0.8)
                D, ci = [fin(v) for v in d], [fin(v) for v in c]
            r.update({"msd batches": self._batches, "fit fraction": 0.8, "diffusion coefficient [m^2/s]": D,
                      "diffusion 95% interval [m^2/s]": ci})
        else:
            r["live excitons"] = int(self._last[2]) if self._last is not None else int(self._n_particles)
            D = []
            if self._metric_rows:  # the flux-gradient D per interface (monte_carlo_results.py:428-442)
                g = self._contacts
                D = contacts.flux_gradient_diffusion_from_counts(
                    (self._pop_sum / self._metric_rows)[None, :], (self._cur_sum / self._metric_rows)[None, :],
                    g["area"], g["dy"], self._dt)
                D = [fin(float(v)) for v in D]
            r["flux-gradient D [m^2/s]"] = D
        return r

    def write_run_report(self, wall_seconds: float) -> dict:
        r = self.run_report(wall_seconds)
        with open(os.path.join(self._output_directory, "run_report.json"), "w") as f:
            json.dump(r, f, indent=2)
            f.write("\n")
        return r

    def close(self):
        for name in ("_msd_file", "_pop_file", "_cur_file"):
            f = getattr(self, name, None)
            if f is not None:
                f.close()
                setattr(self, name, None)
        self._engine.close()


CHUNK = 256  # time steps per engine call in run()


def _no_constant(name: str):
    raise ValueError(f"json: {name} is not a JSON number")


def run(input_json: str, device: int = 0) -> str:
    """src/main.cpp:32-80: read input.json, run the Green-Kubo loop, return the output directory.
    The file is read as strictly as the reference's nlohmann::json reads it (and as cntkmc_run
    does): NaN, Infinity and -Infinity are refused."""
    with open(input_json) as f:
        j = json.load(f, parse_constant=_no_constant)
    if "exciton monte carlo" not in j:
        raise ValueError('json input file does not contain "exciton monte carlo"')
    jm = dict(j["exciton monte carlo"])
    dt = float(jm["monte carlo time step"])
    t0 = time.perf_counter()
    if jm.get("mode") == "contacts":  # main.cpp:85-106, until the contacts time limit
        if "maximum time for contacts simulation [seconds]" not in jm:
            raise ValueError('contacts mode needs "maximum time for contacts simulation [seconds]"')
        sim = monte_carlo(jm, device)
        sim.init()
        sim.save_json_properties()
        sim.track_particles(dt, int(jm.get("number of tracked particles", 100)))  # main.cpp:90-92
        left = sim.steps_until(sim.contacts_max_time(), dt)  # the loop's steps, in chunks of one call
        while left > 0:
            sim.contacts_steps_and_save(min(CHUNK, left), dt)
            left -= CHUNK
        sim.write_run_report(time.perf_counter() - t0)
        out = sim.output_path()
        sim.close()
        return out
    sim = monte_carlo(jm, device)
    sim.kubo_init()
    sim.save_json_properties()
    sim.kubo_create_particles()
    left = sim.steps_until(sim.kubo_max_time(), dt)  # main.cpp:70-76's steps, in chunks of one call
    while left > 0:
        sim.kubo_steps_and_save(min(CHUNK, left), dt)
        left -= CHUNK
    sim.write_run_report(time.perf_counter() - t0)
    out = sim.output_path()
    sim.close()
    return out
