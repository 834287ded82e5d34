"""Benchmark: exciton hops/s of the Green-Kubo hot path on GB300.

Default workload (--workload cfg3), the batched mixed-precision form: 256 independent films of
uneven size in one persistent launch.  Film i (seed i, i = 0..255): tube count uniform in
50..2000, tube lengths lognormal (median 300 nm, sigma 0.5), uniform centres in a 1000 x 1000 x
20 nm box, azimuth U[0, pi), z-tilt U[-5, 5] deg, 1 nm segments, 10 nm hopping cutoff, 2-D
(distance 0.5-10 nm x angle 0-90 deg) Förster-form rate table; 100 excitons per tube injected
uniformly at random sites, Philox key i for film i, exciton velocity 2e5 m/s.  One "step" = all
excitons advanced by one 1 ps MSD bin (one kmc_run call, one persistent launch over all films).
Synthetic films (the reference's meshes are not available).
value: hops/s of the mixed-precision kernel, device time from CUDA events on the launching
stream, max over ranks; e2e: the same metric through the public API from host buffers (films
and table uploaded, neighbour lists built, excitons created, K steps run, MSD read back).
Multi-GPU (torchrun): independent replicas (Philox key rank * 2^32 + film seed), weak scaling, no
collective on the data path.  --impl reference times the reference's algorithm (the oracle's
restatement, which recomputes every neighbour list on every hop like
src/monte_carlo/scatterer.cpp:9-31) on the host cores, with its inputs built by the oracle: the
reference arm never loads the engine's library.
Other workloads (--workload): cfg2 (the 100-tube film with 10^6 excitons, 8 bins per step), cfg4
(10.8 M-site film), contacts (the contacts-mode loop on the cfg2 film) and cfg5: 64
mixed-chirality films whose pair rate tables come from the surrogate network trained on the GPU
in the set-up (untimed); its line adds a "surrogate" object (training throughput, held-out rate
error, D error against the labeller's tables on a mixed film).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FILM = dict(n_tubes=100, length_nm=200.0, box_nm=(500.0, 500.0, 10.0), tilt_deg=5.0, film_seed=1234)
R_MAX, VEL, BIN = 10e-9, 2e5, 1e-12
N_EXC, SEED = 1_000_000, 1
METRIC = "exciton hops/s (Green-Kubo hop kernel)"
UNIT = "hops/s"


def workload(name="cfg3", films=256, table=None):
    """(list of films, rate table, excitons per film, Philox key per film, description).

    ``table`` builds the 2-D Förster-form table from gamma_0 (default: the engine's
    tables.forster_2d; the reference arm passes the oracle's own, equal bit for bit)."""
    from cnt_film_monte_carlo_gb300 import film as F

    if table is None:
        from cnt_film_monte_carlo_gb300 import tables

        table = tables.forster_2d
    tab = table(1e15)
    if name == "cfg4":
        f = F.lognormal_tubes(20000, 500.0, 0.4, (5000.0, 5000.0, 50.0), seed=7)
        return [f], tab, [10_000_000], [7], ("cfg4 film: 20,000 tubes, lognormal length (median 500 nm, sigma 0.4), "
                                             "5x5 um x 50 nm box, 1 nm segments, 10 nm cutoff, 2-D rate table, seed 7")
    if name == "cfg3":
        out, ne = [], []
        for i in range(films):
            rng = np.random.default_rng(i)
            n_t = int(rng.integers(50, 2001))
            out.append(F.lognormal_tubes(n_t, 300.0, 0.5, (1000.0, 1000.0, 20.0), seed=i))
            ne.append(100 * n_t)
        return out, tab, ne, list(range(films)), (
            f"cfg3 batch: {films} films (seeds 0-{films - 1}), tubes U{{50..2000}}, lognormal length (median 300 nm, "
            "sigma 0.5), 1000x1000x20 nm boxes, 1 nm segments, 10 nm cutoff, 2-D rate table, 100 excitons per tube, "
            "one persistent launch")
    if name == "cfg5":
        n_f = CFG5_FILMS if films == 256 else films
        out = [F.lognormal_tubes(1000, 300.0, 0.5, (1000.0, 1000.0, 20.0), seed=5000 + i) for i in range(n_f)]
        # The CPU legs time the same per-hop work (a kind-3 lookup per neighbour pair) on 16 copies
        # of the 2-D table; the GPU arm replaces them with the network's pair tables (cfg5_surrogate).
        t2 = table(1e15)
        pairs = {"kind": 3, "grids": t2["grids"], "rate": np.broadcast_to(t2["rate"], (4, 4) + t2["rate"].shape).copy()}
        return out, pairs, [CFG5_EXC] * n_f, [SEED + i for i in range(n_f)], (
            f"cfg5 batch: {n_f} mixed-chirality films of 1000 tubes ((6,5), (7,5), (8,3), (8,4) uniform per tube), "
            "lognormal length (median 300 nm, sigma 0.5), 1000x1000x20 nm boxes, 1 nm segments, 10 nm cutoff, "
            "16 (donor, acceptor) rate tables of 96 x 91 built by the trained surrogate")
    f = F.straight_tubes(FILM["n_tubes"], FILM["length_nm"], box_nm=FILM["box_nm"], max_tilt_deg=FILM["tilt_deg"],
                         seed=FILM["film_seed"])
    return [f], tab, [N_EXC], [SEED], ("cfg2 film: 100 tubes x 200 nm, 500x500x10 nm, 1 nm segments, 10 nm cutoff, "
                                       "2-D rate table")


CFG5_FILMS, CFG5_EXC = 64, 100_000
CFG5_EPOCHS = 600            # Adam epochs over the 2M labels (4.4 s on a GB300)
CFG5_D_EXCITONS = 2_000_000  # excitons of each D comparison run (95 % interval ~ +-3.5 %)


def cfg5_species(films):
    """Chirality index of every site of the cfg5 films: one of 4, uniform per tube."""
    from cnt_film_monte_carlo_gb300 import surrogate as SG

    return [SG.site_species(f, np.random.default_rng(500 + i).integers(0, 4, f.n_tubes)) for i, f in enumerate(films)]


def cfg5_surrogate(films, device):
    """Per-site chiralities of the cfg5 films, the rate tables of the network trained on the GPU
    (2M samples labelled by the exciton-transfer labeller, 200 epochs) and its report: labelling
    and training throughput, held-out rate error, the time to build the 16 pair tables by the
    labeller and by the network, and the D error the network's tables bring to a mixed film
    against the labeller's own tables."""
    from cnt_film_monte_carlo_gb300 import engine as E
    from cnt_film_monte_carlo_gb300 import exciton as X
    from cnt_film_monte_carlo_gb300 import film as F
    from cnt_film_monte_carlo_gb300 import surrogate as SG

    species = cfg5_species(films)
    e = E.Engine(device)
    lab = X.PairLabeller(e)
    t0 = time.perf_counter()
    train = SG.draw_samples(lab, 2_000_000, seed=100, log_distance=True)
    t_label = time.perf_counter() - t0
    held = SG.draw_samples(lab, 200_000, seed=101)
    dist_g, theta_g = SG.grids()
    net = SG.RateSurrogate(e, lab)
    st = net.fit(train, epochs=CFG5_EPOCHS, seed=1)
    err = net.rate_errors(held)
    t0 = time.perf_counter()
    tab = net.table(dist_g, theta_g)
    t_net_table = time.perf_counter() - t0
    t0 = time.perf_counter()
    lab_tab = SG.labeller_table(lab, dist_g, theta_g)
    t_lab_table = time.perf_counter() - t0
    one_tab = SG.single_table(lab, dist_g, theta_g, species=1)
    lab.close()
    e.close()
    f = F.straight_tubes(300, 80.0, (250.0, 250.0, 10.0), 5.0, 1.0, 21)
    sp = SG.site_species(f, np.random.default_rng(21).integers(0, 4, 300))
    run = (CFG5_D_EXCITONS, 100, BIN, VEL, 77)
    d_lab, c_lab = SG.film_diffusion(f, sp, 4, lab_tab, *run, device=device)
    d_net, c_net = SG.film_diffusion(f, sp, 4, tab, *run, device=device)
    d_one, c_one = SG.film_diffusion(f, sp, 4, one_tab, *run, device=device)
    lab_d, net_d, one = (float(np.mean(d[:2])) for d in (d_lab, d_net, d_one))
    report = {
        "network": "4 -> 64 -> 64 -> 1 GELU, BF16 weight matrices, FP32 sums; labels from exciton_transfer::first_order "
                   "between ~40 nm tubes of (6,5), (7,5), (8,3), (8,4), computed on the GPU (kmc_exciton_rates)",
        "labelling": {"samples": len(train["dist"]), "seconds": t_label, "samples_per_s": len(train["dist"]) / t_label},
        "training": {"samples": len(train["dist"]), "epochs": CFG5_EPOCHS, "distance_sampling": "uniform in ln d",
                     "steps": st["steps"], "seconds": st["seconds"],
                     "samples_per_s": st["steps"] * SG.BATCH / st["seconds"], "first_loss": st["first_loss"],
                     "last_loss": st["last_loss"]},
        "rate_error_held_out": err,
        "pair_tables_seconds": {"labeller": t_lab_table, "network": t_net_table, "tables": "16 x 96 x 91"},
        "d_error": {"film": f"300 tubes x 80 nm, 250x250x10 nm, {CFG5_D_EXCITONS} excitons, 100 x 1 ps, same Philox "
                            "streams",
                    "labeller_in_plane": lab_d, "network_in_plane": net_d, "rel_error": net_d / lab_d - 1,
                    "ci95_labeller": float(np.hypot(c_lab[0], c_lab[1]) / 2),
                    "ci95_network": float(np.hypot(c_net[0], c_net[1]) / 2),
                    "single_table_in_plane": one, "single_table_rel_error": one / lab_d - 1,
                    "single_table": "(7,5) table for every pair: the film without the surrogate"},
    }
    return species, tab, report


def config(desc, n_sites, n_exc, bins_per_step, extra=None):
    c = {"workload": f"{desc}; {n_exc} excitons uniform injection; MSD bin 1 ps; {bins_per_step} bin(s) per step",
         "n_sites": n_sites, "n_excitons": n_exc, "bin_s": BIN,
         "bins_per_step": bins_per_step, "precision": "mixed (FP32 cumulative rates, exact FP64 re-resolve)",
         "l2": "256 MB buffer written between timed steps"}
    if extra:
        c.update(extra)
    return c


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.p is None:
            return
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bytes_per_hop(k_mean):
    """Bytes one hop of the mixed kernel must move in its own layout: the destination site's
    64-byte record (1/total, links, link times, first search level) and the one 64-byte row block
    holding the chosen entry (8 FP32 cumulative values + 8 neighbour ids); rows of 65-512 entries
    add the 32-byte second level."""
    return 128 if k_mean <= 64 else 160


def algorithmic_bytes_per_hop(k_mean):
    """Algorithmic bytes of one hop of a plain CSR walk with an FP32 cumulative table, each
    dependent random access one 32-byte sector: the destination site record (64 B: position,
    row offset, 1/total, links), one column-index sector and the bisection's sectors,
    max(1, ceil(log2 k) - 2) of them (8 FP32 values per sector, the last three probes share one),
    at the measured mean row length k."""
    return 64 + 32 + 32 * max(1, math.ceil(math.log2(max(k_mean, 2.0))) - 2)


class CpuSample:
    """The reference's algorithm on the host cores: the oracle restatement with a fresh neighbour
    search on every hop (scatterer.cpp:9-31), OpenMP over excitons.  A short pilot fixes the number
    of excitons so that one sample (all of them advanced by one 1 ps bin from their injection) takes
    about `seconds` of wall time."""

    def __init__(self, f, tab, seconds=10.0, threads=None, species=None, seed=SEED):
        from oracle import oracle as O

        self.O, self.f, self.tab, self.species, self.seed = O, f, tab, species, seed
        self.threads = threads or os.cpu_count() or 1
        n = max(self.threads * 16, 128)
        sim = self._sim(n)
        t0 = time.perf_counter()
        sim.step(BIN / 20, 1)
        dt = time.perf_counter() - t0
        rate = max(sim.total_hops(), 1) / max(dt, 1e-9)
        hops_per_exc_bin = max(sim.total_hops() / n * 20, 1.0)
        self.n = int(max(self.threads, min(N_EXC, seconds * rate / hops_per_exc_bin)))

    def _sim(self, n):
        f = self.f
        sim = self.O.Sim(f.pos_m(), f.orient, f.left, f.right, self.tab, R_MAX, VEL, n_threads=self.threads,
                         species=self.species)
        sim.create_excitons(1, 0, n, self.seed, use_csr=False)
        return sim

    def run(self):
        sim = self._sim(self.n)
        t0 = time.perf_counter()
        sim.step(BIN, 1)
        dt = time.perf_counter() - t0
        hops = sim.total_hops()
        return hops / dt, f"{self.n} excitons x one 1 ps bin of the same film ({hops} hops, {dt:.2f} s)", dt


def reference_arm(args):
    """The reference's algorithm on the host cores.  Films come from the numpy generator and the
    rate table from the oracle (oracle.forster2d_table, equal bit for bit to the engine's), so this
    process never loads the engine's library."""
    from oracle import oracle as O

    films, tab, ne, seeds, desc = workload(args.workload, args.films, table=O.forster2d_table)
    f = films[0]
    if args.workload == "contacts":
        vals, secs = [], []
        for i in range(args.warmup + args.steps):
            v, sample, dt, threads = contacts_cpu_sample(f, tab, SEED)
            if i >= args.warmup:
                vals.append(v)
                secs.append(dt)
        value = float(np.mean(vals))
        print(json.dumps({"impl": "reference", "metric": CONTACTS_METRIC, "value": value, "unit": UNIT,
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": float(np.mean(secs)) * 1e3, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                          "config": {"workload": f"{desc}; contacts mode, {CONTACTS_SEG} y slabs", "sample": sample},
                          "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                                           "sample": sample},
                          "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    # whole run within a few minutes: every step gets an equal share of ~150 s
    per_step = min(args.cpu_seconds, 150.0 / max(args.steps + args.warmup, 1))
    sp0 = cfg5_species(films[:1])[0] if args.workload == "cfg5" else None
    cs = CpuSample(f, tab, seconds=per_step, species=sp0, seed=seeds[0])
    vals, secs, sample = [], [], ""
    for i in range(args.warmup + args.steps):
        v, sample, dt = cs.run()
        if len(films) > 1:
            sample += f"; film 0 of the {len(films)}-film batch ({f.n_sites} sites)"
        if args.workload == "cfg5":
            sample += "; 16 chirality-pair tables (a per-pair lookup added to the reference's algorithm)"
        if i >= args.warmup:
            vals.append(v)
            secs.append(dt)
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(secs)) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(desc, sum(x.n_sites for x in films), int(sum(ne)), 1,
                             {"sample": sample, "cpu_arm": "a bounded sample of the workload (the excitons of one "
                                                           "film of the batch for one 1 ps bin), timed on the host "
                                                           "cores; hops/s is the comparable figure"}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cs.threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


CONTACTS_SEG, CONTACTS_POP = 10, (200_000, 0)
CONTACTS_METRIC = "exciton hops/s (contacts-mode step: hops, slab metrics, contact repopulation)"


CONTACTS_CPU_POP = (1_000, 0)


def contacts_cpu_sample(f, tab, seed):
    """The reference's contacts loop on the host cores: the oracle's restatement with a fresh
    neighbour search on every hop (scatterer.cpp:9-31), OpenMP over excitons, on the same film
    with contact populations (1000, 0) (about 5,500 excitons): one 1 ps step."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, R_MAX, VEL, n_threads=threads)
    p = CONTACTS_CPU_POP
    sim.contacts_init(CONTACTS_SEG, p[0], p[1], seed, p[0] * (CONTACTS_SEG + 2) + 1024)
    sim.use_csr(False)
    t0 = time.perf_counter()
    sim.contacts_step(BIN, 1)
    dt = time.perf_counter() - t0
    hops = sim.total_hops()
    return hops / dt, (f"oracle contacts loop with the per-hop neighbour search, contact populations {p}, one 1 ps "
                       f"step ({hops} hops, {dt:.2f} s)"), dt, threads


def contacts_arm(args, local, rank, world):
    """--workload contacts: the contacts (steady-state flux) loop on the cfg2 film, 10 y slabs,
    contact populations (200000, 0) (about 1.1 M live excitons), 1 ps steps; one timed step =
    one kmc_contacts_run step (hop launch + metrics + both repopulations, one CUDA graph)."""
    import torch

    from cnt_film_monte_carlo_gb300 import _lib as L
    from cnt_film_monte_carlo_gb300 import engine as E
    from cnt_film_monte_carlo_gb300 import replicas as R

    films, tab, _, _, desc = workload("cfg2")
    f = films[0]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    seed = R.replica_seed(SEED, rank)

    def engine():
        e = E.Engine(local)
        e.load_films([f])
        e.set_table(tab)
        st = e.build(R_MAX)
        g = e.contacts_init(CONTACTS_SEG, CONTACTS_POP, seed, 0)
        return e, st, g

    e, st, g = engine()
    tune = e.autotune(BIN, VEL, trial_steps=2) if not args.no_tune else None
    for _ in range(args.warmup):
        e.contacts_run(1, BIN, VEL, L.KMC_PREC_MIXED)
    h0 = e.stats()["hops"]
    dev_ms, launches, live = 0.0, 0, []
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            _, _, n_live = e.contacts_run(1, BIN, VEL, L.KMC_PREC_MIXED)
            s = e.stats()
            dev_ms += s["last_run_ms"]
            launches += s["last_launches"]
            live.append(int(n_live[0]))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    hops = e.stats()["hops"] - h0
    l2_gbs = e.probe_l2(32 << 20, 200)
    e.close()
    dev_s_max, wall_max, hops_all = R.job_timing(dev_ms / 1e3, wall, hops)
    value = hops_all / dev_s_max
    e2e = None
    if not args.no_e2e:
        t0 = time.perf_counter()
        e3, _, _ = engine()
        if tune:
            e3.set_mixed_variant(tune["variant"])
        for _ in range(args.steps):  # each step: run it, read its slab and interface counts back
            e3.contacts_run(1, BIN, VEL, L.KMC_PREC_MIXED)
        h3 = e3.stats()["hops"]
        e3.close()
        w3 = time.perf_counter() - t0
        h2d = f.n_sites * (3 * 8 * 2 + 2 * 4) + 16 + tab["rate"].nbytes + sum(x.nbytes for x in tab["grids"])
        e2e = {"value": h3 * world / w3, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
               "d2h_bytes_per_step": 8 * (2 * CONTACTS_SEG - 1 + 1), "seconds": w3,
               "includes": "film+table upload and neighbour build (amortised over K), contacts set-up, K steps each "
                           "followed by the read-back of its counts"}
    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    bph = bytes_per_hop(st["k_mean"])
    achieved = hops / (dev_ms / 1e3) * bph / 1e9
    l2 = None
    prof = os.path.join(ROOT, "profiles", "hop_mixed_traffic.json")
    if os.path.exists(prof):
        with open(prof) as fh:
            pj = json.load(fh).get("cfg2")  # the same film
        if pj and "lts_bytes_per_hop" in pj:
            l2_ach = pj["lts_bytes_per_hop"] * hops / (dev_ms / 1e3) / 1e9
            l2 = {"achieved": l2_ach, "peak": l2_gbs, "unit": "GB/s", "frac": l2_ach / l2_gbs,
                  "bytes_per_hop": pj["lts_bytes_per_hop"],
                  "peak_kind": "measured: kmc_probe_l2, 16-byte L2-only loads over a 32 MB buffer",
                  "source": pj["source"] + " (the Green-Kubo launch on the same film)"}
    line = {
        "metric": CONTACTS_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall_max / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": {"workload": f"{desc}; contacts mode: {CONTACTS_SEG} y slabs, contact populations {CONTACTS_POP}, "
                               f"1 ps steps", "n_sites": st["n_sites"], "k_mean": st["k_mean"],
                   "initial_excitons": g["n_initial"], "slots": g["capacity"], "live_excitons": live,
                   "hops_timed": hops, "l2": "256 MB buffer written between timed steps"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_kind": peak_kind, "bytes_per_hop": bph,
                     "note": "algorithmic bytes per hop x hops / device time of the whole contacts step",
                     "l2": l2},
        "gpu_launches": launches, "autotune": tune, "e2e": e2e, "clocks": clk.summary(),
    }
    if world == 1 and not args.no_cpu:
        v, sample, _, threads = contacts_cpu_sample(f, tab, seed)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-exc", type=int, default=None, help="excitons per film (default: the workload's)")
    ap.add_argument("--workload", default="cfg3", choices=["cfg2", "cfg3", "cfg4", "cfg5", "contacts"])
    ap.add_argument("--films", type=int, default=256, help="films of the cfg3 batch (cfg5: default 64)")
    ap.add_argument("--bins-per-step", type=int, default=None,
                    help="1 ps MSD bins advanced per timed step (one kmc_run call; default 1 for cfg3, 8 otherwise)")
    ap.add_argument("--fp64-steps", type=int, default=None,
                    help="plain FP64 comparison steps (default 3; cfg3 and cfg5 1)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="wall seconds of one CPU sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--variant", type=int, default=None)
    ap.add_argument("--order", default="auto", choices=["auto", "slots", "spatial"],
                    help="order in which the mixed kernel takes excitons")
    ap.add_argument("--no-graph", action="store_true", help="launch directly instead of replaying a CUDA graph")
    args = ap.parse_args()
    if args.fp64_steps is None:
        args.fp64_steps = 1 if args.workload in ("cfg3", "cfg5") else 3
    if args.bins_per_step is None:
        args.bins_per_step = 1 if args.workload == "cfg3" else 8
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args)
        return

    import torch

    from cnt_film_monte_carlo_gb300 import _lib as L
    from cnt_film_monte_carlo_gb300 import build as B
    from cnt_film_monte_carlo_gb300 import engine as E
    from cnt_film_monte_carlo_gb300 import replicas as R

    B.build()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    if args.workload == "contacts":
        contacts_arm(args, local, rank, world)
        if dist is not None:
            dist.destroy_process_group()
        return

    films, tab, n_exc, film_seeds, desc = workload(args.workload, args.films)
    keys = [R.replica_seed(sd, rank) for sd in film_seeds]
    cpu_tab, species, surrogate = tab, None, None
    if args.workload == "cfg5":
        species, tab, surrogate = cfg5_surrogate(films, local)
        species = np.concatenate(species)
    if args.n_exc is not None:
        n_exc = [args.n_exc] * len(films)
    n_exc_total = int(sum(n_exc))
    f = films[0]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def load(eng):
        eng.load_films(films)
        if species is not None:
            eng.set_species(species, 4)
        eng.set_table(tab)

    e = E.Engine(local)
    load(e)
    st = e.build(R_MAX)
    e.init_excitons(n_exc, keys, L.KMC_INJECT_UNIFORM)
    bins = args.bins_per_step
    order = {"auto": L.KMC_ORDER_AUTO, "slots": L.KMC_ORDER_SLOTS, "spatial": L.KMC_ORDER_SPATIAL}[args.order]
    e.set_work_order(order)
    e.set_graph(not args.no_graph)
    if args.variant is not None:
        e.set_mixed_variant(args.variant)
    # trials of one step's length, so launches of up to `bins` steps are among the candidates
    tune = e.autotune(BIN, VEL, trial_steps=max(1 if args.workload == "cfg3" else 2, bins)) \
        if not (args.no_tune or args.variant is not None) else None
    for _ in range(args.warmup):
        e.run(bins, BIN, VEL, L.KMC_PREC_MIXED)
    s0 = e.stats()
    h0 = s0["hops"]
    dev_ms, launches = 0.0, 0
    barrier()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e.run(bins, BIN, VEL, L.KMC_PREC_MIXED)
            s = e.stats()
            dev_ms += s["last_run_ms"]
            launches += s["last_launches"]
        barrier()
        wall = time.perf_counter() - t0
    order_used = "spatial" if e.work_order() == L.KMC_ORDER_SPATIAL else "slots"
    s1 = e.stats()
    hops = s1["hops"] - h0
    crossings = s1["crossings"] - s0["crossings"]
    exact = s1["exact_resolves"] - s0["exact_resolves"]
    t_end = e.stats()["steps_done"] * BIN
    # MSD of the last step over every replica's excitons (the path's only exchange)
    last = R.sum_msd(e.msd(0, e.stats()["steps_done"])[:, -1].sum(axis=0))
    d_eff = (last / (n_exc_total * world) / (2 * t_end)).tolist()
    l2_gbs = e.probe_l2(32 << 20, 200)  # L2 read bandwidth, the L2 roofline's denominator
    e.close()
    dev_s = dev_ms / 1e3
    dev_s_max, wall_max, hops_all = R.job_timing(dev_s, wall, hops)
    value = hops_all / dev_s_max

    # plain FP64 kernel on the same workload (same seeds; same hop sequence)
    fp64 = None
    if args.fp64_steps > 0:
        e2 = E.Engine(local)
        load(e2)
        e2.build(R_MAX)
        e2.init_excitons(n_exc, keys, L.KMC_INJECT_UNIFORM)
        e2.run(bins, BIN, VEL, L.KMC_PREC_FP64)  # one warm-up step
        h1 = e2.stats()["hops"]
        ms = 0.0
        for _ in range(args.fp64_steps):
            flush.zero_()
            torch.cuda.synchronize()
            e2.run(bins, BIN, VEL, L.KMC_PREC_FP64)
            ms += e2.stats()["last_run_ms"]
        fp64 = (e2.stats()["hops"] - h1) / (ms / 1e3)
        e2.close()

    # end to end through the public API from host buffers: the flat arrays the C ABI takes
    # (kmc_film) are ready in host memory; their copies to the device are inside the timed region
    e2e = None
    if not args.no_e2e:
        off = np.zeros(len(films) + 1, np.int64)
        off[1:] = np.cumsum([f.n_sites for f in films])
        flat = (off, np.ascontiguousarray(np.concatenate([f.pos_m() for f in films])),
                np.ascontiguousarray(np.concatenate([f.orient for f in films])),
                np.ascontiguousarray(np.concatenate([f.left for f in films]), dtype=np.int32),
                np.ascontiguousarray(np.concatenate([f.right for f in films]), dtype=np.int32))
        barrier()
        t0 = time.perf_counter()
        e3 = E.Engine(local)
        e3.load_arrays(*flat)
        if species is not None:
            e3.set_species(species, 4)
        e3.set_table(tab)
        e3.build(R_MAX)
        e3.init_excitons(n_exc, keys, L.KMC_INJECT_UNIFORM)
        e3.set_work_order(order)
        e3.set_graph(not args.no_graph)
        if tune:
            e3.set_mixed_variant(tune["variant"])
            e3.set_launch_config(128, tune["steps_per_launch"])
        elif args.variant is not None:
            e3.set_mixed_variant(args.variant)
        d2h = 0
        for k in range(args.steps):  # each step: run it, read its MSD sums back
            e3.run(bins, BIN, VEL, L.KMC_PREC_MIXED)
            d2h += e3.msd(k * bins, bins).nbytes
        h3 = e3.stats()["hops"]
        e3.close()
        barrier()
        w3 = time.perf_counter() - t0
        n_all = sum(x.n_sites for x in films)
        h2d = n_all * (3 * 8 * 2 + 2 * 4) + 8 * (len(films) + 1) + tab["rate"].nbytes + sum(g.nbytes for g in tab["grids"])
        if species is not None:
            h2d += species.nbytes
        e2e = {"value": h3 * world / w3, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
               "d2h_bytes_per_step": int(d2h / args.steps), "seconds": w3,
               "includes": "from the flat host arrays of kmc_film: film+table upload and neighbour build (per step: "
                           "amortised over K), exciton creation, K steps each followed by the read-back of its MSD sums"}

    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    bph = bytes_per_hop(st["k_mean"])
    abph = algorithmic_bytes_per_hop(st["k_mean"])
    achieved = hops / dev_s * abph / 1e9
    kernel_achieved = hops / dev_s * bph / 1e9
    spl = tune["steps_per_launch"] if tune else 32  # the engine's default steps per launch
    hop_launches = args.steps * math.ceil(bins / spl)
    traffic = None  # DRAM bytes per hop-kernel launch, from the ncu capture of this workload
    l2 = None
    prof = os.path.join(ROOT, "profiles", "hop_mixed_traffic.json")
    if os.path.exists(prof):
        with open(prof) as fh:
            pj = json.load(fh).get(args.workload)
        if pj:
            traffic = pj["dram_bytes_per_hop"] * hops / max(hop_launches, 1)
        if pj and "lts_bytes_per_hop" in pj:
            # the film's rows stay in L2: L2->SM bytes per hop (ncu) x hops/s against the measured
            # L2 read bandwidth
            l2_ach = pj["lts_bytes_per_hop"] * hops / dev_s / 1e9
            l2 = {"achieved": l2_ach, "peak": l2_gbs, "unit": "GB/s", "frac": l2_ach / l2_gbs,
                  "bytes_per_hop": pj["lts_bytes_per_hop"],
                  "peak_kind": "measured: kmc_probe_l2, 16-byte L2-only loads over a 32 MB buffer",
                  "source": pj["source"]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall_max / args.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32", "data": "synthetic",
        "config": config(desc, st["n_sites"], n_exc_total, bins,
                         {"films": len(films), "k_mean": st["k_mean"], "k_max": st["k_max"], "nnz": st["nnz"],
                          "hops_timed": hops, "crossings_per_hop": crossings / max(hops, 1),
                          "fp64_resolves_per_hop": exact / max(hops, 1),
                          "build_ms": st["build_ms"], "work_order": order_used,
                          "cuda_graph": not args.no_graph}),
        "fp64_plain_value": fp64, "speedup_vs_fp64": (value / world / fp64) if fp64 else None,
        "d_eff_m2_per_s": d_eff,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind, "bytes_per_hop": abph,
                     "note": ("algorithmic bytes per hop (plain CSR walk with FP32 cumulative rows at the measured "
                              "mean row length) x hops / hop-kernel device time; rows the excitons in flight hop "
                              "over are served mostly from L2, so DRAM traffic (traffic, per launch) stays below "
                              "the algorithmic bytes"),
                     "kernel_layout": {"bytes_per_hop": bph, "achieved": kernel_achieved,
                                       "frac": kernel_achieved / peak,
                                       "note": "the two dependent 64-byte lines (site record, row block) this "
                                               "kernel reads per hop, +32 B second level for rows over 64 entries"},
                     "dram_bytes_per_hop": (traffic * max(hop_launches, 1) / hops) if traffic else None,
                     "l2": l2},
        "gpu_launches": launches,
        "autotune": tune,
        "e2e": e2e,
        "clocks": clk.summary(),
    }
    if surrogate is not None:
        line["surrogate"] = surrogate
    if world == 1 and not args.no_cpu:
        cs = CpuSample(f, cpu_tab, seconds=args.cpu_seconds,
                       species=species[:f.n_sites] if species is not None else None)
        v, sample, _ = cs.run()
        if species is not None:
            sample += "; 16 chirality-pair tables (a per-pair lookup added to the reference's algorithm)"
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cs.threads, "kind": "port", "sample": sample}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
