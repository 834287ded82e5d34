"""The benchmark configurations at (or near) full size: size-independent properties.

* cfg 1 (100 tubes x 200 nm film, 10^4 excitons, Philox seed 1234): the mixed and plain FP64
  kernels give the same state for every exciton, and the first excitons equal an oracle run.
* cfg 4 (20,000 lognormal tubes, 10.8 M sites, 10^7 excitons): spatial storage + spatial work
  order (chosen automatically at this size), slot order and the plain FP64 kernel give the same
  state for every exciton.
* cfg 3 batch (the first films of the 256-film set, one launch over all films): the same
  three-way equality, per film.
"""
import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import tables
from oracle import oracle as O

pytestmark = pytest.mark.gpu

V = 2e5
KEYS = ("site", "pos", "delta", "ff", "heading", "draws", "hops")


def run(films, tab, n_exc, seeds, dt, steps, precision, order=L.KMC_ORDER_AUTO):
    e = E.Engine(0)
    e.load_films(films)
    e.set_table(tab)
    st = e.build(10e-9)
    e.set_work_order(order)
    e.init_excitons(n_exc, seeds, L.KMC_INJECT_UNIFORM)
    used = e.work_order()
    e.run(steps, dt, V, precision)
    out = e.excitons(), e.msd(0, steps), e.stats(), st, used
    e.close()
    return out


def assert_same(a, b):
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), k


def test_cfg1_mixed_equals_fp64_and_oracle():
    f = F.straight_tubes(100, 200.0, box_nm=(500.0, 500.0, 10.0), max_tilt_deg=5.0, seed=1234)
    tab = tables.forster_2d(1e15)
    n_exc, seed, dt, steps = 10_000, 1234, 1e-12, 4
    gm, mm, sm, st, _ = run([f], tab, n_exc, seed, dt, steps, L.KMC_PREC_MIXED)
    gf, mf, sf, _, _ = run([f], tab, n_exc, seed, dt, steps, L.KMC_PREC_FP64)
    assert_same(gm, gf)
    assert sm["hops"] == sf["hops"] > 1000 * n_exc * steps
    np.testing.assert_allclose(mm, mf, rtol=1e-12)
    n = 64
    sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, 10e-9, V, n_threads=8)
    sim.create_excitons(1, 0, n, seed)
    sim.step(dt, steps)
    o = sim.excitons()
    for k in ("site", "pos", "delta", "ff", "heading", "draws"):
        assert np.array_equal(gm[k][:n], o[k]), k


def test_cfg4_full_size_orders_and_precisions_agree():
    f = F.lognormal_tubes(20000, 500.0, 0.4, (5000.0, 5000.0, 50.0), seed=7)
    tab = tables.forster_2d(1e15)
    n_exc, dt, steps = 10_000_000, 2e-13, 1
    gs, ms, ss, st, used = run([f], tab, n_exc, 7, dt, steps, L.KMC_PREC_MIXED)
    assert used == L.KMC_ORDER_SPATIAL
    assert st["n_sites"] > 10_000_000 and st["k_mean"] > 30
    go, mo, so, _, used_o = run([f], tab, n_exc, 7, dt, steps, L.KMC_PREC_MIXED, L.KMC_ORDER_SLOTS)
    assert used_o == L.KMC_ORDER_SLOTS
    gf, mf, sf, _, _ = run([f], tab, n_exc, 7, dt, steps, L.KMC_PREC_FP64)
    assert_same(gs, go)
    assert_same(gs, gf)
    assert ss["hops"] == so["hops"] == sf["hops"] > 100 * n_exc
    np.testing.assert_allclose(ms, mf, rtol=1e-12)
    np.testing.assert_allclose(mo, mf, rtol=1e-12)


def test_cfg3_batch_orders_and_precisions_agree():
    films, n_exc = [], []
    for i in range(6):
        rng = np.random.default_rng(i)
        n_t = int(rng.integers(50, 2001))
        films.append(F.lognormal_tubes(n_t, 300.0, 0.5, (1000.0, 1000.0, 20.0), seed=i))
        n_exc.append(100 * n_t)
    tab = tables.forster_2d(1e15)
    seeds = list(range(len(films)))
    dt, steps = 1e-13, 2
    gs, ms, ss, _, used = run(films, tab, n_exc, seeds, dt, steps, L.KMC_PREC_MIXED, L.KMC_ORDER_SPATIAL)
    go, mo, so, _, _ = run(films, tab, n_exc, seeds, dt, steps, L.KMC_PREC_MIXED, L.KMC_ORDER_SLOTS)
    gf, mf, sf, _, _ = run(films, tab, n_exc, seeds, dt, steps, L.KMC_PREC_FP64)
    assert used == L.KMC_ORDER_SPATIAL
    assert_same(gs, go)
    assert_same(gs, gf)
    assert ss["hops"] == so["hops"] == sf["hops"]
    np.testing.assert_allclose(ms, mf, rtol=1e-12)
    np.testing.assert_allclose(mo, mf, rtol=1e-12)


def test_region_injection_with_removal_at_scale():
    # the reference's own set-up (central injection cell, removal slab, reinjection): many
    # excitons leave the removal domain, so the reinjection draw and the per-lane draw ring
    # restart are exercised thousands of times; spatial order and multi-step launches included
    f = F.straight_tubes(100, 200.0, box_nm=(500.0, 500.0, 10.0), max_tilt_deg=5.0, seed=1234)
    tab = tables.forster_2d(1e15)
    n_exc, seed, dt, steps = 400_000, 99, 2e-12, 6
    out = []
    for precision, order, spl in ((L.KMC_PREC_MIXED, L.KMC_ORDER_SPATIAL, 1), (L.KMC_PREC_MIXED, L.KMC_ORDER_SLOTS, 3),
                                  (L.KMC_PREC_FP64, L.KMC_ORDER_AUTO, 1)):
        e = E.Engine(0)
        e.load_films([f])
        e.set_table(tab)
        e.build(10e-9)
        e.set_work_order(order)
        e.set_launch_config(128, spl)
        e.init_excitons([n_exc], [seed], L.KMC_INJECT_REGION, n_sections=3)
        e.run(steps, dt, V, precision)
        out.append((e.excitons(), e.msd(0, steps), e.stats()))
        e.close()
    g0 = out[0][0]
    assert (g0["draws"] > 0).all()
    for g, m, st in out[1:]:
        assert_same(g0, g)
        np.testing.assert_allclose(m, out[0][1], rtol=1e-12)
        assert st["hops"] == out[0][2]["hops"]
    n = 64
    sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, 10e-9, V, n_threads=8)
    sim.create_excitons(0, 3, n, seed)
    sim.step(dt, steps)
    o = sim.excitons()
    for k in ("site", "pos", "delta", "ff", "heading", "draws"):
        assert np.array_equal(g0[k][:n], o[k]), k
