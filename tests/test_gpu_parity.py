"""GPU parity: the CUDA engine through the C ABI against the oracle and the reference's golden
outputs.  Hop-site sequences, exciton states, dwell clocks and positions are compared bit for bit;
per-step MSD sums (accumulated with device atomics in a different order) to 1e-12 relative."""
import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import tables
from helpers import CASES, case_inputs, hop_events, load_case, ref_traces
from oracle import oracle as O

pytestmark = pytest.mark.gpu
MSD_RTOL = 1e-12
PRECISIONS = [L.KMC_PREC_FP64, L.KMC_PREC_MIXED]


def assert_msd_close(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    np.testing.assert_allclose(a, b, rtol=MSD_RTOL, atol=0)


def assert_states_equal(g, o, n=None):
    n = n if n is not None else len(o["site"])
    for k in ("site", "pos", "delta", "ff", "heading", "draws"):
        assert np.array_equal(g[k][:n], o[k][:n]), k


@pytest.fixture(scope="module")
def eng():
    e = E.Engine(0)
    yield e
    e.close()


def test_dwell_uniform_exact_for_every_rand_value(eng):
    # the division-free RN(r / RAND_MAX) of the mixed kernel equals IEEE division for all r
    assert eng.selftest_uniform(0, 1 << 31) == 0


def test_device_log_acos_match_oracle(eng):
    rng = np.random.default_rng(3)
    r = rng.integers(1, 2**31, 400000)
    x = np.concatenate([r / 2147483647.0, rng.uniform(0, 1, 100000), np.exp(rng.uniform(-700, 700, 50000)),
                        [1.0, 0.5, 2.0, 5e-324, 2.2250738585072014e-308, 1 - 2.0**-53, 1 + 2.0**-52]])
    lo, _ = eng.math_probe(x)
    assert np.array_equal(lo.view(np.uint64), O.log_array(x).view(np.uint64))
    c = np.concatenate([rng.uniform(-1, 1, 20000), [1.0, -1.0, 0.5, -0.5, 0.0, 0.9999999999]])
    _, ac = eng.math_probe(c)
    assert np.array_equal(ac, np.array([O.acos(v) for v in c]))


def golden_engine(d):
    ci = case_inputs(d)
    pos, ori, lk, rk = E.trim_sites(ci["pos"], ci["orient"], ci["left"], ci["right"], ci["lim"])
    e = E.Engine(0)
    e.load_arrays(np.array([0, len(lk)], np.int64), pos, ori, lk, rk)
    e.set_table(E.forster_table(ci["gamma"], *ci["grids"]))
    st = e.build(ci["r_max"])
    return e, ci, st, len(lk)


@pytest.mark.parametrize("name", CASES)
def test_golden_neighbor_csr(name):
    d = load_case(name)
    e, ci, st, n = golden_engine(d)
    nb = e.neighbors(n, st["nnz"])
    assert np.array_equal(nb["rowptr"], d["ref_csr_rowptr"])
    assert np.array_equal(nb["col"], d["ref_csr_col"])
    assert np.array_equal(nb["cum"], d["ref_csr_cum"])
    assert np.array_equal(nb["total"], d["ref_total"])
    assert st["k_max"] == int(np.max(np.diff(d["ref_csr_rowptr"])))
    e.close()


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("name", CASES)
def test_golden_green_kubo(name, precision):
    d = load_case(name)
    e, ci, st, n = golden_engine(d)
    n_tr = len(d["ref_trace_len"])
    e.set_trace(n_tr, 1 << 16)
    e.init_excitons(ci["n_exc"], int(d["seed"]), L.KMC_INJECT_REGION, ci["sections"])
    g0 = e.excitons()
    assert np.array_equal(g0["site"], d["ref_site_init"])
    assert np.array_equal(g0["ff"], d["ref_ff_init"])
    assert np.array_equal(g0["heading"], d["ref_heading_init"])
    steps = int(d["steps"])
    half = steps // 2
    e.run(half, ci["dt"], ci["v"], precision)  # two calls: state carried across launches
    e.run(steps - half, ci["dt"], ci["v"], precision)
    g = e.excitons()
    assert np.array_equal(g["site"], d["ref_site"])
    assert np.array_equal(g["pos"].ravel(), d["ref_xpos"])
    assert np.array_equal(g["delta"].ravel(), d["ref_delta"])
    assert np.array_equal(g["ff"], d["ref_ff"])
    assert np.array_equal(g["heading"], d["ref_heading"])
    assert np.array_equal(g["draws"], d["ref_draws"])
    assert e.stats()["hops"] == int(d["ref_hops"][0])
    assert_msd_close(e.msd(0, steps), d["ref_msd"])
    for i, rt in enumerate(ref_traces(d)):
        tr, _ = e.trace(i)
        assert np.array_equal(hop_events(tr)[: len(rt)], rt)
    e.close()


def synthetic_case(table_kind=2, n_tubes=40, length=60.0, box=(120.0, 120.0, 8.0), seed=5, r_max=10e-9):
    f = F.straight_tubes(n_tubes, length, box_nm=box, seed=seed)
    if table_kind == 2:
        tab = tables.forster_2d(1e15)
    else:
        tab = E.forster_table(1e15, (0, 180, 21), (1.5e-9, 10e-9, 11), (-10e-9, 10e-9, 11), (-10e-9, 10e-9, 11))
    return f, tab, r_max


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("table_kind", [2, 4])
def test_uniform_injection_vs_oracle(precision, table_kind):
    f, tab, r_max = synthetic_case(table_kind)
    n_exc, seed, dt, v, steps = 500, 1234, 2e-13, 2e5, 12
    sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, r_max, v)
    sim.set_trace(8, 1 << 18)
    sim.create_excitons(1, 0, n_exc, seed)
    om = sim.step(dt, steps)
    o = sim.excitons()
    e = E.Engine(0)
    e.load_films(f)
    e.set_table(tab)
    st = e.build(r_max)
    csr = sim.build_csr()
    nb = e.neighbors(f.n_sites, st["nnz"])
    assert np.array_equal(nb["col"], csr["col"]) and np.array_equal(nb["cum"], csr["cum"])
    e.set_trace(8, 1 << 18)
    e.init_excitons(n_exc, seed, L.KMC_INJECT_UNIFORM)
    e.run(steps, dt, v, precision)
    assert_states_equal(e.excitons(), o)
    assert_msd_close(e.msd(0, steps), om)
    for i in range(8):
        a, na = e.trace(i)
        b, nb_ = sim.trace(i)
        assert na == nb_ and np.array_equal(a, b)  # hops and free-flight crossings, in order
    assert e.stats()["hops"] == sim.total_hops()
    assert e.stats()["crossings"] == sim.total_crossings()
    e.close()


def test_batched_films_equal_single_films():
    films = [F.straight_tubes(n, 40.0, box_nm=(80, 80, 6), seed=s) for n, s in ((12, 1), (30, 2), (7, 3))]
    tab = tables.forster_2d(1e15)
    n_exc, seeds, dt, v, steps = [70, 200, 33], [11, 22, 33], 1e-13, 2e5, 6
    b = E.Engine(0)
    b.load_films(films)
    b.set_table(tab)
    b.build(10e-9)
    b.init_excitons(n_exc, seeds, L.KMC_INJECT_UNIFORM)
    b.run(steps, dt, v, L.KMC_PREC_MIXED)
    gb = b.excitons()
    mb = b.msd(0, steps)
    off = 0
    for i, f in enumerate(films):
        s = E.Engine(0)
        s.load_films(f)
        s.set_table(tab)
        s.build(10e-9)
        s.init_excitons(n_exc[i], seeds[i], L.KMC_INJECT_UNIFORM)
        s.run(steps, dt, v, L.KMC_PREC_FP64)
        gs = s.excitons()
        for k in ("site", "pos", "delta", "ff", "draws"):
            assert np.array_equal(gb[k][off:off + n_exc[i]], gs[k]), (i, k)
        assert_msd_close(mb[i], s.msd(0, steps)[0])
        off += n_exc[i]
        s.close()
    b.close()


def isolated_film():
    """Tube A: sites at x = 0, 1, 2, 7, 12 nm (the last two have no neighbour within 3 nm but keep
    their tube links); tube B: x = 0..4 nm at y = 1.5 nm; three single sites far away (no links,
    no neighbours).  Empty neighbour lists are undefined behaviour in the reference; here an
    exciton there stays (update_state returns the site) and keeps flying along its tube."""
    xa = [0.0, 1.0, 2.0, 7.0, 12.0]
    pos = [[x, 0.0, 0.0] for x in xa] + [[x, 1.5, 0.0] for x in range(5)] + [[100.0 + 20 * k, 50.0, 0.0] for k in range(3)]
    n = len(pos)
    left = np.full(n, -1, np.int32)
    right = np.full(n, -1, np.int32)
    for a, b in ((0, 5), (5, 10)):
        for i in range(a, b):
            left[i] = i - 1 if i > a else -1
            right[i] = i + 1 if i + 1 < b else -1
    ori = np.tile([1.0, 0.0, 0.0], (n, 1))
    return np.asarray(pos) * 1e-9, ori, left, right


def test_isolated_sites_and_empty_lists():
    pos, ori, lk, rk = isolated_film()
    tab = tables.forster_2d(1e13)  # slow rates: dwell times longer than the 5 nm link flight
    sim = O.Sim(pos, ori, lk, rk, tab, 3e-9, 2e5)
    sim.set_trace(32, 1 << 16)
    sim.create_excitons(1, 0, 300, 5)
    om = sim.step(1e-13, 6)
    assert sim.total_crossings() > 0
    for prec in PRECISIONS:
        e = E.Engine(0)
        e.load_arrays(np.array([0, len(lk)], np.int64), pos, ori, lk, rk)
        e.set_table(tab)
        st = e.build(3e-9)
        assert st["isolated"] == 5
        e.set_trace(32, 1 << 16)
        e.init_excitons(300, 5, L.KMC_INJECT_UNIFORM)
        e.run(6, 1e-13, 2e5, prec)
        assert_states_equal(e.excitons(), sim.excitons())
        assert_msd_close(e.msd(0, 6), om)
        for i in range(32):
            assert np.array_equal(e.trace(i)[0], sim.trace(i)[0])
        e.close()


def test_hop_cap_reports_error_and_context_recovers():
    f, tab, r_max = synthetic_case(2, n_tubes=10, length=20.0, box=(40, 40, 4))
    e = E.Engine(0)
    e.load_films(f)
    e.set_table(tab)
    e.build(r_max)
    e.init_excitons(64, 1, L.KMC_INJECT_UNIFORM)
    e.set_hop_cap(3)
    with pytest.raises(L.KmcError) as ex:
        e.run(1, 1e-12, 2e5, L.KMC_PREC_MIXED)
    assert ex.value.code == L.KMC_ERR_HOP_CAP
    e.set_hop_cap(10**9)
    e.init_excitons(64, 1, L.KMC_INJECT_UNIFORM)
    e.run(2, 1e-13, 2e5, L.KMC_PREC_MIXED)
    assert e.stats()["hops"] > 0
    e.close()


def test_argument_errors():
    e = E.Engine(0)
    with pytest.raises(L.KmcError) as ex:
        e.run(1, 1e-13, 2e5)
    assert ex.value.code == L.KMC_ERR_STATE
    f, tab, r_max = synthetic_case(2, n_tubes=4, length=10.0, box=(20, 20, 2))
    bad = f.right.copy()
    bad[3] = f.n_sites + 5  # a link outside the film: reported, the film stays unloaded
    with pytest.raises(L.KmcError) as ex:
        e.load_arrays(np.array([0, f.n_sites], np.int64), f.pos_m(), f.orient, f.left, bad)
    assert ex.value.code == L.KMC_ERR_ARG and "bad link at 3" in str(ex.value)
    e.set_table(tab)
    with pytest.raises(L.KmcError) as ex:
        e.build(r_max)
    assert ex.value.code == L.KMC_ERR_STATE
    e.close()
    e = E.Engine(0)
    e.load_films(f)
    with pytest.raises(L.KmcError):
        e.build(r_max)  # no table yet
    e.set_table(tab)
    with pytest.raises(L.KmcError):
        e.build(-1.0)
    e.build(r_max)
    with pytest.raises(L.KmcError):
        e.init_excitons(10, 1, L.KMC_INJECT_REGION, 4)  # even number of sections
    for n_trace, cap in ((1 << 20, 1 << 17), (2**62, 2**2), (-1, 8), (4, 0)):  # too large to index, or bad
        with pytest.raises(L.KmcError) as ex:
            e.set_trace(n_trace, cap)
        assert ex.value.code == L.KMC_ERR_ARG
    e.set_trace(4, 1 << 10)
    with pytest.raises(L.KmcError) as ex:  # refused before anything is allocated
        e.init_excitons(2**31 + 1, 1, L.KMC_INJECT_UNIFORM)
    assert ex.value.code == L.KMC_ERR_ARG and "2^31" in str(ex.value)
    e.close()


def test_launch_shape_does_not_change_results():
    f, tab, r_max = synthetic_case(2, n_tubes=20, length=40.0, box=(80, 80, 6))
    out = []
    for block, spl in ((128, 32), (64, 1), (256, 5)):
        e = E.Engine(0)
        e.load_films(f)
        e.set_table(tab)
        e.build(r_max)
        e.set_launch_config(block, spl)
        e.init_excitons(1000, 3, L.KMC_INJECT_UNIFORM)
        e.run(7, 1e-13, 2e5, L.KMC_PREC_MIXED)
        out.append(e.excitons())
        e.close()
    for o in out[1:]:
        assert_states_equal(o, out[0])


@pytest.mark.parametrize("box,n_tubes,r_max,kmin", [((60, 60, 4), 40, 12e-9, 65), ((40, 40, 4), 60, 20e-9, 513)])
def test_long_rows_match_oracle(box, n_tubes, r_max, kmin):
    # neighbour rows beyond 64 entries (three-level search) and beyond 512 (FP32 bisection)
    f = F.straight_tubes(n_tubes, 40.0, box_nm=box, seed=3)
    tab = tables.forster_2d(1e15)
    sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, r_max, 2e5, n_threads=4)
    sim.create_excitons(1, 0, 400, 9)
    om = sim.step(2e-14, 4)
    for prec in PRECISIONS:
        e = E.Engine(0)
        e.load_films(f)
        e.set_table(tab)
        st = e.build(r_max)
        assert st["k_max"] >= kmin
        e.init_excitons(400, 9, L.KMC_INJECT_UNIFORM)
        e.run(4, 2e-14, 2e5, prec)
        assert_states_equal(e.excitons(), sim.excitons())
        assert_msd_close(e.msd(0, 4), om)
        e.close()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_msd_batches_and_diffusion_fit_match_oracle(precision):
    from cnt_film_monte_carlo_gb300 import diffusion

    f, tab, r_max = synthetic_case(2, n_tubes=30, length=50.0, box=(100, 100, 6))
    n_exc, seed, dt, v, steps, B = 2000, 17, 1e-13, 2e5, 10, 8
    sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, r_max, v)
    sim.create_excitons(1, 0, n_exc, seed)
    ob = sim.step_batches(dt, steps, B)
    for films in ([f], [f, f]):  # single film (shared bins off: batches > 1) and two films (global atomics)
        e = E.Engine(0)
        e.load_films(films)
        e.set_table(tab)
        e.build(r_max)
        e.set_msd_batches(B)
        e.init_excitons(n_exc, seed, L.KMC_INJECT_UNIFORM)
        e.run(steps, dt, v, precision)
        gb = e.msd_batches(0, steps)
        for k in range(len(films)):
            np.testing.assert_allclose(gb[k], ob, rtol=MSD_RTOL)
            np.testing.assert_allclose(e.msd(0, steps)[k], ob.sum(axis=1), rtol=MSD_RTOL)
        t = np.arange(1, steps + 1) * dt
        dg, cg = diffusion.fit(gb[0], n_exc, t)
        do, co = diffusion.fit(ob, n_exc, t)
        np.testing.assert_allclose(dg, do, rtol=1e-9)
        np.testing.assert_allclose(cg, co, rtol=1e-6)
        e.close()


def test_mixed_variants_and_autotune_do_not_change_results():
    f, tab, r_max = synthetic_case(2, n_tubes=20, length=40.0, box=(80, 80, 6))
    states = []
    for variant in range(6):
        e = E.Engine(0)
        e.load_films(f)
        e.set_table(tab)
        e.build(r_max)
        e.set_mixed_variant(variant)
        e.init_excitons(3000, 4, L.KMC_INJECT_UNIFORM)
        e.run(5, 1e-13, 2e5, L.KMC_PREC_MIXED)
        states.append((e.excitons(), e.msd(0, 5), e.stats()["hops"]))
        e.close()
    e = E.Engine(0)
    e.load_films(f)
    e.set_table(tab)
    e.build(r_max)
    e.init_excitons(3000, 4, L.KMC_INJECT_UNIFORM)
    choice = e.autotune(1e-13, 2e5, trial_steps=2)
    assert choice["variant"] in range(6) and choice["hops_per_s"] > 0
    e.run(5, 1e-13, 2e5, L.KMC_PREC_MIXED)
    states.append((e.excitons(), e.msd(0, 5), e.stats()["hops"]))
    e.close()
    for g, m, h in states[1:]:
        assert_states_equal(g, states[0][0])
        assert_msd_close(m, states[0][1])
        assert h == states[0][2]


def test_work_order_and_graph_do_not_change_results():
    # two films so that the spatial order interleaves nothing across films; region injection so
    # that removal/reinjection moves excitons between cells between launches
    films = [F.straight_tubes(n, 40.0, box_nm=(80, 80, 6), seed=s) for n, s in ((24, 5), (9, 6))]
    tab = tables.forster_2d(1e15)
    runs = []
    for order, graph, spl in ((L.KMC_ORDER_SLOTS, False, 1), (L.KMC_ORDER_SPATIAL, False, 1),
                              (L.KMC_ORDER_SPATIAL, True, 2), (L.KMC_ORDER_AUTO, True, 1)):
        e = E.Engine(0)
        e.load_films(films)
        e.set_table(tab)
        e.build(10e-9)
        e.set_work_order(order)
        e.set_graph(graph)
        e.set_launch_config(128, spl)
        e.init_excitons([4000, 1500], [3, 4], L.KMC_INJECT_REGION, n_sections=3)
        if order == L.KMC_ORDER_SPATIAL:
            assert e.work_order() == L.KMC_ORDER_SPATIAL
        e.run(3, 1e-13, 2e5, L.KMC_PREC_MIXED)
        e.run(2, 1e-13, 2e5, L.KMC_PREC_MIXED)  # second run: the cached graph is updated in place
        runs.append((e.excitons(), e.msd(0, 5), e.stats()["hops"]))
        e.close()
    for g, m, h in runs[1:]:
        assert_states_equal(g, runs[0][0])
        assert_msd_close(m, runs[0][1])
        assert h == runs[0][2]


def test_step_end_batching_does_not_change_results():
    # the mixed kernel batches the ends of short steps across a warp when the previous run's steps
    # averaged fewer than 64 hops: a long step (no batching next), short steps (batching off),
    # short steps again (batching on), each against the plain FP64 kernel doing the same runs
    films = [F.straight_tubes(60, 80.0, box_nm=(150, 150, 8), seed=12)]
    tab = tables.forster_2d(1e15)
    out = {}
    for prec in (L.KMC_PREC_MIXED, L.KMC_PREC_FP64):
        e = E.Engine(0)
        e.load_films(films)
        e.set_table(tab)
        e.build(10e-9)
        e.init_excitons([20000], [17], L.KMC_INJECT_REGION, n_sections=3)
        for n, dt in ((1, 3e-13), (40, 1e-15), (40, 1e-15), (1, 3e-13)):
            e.run(n, dt, 2e5, prec)
        out[prec] = (e.excitons(), e.msd(0, 82), e.stats()["hops"])
        e.close()
    g, m, h = out[L.KMC_PREC_MIXED]
    assert_states_equal(g, out[L.KMC_PREC_FP64][0])
    assert_msd_close(m, out[L.KMC_PREC_FP64][1])
    assert h == out[L.KMC_PREC_FP64][2] and h > 20000 * 100


def test_long_run_launched_directly_equals_graph_runs():
    # a run of more than 256 launches is launched without a CUDA graph; the same steps as three
    # graph-captured calls give the same state and MSD
    films = [F.straight_tubes(30, 60.0, box_nm=(100, 100, 6), seed=21)]
    tab = tables.forster_2d(1e15)
    out = []
    for chunks in ((300,), (100, 100, 100)):
        e = E.Engine(0)
        e.load_films(films)
        e.set_table(tab)
        e.build(10e-9)
        e.set_launch_config(128, 1)
        e.init_excitons([5000], [8], L.KMC_INJECT_UNIFORM)
        for n in chunks:
            e.run(n, 1e-15, 2e5, L.KMC_PREC_MIXED)
        out.append((e.excitons(), e.msd(0, 300), e.stats()))
        e.close()
    assert out[0][2]["last_launches"] >= 300 and out[0][2]["steps_done"] == 300
    assert_states_equal(out[0][0], out[1][0])
    assert_msd_close(out[0][1], out[1][1])
    assert out[0][2]["hops"] == out[1][2]["hops"]


@pytest.mark.parametrize("table_kind", [2, 4])
def test_random_geometry_csr_matches_oracle(table_kind):
    # sites at random points with random axes (each a one-site tube): pair distances and angles
    # sweep the table grids densely, so every nearest-grid tie and window edge is exercised
    rng = np.random.default_rng(11)
    n = 3000
    pos = rng.uniform(0, 40e-9, size=(n, 3))
    ax = rng.normal(size=(n, 3))
    ax /= np.linalg.norm(ax, axis=1)[:, None]
    lk = np.full(n, -1, np.int32)
    rk = np.full(n, -1, np.int32)
    if table_kind == 2:
        tab = tables.forster_2d(1e15)
    else:
        tab = E.forster_table(1e15, (0, 180, 21), (1.5e-9, 10e-9, 11), (-10e-9, 10e-9, 11), (-10e-9, 10e-9, 11))
    sim = O.Sim(pos, ax, lk, rk, tab, 8e-9, 2e5, n_threads=4)
    csr = sim.build_csr()
    e = E.Engine(0)
    e.load_arrays(np.array([0, n], np.int64), pos, ax, lk, rk)
    e.set_table(tab)
    st = e.build(8e-9)
    nb = e.neighbors(n, st["nnz"])
    for k in ("rowptr", "col", "cum", "total"):
        assert np.array_equal(nb[k], csr[k]), k
    e.close()


@pytest.mark.parametrize("offset", [0.0, 2.5e-6])
def test_window_edges_match_oracle(offset):
    # pairs at distances within a few ulps of the window edges (0.4 nm and the cutoff) in every
    # direction: the FP32 screen must hand all of them to the FP64 test, whose answer decides
    r = 8e-9
    rng = np.random.default_rng(5)
    centres = offset + rng.uniform(20e-9, 60e-9, size=(60, 3))
    pos = [centres]
    for edge in (r, 0.4e-9):
        for ulps in (-3, -1, 0, 1, 3):
            d = np.full(len(centres), edge)
            for _ in range(abs(ulps)):
                d = np.nextafter(d, np.inf if ulps > 0 else -np.inf)
            u = rng.normal(size=(len(centres), 3))
            u /= np.linalg.norm(u, axis=1)[:, None]
            pos.append(centres + d[:, None] * u)
    pos = np.concatenate(pos)
    n = len(pos)
    ax = rng.normal(size=(n, 3))
    ax /= np.linalg.norm(ax, axis=1)[:, None]
    lk = np.full(n, -1, np.int32)
    rk = np.full(n, -1, np.int32)
    tab = tables.forster_2d(1e15)
    sim = O.Sim(pos, ax, lk, rk, tab, r, 2e5, n_threads=4)
    csr = sim.build_csr()
    e = E.Engine(0)
    e.load_arrays(np.array([0, n], np.int64), pos, ax, lk, rk)
    e.set_table(tab)
    st = e.build(r)
    nb = e.neighbors(n, st["nnz"])
    for k in ("rowptr", "col", "cum", "total"):
        assert np.array_equal(nb[k], csr[k]), k
    e.close()


@pytest.mark.parametrize("precision", [L.KMC_PREC_FP64, L.KMC_PREC_MIXED])
def test_zero_rate_entries_match_oracle(precision):
    # a table with zero rates in whole bands: rows get runs of equal cumulative values, which
    # update_state skips (first cum > dice); the FP32 search must agree on every tie
    f, tab, r_max = synthetic_case(2)
    rate = tab["rate"].copy()
    rate[:, 30:60] = 0.0        # angles 30-59 deg
    rate[40:70, :] = 0.0        # distances ~4.4-7.6 nm
    tab = {"kind": 2, "grids": tab["grids"], "rate": rate}
    n_exc, seed, dt, v, steps = 800, 77, 2e-13, 2e5, 8
    sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, r_max, v)
    sim.create_excitons(1, 0, n_exc, seed)
    om = sim.step(dt, steps)
    o = sim.excitons()
    e = E.Engine(0)
    e.load_films(f)
    e.set_table(tab)
    e.build(r_max)
    e.init_excitons(n_exc, seed, L.KMC_INJECT_UNIFORM)
    e.run(steps, dt, v, precision)
    assert_states_equal(e.excitons(), o)
    assert_msd_close(e.msd(0, steps), om)
    assert e.stats()["hops"] == sim.total_hops()
    e.close()


def bad_table(kind):
    """The 2-D Förster-form table with bad values planted at a few grid points: NaN (rows with a
    NaN total: excitons landing there get a NaN dwell clock and never hop again), +inf (rows with
    an infinite total: zero dwell times, the selection clamps to the last neighbour) or negative
    rates (rows whose cumulative values fall; a few rows with a negative total)."""
    base = tables.forster_2d(1e15)
    r = base["rate"].copy()
    if kind == "nan":
        r[50, 10:20] = np.nan
    elif kind == "inf":
        r[80, 45] = np.inf
    else:
        r[:, 60:70] *= -1.0
        r[5:9, 60:62] *= 1e3
    return {"kind": 2, "grids": base["grids"], "rate": r}


def same_bits_or_both_nan(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype.kind != "f":
        return np.array_equal(a, b)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("kind", ["nan", "inf", "neg"])
def test_bad_table_values_follow_the_oracle(kind, precision):
    # the reference has no check on its table; NaN, infinite and negative rates flow through
    # its prefix sum, dwell time and bisection (scatterer.cpp:9-31, scatterer.h:74-93).  The
    # engine routes such rows to the FP64 bisection and must land where the oracle lands
    f = F.straight_tubes(40, 60.0, box_nm=(120.0, 120.0, 8.0), seed=5)
    tab = bad_table(kind)
    n_exc, seed, dt, v, steps = 800, 77, 2e-13, 2e5, 8
    sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, 10e-9, v)
    csr = sim.build_csr()
    bad_rows = {"nan": np.isnan(csr["total"]), "inf": np.isinf(csr["total"]),
                "neg": csr["total"] < 0}[kind]
    assert np.any(bad_rows)
    sim.create_excitons(1, 0, n_exc, seed)
    om = sim.step(dt, steps)
    o = sim.excitons()
    e = E.Engine(0)
    e.load_films(f)
    e.set_table(tab)
    st = e.build(10e-9)
    nb = e.neighbors(f.n_sites, st["nnz"])
    for k in ("rowptr", "col", "cum", "total"):
        assert same_bits_or_both_nan(nb[k], csr[k]), k
    e.init_excitons(n_exc, seed, L.KMC_INJECT_UNIFORM)
    e.run(steps, dt, v, precision)
    g = e.excitons()
    for k in ("site", "pos", "delta", "ff", "heading", "draws"):
        assert same_bits_or_both_nan(g[k], o[k]), k
    if kind == "nan":
        assert np.isnan(g["ff"]).sum() > 100  # excitons frozen on NaN rows
    assert e.stats()["hops"] == sim.total_hops()
    np.testing.assert_allclose(e.msd(0, steps).ravel(), om.ravel(), rtol=MSD_RTOL, atol=0)
    e.close()


def test_empty_injection_region_is_refused():
    # the central injection cell of this trimmed film holds no site: the reference divides by
    # zero there (std::rand() % 0, monte_carlo.cpp:311); the engine refuses, as the oracle does
    f = F.straight_tubes(14, 25.0, box_nm=(40, 40, 8), seed=5)
    pos, ori, lk, rk = E.trim_sites(f.pos_m(), f.orient, f.left, f.right, [5e-9, 35e-9, -1, 1, -1, 1])
    e = E.Engine(0)
    e.load_arrays(np.array([0, len(lk)], np.int64), pos, ori, lk, rk)
    e.set_table(tables.forster_2d(1e13))
    e.build(6e-9)
    with pytest.raises(L.KmcError) as ex:
        e.init_excitons(96, 3, L.KMC_INJECT_REGION, 5)
    assert ex.value.code == L.KMC_ERR_ARG and "no injection site" in str(ex.value)
    e.init_excitons(96, 3, L.KMC_INJECT_REGION, 3)  # the 3-section region holds sites
    e.close()
