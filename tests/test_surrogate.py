"""The learned pair-rate surrogate on the CPU: the labeller that stands in for exciton_transfer,
pinned to the reference's Förster form, the oracle network's gradient against finite
differences, and the host-side argument checks of the C ABI (no device calls)."""
import math

import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import surrogate as SG
from cnt_film_monte_carlo_gb300 import tables
from oracle import mlp as M


def test_neutral_labeller_is_the_forster_table_bit_for_bit():
    # equal chiralities, no floor, no near field: gamma_0 cos^2(theta) (1 nm / d)^6 of
    # create_forster_scatt_table (monte_carlo.cpp:174-187) as kmc_forster2d_table builds it
    t = tables.forster_2d(1e15, (0.5e-9, 10e-9, 96), (0.0, 90.0, 91))
    dist, theta = t["grids"]
    i, k = np.meshgrid(np.arange(len(dist)), np.arange(len(theta)), indexing="ij")
    z = np.zeros(i.size, np.int32)
    got = E.species_rates(SG.neutral_model(1), dist[i.ravel()], theta[k.ravel()], z, z)
    assert np.array_equal(got, t["rate"].ravel())


def test_labeller_matches_oracle():
    model = SG.species_model()
    s = SG.draw_samples(model, 20000, seed=3)
    want = M.species_rates(model, s["dist"], s["theta"], s["donor"], s["acceptor"])
    np.testing.assert_allclose(np.exp(s["log_rate"]), want, rtol=1e-13)
    # the chirality factor: downhill and same-chirality transfers are not damped, uphill ones are
    S = SG.n_species(model)
    d = np.full(S * S, 2e-9)
    th = np.zeros(S * S)
    a, b = np.divmod(np.arange(S * S), S)
    r = E.species_rates(model, d, th, a, b).reshape(S, S)
    e = model["energy"]
    lo, hi = int(np.argmin(e)), int(np.argmax(e))
    assert r[hi, lo] > 10 * r[lo, hi]


def test_labeller_table_layout():
    model = SG.species_model()
    dist, theta = SG.grids(7, 5)
    t = SG.labeller_table(model, dist, theta)
    assert t["kind"] == L.KMC_TABLE_2D_SPECIES and t["rate"].shape == (4, 4, 7, 5)
    a, b, i, k = 2, 3, 4, 1
    want = M.species_rates(model, [dist[i]], [theta[k]], [a], [b])[0]
    assert t["rate"][a, b, i, k] == pytest.approx(want, rel=1e-13)
    single = SG.single_table(model, dist, theta, species=1)
    assert single["kind"] == L.KMC_TABLE_2D and np.array_equal(single["rate"], t["rate"][1, 1])


def test_labeller_rejects_bad_arguments():
    model = SG.species_model()
    with pytest.raises(L.KmcError):
        E.species_rates(model, [1e-9], [0.0], [0], [4])  # species out of range
    bad = dict(model, width=0.0)
    with pytest.raises(L.KmcError):
        E.species_rates(bad, [1e-9], [0.0], [0], [1])


def test_bf16_rounding_known_answers():
    x = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, 1 + 2 ** -9, -2.5, 3.140625, 1e-20], np.float32)
    got = M.bf16(x)
    want = np.array([1.0, 1.0, 1 + 2 ** -6, 1.0, -2.5, 3.140625], np.float32)
    assert got[:6].tolist() == want[:6].tolist()
    assert got[6].view(np.uint32) & 0xFFFF == 0 and abs(got[6] / np.float32(1e-20) - 1) < 2 ** -8


def oracle_problem(n=300, S=3, seed=1):
    rng = np.random.default_rng(seed)
    params = (rng.standard_normal(M.n_params(S)) * 0.3).astype(np.float32)
    dist = rng.uniform(0.5e-9, 10e-9, n)
    theta = rng.uniform(0, math.pi / 2, n)
    pair = rng.integers(0, S * S, n)
    feat = M.features(dist, theta, 0.5e-9, 10e-9)
    target = rng.standard_normal(n).astype(np.float32)
    return params, S, feat, pair, target


def test_oracle_gradient_matches_finite_differences():
    params, S, feat, pair, target = oracle_problem()
    p64 = params.astype(np.float64)
    _, g = M.loss_and_grad(p64, S, feat, pair, target, quantize=False)
    rng = np.random.default_rng(5)
    idx = np.concatenate([rng.choice(np.arange(M.OFF_W1, M.OFF_B1), 6), rng.choice(np.arange(M.OFF_B1, M.OFF_W2), 3),
                          rng.choice(np.arange(M.OFF_W2, M.OFF_B2), 10), rng.choice(np.arange(M.OFF_B2, M.OFF_W3), 3),
                          rng.choice(np.arange(M.OFF_W3, M.OFF_B3), 4), [M.OFF_B3],
                          np.arange(M.OFF_E, M.n_params(S))])

    def loss_at(p):
        y, _ = M.forward(p, S, feat, pair, quantize=False)
        return float(np.mean((y - target.astype(np.float64)) ** 2))

    h = 1e-6
    for i in idx:
        pp, pm = p64.copy(), p64.copy()
        pp[i] += h
        pm[i] -= h
        fd = (loss_at(pp) - loss_at(pm)) / (2 * h)
        assert fd == pytest.approx(g[i], rel=2e-5, abs=1e-9), i
    assert np.all(g[M.OFF_B3 + 1:M.OFF_E] == 0)  # padding


def test_oracle_adam_first_step_moves_by_lr():
    rng = np.random.default_rng(2)
    p = rng.standard_normal(50).astype(np.float32)
    g = rng.standard_normal(50)
    q, m, v = M.adam(p, np.zeros(50), np.zeros(50), g, 1, 1e-3)
    # bias-corrected first step: m_hat / sqrt(v_hat) = sign(g)
    np.testing.assert_allclose(p.astype(np.float64) - q, 1e-3 * np.sign(g), rtol=1e-4, atol=1e-7)


def test_parameter_layout():
    assert L.KMC_MLP_PARAMS(4) == M.n_params(4) == 4548 + 32
    assert M.OFF_B3 == 4544 and M.OFF_W2 == 320


def test_site_species_follows_tubes():
    from cnt_film_monte_carlo_gb300 import film as F

    f = F.straight_tubes(5, [3.0, 1.0, 4.0, 2.0, 5.0], (50.0, 50.0, 5.0), 5.0, 1.0, 0)
    sp = SG.site_species(f, [3, 0, 2, 1, 3])
    assert sp.tolist() == [3] * 3 + [0] + [2] * 4 + [1] * 2 + [3] * 5
    assert sp.dtype == np.int32 and len(sp) == f.n_sites


def test_samples_are_reproducible_and_cover_the_pairs():
    model = SG.species_model()
    a = SG.draw_samples(model, 4000, seed=8)
    b = SG.draw_samples(model, 4000, seed=8)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert set(np.unique(a["pair"]).tolist()) == set(range(16))
    assert np.all(a["pair"] == a["donor"] * 4 + a["acceptor"])
    assert a["dist"].min() >= SG.D_RANGE[0] and a["dist"].max() <= SG.D_RANGE[1]
    assert a["theta"].min() >= 0 and a["theta"].max() <= math.pi / 2


def test_surrogate_calls_fail_loudly_without_a_device_or_network():
    # without a GPU the context cannot be created; with one, reading parameters before
    # kmc_mlp_init is a state error (checked on the GPU in test_gpu_surrogate)
    import ctypes as C

    lib = L.load()
    st = C.c_int(0)
    h = lib.kmc_create(0, C.byref(st))
    if h:
        lib.kmc_destroy(h)
        pytest.skip("a CUDA device is present")
    assert st.value == L.KMC_ERR_NO_DEVICE
    with pytest.raises(L.KmcError):
        E.Engine(0)


def mixed_film(seed=3, n_tubes=30, length=25.0, box=(50.0, 50.0, 8.0), S=4):
    from cnt_film_monte_carlo_gb300 import film as F

    f = F.straight_tubes(n_tubes, length, box, 5.0, 1.0, seed)
    return f, SG.site_species(f, np.random.default_rng(seed).integers(0, S, n_tubes))


def test_oracle_species_tables_are_exact_sums():
    # the oracle's chirality-pair rows: with an index-valued 2-D table the row differences give
    # each entry's grid cell exactly; the pair-table row is then the FP64 running sum of the
    # pair tables' values in list order (find_neighbors, scatterer.cpp:78-80)
    from oracle import oracle as O

    f, sp = mixed_film()
    dist, theta = SG.grids(30, 21)
    nd, nt = len(dist), len(theta)
    idx = {"kind": 2, "grids": [dist, theta], "rate": np.arange(1, nd * nt + 1, dtype=np.float64).reshape(nd, nt)}
    ci = O.Sim(f.pos_m(), f.orient, f.left, f.right, idx, 10e-9, 2e5).build_csr()
    lab = SG.labeller_table(SG.species_model(), dist, theta)
    cs = O.Sim(f.pos_m(), f.orient, f.left, f.right, lab, 10e-9, 2e5, species=sp).build_csr()
    assert np.array_equal(cs["rowptr"], ci["rowptr"]) and np.array_equal(cs["col"], ci["col"])
    flat = lab["rate"].reshape(4, 4, nd * nt)
    for s in range(f.n_sites):
        r0, r1 = ci["rowptr"][s], ci["rowptr"][s + 1]
        cells = np.diff(np.concatenate([[0.0], ci["cum"][r0:r1]])).astype(np.int64) - 1
        run = 0.0
        for j in range(r1 - r0):
            v = float(flat[sp[s], sp[ci["col"][r0 + j]], cells[j]])
            run = v if j == 0 else run + v
            assert cs["cum"][r0 + j] == run
        assert cs["total"][s] == (run if r1 > r0 else 0.0)


def test_oracle_identical_pair_tables_equal_the_2d_table():
    from oracle import oracle as O

    f, sp = mixed_film(seed=5)
    t2 = SG.single_table(SG.species_model(), *SG.grids(40, 31), species=3)
    t3 = {"kind": 3, "grids": t2["grids"], "rate": np.broadcast_to(t2["rate"], (4, 4) + t2["rate"].shape).copy()}
    a = O.Sim(f.pos_m(), f.orient, f.left, f.right, t3, 10e-9, 2e5, species=sp)
    b = O.Sim(f.pos_m(), f.orient, f.left, f.right, t2, 10e-9, 2e5)
    ca, cb = a.build_csr(), b.build_csr()
    for k in ("rowptr", "col", "cum", "total"):
        assert np.array_equal(ca[k], cb[k]), k
    # same hops on both: the Green-Kubo step reads only the rows
    for sim in (a, b):
        sim.create_excitons(1, 0, 200, 9)
        sim.step(1e-13, 2)
    ea, eb = a.excitons(), b.excitons()
    assert np.array_equal(ea["site"], eb["site"]) and a.total_hops() == b.total_hops() > 0
