"""Property tests of the library's host-side C-ABI functions on random inputs (CPU; hypothesis).

* kmc_trim_sites against the oracle's trim_scats (monte_carlo.h:722-782) on random films and
  limits, bit for bit, and the kept links stay symmetric and inside the kept sites;
* kmc_forster_table (create_forster_scatt_table, monte_carlo.cpp:156-200) and
  kmc_forster2d_table against the oracle on random grids, bit for bit;
* kmc_read_mesh reads back what film.write_mesh wrote, for random films;
* kmc_fit_diffusion on exactly linear batch sums: D is the batches' mean slope / 2, and the 95 %
  interval is Student's t quantile (scipy) x the batches' standard error.

The fixed cases of these functions (and their agreement with the reference's own code) are in
test_abi.py, test_tables.py and test_diffusion.py.
"""
import numpy as np
import pytest

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")
stats = pytest.importorskip("scipy.stats")

from cnt_film_monte_carlo_gb300 import diffusion  # noqa: E402
from cnt_film_monte_carlo_gb300 import engine as E  # noqa: E402
from cnt_film_monte_carlo_gb300 import film as F  # noqa: E402
from oracle import oracle as O  # noqa: E402

SETTINGS = hyp.settings(max_examples=150, deadline=None, database=None, derandomize=True)


@st.composite
def films(draw, max_tubes=6):
    n_tubes = draw(st.integers(1, max_tubes))
    lengths = draw(st.lists(st.floats(0.5, 14.0), min_size=n_tubes, max_size=n_tubes))
    box = draw(st.tuples(st.floats(1.0, 40.0), st.floats(1.0, 40.0), st.floats(0.5, 5.0)))
    seed = draw(st.integers(0, 2**31 - 1))
    return F.straight_tubes(n_tubes, lengths, box_nm=box, max_tilt_deg=draw(st.floats(0.0, 30.0)), seed=seed)


@st.composite
def limits(draw):
    """Trim limits in metres: intervals that cut the film anywhere, empty ones, reversed ones."""
    out = []
    for hi_box in (40e-9, 40e-9, 5e-9):
        a = draw(st.floats(-5e-9, hi_box + 5e-9))
        b = draw(st.floats(-5e-9, hi_box + 5e-9))
        out += [a, b] if draw(st.booleans()) else [min(a, b), max(a, b)]
    return out


@SETTINGS
@hyp.given(films(), limits())
def test_trim_matches_oracle_on_random_films(f, lim):
    p = f.pos_m()
    a = E.trim_sites(p, f.orient, f.left, f.right, lim)
    b = O.trim(p, f.orient, f.left, f.right, lim)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    pos, _, lk, rk = a
    n = len(lk)
    assert n <= f.n_sites
    assert np.all((lk >= -1) & (lk < n)) and np.all((rk >= -1) & (rk < n))
    for i in range(n):
        if lk[i] >= 0:
            assert rk[lk[i]] == i
        if rk[i] >= 0:
            assert lk[rk[i]] == i
    # every kept position is one of the film's, each kept once
    keys = {tuple(r) for r in p}
    assert all(tuple(r) in keys for r in pos)
    assert len({tuple(r) for r in pos}) == n


def grid(lo_min, lo_max, span_max, n_max):
    return st.tuples(st.floats(lo_min, lo_max), st.floats(0.0, span_max), st.integers(1, n_max)).map(
        lambda t: (t[0], t[0] + t[1], t[2]))


@SETTINGS
@hyp.given(st.floats(1e10, 1e16), grid(0.0, 90.0, 90.0, 7), grid(0.5e-9, 5e-9, 5e-9, 5),
           grid(-10e-9, 0.0, 20e-9, 4), grid(-10e-9, 0.0, 20e-9, 4))
def test_forster_table_matches_oracle_on_random_grids(gamma, th, z, a1, a2):
    t1 = E.forster_table(gamma, th, z, a1, a2)
    t2 = O.forster_table(gamma, th, z, a1, a2)
    assert np.array_equal(t1["rate"], t2["rate"], equal_nan=True)
    for g1, g2 in zip(t1["grids"], t2["grids"]):
        assert np.array_equal(g1, g2)
    for g, spec in zip(t1["grids"], (th, z, a1, a2)):
        assert len(g) == spec[2]
    for g, spec in zip(t1["grids"][1:], (z, a1, a2)):  # arma::linspace ends on the last value (metres)
        assert g[-1] == spec[1]


@SETTINGS
@hyp.given(st.floats(1e10, 1e16), grid(0.2e-9, 2e-9, 20e-9, 40), grid(0.0, 45.0, 90.0, 40))
def test_forster2d_table_matches_oracle_on_random_grids(gamma, dd, th):
    t1 = E.forster2d_table(gamma, dd, th)
    t2 = O.forster2d_table(gamma, dd, th)
    assert np.array_equal(t1["rate"], t2["rate"])
    for g1, g2 in zip(t1["grids"], t2["grids"]):
        assert np.array_equal(g1, g2)
    assert np.all(t1["rate"] >= 0)


@SETTINGS
@hyp.given(st.integers(1, 6), st.floats(0.5, 12.0), st.integers(0, 2**31 - 1))
def test_mesh_round_trip_on_random_films(tmp_path_factory, n_tubes, length, seed):
    f = F.straight_tubes(n_tubes, length, box_nm=(30, 30, 3), max_tilt_deg=20.0, seed=seed)
    d = tmp_path_factory.mktemp("mesh")
    F.write_mesh(f, str(d))
    pos, ori, lk, rk = E.read_mesh(str(d))
    assert np.array_equal(pos, f.pos_m()) and np.array_equal(ori, f.orient)
    assert np.array_equal(lk, f.left) and np.array_equal(rk, f.right)


@SETTINGS
@hyp.given(st.integers(2, 48), st.integers(3, 40), st.integers(0, 2**31 - 1), st.floats(0.1, 1.0))
def test_fit_on_exactly_linear_sums(batches, n_steps, seed, frac):
    rng = np.random.default_rng(seed)
    times = np.cumsum(rng.uniform(0.5e-13, 2e-12, n_steps))
    counts = rng.integers(1, 1000, batches).astype(np.int64)
    slope = rng.uniform(1e-6, 1e-3, (batches, 3))  # D of each batch and axis, m^2/s
    icpt = rng.uniform(0.0, 1e-16, (batches, 3))
    per = 2.0 * slope[None] * times[:, None, None] + icpt[None]  # mean squared displacement
    msd = per * counts[None, :, None]
    D, ci = diffusion.fit_counts(msd, counts, times, frac)
    np.testing.assert_allclose(D, slope.mean(axis=0), rtol=1e-9)
    se = slope.std(axis=0, ddof=1) / np.sqrt(batches)
    q = stats.t.ppf(0.975, batches - 1)
    np.testing.assert_allclose(ci, q * se, rtol=1e-8 if batches <= 32 else 2e-8, atol=1e-9 * np.abs(D).max())


def test_t_quantiles_of_small_fits_are_exact():
    """The 95 % interval of a fit over B <= 32 batches uses the quantile itself, not an
    expansion: batch slopes 0, 1, ..., B - 1 give t(0.975, B - 1) x their standard error to
    within a few ulps."""
    times = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    for batches in range(2, 33):
        slope = np.zeros((batches, 3))
        slope[:, 0] = np.arange(batches, dtype=np.float64)
        msd = 2.0 * slope[None] * times[:, None, None]
        D, ci = diffusion.fit_counts(msd, np.ones(batches, np.int64), times, 1.0)
        se = np.std(np.arange(batches, dtype=np.float64), ddof=1) / np.sqrt(batches)
        assert ci[0] == pytest.approx(stats.t.ppf(0.975, batches - 1) * se, rel=2e-15)


def test_trim_refuses_links_outside_the_film():
    f = F.straight_tubes(3, 5.0, box_nm=(20, 20, 2), seed=1)
    lim = [-1, 1, -1, 1, -1, 1]
    for field, bad in (("left", f.n_sites), ("right", -2), ("left", 2**31 - 1)):
        lk, rk = f.left.copy(), f.right.copy()
        (lk if field == "left" else rk)[2] = bad
        with pytest.raises(E.L.KmcError) as ei:
            E.trim_sites(f.pos_m(), f.orient, lk, rk, lim)
        assert ei.value.code == E.L.KMC_ERR_ARG


@pytest.mark.parametrize("n", [float("nan"), 0.0, 0.5, -3.0, 1e300, float("inf")])
def test_tables_refuse_bad_point_counts(n):
    with pytest.raises(E.L.KmcError) as ei:
        E.forster2d_table(1e15, (0.5e-9, 10e-9, n), (0.0, 90.0, 5))
    assert ei.value.code == E.L.KMC_ERR_ARG
    with pytest.raises(E.L.KmcError) as ei:
        E.forster_table(1e15, (0.0, 90.0, 3), (1e-9, 2e-9, 2), (0.0, 1e-9, n), (0.0, 1e-9, 2))
    assert ei.value.code == E.L.KMC_ERR_ARG


def _write_mesh_files(d, texts):
    names = ["single_cnt.pos.x.dat", "single_cnt.pos.y.dat", "single_cnt.pos.z.dat",
             "single_cnt.orient.x.dat", "single_cnt.orient.y.dat", "single_cnt.orient.z.dat"]
    for name, t in zip(names, texts):
        (d / name).write_bytes(t if isinstance(t, bytes) else t.encode())


def test_mesh_reader_refuses_malformed_files(tmp_path_factory):
    good = "1 2 3\n4 5 6\n"
    cases = {
        "token": ["1 2 3\n4 x 6\n"] + [good] * 5,
        "trailing text": ["1 2 3 # three\n4 5 6\n"] + [good] * 5,
        "ragged": ["1 2 3\n4 5\n"] + [good] * 5,
        "shape": [good] * 5 + ["1 2\n3 4\n5 6\n"],
        "missing": [good] * 5,
    }
    for name, texts in cases.items():
        d = tmp_path_factory.mktemp("bad_mesh")
        _write_mesh_files(d, texts)
        with pytest.raises(E.L.KmcError) as ei:
            E.read_mesh(str(d))
        assert ei.value.code == E.L.KMC_ERR_IO, name
    # blank lines, CRLF endings, commas and exponents are read
    d = tmp_path_factory.mktemp("ok_mesh")
    _write_mesh_files(d, ["1,2,3\r\n\r\n4e0 5 6\r\n"] * 6)
    pos, ori, lk, rk = E.read_mesh(str(d))
    assert np.array_equal(ori[:, 0], [1, 2, 3, 4, 5, 6]) and np.array_equal(lk, [-1, 0, 1, -1, 3, 4])


@SETTINGS
@hyp.given(st.lists(st.binary(max_size=64) | st.text(alphabet="0123456789 .,-+eE\n\r\tnaif", max_size=64),
                    min_size=6, max_size=6))
def test_mesh_reader_never_crashes(tmp_path_factory, texts):
    """Any six files give either a mesh or KMC_ERR_IO."""
    d = tmp_path_factory.mktemp("fuzz_mesh")
    _write_mesh_files(d, texts)
    try:
        pos, ori, lk, rk = E.read_mesh(str(d))
    except E.L.KmcError as e:
        assert e.code == E.L.KMC_ERR_IO
        return
    n = len(lk)
    assert pos.shape == (n, 3) and ori.shape == (n, 3)
    assert np.all((lk >= -1) & (lk < n)) and np.all((rk >= -1) & (rk < n))


def test_tables_past_2_to_34_entries_are_refused_before_allocation():
    big = (0.0, 1.0, 2**31 - 1)
    with pytest.raises(E.L.KmcError, match="too large") as ei:
        E.forster_table(1e15, big, big, big, big)
    assert ei.value.code == E.L.KMC_ERR_ARG
    with pytest.raises(E.L.KmcError, match="too large"):
        E.forster2d_table(1e15, (0.5e-9, 10e-9, 2**31 - 1), (0.0, 90.0, 2**20))
