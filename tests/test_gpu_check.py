"""The KMC_CHECK build (libcntkmc_check.so) on the GPU.

Its hop, neighbour-build and contacts kernels bounds-check every site, row-block and link index
they follow, the MSD and slab bins they add to and the Philox counters they store.  On correct
inputs it must give the normal library's results bit for bit with the error word clear: the
golden cases (against the reference's own outputs), two films in both precisions with region
injection (reinjections) and a contacts run.  One check is made to fire by an input the API
accepts: an exciton restored with its Philox counter two draws short of 2^64 wraps it during the
step, which only the checked build reports (KMC_ERR_CHECK); the wrap changes which random
numbers are drawn, never an address.
"""
import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import tables
from helpers import CASES, CONTACT_CASES, case_inputs, contacts_inputs, load_case
from test_gpu_resume import KEYS

pytestmark = pytest.mark.gpu

V, BIN = 2e5, 1e-12


def films_run(checked, precision, steps=20):
    fs = [F.straight_tubes(60, 150.0, box_nm=(300.0, 300.0, 10.0), max_tilt_deg=5.0, seed=21),
          F.lognormal_tubes(80, 120.0, 0.5, (250.0, 250.0, 12.0), seed=22)]
    e = E.Engine(0, checked=checked)
    e.load_films(fs)
    e.set_table(tables.forster_2d(1e15))
    nb = e.build(10e-9)
    e.set_msd_batches(4)
    e.init_excitons([1200, 700], [3, 4], L.KMC_INJECT_REGION, 5)
    e.run(steps, BIN, V, precision)
    out = {"x": e.excitons(), "msd": e.msd_batches(0, steps), "stats": e.stats(), "nbr": nb}
    out["rows"] = e.neighbors(int(nb["n_sites"]), int(nb["nnz"]))
    e.close()
    return out


@pytest.mark.parametrize("precision", [L.KMC_PREC_MIXED, L.KMC_PREC_FP64])
def test_checked_build_equals_normal_build(precision):
    a, b = films_run(False, precision), films_run(True, precision)
    for k in KEYS:
        assert np.array_equal(a["x"][k], b["x"][k]), k
    for k in ("rowptr", "col", "cum", "total"):
        assert np.array_equal(a["rows"][k], b["rows"][k]), k
    assert a["stats"]["hops"] == b["stats"]["hops"] > 0
    np.testing.assert_allclose(a["msd"], b["msd"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("precision", [L.KMC_PREC_MIXED, L.KMC_PREC_FP64])
@pytest.mark.parametrize("name", CASES)
def test_checked_build_on_golden_cases(name, precision):
    # the reference's own rows and exciton states (golden fixtures), through the checked build
    d = load_case(name)
    ci = case_inputs(d)
    pos, ori, lk, rk = E.trim_sites(ci["pos"], ci["orient"], ci["left"], ci["right"], ci["lim"])
    e = E.Engine(0, checked=True)
    e.load_arrays(np.array([0, len(lk)], np.int64), pos, ori, lk, rk)
    e.set_table(E.forster_table(ci["gamma"], *ci["grids"]))
    st = e.build(ci["r_max"])
    nb = e.neighbors(len(lk), st["nnz"])
    assert np.array_equal(nb["rowptr"], d["ref_csr_rowptr"]) and np.array_equal(nb["col"], d["ref_csr_col"])
    assert np.array_equal(nb["cum"], d["ref_csr_cum"])
    e.init_excitons(ci["n_exc"], int(d["seed"]), L.KMC_INJECT_REGION, ci["sections"])
    e.run(int(d["steps"]), ci["dt"], ci["v"], precision)
    g = e.excitons()
    assert np.array_equal(g["site"], d["ref_site"])
    assert np.array_equal(g["pos"].ravel(), d["ref_xpos"])
    assert np.array_equal(g["delta"].ravel(), d["ref_delta"])
    assert np.array_equal(g["ff"], d["ref_ff"])
    assert np.array_equal(g["draws"], d["ref_draws"])
    assert e.stats()["hops"] == int(d["ref_hops"][0])
    e.close()


def test_checked_build_contacts():
    d = load_case(CONTACT_CASES[0])
    c = contacts_inputs(d)
    res = []
    for checked in (False, True):
        e = E.Engine(0, checked=checked)
        e.load_arrays(np.array([0, len(c["left"])], np.int64), c["pos"], c["orient"], c["left"], c["right"])
        e.set_table(c["table"])
        e.build(c["r_max"])
        e.contacts_init(c["n_seg"], c["pops"], c["seed"], len(d["ref_site"]) + 64)
        pop, cur, live = e.contacts_run(c["steps"], c["dt"], c["v"], L.KMC_PREC_MIXED)
        res.append((pop, cur, live, e.excitons()))
        e.close()
    (pa, ca, la, xa), (pb, cb, lb, xb) = res
    assert np.array_equal(pa, pb) and np.array_equal(ca, cb) and np.array_equal(la, lb)
    assert np.array_equal(pa.ravel(), d["ref_pop"])
    for k in KEYS:
        assert np.array_equal(xa[k], xb[k]), k


@pytest.mark.parametrize("precision", [L.KMC_PREC_MIXED, L.KMC_PREC_FP64])
def test_philox_counter_wrap_is_reported(precision):
    f = F.straight_tubes(30, 100.0, box_nm=(150.0, 150.0, 8.0), max_tilt_deg=5.0, seed=9)
    codes = []
    for checked in (False, True):
        e = E.Engine(0, checked=checked)
        e.load_films([f])
        e.set_table(tables.forster_2d(1e15))
        e.build(10e-9)
        e.init_excitons(64, 5, L.KMC_INJECT_UNIFORM)
        s = e.excitons()
        s["draws"][7] = np.uint64(2**64 - 2)
        e.set_excitons(s)
        try:
            e.run(1, BIN, V, precision)
            codes.append(L.KMC_OK)
        except L.KmcError as ex:
            codes.append(ex.code)
        e.close()
    assert codes == [L.KMC_OK, L.KMC_ERR_CHECK]
