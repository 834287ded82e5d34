"""The benchmark film at full size on the GPU: size-independent properties.

Film: 100 straight (7,5)-like tubes of 200 nm in a 500 x 500 x 10 nm box, 1 nm segments,
10 nm cutoff, 2-D (distance, angle) table; 1,000,000 excitons injected uniformly.
  * mixed and FP64 kernels give the same hop sequence for every exciton (states bit-equal);
  * exciton streams are independent, so the first excitons equal an oracle run of just them;
  * MSD sums equal the host sum of the returned displacements.
"""
import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from cnt_film_monte_carlo_gb300 import film as F
from cnt_film_monte_carlo_gb300 import tables
from oracle import oracle as O

pytestmark = pytest.mark.gpu

N_EXC, SEED, DT, V, STEPS = 1_000_000, 1, 1e-13, 2e5, 3


@pytest.fixture(scope="module")
def bench_film():
    f = F.straight_tubes(100, 200.0, box_nm=(500.0, 500.0, 10.0), max_tilt_deg=5.0, seed=1234)
    return f, tables.forster_2d(1e15)


def run(f, tab, precision):
    e = E.Engine(0)
    e.load_films(f)
    e.set_table(tab)
    st = e.build(10e-9)
    e.init_excitons(N_EXC, SEED, L.KMC_INJECT_UNIFORM)
    e.run(STEPS, DT, V, precision)
    out = e.excitons(), e.msd(0, STEPS), e.stats(), st
    e.close()
    return out


def test_full_size_mixed_equals_fp64_and_oracle(bench_film):
    f, tab = bench_film
    gm, mm, sm, st = run(f, tab, L.KMC_PREC_MIXED)
    gf, mf, sf, _ = run(f, tab, L.KMC_PREC_FP64)
    assert 30 < st["k_mean"] < 80
    for k in ("site", "pos", "delta", "ff", "heading", "draws", "hops"):
        assert np.array_equal(gm[k], gf[k]), k
    assert sm["hops"] == sf["hops"] and sm["hops"] > N_EXC * STEPS
    np.testing.assert_allclose(mm, mf, rtol=1e-12)
    last = (gm["delta"] ** 2).sum(axis=0)
    np.testing.assert_allclose(mm[0, -1], last, rtol=1e-12)
    n = 300
    sim = O.Sim(f.pos_m(), f.orient, f.left, f.right, tab, 10e-9, V, n_threads=4)
    sim.create_excitons(1, 0, n, SEED)
    sim.step(DT, STEPS)
    o = sim.excitons()
    for k in ("site", "pos", "delta", "ff", "heading", "draws"):
        assert np.array_equal(gm[k][:n], o[k]), k
