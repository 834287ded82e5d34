"""Known answers computed by hand, for the oracle (CPU) and the engine (GPU, through the C ABI).

* Förster rate of a two-site geometry (create_forster_scatt_table, monte_carlo.cpp:156-200, read
  through find_neighbors' pair geometry, scatterer.cpp:34-83): two single-site tubes 3.2 nm apart
  along z with no axial offset.  Parallel (theta = 0): rate = g0 (1 nm / zsh)^6.  Perpendicular:
  rate = g0 cos^2(90 deg x 3.141592/180) (1 nm / zsh)^6 -- not zero, because the reference scales
  its theta grid with pi = 3.141592 (helper/constants.h:10).  zsh is the z-shift grid point.
* Free flight (particle::fly, particle.cpp:9-54): a three-site tube with a cutoff below its 1 nm
  spacing has no neighbours, so an exciton only flies and bounces between the tube ends; after a
  time t its position is the unfolded coordinate x0 + h v t reflected into [0, 2 nm].
* The L2 probe behind the L2 roofline separates an L2-resident buffer from one far larger than L2.
"""
import numpy as np
import pytest

from cnt_film_monte_carlo_gb300 import _lib as L
from cnt_film_monte_carlo_gb300 import engine as E
from oracle import oracle as O

G0 = 1e15
GRID = ([0, 180, 21], [1.5e-9, 10e-9, 11], [-10e-9, 10e-9, 11], [-10e-9, 10e-9, 11])
V = 2e5


def two_sites(perpendicular):
    pos = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 3.2]]) * 1e-9
    orient = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0] if perpendicular else [1.0, 0.0, 0.0]])
    lr = np.array([-1, -1], np.int32)
    return pos, orient, lr


def hand_rate(perpendicular):
    zsh = O.linspace(*GRID[1])
    z = zsh[np.argmin(np.abs(zsh - 3.2e-9))]
    ang = np.cos(90 * 3.141592 / 180) ** 2 if perpendicular else 1.0
    return G0 * ang * (1e-9 / z) ** 6


@pytest.mark.parametrize("perpendicular", [False, True])
def test_forster_pair_rate_oracle(perpendicular):
    pos, orient, lr = two_sites(perpendicular)
    tab = O.forster_table(G0, *GRID)
    sim = O.Sim(pos, orient, lr, lr, tab, 10e-9, V)
    csr = sim.build_csr()
    want = hand_rate(perpendicular)
    assert list(csr["rowptr"]) == [0, 1, 2] and list(csr["col"]) == [1, 0]
    np.testing.assert_allclose(csr["cum"], [want, want], rtol=1e-12)
    np.testing.assert_allclose(csr["total"], [want, want], rtol=1e-12)
    if perpendicular:
        assert 0 < want < 1.0  # the truncated pi leaves a rate of ~0.1 /s


def bounce_expected(x0, right, t):
    y = np.mod(x0 + (1 if right else -1) * V * t, 4e-9)
    x = np.where(y <= 2e-9, y, 4e-9 - y)
    heading = (y < 2e-9) if right else (y >= 2e-9)
    return x, heading


def tube3():
    pos = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [2.0, 0.0, 0.0]]) * 1e-9
    orient = np.tile([1.0, 0.0, 0.0], (3, 1))
    return pos, orient, np.array([-1, 0, 1], np.int32), np.array([1, 2, -1], np.int32)


def check_bounce(site0, heading0, pos, heading, t):
    x0 = np.array([0.0, 1e-9, 2e-9])[site0]
    for i in range(len(site0)):
        x, h = bounce_expected(x0[i], bool(heading0[i]), t)
        assert abs(pos[i, 0] - x) < 1e-20, (i, pos[i, 0], x)
        assert pos[i, 1] == 0.0 and pos[i, 2] == 0.0
        assert bool(heading[i]) == bool(h), i


def test_free_flight_bounces_oracle():
    pos, orient, left, right = tube3()
    tab = O.forster_table(G0, *GRID)
    sim = O.Sim(pos, orient, left, right, tab, 0.9e-9, V)
    n, dt = 64, 1.3e-14
    sim.create_excitons(1, 0, n, 11)
    s0 = sim.excitons()
    for k in range(1, 4):
        sim.step(dt, 1)
        s = sim.excitons()
        check_bounce(s0["site"], s0["heading"], s["pos"], s["heading"], k * dt)
    assert sim.total_hops() == 0 and sim.total_crossings() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("perpendicular", [False, True])
def test_forster_pair_rate_engine(perpendicular):
    pos, orient, lr = two_sites(perpendicular)
    e = E.Engine(0)
    e.load_arrays(np.array([0, 2], np.int64), pos, orient, lr, lr)
    e.set_table(O.forster_table(G0, *GRID))
    st = e.build(10e-9)
    g = e.neighbors(2, st["nnz"])
    e.close()
    want = hand_rate(perpendicular)
    assert list(g["rowptr"]) == [0, 1, 2] and list(g["col"]) == [1, 0]
    np.testing.assert_allclose(g["cum"], [want, want], rtol=1e-12)
    np.testing.assert_allclose(g["total"], [want, want], rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [L.KMC_PREC_FP64, L.KMC_PREC_MIXED])
def test_free_flight_bounces_engine(precision):
    pos, orient, left, right = tube3()
    e = E.Engine(0)
    e.load_arrays(np.array([0, 3], np.int64), pos, orient, left, right)
    e.set_table(O.forster_table(G0, *GRID))
    e.build(0.9e-9)
    n, dt = 64, 1.3e-14
    e.init_excitons(n, 11, L.KMC_INJECT_UNIFORM)
    s0 = e.excitons()
    for k in range(1, 4):
        e.run(1, dt, V, precision)
        s = e.excitons()
        check_bounce(s0["site"], s0["heading"], s["pos"], s["heading"], k * dt)
    assert e.stats()["hops"] == 0
    e.close()


@pytest.mark.gpu
def test_l2_probe_separates_l2_from_hbm():
    # the L2 roofline's denominator: an L2-resident buffer streams well above HBM speed, one far
    # larger than the L2 at about the HBM copy rate
    e = E.Engine(0)
    l2 = e.probe_l2(32 << 20, 200)
    hbm = e.probe_l2(512 << 20, 20)
    e.close()
    assert l2 > 1.5 * hbm > 3000.0
