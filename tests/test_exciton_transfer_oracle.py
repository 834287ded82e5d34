"""The CPU restatement of exciton_transfer's tube geometry and Coulomb sum (oracle/
exciton_transfer.py), which future device kernels for the labeller are checked against.  The
reference's own code cannot be compiled here (it needs Armadillo's complex types and eig_sym), so
the restatement is checked against the tube-geometry closed forms (Saito, Dresselhaus &
Dresselhaus), the calculate_J double loop as written, and identities of the sum."""
import math

import numpy as np
import pytest

from oracle import exciton_transfer as X

CHIRALITIES = [(6, 5), (7, 5), (8, 3), (8, 4), (10, 0), (5, 5)]


@pytest.mark.parametrize("n,m", CHIRALITIES)
def test_tube_geometry_closed_forms(n, m):
    g = X.cnt_geometry(n, m, 2)
    dR = math.gcd(2 * n + m, 2 * m + n)
    assert g["Nu"] == 2 * (n * n + n * m + m * m) // dR
    ch_len = X.A_L * math.sqrt(n * n + n * m + m * m)
    assert g["ch_len"] == pytest.approx(ch_len, rel=1e-12)
    assert np.linalg.norm(g["t_vec"]) == pytest.approx(math.sqrt(3) * ch_len / dR, rel=1e-12)
    assert g["radius"] == pytest.approx(ch_len / (2 * 3.141592), rel=1e-15)
    # the rotated frame: chiral vector along x, translation vector along y
    assert abs(g["ch"][1]) < 1e-15 * ch_len and abs(g["t_vec"][0]) < 1e-15 * ch_len
    # unit cells inside one period, on the cylinder
    p = g["pos_u_2d"]
    assert p[:, 0].min() >= 0 and p[:, 0].max() <= g["ch"][0]
    assert p[:, 1].min() >= 0 and p[:, 1].max() <= g["t_vec"][1]
    q = g["pos_u_3d"]
    np.testing.assert_allclose(np.hypot(q[:, 0], q[:, 2]), g["radius"], rtol=1e-14)


@pytest.mark.parametrize("n,m", CHIRALITIES)
def test_unit_cells_form_the_graphene_lattice(n, m):
    # every A atom's nearest A neighbours (periodic images across the chiral and translation
    # periods included) sit one lattice constant away, and no two unit cells coincide
    g = X.cnt_geometry(n, m, 1)
    p = g["pos_u_2d"]
    ch, tv = g["ch"], g["t_vec"]
    images = np.concatenate([p + a * ch + b * tv for a in (-1, 0, 1) for b in (-1, 0, 1)])
    d = np.linalg.norm(p[:, None, :] - images[None, :, :], axis=2)
    d[d < 1e-3 * X.A_L] = np.inf  # the atom itself
    np.testing.assert_allclose(d.min(axis=1), X.A_L, rtol=1e-9)
    assert np.all((d < 0.999 * X.A_L).sum(axis=1) == 0)
    # and the A-B bond is a_cc
    assert np.linalg.norm(g["acc"]) == pytest.approx(X.A_L / math.sqrt(3), rel=1e-12)


def test_lattice_constant_keeps_the_single_precision_square_root():
    # cnt.h:26 takes sqrt(float(3.0)): the lattice constant differs from sqrt(3) a_cc in the 8th digit
    assert X.A_L == float(np.float32(math.sqrt(3.0))) * 1.42e-10
    assert abs(X.A_L / (math.sqrt(3) * 1.42e-10) - 1) > 1e-9


def small_pair():
    return X.cnt_geometry(5, 0, 3), X.cnt_geometry(5, 5, 4)


def test_coulomb_sum_equals_the_double_loop():
    gi, gf = small_pair()
    for ik_i, ik_f, shifts, z, ang in [(0, 0, (0.0, 0.0), 2e-9, 0.0), (1, -2, (1e-10, -3e-10), 1.5e-9, 0.7),
                                       (3, 2, (0.0, 5e-10), 3e-9, 1.9)]:
        a = X.coulomb_j(gi, gf, ik_i, ik_f, shifts, z, ang, block=7)
        b = X.coulomb_j_loops(gi, gf, ik_i, ik_f, shifts, z, ang)
        assert abs(a - b) <= 1e-12 * abs(b)


def test_coulomb_sum_identities():
    gi, gf = small_pair()
    # real kernel 1/|R|: flipping both momenta conjugates J
    a = X.coulomb_j(gi, gf, 2, -1, (0.0, 0.0), 2e-9, 0.4)
    b = X.coulomb_j(gi, gf, -2, 1, (0.0, 0.0), 2e-9, 0.4)
    assert abs(a - b.conjugate()) <= 1e-12 * abs(a)
    # zero momenta: a sum of positive terms
    c = X.coulomb_j(gi, gf, 0, 0, (0.0, 0.0), 2e-9, 0.4)
    assert abs(c.imag) < 1e-12 * c.real and c.real > 0
    # far field at zero momenta: N_i N_f / separation (the tubes are ~2 nm long, 1 um apart)
    z = 1e-6
    far = X.coulomb_j(gi, gf, 0, 0, (0.0, 0.0), z, 0.3)
    n_i, n_f = len(X.unit_cells_2d(gi)), len(X.unit_cells_2d(gf))
    assert far.real == pytest.approx(n_i * n_f / z, rel=1e-5) and abs(far.imag) < 1e-12 * far.real
    # at nonzero momenta a whole tube's phases cancel, so the monopole term vanishes
    ei = np.exp(-1j * (X.unit_cells_2d(gi) @ (1 * gi["dk_l"]))).sum()
    assert abs(ei) < 1e-6 * n_i


@pytest.mark.parametrize("n,m,nk", [(5, 5, 6), (10, 0, 9), (7, 5, 12), (8, 4, 30)])
def test_tight_binding_bands_are_zone_folded_graphene(n, m, nk, monkeypatch):
    # with pi exact, the tube Hamiltonian's eigenvalues are graphene's nearest-neighbour bands on
    # the tube's cutting lines to rounding
    monkeypatch.setattr(X, "PI", math.pi)
    g = X.cnt_geometry(n, m, nk)
    np.testing.assert_allclose(X.electron_bands(g), X.zone_folded_bands(g), rtol=0, atol=1e-12 * X.T0)


def test_reference_pi_shifts_the_bands_slightly():
    # exciton_transfer's pi = 3.141592 enters the reciprocal vectors, so b.a != 2 pi and the
    # axial momenta sit 2e-7 off the Brillouin-zone grid: bands move by ~1e-5 t0
    g = X.cnt_geometry(7, 5, 12)
    d = np.abs(X.electron_bands(g) - X.zone_folded_bands(g)).max() / X.T0
    assert 1e-8 < d < 1e-4


def test_band_gaps_and_eigenvector_phases():
    # armchair (5,5) is metallic (a k point of a 6-cell grid hits the Dirac point), (7,5) has
    # E11 ~ 2 t0 a_cc / d = 0.94 eV
    g = X.cnt_geometry(5, 5, 6)
    assert np.abs(X.electron_bands(g)).min() < 1e-5 * X.EV
    g = X.cnt_geometry(7, 5, 60)
    gap = 2 * np.abs(X.electron_bands(g)).min() / X.EV
    assert 0.9 < gap < 1.0
    E, C = X.electron_bands(X.cnt_geometry(5, 0, 4), vectors=True)
    first = C[:, 0, :]
    assert np.all(np.abs(first.imag) < 1e-12) and np.all(first.real >= 0)
    for k in range(C.shape[0]):
        np.testing.assert_allclose(C[k].conj().T @ C[k], np.eye(C.shape[1]), atol=1e-12)


def test_vq_equals_the_loops_as_written():
    g = X.cnt_geometry(5, 0, 5)
    a = X.calculate_vq(g, (-2, 3), (0, 4), 5)
    b = X.calculate_vq_loops(g, (-2, 3), (0, 4), 5)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())


def test_vq_identities():
    g = X.cnt_geometry(7, 5, 11)
    v = X.calculate_vq(g, (-2, 3), (0, 3), 11)
    # q = 0: the plain sum of the potential over each sublattice pair's positions
    rel = X.vq_positions(g, 11)
    coeff = (4. * X.PI * X.EPS0 * X.UPP / X.Q0 / X.Q0) ** 2
    pot = X.UPP / np.sqrt(coeff * (rel[..., 0] ** 2 + rel[..., 1] ** 2) + 1)
    q0 = v[2, 0]  # iq = 0, mu = 0
    np.testing.assert_allclose(q0.real, pot.sum(axis=1) / (2 * g["Nu"] * 11), rtol=1e-12)
    assert np.all(q0.imag == 0)
    # same-sublattice sums agree (A-A and B-B see the same lattice); A-B and B-A are mirror
    # images, conjugate up to the one-sided fold at +-ch/2
    np.testing.assert_allclose(v[..., 0], v[..., 3], rtol=1e-9, atol=1e-12 * np.abs(v).max())
    assert np.abs(v[..., 1] - np.conj(v[..., 2])).max() < 1e-2 * np.abs(v).max()
    # an even cell count is made odd, as the reference does
    assert X.vq_positions(g, 10).shape == X.vq_positions(g, 11).shape


@pytest.mark.parametrize("n,m,nk", [(7, 5, 6), (8, 4, 10), (5, 5, 6), (10, 0, 5)])
def test_k2_extended_bands_relabel_the_full_unit_cell_bands(n, m, nk, monkeypatch):
    # the K2-extended grid (Q cutting lines x Nu/Q nk points) holds the same k points as the
    # full-unit-cell grid (Nu lines x nk points): with pi exact, the same energies
    monkeypatch.setattr(X, "PI", math.pi)
    g = X.cnt_geometry(n, m, nk)
    assert g["M"] is not None and g["Nu"] % g["Q"] == 0
    E, _ = X.k2_extended(g)
    np.testing.assert_allclose(np.sort(E.ravel()), np.sort(X.electron_bands(g).ravel()), rtol=0, atol=1e-11 * X.T0)


def test_two_band_eigenpairs_and_valleys():
    g = X.cnt_geometry(7, 5, 8)
    E, W = X.k2_extended(g)
    d = [(g["a1"] + g["a2"]) / 3., (g["a1"] - 2. * g["a2"]) / 3., (g["a2"] - 2. * g["a1"]) / 3.]
    for ik in (0, 17, 555, 1743):
        k = 0 * g["K1"] + ik * g["dk_l"]
        f = sum(np.exp(1j * float(k @ v)) for v in d)
        H = np.array([[0, -X.T0 * f], [-X.T0 * np.conj(f), 0]])
        psi = W[0][:, :, ik]  # [atom][band]
        for band in (0, 1):
            np.testing.assert_allclose(H @ psi[:, band], E[band, ik, 0] * psi[:, band], atol=1e-12 * X.T0)
        np.testing.assert_allclose(psi.conj().T @ psi, np.eye(2), atol=1e-14)
    valleys = X.find_valleys(E)
    assert valleys, "no valley"
    (a, b) = valleys[0]
    assert E[1][a] == pytest.approx(E[1][b], rel=1e-6)  # K and K' valleys
    assert E[1][a] == E[1].min()
    # E11 of (7,5) in this tight binding: 2 x the valley energy, ~0.94 eV
    assert 0.9 < 2 * E[1].min() / X.EV < 1.0


@pytest.mark.parametrize("n,m,cells", [(5, 5, 4), (8, 4, 2)])
def test_polarization_equals_the_loops_and_is_symmetric(n, m, cells):
    g = X.cnt_geometry(n, m, cells)
    E, W = X.k2_extended(g)
    ikr, mur = (0, g["Nu"] // g["Q"] * cells), (0, g["Q"])
    # the q range of calculate_exciton_dispersion (cnt.cpp:1069-1070)
    iqr, muqr = (-(ikr[1] - 1), ikr[1]), (-(mur[1] - 1), mur[1])
    a = X.calculate_polarization(g, iqr, muqr, E, W, ikr, mur)
    b = X.calculate_polarization_loops(g, iqr, muqr, E, W, ikr, mur)
    # at q = 0 (same k) valence and conduction states are orthogonal and PI is rounding noise
    # (~1e-12 against ~1e20), hence the absolute floor
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())
    assert np.all(a >= 0)  # every term is a squared overlap over a positive gap
    assert a[ikr[1] - 1, mur[1] - 1] < 1e-20 * a.max()
    # time reversal: |f(-k)| = |f(k)|
    np.testing.assert_allclose(a, a[::-1, ::-1], rtol=1e-10, atol=1e-12 * a.max())


def test_dielectric_function():
    g = X.cnt_geometry(5, 5, 3)
    E, W = X.k2_extended(g)
    ikr, mur = (0, g["Nu"] // g["Q"] * 3), (0, g["Q"])
    iqr, muqr = (-(ikr[1] - 1), ikr[1]), (-(mur[1] - 1), mur[1])
    pi = X.calculate_polarization(g, iqr, muqr, E, W, ikr, mur)
    vq = X.calculate_vq(g, iqr, muqr, 3)
    eps = X.calculate_dielectric(vq, pi)
    np.testing.assert_allclose(eps, 1 + vq.real.mean(axis=2) * pi, rtol=1e-15)
    # no interband polarisation at q = 0: eps = 1 there; the positive Ohno potential screens
    # every other q
    q0 = (ikr[1] - 1, mur[1] - 1)
    assert eps[q0] == pytest.approx(1.0, abs=1e-12)
    mask = np.ones_like(eps, bool)
    mask[q0] = False
    assert np.all(eps[mask] > 1.0)


def test_relevant_states_around_the_valleys():
    # the states within 1 eV of each valley bottom (calculate_exciton_dispersion's window,
    # cnt.cpp:1066): contiguous in ik around the bottom, all below the window, and the two
    # equivalent valleys keep the same number of states
    g = X.cnt_geometry(7, 5, 10)
    E, _ = X.k2_extended(g)
    valleys = X.find_valleys(E)
    rel = X.find_relev_ik_range(E, valleys[0], 1.0 * X.EV)
    nk = E.shape[1]
    assert len(rel) == 2 and len(rel[0]) == len(rel[1]) > 1
    for states, (ikb, mub) in zip(rel, valleys[0]):
        iks = [ik for ik, mu in states]
        assert all(mu == mub for _, mu in states)
        steps = [(b - a) % nk for a, b in zip(iks, iks[1:])]
        assert steps == [1] * len(steps)  # contiguous, wrapping across the zone edge
        assert ikb in iks
        assert max(E[1, ik, mub] for ik in iks) < E[1, ikb, mub] + 1.0 * X.EV


@pytest.fixture(scope="module")
def excitons_84():
    g = X.cnt_geometry(8, 4, 12)
    return X.exciton_dispersion(g), X.exciton_dispersion(g, interaction=False)


def test_bse_without_interaction_gives_the_free_pairs(excitons_84):
    # vq = 0, eps = 1: the kernels are diagonal with the pair energies E_c(k) - E_v(k - k_cm)
    _, free = excitons_84
    E = free["energy"]
    nk = E.shape[1]
    v1 = free["relev"][0]
    for a, ik_cm in enumerate(range(*free["ik_cm_range"])):
        pairs = sorted(E[1, ik, mu] - E[0, (ik - ik_cm) % nk, mu] for ik, mu in v1)
        for key in ("A1", "A2_triplet", "A2_singlet"):
            np.testing.assert_allclose(free[key][a], pairs, rtol=0, atol=1e-12 * X.T0)


def test_bse_binds_the_a_excitons(excitons_84):
    ex, free = excitons_84
    k0 = -ex["ik_cm_range"][0]
    gap = 2 * ex["energy"][1].min()
    assert free["A1"][k0].min() == pytest.approx(gap, rel=1e-12)
    for k11, k12, kx in ex["kernels"]:
        for k in (k11, k12, kx):
            assert np.abs(k - k.conj().T).max() == 0.0
    # screened attraction binds the lowest exciton well below the band gap; exchange pushes the
    # singlet above the triplet; screening never anti-screens
    assert 0.2 * gap < ex["A1"][k0].min() < 0.8 * gap
    assert ex["A2_singlet"][k0].min() > ex["A2_triplet"][k0].min()
    assert ex["eps"].min() >= 1.0


def test_first_order_rate_of_the_restated_model(excitons_84):
    # the reference's first-order transfer rate between two parallel (8,4) tubes of 12 unit cells
    # (13.5 nm): positive, falling with the centre distance, of the Förster form's order at a few
    # nanometres (gamma_0 (1 nm / d)^6 = 1.4e12 /s at 3 nm)
    ex, _ = excitons_84
    g = X.cnt_geometry(8, 4, 12)
    rates = [X.first_order(g, ex, g, ex, z) for z in (1.5e-9, 3e-9, 6e-9)]
    assert rates[0] > rates[1] > rates[2] > 0
    assert 1e11 < rates[1] < 1e14
    # the matrix element does not depend on the phase of the exciton eigenvectors
    st = X.relevant_states(ex, ex["A2_singlet"].min())[0]
    q = X.q_partial(g, ex, st)
    ex2 = dict(ex, A2_singlet_psi=[p * np.exp(0.7j) for p in ex["A2_singlet_psi"]])
    assert abs(X.q_partial(g, ex2, st)) == pytest.approx(abs(q), rel=1e-12)
