"""CPU oracle for exciton_transfer's tube geometry, bands and Coulomb sum -- TEST INFRASTRUCTURE ONLY.

Only the tests use this module, to check future device kernels; the product never calls it.

What it restates (reference project paths):

* ``cnt_geometry``: ``cnt::get_parameters`` (src/exciton_transfer/cnt.cpp:16-60, 81-86) and
  ``cnt::get_atom_coordinates`` (cnt.cpp:120-210).  The graphene lattice constant is
  a_l = sqrt(float(3)) a_cc (cnt.h:25-26: the square root is taken in single precision), pi is
  3.141592 (src/exciton_transfer/constants.h:10), the lattice is rotated so that the chiral
  vector lies along x, and the unit-cell (A-atom) positions are wrapped into the chiral period.
* ``unit_cells_3d`` / ``unit_cells_2d``: the lambdas make_Ru_3d / make_Ru_2d of
  ``exciton_transfer::calculate_J`` (exciton_transfer.cpp:310-355): every graphene unit cell of
  the whole tube, centred on its axis, shifted along it and in z, rotated about z.
* ``coulomb_j``: calculate_J (exciton_transfer.cpp:357-377),
  J = sum_i sum_j exp(-i k_i . r_i) exp(+i k_f . r_j) / |R_i - R_j|.
* ``electron_bands``: cnt::electron_full_unit_cell (cnt.cpp:212-300), the nearest-neighbour
  tight-binding bands of the full tube unit cell; ``zone_folded_bands`` is the closed form it
  must equal (graphene bands on the tube's cutting lines).
* ``electron_energy`` / ``k2_extended`` / ``find_valleys`` / ``find_relev_ik_range``: the
  two-band bands of the K2-extended representation, their valleys and the states within an
  energy window of each valley bottom (cnt.cpp:302-505, 1061-1066).
* ``calculate_polarization`` / ``calculate_dielectric``: the static polarisation of the
  K2-extended bands and the dielectric function (cnt.cpp:634-757).
* ``calculate_a_excitons``: the Bethe-Salpeter kernels and A-exciton energies
  (cnt.cpp:783-1000).
* ``relevant_states``, ``q_partial``, ``first_order``: the thermal A2-singlet states, the
  Q matrix element and the first-order transfer rate (exciton_transfer.cpp:226-304, 380-424;
  exciton_transfer.h:30-33, 167-196).
* ``calculate_vq``: cnt::calculate_vq (cnt.cpp:520-631), the Fourier sums of the Ohno
  potential per sublattice pair that the dielectric function and the Bethe-Salpeter kernel use.

Parity: pinned against the reference's own code.  oracle/_ref/ref_exciton is cnt.cpp and
exciton_transfer.cpp compiled unchanged against a second Armadillo shim (oracle/shim_et), and
tests/golden/ref_et_*.npz hold what it computes for four tube pairs (the two pairs of the
reference's input.json and two of the surrogate's chiralities).  This restatement reproduces
them: lattice vectors, K2-extended parameters, valleys and relevant-state windows exactly; bands,
vq, PI, eps and the A-exciton energies to ~1e-15 relative; J to ~1e-14; |Q|, M and the
first-order rate to ~1e-12 (tests/test_exciton_transfer_golden.py).  Eigenvector phases are not
compared (neither LAPACK's nor the shim's Jacobi fixes them); everything compared is phase-free.
The older tests also check tube-geometry invariants, a brute-force double loop, far-field and
conjugation identities, and the bands against zone-folded graphene.
"""
from __future__ import annotations

import math

import numpy as np

A_CC = 1.42e-10                               # carbon-carbon distance, m (cnt.h:25)
A_L = float(np.sqrt(np.float32(3.0))) * A_CC  # cnt.h:26: std::sqrt(float(3.0)) * a_cc
PI = 3.141592                                 # constants.h:10


def cnt_geometry(n: int, m: int, n_cells: int) -> dict:
    """Lattice vectors (rotated frame), radius, translation vector, the Nu unit-cell positions in
    the unrolled sheet and on the cylinder, and the axial k step dk_l = K2 / n_cells."""
    s3 = math.sqrt(3.0)
    a1 = np.array([A_L * s3 / 2.0, +A_L / 2.0])
    a2 = np.array([A_L * s3 / 2.0, -A_L / 2.0])
    b1 = np.array([1.0 / math.sqrt(3.0) * 2.0 * PI / A_L, +2.0 * PI / A_L])
    b2 = np.array([1.0 / math.sqrt(3.0) * 2.0 * PI / A_L, -2.0 * PI / A_L])
    acc = 1.0 / 3.0 * (a1 + a2)
    ch = float(n) * a1 + float(m) * a2
    ch_len = float(np.linalg.norm(ch))
    radius = ch_len / 2.0 / PI
    dR = math.gcd(2 * n + m, n + 2 * m)
    t1 = (2 * m + n) // dR
    t2 = -(2 * n + m) // dR
    tv = float(t1) * a1 + float(t2) * a2
    Nu = int(2 * (n * n + m * m + n * m) / dR)
    c = ch[0] / np.linalg.norm(ch)
    s = ch[1] / np.linalg.norm(ch)

    def rot(v):  # [[c, s], [-s, c]] v
        return np.array([c * v[0] + s * v[1], -s * v[0] + c * v[1]])

    ch, tv, a1, a2, b1, b2, acc = (rot(v) for v in (ch, tv, a1, a2, b1, b2, acc))
    t3 = np.array([0.0, tv[1], 0.0])
    K2 = (float(m) * b1 - float(n) * b2) / float(Nu)
    dk_l = K2 / float(n_cells)
    K1 = (-float(t2) * b1 + float(t1) * b2) / float(Nu)
    # K2-extended representation (cnt.cpp:88-114): the first p with (1 + t2 p) divisible by t1
    p_min = (1. / float(t1) + 1. / float(n)) / (float(m) / float(n) - float(t2) / float(t1))
    p_max = (1. / float(t1) + float(Nu) / float(n)) / (float(m) / float(n) - float(t2) / float(t1))
    M = Q = None
    for pp in range(math.ceil(p_min), math.ceil(p_max)):
        if (1 + t2 * pp) % t1 == 0:
            qq = (1 + t2 * pp) // t1
            M = m * pp - n * qq
            Q = math.gcd(Nu, M)
            break
    # unit-cell (A-atom) and B-atom positions inside the chiral period
    pos_a, pos_b = [], []

    def wrap(p):
        for d in range(2):
            if p[d] > ch[d]:
                p[d] -= ch[d]
            if p[d] < 0.0:
                p[d] += ch[d]
        return p

    for i in range(0, t1 + n + 1):
        for j in range(t2, m + 1):
            f1 = (t2 * i) / t1 <= j
            f2 = (m * i) / n >= j
            f3 = (t2 * (i - n)) / t1 > (j - m)
            f4 = (m * (i - t1)) / n < (j - t2)
            if f1 and f2 and f3 and f4:
                p = float(i) * a1 + float(j) * a2
                q = p + acc
                pos_a.append(wrap(p))
                pos_b.append(wrap(q))
    pos_a, pos_b = np.array(pos_a), np.array(pos_b)
    if len(pos_a) != Nu:
        raise ValueError(f"({n},{m}): found {len(pos_a)} unit cells, expected {Nu}")

    def roll(p2):
        return np.stack([radius * np.cos(p2[:, 0] / radius), p2[:, 1], radius * np.sin(p2[:, 0] / radius)], 1)

    pos_2d = np.concatenate([pos_a, pos_b])
    return {"n": n, "m": m, "a1": a1, "a2": a2, "b1": b1, "b2": b2, "acc": acc, "ch": ch, "ch_len": ch_len,
            "radius": radius, "t_vec": tv, "t_vec_3d": t3, "Nu": Nu, "t1": t1, "t2": t2, "dR": dR, "K1": K1, "K2": K2,
            "M": M, "Q": Q,
            "pos_u_2d": pos_a, "pos_u_3d": roll(pos_a), "pos_2d": pos_2d, "pos_3d": roll(pos_2d), "dk_l": dk_l,
            "n_cells": n_cells}


EV = 1.6e-19       # constants.h:12
T0 = 2.7 * EV      # nearest-neighbour hopping, cnt.h:29 (on-site e2p = 0, overlap s0 = 0)


def electron_bands(g: dict, vectors: bool = False):
    """cnt::electron_full_unit_cell (cnt.cpp:212-300): the 2Nu x 2Nu nearest-neighbour
    tight-binding Hamiltonian of one tube unit cell with Bloch phases exp(i k l T) across the
    translation period, at k = (n - nk/2) |dk_l| for n < nk = number of unit cells; energies
    ascending [2Nu][nk] (J) and, with vectors, eigenvectors [nk][2Nu][2Nu] with the reference's
    phase fix (first component real and non-negative)."""
    p = g["pos_3d"]
    t3 = g["t_vec_3d"]
    N2 = len(p)
    nn = []
    for i in range(N2):
        row = []
        for j in range(N2):
            for l in (-1, 0, 1):
                dR = np.linalg.norm(p[i] - p[j] + float(l) * t3)
                if i != j and dR < 1.4 * A_CC:
                    row.append((j, l))
        if len(row) != 3:
            raise ValueError(f"atom {i}: {len(row)} nearest neighbours")
        nn.append(row)
    nk = g["n_cells"]
    t_len = float(np.linalg.norm(t3))
    dk = float(np.linalg.norm(g["dk_l"]))
    E = np.zeros((N2, nk))
    C = np.zeros((nk, N2, N2), complex) if vectors else None
    for n in range(nk):
        wave_vec = float(n - nk // 2) * dk
        H = np.zeros((N2, N2), complex)
        for i in range(N2):
            for j, l in nn[i]:
                H[i, j] += T0 * np.exp(1j * wave_vec * float(l) * t_len)
        e, c = np.linalg.eigh(H)
        E[:, n] = e
        if vectors:
            phi = np.conj(c[0, :]) / np.abs(c[0, :])
            C[n] = c * phi[None, :]
    return (E, C) if vectors else E


def zone_folded_bands(g: dict) -> np.ndarray:
    """Nearest-neighbour graphene bands +-t0 |1 + exp(i k.a1) + exp(i k.a2)| on the tube's
    cutting lines k = mu K1 + kappa K2/|K2| (mu < Nu), at the axial momenta of electron_bands."""
    nk = g["n_cells"]
    dk = float(np.linalg.norm(g["dk_l"]))
    K2h = g["K2"] / np.linalg.norm(g["K2"])
    out = np.zeros((2 * g["Nu"], nk))
    for n in range(nk):
        kappa = float(n - nk // 2) * dk
        ks = np.arange(g["Nu"])[:, None] * g["K1"][None, :] + kappa * K2h[None, :]
        f = np.abs(1 + np.exp(1j * (ks @ g["a1"])) + np.exp(1j * (ks @ g["a2"])))
        out[:, n] = np.sort(np.concatenate([-T0 * f, T0 * f]))
    return out


def electron_energy(g: dict, ik_range, mu_range):
    """cnt::electron_energy (cnt.cpp:302-345): two-band graphene tight binding at
    k = mu K1 + ik dk_l, f(k) summed over the three bond vectors; energies [2][nk][n_mu]
    (valence -t0|f|, conduction +t0|f|) and wavefunctions [n_mu][2 atoms][2 bands][nk]."""
    a1, a2 = g["a1"], g["a2"]
    d = [(a1 + a2) / 3., (a1 - 2. * a2) / 3., (a2 - 2. * a1) / 3.]
    nk, n_mu = ik_range[1] - ik_range[0], mu_range[1] - mu_range[0]
    energy = np.zeros((2, nk, n_mu))
    wf = np.zeros((n_mu, 2, 2, nk), complex)
    for b, mu in enumerate(range(*mu_range)):
        for a, ik in enumerate(range(*ik_range)):
            k = float(mu) * g["K1"] + float(ik) * g["dk_l"]
            fk = sum(np.exp(1j * float(k @ v)) for v in d)
            energy[1, a, b] = +T0 * abs(fk)
            energy[0, a, b] = -T0 * abs(fk)
            wf[b, 0, 1, a] = wf[b, 0, 0, a] = 1. / math.sqrt(2.)
            wf[b, 1, 1, a] = -1. / math.sqrt(2.) * np.conj(fk) / abs(fk)
            wf[b, 1, 0, a] = +1. / math.sqrt(2.) * np.conj(fk) / abs(fk)
    return energy, wf


def k2_extended(g: dict):
    """The K2-extended grid of calculate_exciton_dispersion (cnt.cpp:1061-1064)."""
    return electron_energy(g, (0, g["Nu"] // g["Q"] * g["n_cells"]), (0, g["Q"]))


def find_valleys(energy) -> list:
    """cnt::find_valleys (cnt.cpp:362-410): conduction-band minima along ik (periodic) on each
    cutting line, sorted by energy and paired.  The reference sorts with std::sort, which orders
    equal energies arbitrarily; this restatement keeps their grid order."""
    e = energy[1]
    nk, n_mu = e.shape
    idx = [(ik, mu) for ik in range(nk) for mu in range(n_mu)
           if e[ik, mu] < e[(ik - 1) % nk, mu] and e[ik, mu] < e[(ik + 1) % nk, mu]]
    idx.sort(key=lambda v: e[v[0], v[1]])
    return [(idx[2 * i], idx[2 * i + 1]) for i in range(len(idx) // 2)]


def find_relev_ik_range(energy, valley_pair, delta_energy: float, ik_range=None, mu_range=(0, 0)) -> list:
    """cnt::find_relev_ik_range (cnt.cpp:419-505) for one valley pair: starting at each valley
    bottom, walk outwards along its cutting line (periodic in ik) one step at a time on both
    sides, keeping states below bottom + delta_energy, until a step keeps none; returns, per
    valley, the (ik, mu) list in ik order around the bottom."""
    e = energy[1]
    nk = e.shape[0]
    ik0 = 0 if ik_range is None else ik_range[0]
    out = []
    for (ikb_idx, mub_idx) in valley_pair:
        ik_bottom, mu_bottom = ikb_idx + ik0, mub_idx + mu_range[0]
        max_e = e[ikb_idx, mub_idx] + delta_energy
        states = [(ik_bottom, mu_bottom)]
        count, in_range = 0, True
        while in_range:
            in_range = False
            count += 1
            ik = ik_bottom + count
            while ik >= ik0 + nk:
                ik -= nk
            if e[ik - ik0, mub_idx] < max_e:
                states.append((ik, mu_bottom))
                in_range = True
            ik = ik_bottom - count
            while ik < ik0:
                ik += nk
            if e[ik - ik0, mub_idx] < max_e:
                states.insert(0, (ik, mu_bottom))
                in_range = True
        out.append(states)
    return out


def _kq(g, ik, mu_k, iq, mu_q, ik_range, mu_range):
    """get_kq of calculate_polarization (cnt.cpp:650-668): k + q wrapped into the K2-extended zone
    (a wrap across the cutting lines moves ik by nk_K1 M)."""
    n_mu, nk = mu_range[1] - mu_range[0], ik_range[1] - ik_range[0]
    mu_kq = mu_k + mu_q
    w = np.floor_divide(mu_kq - mu_range[0], n_mu)
    mu_kq = mu_kq - w * n_mu
    ikq = ik + iq + w * g["n_cells"] * g["M"]
    ikq = ik_range[0] + np.mod(ikq - ik_range[0], nk)
    return ikq, mu_kq


def calculate_polarization(g: dict, iq_range, mu_q_range, energy, wf, ik_range, mu_range) -> np.ndarray:
    """cnt::calculate_polarization (cnt.cpp:634-720): PI(q, mu_q) = 2 sum_{k, mu_k}
    |<v(k)|c(k+q)>|^2 / (E_c(k+q) - E_v(k)) + |<c(k)|v(k+q)>|^2 / (E_c(k) - E_v(k+q)) over the
    K2-extended bands (energy [2][nk][n_mu], wavefunctions [n_mu][atom][band][nk])."""
    nk, n_mu = ik_range[1] - ik_range[0], mu_range[1] - mu_range[0]
    ik, mu_k = np.meshgrid(np.arange(*ik_range), np.arange(*mu_range), indexing="ij")
    ik_i, mu_i = ik - ik_range[0], mu_k - mu_range[0]
    psi = np.transpose(wf, (0, 3, 2, 1))  # [mu][k][band][atom]
    out = np.zeros((iq_range[1] - iq_range[0], mu_q_range[1] - mu_q_range[0]))
    for a, iq in enumerate(range(*iq_range)):
        for b, mu_q in enumerate(range(*mu_q_range)):
            ikq, mu_kq = _kq(g, ik, mu_k, iq, mu_q, ik_range, mu_range)
            kq_i, mkq_i = ikq - ik_range[0], mu_kq - mu_range[0]
            vk, ck = psi[mu_i, ik_i, 0], psi[mu_i, ik_i, 1]
            vkq, ckq = psi[mkq_i, kq_i, 0], psi[mkq_i, kq_i, 1]
            t1 = np.abs((np.conj(vk) * ckq).sum(-1)) ** 2 / (energy[1, kq_i, mkq_i] - energy[0, ik_i, mu_i])
            t2 = np.abs((np.conj(ck) * vkq).sum(-1)) ** 2 / (energy[1, ik_i, mu_i] - energy[0, kq_i, mkq_i])
            out[a, b] = (t1 + t2).sum()
    return 2 * out


def calculate_polarization_loops(g: dict, iq_range, mu_q_range, energy, wf, ik_range, mu_range) -> np.ndarray:
    """calculate_polarization's loops as written, with get_kq's while loops (small grids only)."""
    nk, n_mu = ik_range[1] - ik_range[0], mu_range[1] - mu_range[0]
    out = np.zeros((iq_range[1] - iq_range[0], mu_q_range[1] - mu_q_range[0]))
    for iq in range(*iq_range):
        for mu_q in range(*mu_q_range):
            acc = 0.0
            for ik in range(*ik_range):
                for mu_k in range(*mu_range):
                    mu_kq, ikq = mu_k + mu_q, ik + iq
                    while mu_kq >= mu_range[1]:
                        mu_kq -= n_mu
                        ikq += g["n_cells"] * g["M"]
                    while mu_kq < mu_range[0]:
                        mu_kq += n_mu
                        ikq -= g["n_cells"] * g["M"]
                    while ikq >= ik_range[1]:
                        ikq -= nk
                    while ikq < ik_range[0]:
                        ikq += nk
                    a, m_ = ik - ik_range[0], mu_k - mu_range[0]
                    c, mq = ikq - ik_range[0], mu_kq - mu_range[0]
                    acc += abs(np.vdot(wf[m_][:, 0, a], wf[mq][:, 1, c])) ** 2 / (energy[1, c, mq] - energy[0, a, m_])
                    acc += abs(np.vdot(wf[m_][:, 1, a], wf[mq][:, 0, c])) ** 2 / (energy[1, a, m_] - energy[0, c, mq])
            out[iq - iq_range[0], mu_q - mu_q_range[0]] = acc
    return 2 * out


def calculate_dielectric(vq: np.ndarray, pi: np.ndarray) -> np.ndarray:
    """cnt::calculate_dielectric (cnt.cpp:735-757) on matching (q, mu) grids:
    eps = 1 + Re(mean of vq over the four sublattice pairs) PI."""
    return 1. + np.real(vq.mean(axis=2)) * pi


def calculate_a_excitons(energy, wf, relev, vq, vq_ranges, eps, ik_cm_range, ik_range, mu_range) -> dict:
    """cnt::calculate_A_excitons (cnt.cpp:783-1000): for each centre-of-mass momentum ik_cm the
    Bethe-Salpeter kernels between the relevant states of the two valleys (relev, from
    find_relev_ik_range): kernel_11 (band energies minus the screened direct term within valley
    1), kernel_12 (direct term across the valleys) and the exchange kernel; each is filled on one
    triangle, completed with its conjugate transpose (Armadillo's .t()) and its diagonal halved.
    Eigen-decompositions give the A1 (K11 - K12), A2 triplet (K11 + K12) and A2 singlet
    (K11 + K12 + 2 Kx) excitons.  vq [iq][mu][4] and eps [iq][mu] on vq_ranges = (iq0, mu0)."""
    nk = ik_range[1] - ik_range[0]
    iq0, mu0 = vq_ranges
    v1, v2 = relev
    n = len(v1)

    def ikv(ik_c, ik_cm):
        return ik_range[0] + (ik_c - ik_cm - ik_range[0]) % nk

    def ikc(ik_v, ik_cm):
        return ik_range[0] + (ik_v + ik_cm - ik_range[0]) % nk

    def psi(mu, atom, band, ik):
        return wf[mu - mu_range[0]][atom, band, ik - ik_range[0]]

    def direct(ik_c, mu_c, ik_v, mu_v, ik_cp, mu_cp, ik_vp, mu_vp):
        dk = ik_range[0] + (ik_c - ik_cp - ik_range[0]) % nk
        dmu = mu_c - mu_cp
        acc = 0j
        for i in range(2):
            for j in range(2):
                acc += (np.conj(psi(mu_c, i, 1, ik_c)) * psi(mu_v, j, 0, ik_v) * psi(mu_cp, i, 1, ik_cp)
                        * np.conj(psi(mu_vp, j, 0, ik_vp)) * vq[dk - iq0, dmu - mu0, 2 * i + j] / eps[dk - iq0, dmu - mu0])
        return acc

    def exchange(ik_cm, ik_c, mu_c, ik_v, mu_v, ik_cp, mu_cp, ik_vp, mu_vp):
        acc = 0j
        for i in range(2):
            for j in range(2):
                acc += (np.conj(psi(mu_c, i, 1, ik_c)) * psi(mu_v, i, 0, ik_v) * psi(mu_cp, j, 1, ik_cp)
                        * np.conj(psi(mu_vp, j, 0, ik_vp)) * vq[ik_cm - iq0, 0 - mu0, 2 * i + j])
        return acc

    out = {"A1": [], "A2_triplet": [], "A2_singlet": [], "kernels": []}
    for ik_cm in range(*ik_cm_range):
        k11 = np.zeros((n, n), complex)
        k12 = np.zeros((n, n), complex)
        kx = np.zeros((n, n), complex)
        for c in range(n):
            ik_c, mu_c = v1[c]
            ik_v, mu_v = ikv(ik_c, ik_cm), mu_c
            k11[c, c] += energy[1, ik_c - ik_range[0], mu_c - mu_range[0]] - energy[0, ik_v - ik_range[0], mu_c - mu_range[0]]
            for cp in range(c + 1):
                ik_cp, mu_cp = v1[cp]
                ik_vp, mu_vp = ikv(ik_cp, ik_cm), mu_cp
                k11[c, cp] -= direct(ik_c, mu_c, ik_v, mu_v, ik_cp, mu_cp, ik_vp, mu_vp)
                kx[c, cp] += 2 * exchange(ik_cm, ik_c, mu_c, ik_v, mu_v, ik_cp, mu_cp, ik_vp, mu_vp)
            for vp in range(c, n):
                ik_vp, mu_vp = v2[vp]
                ik_cp, mu_cp = ikc(ik_vp, ik_cm), mu_vp
                k12[c, n - 1 - vp] -= direct(ik_c, mu_c, ik_v, mu_v, ik_cp, mu_cp, ik_vp, mu_vp)
        for k in (k11, k12, kx):
            k += k.conj().T
            k[np.diag_indices(n)] /= 2
        out["A1"].append(np.linalg.eigvalsh(k11 - k12))
        out["A2_triplet"].append(np.linalg.eigvalsh(k11 + k12))
        e_s, v_s = np.linalg.eigh(k11 + k12 + 2 * kx)
        out["A2_singlet"].append(e_s)
        # A2 singlet states over both valleys (cnt.cpp:962-965): +v/sqrt2 on each
        out.setdefault("A2_singlet_psi", []).append(np.vstack([v_s, v_s]) / math.sqrt(2.))
        # indices of the (conduction, valence) states of each row (cnt.cpp:969-997)
        idx = np.zeros((4, 2 * n), int)
        for c in range(n):
            ik_c, mu_c = v1[c]
            idx[:, c] = (ik_c - ik_range[0], mu_c - mu_range[0], ikv(ik_c, ik_cm) - ik_range[0], mu_c - mu_range[0])
        for v in range(n):
            ik_v, mu_v = v2[v]
            idx[:, 2 * n - 1 - v] = (ikc(ik_v, ik_cm) - ik_range[0], mu_v - mu_range[0], ik_v - ik_range[0],
                                     mu_v - mu_range[0])
        out.setdefault("ik_idx", []).append(idx)
        out["kernels"].append((k11, k12, kx))
    for key in ("A1", "A2_triplet", "A2_singlet"):
        out[key] = np.array(out[key])
    return out


def exciton_dispersion(g: dict, window_ev: float = 1.0, interaction: bool = True) -> dict:
    """calculate_exciton_dispersion (cnt.cpp:1056-1080) on the tube of g: K2-extended bands, the
    lowest valley pair (_i_sub = 0, cnt.h:117), the states within window_ev of its bottom, vq,
    PI and eps over the full q range, and the A excitons for k_cm within +-(states per valley).
    interaction=False zeroes vq (eps = 1): the kernels hold the bare pair energies."""
    E, W = k2_extended(g)
    ik_range, mu_range = (0, E.shape[1]), (0, E.shape[2])
    relev = find_relev_ik_range(E, find_valleys(E)[0], window_ev * EV)
    iq_range = (-(ik_range[1] - 1), ik_range[1])
    mq_range = (-(mu_range[1] - 1), mu_range[1])
    vq = calculate_vq(g, iq_range, mq_range, g["n_cells"])
    if not interaction:
        vq = np.zeros_like(vq)
    pi = calculate_polarization(g, iq_range, mq_range, E, W, ik_range, mu_range)
    eps = calculate_dielectric(vq, pi)
    n = len(relev[0])
    ex = calculate_a_excitons(E, W, relev, vq, (iq_range[0], mq_range[0]), eps, (-n, n), ik_range, mu_range)
    ex.update({"relev": relev, "energy": E, "wavefunc": W, "ik_cm_range": (-n, n), "vq": vq, "eps": eps})
    return ex


KB = 1.3865e-23        # constants.h:14
HB = 6.5e-16 * EV      # constants.h:13
BROADENING = 4e-3 * EV  # exciton_transfer.h:42


def lorentzian(e, broadening=BROADENING):
    """exciton_transfer.h:30-33"""
    return (1. / PI) * broadening / (e * e + broadening * broadening)


def relevant_states(ex: dict, min_energy: float, temperature: float = 300.) -> list:
    """get_relevant_states (exciton_transfer.cpp:226-250) of the A2 singlet: (energy, ik_cm,
    ik_cm_idx, i_principal) with energy within |ln 1e-3| kT of min_energy, by energy."""
    thr = min_energy + abs(math.log(1.e-3) * KB * temperature)
    e = ex["A2_singlet"]
    st = [(e[a, i], a + ex["ik_cm_range"][0], a, i) for i in range(e.shape[1]) for a in range(e.shape[0])
          if e[a, i] <= thr]
    return sorted(st, key=lambda t: t[0])


def q_partial(g: dict, ex: dict, state) -> complex:
    """The per-state factor of calculate_Q (exciton_transfer.cpp:276-297)."""
    _, ik_cm, a, i_n = state
    W = ex["wavefunc"]
    idx = ex["ik_idx"][a]
    k = ik_cm * g["dk_l"]
    ef = np.array([1.0 + 0j, np.exp(1j * float(k @ g["acc"]))])
    acc = 0j
    for r in range(idx.shape[1]):
        cc = W[idx[1, r]][:, 1, idx[0, r]]
        cv = W[idx[3, r]][:, 0, idx[2, r]]
        acc += ex["A2_singlet_psi"][a][r, i_n] * np.sum(cc * np.conj(cv) * ef)
    return acc


def length_m(g: dict) -> float:
    return float(g["n_cells"]) * float(np.linalg.norm(g["t_vec"]))


def area_u(g: dict) -> float:
    """cnt::Au (cnt.h:346-349): the graphene unit-cell area."""
    return abs(g["a1"][0] * g["a2"][1] - g["a1"][1] * g["a2"][0])


def q_coeff(gd: dict, ga: dict) -> float:
    """The prefactor of calculate_Q (exciton_transfer.cpp:299-301)."""
    return (Q0 ** 2 * area_u(gd) * area_u(ga)) / (16 * PI ** 3 * EPS0 * gd["radius"] * ga["radius"]
                                                   * math.sqrt(length_m(gd) * length_m(ga)))


def calculate_q(gd: dict, exd: dict, ga: dict, exa: dict, d_state, a_state) -> complex:
    """calculate_Q (exciton_transfer.cpp:273-304) of one donor/acceptor state pair."""
    return q_coeff(gd, ga) * np.conj(q_partial(gd, exd, d_state)) * q_partial(ga, exa, a_state)


def first_order(gd: dict, exd: dict, ga: dict, exa: dict, z_shift: float, axis_shifts=(0., 0.), theta: float = 0.,
                temperature: float = 300.) -> float:
    """exciton_transfer::first_order (exciton_transfer.cpp:380-424): the thermal, Lorentzian-matched
    sum of (2 pi / hbar) |Q J|^2 / (L_d L_a) over donor/acceptor A2-singlet states."""
    min_energy = exd["A2_singlet"].min()
    ds = relevant_states(exd, min_energy, temperature)
    as_ = relevant_states(exa, min_energy, temperature)
    Z = sum(math.exp(-d[0] / (KB * temperature)) for d in ds)
    rate = 0.0
    for d in ds:
        for a in as_:
            if not lorentzian(d[0] - a[0]) > 1.e-2 * lorentzian(0.0):
                continue
            Q = calculate_q(gd, exd, ga, exa, d, a)
            J = coulomb_j(gd, ga, d[1], a[1], axis_shifts, z_shift, theta)
            M = abs(Q * J) / math.sqrt(length_m(gd) * length_m(ga))
            rate += (2 * PI / HB) * (math.exp(-d[0] / (KB * temperature)) / Z) * M ** 2 * lorentzian(d[0] - a[0])
    return rate


EPS0 = 8.85e-12    # constants.h:17
Q0 = 1.6e-19       # constants.h:18
UPP = 11.3 * EV    # Ohno potential constant, cnt.h:32


def vq_positions(g: dict, n_cells: int) -> np.ndarray:
    """The relative positions of calculate_vq (cnt.cpp:532-567): atoms of each sublattice pair
    (aa, ab, ba, bb) relative to the first A / B atom, folded once into +-ch/2 along the
    circumference, repeated over an odd number of unit cells centred on 0: [4][Nu n][2]."""
    if n_cells % 2 == 0:
        n_cells += 1
    a, b = g["pos_u_2d"], g["pos_2d"][g["Nu"]:]
    half = g["ch"][0] / 2
    rel = [a - a[0], a - b[0], b - a[0], b - b[0]]
    for r in rel:
        r[r[:, 0] > half, 0] -= g["ch"][0]
    h = n_cells // 2
    return np.stack([np.concatenate([r + i * g["t_vec"] for i in range(-h, h + 1)]) for r in rel])


def calculate_vq(g: dict, iq_range, mu_range, n_cells: int) -> np.ndarray:
    """cnt::calculate_vq (cnt.cpp:520-631): the Ohno potential U / sqrt(c |R|^2 + 1),
    c = (4 pi eps0 U / q0^2)^2, Fourier-summed as sum_R exp(i q.R) over vq_positions for
    q = iq dk_l + mu K1, divided by 2 Nu n: [nq][n_mu][4] complex."""
    rel = vq_positions(g, n_cells)
    n_eff = rel.shape[1] // g["Nu"]
    coeff = (4. * PI * EPS0 * UPP / Q0 / Q0) ** 2
    pot = UPP / np.sqrt(coeff * (rel[..., 0] ** 2 + rel[..., 1] ** 2) + 1)
    out = np.zeros((iq_range[1] - iq_range[0], mu_range[1] - mu_range[0], 4), complex)
    for a, iq in enumerate(range(*iq_range)):
        for b, mu in enumerate(range(*mu_range)):
            q = iq * g["dk_l"] + mu * g["K1"]
            out[a, b] = (np.exp(1j * (rel @ q)) * pot).sum(axis=1)
    return out / (2 * g["Nu"] * n_eff)


def calculate_vq_loops(g: dict, iq_range, mu_range, n_cells: int) -> np.ndarray:
    """calculate_vq's loops as written, term by term (small tubes only)."""
    rel = vq_positions(g, n_cells)
    n_eff = rel.shape[1] // g["Nu"]
    coeff = (4. * PI * EPS0 * UPP / Q0 / Q0) ** 2
    out = np.zeros((iq_range[1] - iq_range[0], mu_range[1] - mu_range[0], 4), complex)
    for a, iq in enumerate(range(*iq_range)):
        for b, mu in enumerate(range(*mu_range)):
            q = iq * g["dk_l"] + mu * g["K1"]
            for i in range(4):
                acc = 0j
                for R in rel[i]:
                    acc += complex(np.exp(1j * float(q @ R))) * UPP / math.sqrt(coeff * (R[0] ** 2 + R[1] ** 2) + 1)
                out[a, b, i] = acc
    return out / (2 * g["Nu"] * n_eff)


def unit_cells_3d(g: dict, shift_along_axis: float, z_shift: float, angle: float) -> np.ndarray:
    """make_Ru_3d: all unit cells of the tube, centred in y, shifted, rotated about z."""
    cells = np.concatenate([g["pos_u_3d"] + i * g["t_vec_3d"] for i in range(g["n_cells"])])
    y_max, y_min = cells[:, 1].max(), cells[:, 1].min()
    cells[:, 1] -= (y_max + y_min) / 2.0
    cells[:, 1] += shift_along_axis
    cells[:, 2] += z_shift
    x = cells[:, 0] * math.cos(angle) - cells[:, 1] * math.sin(angle)
    y = cells[:, 0] * math.sin(angle) + cells[:, 1] * math.cos(angle)
    cells[:, 0], cells[:, 1] = x, y
    return cells


def unit_cells_2d(g: dict) -> np.ndarray:
    """make_Ru_2d: all unit cells of the tube in the unrolled sheet."""
    return np.concatenate([g["pos_u_2d"] + i * g["t_vec"] for i in range(g["n_cells"])])


def coulomb_j(gi: dict, gf: dict, ik_i: int, ik_f: int, shifts=(0.0, 0.0), z_shift: float = 0.0,
              angle: float = 0.0, block: int = 4096) -> complex:
    """calculate_J for the centre-of-mass momenta ik_i dk_l(i) and ik_f dk_l(f)."""
    Ri = unit_cells_3d(gi, shifts[0], 0.0, 0.0)
    Rf = unit_cells_3d(gf, shifts[1], z_shift, angle)
    ki = ik_i * gi["dk_l"]
    kf = ik_f * gf["dk_l"]
    ei = np.exp(-1j * (unit_cells_2d(gi) @ ki))
    ef = np.exp(+1j * (unit_cells_2d(gf) @ kf))
    J = 0j
    for a in range(0, len(Ri), block):
        d = np.linalg.norm(Ri[a:a + block, None, :] - Rf[None, :, :], axis=2)
        J += complex(ei[a:a + block] @ (ef[None, :] / d).sum(axis=1))
    return J


def coulomb_j_loops(gi: dict, gf: dict, ik_i: int, ik_f: int, shifts=(0.0, 0.0), z_shift: float = 0.0,
                    angle: float = 0.0) -> complex:
    """The double loop of calculate_J as written (small tubes only)."""
    Ri = unit_cells_3d(gi, shifts[0], 0.0, 0.0)
    Rf = unit_cells_3d(gf, shifts[1], z_shift, angle)
    ri, rf = unit_cells_2d(gi), unit_cells_2d(gf)
    ki = ik_i * gi["dk_l"]
    kf = ik_f * gf["dk_l"]
    f_exp = [complex(np.exp(+1j * float(kf @ rf[j]))) for j in range(len(rf))]
    J = 0j
    for i in range(len(ri)):
        i_exp = complex(np.exp(-1j * float(ki @ ri[i])))
        for j in range(len(rf)):
            J += i_exp * f_exp[j] / float(np.linalg.norm(Ri[i] - Rf[j]))
    return J
