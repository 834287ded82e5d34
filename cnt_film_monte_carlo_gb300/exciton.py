"""The reference's exciton-transfer physics on the GPU: the labeller of pair transfer rates.

``Tube`` is one carbon nanotube's exciton model, the reference's ``cnt`` after
``calculate_exciton_dispersion`` (src/exciton_transfer/cnt.cpp:1056-1080): lattice, K2-extended
bands, valleys, the screened Coulomb interaction and the A excitons from a Bethe-Salpeter
equation, computed by the library's kernels (vq, polarisation, kernel assembly and a batched
Jacobi eigen-solver).  ``rates`` is ``exciton_transfer::first_order``
(src/exciton_transfer/exciton_transfer.cpp:380-424) at many geometries, with the Coulomb sum J
on the GPU; ``davoody_table`` is ``monte_carlo::create_davoody_scatt_table``
(src/monte_carlo/monte_carlo.cpp:64-153), a 4-D rate table the engine reads
(``Engine.set_table``).

A geometry is (z_shift [m], axis shift 1 [m], axis shift 2 [m], theta [rad]): the donor tube
along y shifted along its axis, the acceptor shifted along its own axis and by z_shift in z,
then rotated by theta about z.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from . import engine as E

TEMPERATURE = 300.0            # K, exciton_transfer.h:40
BROADENING = 4e-3 * 1.6e-19     # J (4 meV), exciton_transfer.h:41


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Tube:
    """The exciton model of an (n, m) tube of ``cells`` unit cells, computed on ``engine``'s GPU."""

    def __init__(self, engine, n: int, m: int, cells: int):
        self.engine = engine
        self.lib = engine.lib
        h = C.c_void_p()
        engine._check(self.lib.kmc_cnt_create(engine.h, int(n), int(m), int(cells), C.byref(h)))
        self.h = h
        info = L.kmc_cnt_info()
        self.lib.kmc_cnt_get_info(self.h, C.byref(info))
        self.info = {k: getattr(info, k) for k, _ in L.kmc_cnt_info._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.kmc_cnt_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def array(self, which: int) -> np.ndarray:
        """One of the model's arrays (include/cntkmc.h, KMC_CNT_*), shaped."""
        i = self.info
        nr, nkc = i["n_relevant"], 2 * i["n_relevant"]
        shapes = {
            L.KMC_CNT_GEOMETRY: ((26,), np.float64), L.KMC_CNT_POS_U_3D: ((i["Nu"], 3), np.float64),
            L.KMC_CNT_BANDS: ((2, i["nk"], i["n_mu"]), np.float64),
            L.KMC_CNT_VALLEYS: ((i["n_valley_pairs"], 2, 2), np.int32), L.KMC_CNT_RELEVANT: ((2, nr, 2), np.int32),
            L.KMC_CNT_VQ: ((i["nq"], i["nmq"], 4), np.complex128), L.KMC_CNT_PI: ((i["nq"], i["nmq"]), np.float64),
            L.KMC_CNT_EPS: ((i["nq"], i["nmq"]), np.float64), L.KMC_CNT_A1: ((i["nk_cm"], nr), np.float64),
            L.KMC_CNT_A2_TRIPLET: ((i["nk_cm"], nr), np.float64), L.KMC_CNT_A2_SINGLET: ((i["nk_cm"], nr), np.float64),
            L.KMC_CNT_IK_IDX: ((i["nk_cm"], 4, nkc), np.int32), L.KMC_CNT_Q_PARTIAL: ((i["nk_cm"], nr), np.complex128),
        }
        shape, dt = shapes[which]
        out = np.zeros(shape, dtype=dt)
        count = out.size * (2 if dt == np.complex128 else 1)
        self.engine._check(self.lib.kmc_cnt_get_array(self.h, which, out.ctypes.data_as(C.c_void_p), count))
        return out

    def geometry(self) -> dict:
        g = self.array(L.KMC_CNT_GEOMETRY)
        names = ("a1", "a2", "b1", "b2", "acc", "ch", "t_vec", "K1", "K2", "dk_l")
        out = {k: g[2 * i:2 * i + 2] for i, k in enumerate(names)}
        out.update(t_vec_3d=g[20:23], radius=g[23], ch_len=g[24], length=g[25])
        return out


def _cfg(temperature, broadening, precision):
    return L.kmc_transfer_cfg(float(temperature), float(broadening), int(precision))


def coulomb_j(engine, donor: Tube, acceptor: Tube, ik_cm_pairs, geometry, precision=L.KMC_PREC_FP64) -> np.ndarray:
    """calculate_J for (donor ik_cm, acceptor ik_cm) pairs at one geometry (complex)."""
    pairs = np.ascontiguousarray(ik_cm_pairs, dtype=np.int32).reshape(-1, 2)
    g = _f64(geometry)
    if g.size != 4:
        raise L.KmcError(L.KMC_ERR_ARG, "coulomb_j: geometry is (z_shift, ash1, ash2, theta)")
    out = np.zeros((len(pairs), 2))
    engine._check(engine.lib.kmc_exciton_j(engine.h, donor.h, acceptor.h, len(pairs), L.ptr(pairs, C.c_int32),
                                           L.ptr(g, C.c_double), int(precision), L.ptr(out, C.c_double)))
    return out[:, 0] + 1j * out[:, 1]


def rates(engine, donor: Tube, acceptor: Tube, geometries, temperature=TEMPERATURE, broadening=BROADENING,
          precision=L.KMC_PREC_MIXED) -> np.ndarray:
    """first_order at geometries [n][4] = (z_shift, ash1, ash2, theta); 1/s."""
    g = _f64(geometries).reshape(-1, 4)
    out = np.zeros(len(g))
    cfg = _cfg(temperature, broadening, precision)
    engine._check(engine.lib.kmc_exciton_rates(engine.h, donor.h, acceptor.h, C.byref(cfg), len(g),
                                               L.ptr(g, C.c_double), L.ptr(out, C.c_double)))
    return out


def davoody_table(engine, donor: Tube, acceptor: Tube, theta_deg=(0, 180, 21), zshift=(1.5e-9, 10e-9, 11),
                  ash1=(-10e-9, 10e-9, 11), ash2=(-10e-9, 10e-9, 11), temperature=TEMPERATURE,
                  broadening=BROADENING, precision=L.KMC_PREC_MIXED) -> dict:
    """create_davoody_scatt_table on the reference's default grids (input.json:47-50): a KMC_TABLE_4D
    table dict for Engine.set_table."""
    specs = [_f64(x) for x in (theta_deg, zshift, ash1, ash2)]
    n = [E._grid_n(x, "davoody_table") for x in specs]
    E._table_size(n, "davoody_table")
    g = [np.zeros(k) for k in n]
    rate = np.zeros(n)
    cfg = _cfg(temperature, broadening, precision)
    engine._check(engine.lib.kmc_davoody_table(engine.h, donor.h, acceptor.h, C.byref(cfg),
                                               *(L.ptr(x, C.c_double) for x in specs),
                                               *(L.ptr(x, C.c_double) for x in g), L.ptr(rate, C.c_double)))
    return {"kind": L.KMC_TABLE_4D, "grids": g, "rate": rate}


# ---------------------------------------------------------------- pair-rate labels of mixed films
CHIRALITIES = ((6, 5), (7, 5), (8, 3), (8, 4))
# tube lengths in unit cells, ~40 nm each ((6,5) 4.06 nm, (7,5) 4.45 nm, (8,3) 4.20 nm and
# (8,4) 1.13 nm per cell): long enough that every tube has seven thermally relevant A2-singlet
# states (three-cell tubes keep only the dark k_cm = 0 state, so most pairs get no rate at all)
CELLS = {(6, 5): 10, (7, 5): 9, (8, 3): 10, (8, 4): 36}
VDW_GAP = 0.34e-9      # closest wall-to-wall distance of two tubes (graphite interlayer spacing), m
RATE_FLOOR = 1e3       # 1/s: labels of dark pairs (rounding residue, ~1e-20 /s) are raised to it


class PairLabeller:
    """first_order rates between segments of a mixed-chirality film, labelled by the reference's
    exciton model on the GPU.

    A sample (centre distance d, folded angle theta, donor chirality a, acceptor chirality b) is
    the rate between two whole tubes of those chiralities (lengths ``CELLS``) whose axes cross at
    that distance and angle with no axial shifts: geometry (max(d, d_contact), 0, 0, theta).
    Tubes cannot interpenetrate, so below their contact distance d_contact = r_a + r_b + 0.34 nm
    the label is the contact-distance rate.  The reference's own davoody table likewise applies
    whole-tube rates (its input: (4,2) tubes of 10 cells) to the segments of its meshes.
    Rates below RATE_FLOOR (pairs whose matched states are all dark) are raised to it."""

    def __init__(self, engine, chiralities=CHIRALITIES, cells=None, precision=L.KMC_PREC_MIXED):
        self.engine = engine
        self.chiralities = tuple(chiralities)
        cells = cells or CELLS
        self.tubes = [Tube(engine, n, m, cells[(n, m)]) for n, m in self.chiralities]
        self.radius = np.array([t.info["radius"] for t in self.tubes])
        self.precision = precision

    @property
    def n_species(self) -> int:
        return len(self.tubes)

    def contact(self, a: int, b: int) -> float:
        return float(self.radius[a] + self.radius[b] + VDW_GAP)

    def rates(self, dist, theta, donor, acceptor) -> np.ndarray:
        dist, theta = _f64(dist), _f64(theta)
        donor, acceptor = np.asarray(donor), np.asarray(acceptor)
        out = np.zeros(len(dist))
        for a in range(self.n_species):
            for b in range(self.n_species):
                sel = np.nonzero((donor == a) & (acceptor == b))[0]
                if len(sel) == 0:
                    continue
                geo = np.zeros((len(sel), 4))
                geo[:, 0] = np.maximum(dist[sel], self.contact(a, b))
                geo[:, 3] = theta[sel]
                out[sel] = rates(self.engine, self.tubes[a], self.tubes[b], geo, precision=self.precision)
        return np.maximum(out, RATE_FLOOR)

    def table(self, dist, theta) -> dict:
        """The labeller's own KMC_TABLE_2D_SPECIES table on (distance, folded angle) grids."""
        dist, theta = _f64(dist), _f64(theta)
        S = self.n_species
        a, b, i, k = np.meshgrid(np.arange(S), np.arange(S), np.arange(len(dist)), np.arange(len(theta)),
                                 indexing="ij")
        r = self.rates(dist[i.ravel()], theta[k.ravel()], a.ravel(), b.ravel())
        return {"kind": L.KMC_TABLE_2D_SPECIES, "grids": [dist, theta], "rate": r.reshape(S, S, len(dist), len(theta))}

    def close(self):
        for t in self.tubes:
            t.close()
