"""ctypes bindings of libcntkmc.so (include/cntkmc.h).

The shared library is built in-tree by ``cnt_film_monte_carlo_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback for any engine call.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcntkmc.so")
LIB_CHECK_PATH = os.path.join(HERE, "libcntkmc_check.so")  # the KMC_CHECK build (device bounds checks)

KMC_OK = 0
KMC_ERR_ARG = -1
KMC_ERR_CUDA = -2
KMC_ERR_STATE = -3
KMC_ERR_IO = -4
KMC_ERR_HOP_CAP = -5
KMC_ERR_NOMEM = -6
KMC_ERR_NO_DEVICE = -7
KMC_ERR_CAPACITY = -8
KMC_ERR_CHECK = -9
KMC_TABLE_4D = 4
KMC_TABLE_2D = 2
KMC_TABLE_2D_SPECIES = 3
KMC_MAX_SPECIES = 8
KMC_MLP_HIDDEN = 64
KMC_INJECT_REGION = 0
KMC_INJECT_UNIFORM = 1
KMC_PREC_FP64 = 0
KMC_PREC_MIXED = 1
KMC_ORDER_AUTO = -1
KMC_ORDER_SLOTS = 0
KMC_ORDER_SPATIAL = 1
KMC_NOALLOC_MAX_SITES = 65536
KMC_NOALLOC_MAX_CELLS = 65536
KMC_CNT_MAX_RELEVANT = 64
(KMC_CNT_GEOMETRY, KMC_CNT_POS_U_3D, KMC_CNT_BANDS, KMC_CNT_VALLEYS, KMC_CNT_RELEVANT, KMC_CNT_VQ, KMC_CNT_PI,
 KMC_CNT_EPS, KMC_CNT_A1, KMC_CNT_A2_TRIPLET, KMC_CNT_A2_SINGLET, KMC_CNT_IK_IDX, KMC_CNT_Q_PARTIAL) = range(13)

PD = C.POINTER(C.c_double)
PI32 = C.POINTER(C.c_int32)
PI64 = C.POINTER(C.c_int64)
PU64 = C.POINTER(C.c_uint64)
PF32 = C.POINTER(C.c_float)


def KMC_MLP_PARAMS(n_species: int) -> int:
    return 4548 + 2 * n_species * n_species


class kmc_film(C.Structure):
    _fields_ = [("n_films", C.c_int32), ("film_site_offsets", PI64), ("pos", PD), ("orient", PD), ("left", PI32),
                ("right", PI32)]


class kmc_table(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n", C.c_int32 * 4), ("grid", PD * 4), ("rate", PD)]


class kmc_inject(C.Structure):
    _fields_ = [("mode", C.c_int32), ("n_sections", C.c_int32), ("n_excitons", PI64), ("seeds", PU64)]


class kmc_nbr_stats(C.Structure):
    _fields_ = [("n_sites", C.c_int64), ("nnz", C.c_int64), ("k_mean", C.c_double), ("k_max", C.c_int32),
                ("n_cells", C.c_int64), ("isolated", C.c_int64), ("exact_only", C.c_int64), ("build_ms", C.c_double)]


class kmc_run_stats(C.Structure):
    _fields_ = [("hops", C.c_int64), ("crossings", C.c_int64), ("exact_resolves", C.c_int64),
                ("steps_done", C.c_int64), ("last_run_ms", C.c_double), ("last_launches", C.c_int32)]


class kmc_tune_result(C.Structure):
    _fields_ = [("variant", C.c_int32), ("steps_per_launch", C.c_int32), ("hops_per_s", C.c_double)]


class kmc_contacts(C.Structure):
    _fields_ = [("n_segments", C.c_int32), ("contact_pop", C.c_int64 * 2), ("seed", C.c_uint64),
                ("capacity", C.c_int64)]


class kmc_contacts_info(C.Structure):
    _fields_ = [("ymin", C.c_double), ("ymax", C.c_double), ("dy", C.c_double), ("n_initial", C.c_int64),
                ("n_contact", C.c_int64 * 2), ("capacity", C.c_int64)]


class kmc_mlp_shape(C.Structure):
    _fields_ = [("n_species", C.c_int32), ("d_min", C.c_double), ("d_max", C.c_double), ("log_mean", C.c_double),
                ("log_scale", C.c_double)]


class kmc_species_model(C.Structure):
    _fields_ = [("n_species", C.c_int32), ("gamma_0", C.c_double), ("energy", PD), ("diameter", PD),
                ("diameter_ref", C.c_double), ("width", C.c_double), ("kT", C.c_double), ("floor", C.c_double),
                ("near_field", C.c_double)]


class kmc_mlp_train_cfg(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_double), ("lr_final", C.c_double),
                ("beta1", C.c_double), ("beta2", C.c_double), ("eps", C.c_double)]


class kmc_mlp_train_stats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("first_loss", C.c_double), ("last_loss", C.c_double), ("seconds", C.c_double)]


class kmc_cnt_info(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("n", "m", "cells", "Nu", "M", "Q", "t1", "t2", "nk", "n_mu", "n_valley_pairs",
                                         "n_relevant", "iq0", "nq", "mq0", "nmq", "ik_cm0", "nk_cm")] + \
               [("radius", C.c_double), ("length", C.c_double), ("area_u", C.c_double)]


class kmc_transfer_cfg(C.Structure):
    _fields_ = [("temperature", C.c_double), ("broadening", C.c_double), ("precision", C.c_int32)]


# every symbol include/cntkmc.h declares, with (restype, argtypes)
SIGNATURES = {
    "kmc_create": (C.c_void_p, [C.c_int, C.POINTER(C.c_int)]),
    "kmc_destroy": (None, [C.c_void_p]),
    "kmc_last_error": (C.c_char_p, [C.c_void_p]),
    "kmc_load_film": (C.c_int, [C.c_void_p, C.POINTER(kmc_film)]),
    "kmc_set_rate_table": (C.c_int, [C.c_void_p, C.POINTER(kmc_table)]),
    "kmc_build_neighbors": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(kmc_nbr_stats)]),
    "kmc_init_excitons": (C.c_int, [C.c_void_p, C.POINTER(kmc_inject)]),
    "kmc_run": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_int32]),
    "kmc_get_msd": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, PD]),
    "kmc_set_msd_batches": (C.c_int, [C.c_void_p, C.c_int32]),
    "kmc_get_msd_batches": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, PD]),
    "kmc_fit_diffusion": (C.c_int, [PD, PI64, PD, C.c_int64, C.c_int32, C.c_double, PD, PD]),
    "kmc_contacts_init": (C.c_int, [C.c_void_p, C.POINTER(kmc_contacts), C.POINTER(kmc_contacts_info), PD, PI64]),
    "kmc_contacts_run": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, C.c_double, C.c_int32, PI64, PI64, PI64]),
    "kmc_contacts_track": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_double, C.c_double, C.c_int64, PD, PI64,
                                     PI32]),
    "kmc_get_excitons": (C.c_int, [C.c_void_p, PI32, PD, PD, PD, PI32, PU64, PI64]),
    "kmc_set_excitons": (C.c_int, [C.c_void_p, PI32, PD, PD, PD, PI32, PU64, PI64]),
    "kmc_num_excitons": (C.c_int64, [C.c_void_p]),
    "kmc_get_run_stats": (C.c_int, [C.c_void_p, C.POINTER(kmc_run_stats)]),
    "kmc_get_neighbors": (C.c_int, [C.c_void_p, PI64, PI32, PD, PD]),
    "kmc_set_trace": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64]),
    "kmc_get_trace": (C.c_int64, [C.c_void_p, C.c_int64, PI32, C.c_int64]),
    "kmc_set_hop_cap": (C.c_int, [C.c_void_p, C.c_int64]),
    "kmc_trim_sites": (C.c_int, [C.c_int64, PD, PD, PI32, PI32, PD, PI64]),
    "kmc_domain": (C.c_int, [C.c_int64, PD, PD, PD]),
    "kmc_forster_table": (C.c_int, [C.c_double, PD, PD, PD, PD, PD, PD, PD, PD, PD]),
    "kmc_forster2d_table": (C.c_int, [C.c_double, PD, PD, PD, PD, PD]),
    "kmc_read_mesh": (C.c_int, [C.c_char_p, PI64, PI64, PD, PD, PI32, PI32]),
    "kmc_selftest_uniform": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64, PU64]),
    "kmc_math_probe": (C.c_int, [C.c_void_p, PD, C.c_int64, PD, PD]),
    "kmc_probe_l2": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, PD]),
    "kmc_set_launch_config": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "kmc_set_mixed_variant": (C.c_int, [C.c_void_p, C.c_int32]),
    "kmc_set_work_order": (C.c_int, [C.c_void_p, C.c_int32]),
    "kmc_get_work_order": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "kmc_set_graph": (C.c_int, [C.c_void_p, C.c_int32]),
    "kmc_autotune": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int64, C.c_void_p]),
    "kmc_build_neighbors_noalloc": (C.c_int, [PD, PD, C.c_int64, C.POINTER(kmc_table), C.c_double, PI64, PI32, PD, PD,
                                              C.c_int64, PI64, C.c_void_p, C.c_char_p, C.c_int64]),
    "kmc_set_site_species": (C.c_int, [C.c_void_p, PI32, C.c_int32]),
    "kmc_species_rates": (C.c_int, [C.POINTER(kmc_species_model), C.c_int64, PD, PD, PI32, PI32, PD]),
    "kmc_mlp_init": (C.c_int, [C.c_void_p, C.POINTER(kmc_mlp_shape), C.c_uint64]),
    "kmc_mlp_set_params": (C.c_int, [C.c_void_p, PF32, C.c_int64]),
    "kmc_mlp_get_params": (C.c_int, [C.c_void_p, PF32, C.c_int64]),
    "kmc_mlp_set_samples": (C.c_int, [C.c_void_p, C.c_int64, PD, PD, PI32, PD]),
    "kmc_mlp_gradient": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, PF32, PD]),
    "kmc_mlp_train": (C.c_int, [C.c_void_p, C.POINTER(kmc_mlp_train_cfg), C.POINTER(kmc_mlp_train_stats)]),
    "kmc_mlp_predict": (C.c_int, [C.c_void_p, C.c_int64, PD, PD, PI32, PD]),
    "kmc_mlp_rate_table": (C.c_int, [C.c_void_p, C.c_int32, PD, C.c_int32, PD, PD]),
    "kmc_version": (C.c_char_p, []),
    "kmc_cnt_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "kmc_cnt_destroy": (None, [C.c_void_p]),
    "kmc_cnt_get_info": (C.c_int, [C.c_void_p, C.POINTER(kmc_cnt_info)]),
    "kmc_cnt_get_array": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64]),
    "kmc_exciton_j": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, PI32, PD, C.c_int32, PD]),
    "kmc_exciton_rates": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(kmc_transfer_cfg), C.c_int64, PD,
                                    PD]),
    "kmc_davoody_table": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(kmc_transfer_cfg), PD, PD, PD, PD,
                                    PD, PD, PD, PD, PD]),
}

_libs = {}


def load(checked: bool = False):
    """Load libcntkmc.so, or with checked=True libcntkmc_check.so (the same ABI with device bounds
    checks); fails loudly if it has not been built.  Both may be loaded in one process: each is
    opened locally and binds its own symbols."""
    path = LIB_CHECK_PATH if checked else LIB_PATH
    if path not in _libs:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run cnt_film_monte_carlo_gb300.build.build() first")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _libs[path] = lib
    return _libs[path]


def ptr(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


class KmcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cntkmc error {code}: {msg}")
        self.code = code
