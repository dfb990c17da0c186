"""ctypes binding of libstarfish_gpu.so (include/starfish_gpu.h).

This is the same binding a Java host makes through JNI; the Python classes in
``starfish_gb300.plugin`` sit on top of it and mirror the reference's plugin
classes.  Loading fails loudly when the library is missing: there is no CPU
fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstarfish_gpu.so")

# status codes and enumerations (include/starfish_gpu.h)
SF_OK, SF_ERR_ARG, SF_ERR_CUDA, SF_ERR_NOT_CONVERGED, SF_ERR_DIVERGED = 0, 1, 2, 3, 4
SF_ERR_TIMEOUT, SF_ERR_OOM, SF_ERR_STATE = 5, 6, 7
DOMAIN_XY, DOMAIN_RZ, DOMAIN_ZR = 0, 1, 2
NODE_OPEN, NODE_DIRICHLET, NODE_INSULATOR, NODE_INTERNAL = -1, 0, 1, 2
DB_OPEN, DB_DIRICHLET, DB_NEUMANN, DB_PERIODIC, DB_SYMMETRY, DB_MESH, DB_SINK = -1, 0, 1, 2, 3, 4, 5
FACE_RIGHT, FACE_TOP, FACE_LEFT, FACE_BOTTOM = 0, 1, 2, 3
BT_DIRICHLET, BT_OPEN, BT_SINK, BT_VIRTUAL = 0, 1, 2, 3
SURF_PASS, SURF_ABSORB, SURF_NONE, SURF_SPECULAR, SURF_DIFFUSE = -1, 0, 1, 2, 3
FIELD_ND, FIELD_U, FIELD_V, FIELD_W, FIELD_COUNT, FIELD_NODE_VOL = 0, 1, 2, 3, 4, 5
FIELD_PHI, FIELD_RHO, FIELD_EFI, FIELD_EFJ, FIELD_NE = 10, 11, 12, 13, 14
PUSH_STATS, PUSH_MOMENTS, PUSH_SAMPLE, PUSH_NOWAIT = 1, 2, 4, 8
FIELD_ND_AVE, FIELD_U_AVE, FIELD_V_AVE, FIELD_W_AVE, FIELD_T = 20, 21, 22, 23, 24
FIELD_T1, FIELD_T2, FIELD_T3, FIELD_P, FIELD_MPC = 25, 26, 27, 28, 29

_STATUS = {1: "SF_ERR_ARG", 2: "SF_ERR_CUDA", 3: "SF_ERR_NOT_CONVERGED", 4: "SF_ERR_DIVERGED",
           5: "SF_ERR_TIMEOUT", 6: "SF_ERR_OOM", 7: "SF_ERR_STATE"}


class SfError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


class MeshDesc(C.Structure):
    _fields_ = [("ni", C.c_int32), ("nj", C.c_int32), ("x0", C.c_double * 2),
                ("dh", C.c_double * 2), ("domain_type", C.c_int32),
                ("node_type", C.c_void_p), ("bc_value", C.c_void_p), ("node_vol", C.c_void_p),
                ("face_type", C.c_void_p), ("n_segments", C.c_int32), ("seg_xy", C.c_void_p),
                ("seg_btype", C.c_void_p), ("node_seg_ptr", C.c_void_p),
                ("node_seg_idx", C.c_void_p)]


class PushStats(C.Structure):
    _fields_ = [("n_sum", C.c_double), ("p_sum", C.c_double * 3), ("e_sum", C.c_double),
                ("boundary_charge", C.c_double), ("np", C.c_int64), ("n_removed", C.c_int64),
                ("n_slow", C.c_int64), ("n_bounce_limited", C.c_int64)]

    def as_dict(self):
        return {"n_sum": self.n_sum, "p_sum": list(self.p_sum), "e_sum": self.e_sum,
                "boundary_charge": self.boundary_charge, "np": self.np,
                "n_removed": self.n_removed, "n_slow": self.n_slow,
                "n_bounce_limited": self.n_bounce_limited}


class PoissonParams(C.Structure):
    _fields_ = [("n0", C.c_double), ("kTe0", C.c_double), ("phi0", C.c_double),
                ("eps", C.c_double), ("tol", C.c_double), ("max_it", C.c_int32),
                ("cycles", C.c_int32), ("use_learned", C.c_int32), ("linear", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("newton_it", C.c_int32), ("vcycles", C.c_int32), ("residual", C.c_double),
                ("residual_inf", C.c_double), ("initial_residual", C.c_double),
                ("ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


EXPORTS = {
    # name: (restype, argtypes)
    "sf_version": (C.c_char_p, []),
    "sf_last_error": (C.c_char_p, [C.c_void_p]),
    "sf_ctx_create": (C.c_int, [C.POINTER(MeshDesc), C.c_int, C.POINTER(C.c_void_p)]),
    "sf_ctx_destroy": (C.c_int, [C.c_void_p]),
    "sf_ctx_set_seed": (C.c_int, [C.c_void_p, C.c_uint64]),
    "sf_build_node_segments": (C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    "sf_species_add": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int64,
                                 C.c_double, C.POINTER(C.c_int32)]),
    "sf_species_set_surface": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                         C.c_double, C.c_double]),
    "sf_species_set_surface_product": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_double]),
    "sf_species_set_sort_interval": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "sf_species_set_sort_block": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "sf_species_particle_steps": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]),
    "sf_species_set_weighted": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "sf_particles_append_lc_w": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "sf_particles_download_weights": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p,
                                                C.POINTER(C.c_int64)]),
    "sf_particles_append": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_int32, C.c_double]),
    "sf_particles_append_lc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p]),
    "sf_particles_count": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]),
    "sf_particles_download": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p,
                                        C.POINTER(C.c_int64)]),
    "sf_particles_sort": (C.c_int, [C.c_void_p, C.c_int32]),
    "sf_particles_clear": (C.c_int, [C.c_void_p, C.c_int32]),
    "sf_set_efield": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "sf_get_field": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "sf_push_deposit": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_int32,
                                  C.POINTER(PushStats)]),
    "sf_push_deposit_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_int32,
                                          C.POINTER(PushStats)]),
    "sf_get_surface_flux": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "sf_reset_surface_flux": (C.c_int, [C.c_void_p, C.c_int32]),
    "sf_ctx_get_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "sf_timing_enable": (C.c_int, [C.c_void_p, C.c_int32]),
    "sf_timing_get": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_double),
                                C.POINTER(C.c_int64)]),
    "sf_timing_reset": (C.c_int, [C.c_void_p]),
    "sf_launch_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.c_int32]),
    "sf_update_rho": (C.c_int, [C.c_void_p]),
    "sf_set_bc_values": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sf_poisson_nl": (C.c_int, [C.c_void_p, C.POINTER(PoissonParams), C.c_void_p, C.c_void_p,
                                C.POINTER(SolveStats)]),
    "sf_efield": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "sf_boltzmann": (C.c_int, [C.c_void_p, C.c_void_p]),
    "sf_source_maxwellian": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_double, C.c_double,
                                       C.c_double, C.c_double, C.POINTER(C.c_double),
                                       C.POINTER(C.c_int64)]),
    "sf_source_uniform": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                    C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "sf_source_preload": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double,
                                    C.POINTER(C.c_int64)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libstarfish_gpu.so not found at {path}; run "
                           "`python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = C.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, ctx=None):
    if rc != SF_OK:
        msg = load().sf_last_error(ctx)
        raise SfError(rc, (msg or b"").decode())


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def build_node_segments(ni, nj, x0, dh, seg_xy):
    """Per-node segment lists (Mesh.setNodeControlVolumes) computed by the library."""
    L = load()
    seg_xy = np.ascontiguousarray(seg_xy, np.float64).reshape(-1)
    nseg = seg_xy.size // 4
    x0 = np.ascontiguousarray(x0, np.float64)
    dh = np.ascontiguousarray(dh, np.float64)
    nnz = C.c_int64(0)
    check(L.sf_build_node_segments(ni, nj, ptr(x0), ptr(dh), nseg, ptr(seg_xy), None, None,
                                   C.byref(nnz)))
    p = np.zeros(ni * nj + 1, np.int32)
    idx = np.zeros(max(nnz.value, 1), np.int32)
    check(L.sf_build_node_segments(ni, nj, ptr(x0), ptr(dh), nseg, ptr(seg_xy), ptr(p), ptr(idx),
                                   C.byref(nnz)))
    return p, idx[:nnz.value]


class Sigma(C.Structure):
    _fields_ = [("model", C.c_int32), ("c", C.c_double * 4), ("diam", C.c_double),
                ("T_ref", C.c_double), ("omega", C.c_double), ("vss_alpha", C.c_double)]


SIGMA_CONST, SIGMA_INV, SIGMA_POLY, SIGMA_LN, SIGMA_BIRD463 = 0, 1, 2, 3, 4
MCC_MEX, MCC_CEX, MCC_IONIZATION = 0, 1, 2
EXPORTS.update({
    "sf_dsmc": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(Sigma), C.c_double, C.c_double,
                          C.POINTER(C.c_int64)]),
    "sf_dsmc_get_counts": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "sf_dsmc_pair": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(Sigma), C.POINTER(Sigma), C.c_double,
                               C.c_double, C.POINTER(C.c_int64)]),
    "sf_dsmc_pair_get_counts": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "sf_mcc_set_target": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p]),
    "sf_mcc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(Sigma), C.c_double,
                         C.POINTER(C.c_int64)]),
    "sf_mcc_ionization": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(Sigma), C.c_double,
                                    C.c_double, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int64)]),
    "sf_mcc_get_sums": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
})
EXPORTS.update({
    "sf_unet_init": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_uint64]),
    "sf_unet_set_tensor_cores": (C.c_int, [C.c_void_p, C.c_int32]),
    "sf_unet_tensor_core_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "sf_unet_tensor_core_wait_test": (C.c_int, [C.c_void_p]),
    "sf_unet_set_training": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.c_int32]),
    "sf_unet_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "sf_unet_debug": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.POINTER(C.c_int64)]),
    "sf_unet_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
})
EXPORTS.update({
    "sf_samples_clear": (C.c_int, [C.c_void_p, C.c_int32]),
    "sf_samples_compute": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.POINTER(C.c_int64)]),
})


class BatchStats(C.Structure):
    _fields_ = [("particles", C.c_int64), ("device_phase_ms", C.c_double), ("solve_ms_sum", C.c_double),
                ("solve_ms_max", C.c_double), ("newton_it_mean", C.c_double), ("newton_it_max", C.c_int32),
                ("capacity_overflow", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


EXPORTS.update({
    "sf_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_int32, C.c_int32,
                                  C.POINTER(C.c_void_p)]),
    "sf_batch_destroy": (C.c_int, [C.c_void_p]),
    "sf_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "sf_batch_set_source": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_double, C.c_double, C.c_double]),
    "sf_batch_step": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(PoissonParams), C.POINTER(BatchStats)]),
    "sf_batch_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p]),
})
