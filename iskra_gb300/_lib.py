"""ctypes binding of libiskra_gpu.so (the C ABI declared in include/iskra_gpu.h).

The library is built in-tree by ``iskra_gb300.build``.  There is no fallback:
if the shared library or a CUDA device is missing, loading fails loudly.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_uint8, c_uint32, c_uint64, c_void_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libiskra_gpu.so")

ISKRA_OK = 0
ERRORS = {
    1: "ISKRA_EINVAL", 2: "ISKRA_ENOMEM", 3: "ISKRA_ECAPACITY", 4: "ISKRA_EDOMAIN", 5: "ISKRA_EPROB",
    6: "ISKRA_ENAN", 7: "ISKRA_ETIMEDOUT", 8: "ISKRA_ECUDA", 9: "ISKRA_ENOTCONV",
}
BND_NONE, BND_WRAP, BND_DISCARD = 0, 1, 2
FIELD_RHO, FIELD_PHI, FIELD_E = 0, 1, 2
SURF_ABSORB, SURF_REFLECT, SURF_PERIODIC, SURF_FIXED, SURF_FLOATING = 1, 2, 3, 4, 5
MCC_ELASTIC_ISOTROPIC, MCC_ELASTIC_BACKWARD, MCC_INELASTIC_BACKWARD, MCC_EXCITATION, MCC_IONIZATION = range(5)


class IskraError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Grid(ctypes.Structure):
    _fields_ = [("nx", c_int32), ("ny", c_int32), ("dx", c_double), ("dy", c_double),
                ("ox", c_double), ("oy", c_double), ("bc", c_int32 * 4)]


dp = POINTER(c_double)
u8p = POINTER(c_uint8)
u32p = POINTER(c_uint32)
i64p = POINTER(c_int64)
ip = POINTER(c_int)
i32p = POINTER(c_int32)
f32p = POINTER(ctypes.c_float)
CTX = c_void_p

# (name, restype, argtypes) of every exported entry point, in header order
SIGNATURES = [
    ("iskra_ctx_create", c_int, [POINTER(Grid), c_uint64, POINTER(c_void_p)]),
    ("iskra_ctx_destroy", c_int, [CTX]),
    ("iskra_last_error", c_char_p, [CTX]),
    ("iskra_sync", c_int, [CTX]),
    ("iskra_stream", c_int, [CTX, POINTER(c_uint64)]),
    ("iskra_species_create", c_int, [CTX, c_double, c_double, c_double, c_int64, ip]),
    ("iskra_species_upload", c_int, [CTX, c_int, dp, dp, dp, u32p, c_int64, c_int64]),
    ("iskra_species_download", c_int, [CTX, c_int, dp, dp, dp, u32p, c_int64, i64p]),
    ("iskra_species_count", c_int, [CTX, c_int, i64p]),
    ("iskra_species_set_boundary", c_int, [CTX, c_int, c_int, c_int]),
    ("iskra_species_absorbed", c_int, [CTX, c_int, i64p]),
    ("iskra_species_sort", c_int, [CTX, c_int]),
    ("iskra_tracker_create", c_int, [CTX, c_int]),
    ("iskra_tracker_add_surface", c_int, [CTX, u8p, c_int, c_int, c_double, ip]),
    ("iskra_tracker_hits", c_int, [CTX, c_int, c_int, i64p]),
    ("iskra_source_create", c_int, [CTX, c_int, c_double, dp, dp, dp, dp, ip]),
    ("iskra_source_sample", c_int, [CTX, c_int, c_double, c_uint64]),
    ("iskra_source_set_every_step", c_int, [CTX, c_int, c_int]),
    ("iskra_dsmc_create", c_int, [CTX, c_int, c_int, dp, dp, c_int, ip]),
    ("iskra_dsmc_perform", c_int, [CTX, c_int, c_double, c_uint64, c_uint64]),
    ("iskra_dsmc_state", c_int, [CTX, c_int, dp, u32p]),
    ("iskra_field_upload_E", c_int, [CTX, dp]),
    ("iskra_field_download", c_int, [CTX, c_int, dp]),
    ("iskra_field_download_async", c_int, [CTX, c_int, dp]),
    ("iskra_advance", c_int, [CTX, c_int, c_double]),
    ("iskra_advance_all", c_int, [CTX, c_double]),
    ("iskra_density", c_int, [CTX, c_int, dp]),
    ("iskra_charge_density", c_int, [CTX]),
    ("iskra_set_background", c_int, [CTX, dp]),
    ("iskra_poisson_create", c_int, [CTX, c_double]),
    ("iskra_poisson_apply_dirichlet", c_int, [CTX, u8p, c_double]),
    ("iskra_poisson_apply_periodic", c_int, [CTX, c_int]),
    ("iskra_poisson_add_dof", c_int, [CTX, ip]),
    ("iskra_poisson_apply_neumann", c_int, [CTX, u8p, c_int]),
    ("iskra_poisson_apply_neumann_gauss", c_int, [CTX, u8p, c_int]),
    ("iskra_poisson_set_sigma", c_int, [CTX, c_int, c_double]),
    ("iskra_poisson_get_sigma", c_int, [CTX, c_int, dp]),
    ("iskra_poisson_drive_dirichlet", c_int, [CTX, u8p, c_double, c_double, c_double, c_double]),
    ("iskra_poisson_solve", c_int, [CTX, c_double, c_int, ip, dp]),
    ("iskra_poisson_solve_host", c_int, [CTX, dp, c_double, c_int, dp, ip, dp]),
    ("iskra_poisson_set_warm_start", c_int, [CTX, c_int]),
    ("iskra_poisson_set_method", c_int, [CTX, c_int, ip]),
    ("iskra_mcc_create", c_int, [CTX, c_int, c_int, ip, dp, i32p, dp, dp, c_double, c_double, c_double, dp, c_int,
                                 dp, ip]),
    ("iskra_mcc_perform", c_int, [CTX, c_int, c_double, c_uint64, c_uint64]),
    ("iskra_mcc_counts", c_int, [CTX, c_int, i64p]),
    ("iskra_mcc_sigma", c_int, [CTX, c_int, c_int, dp, c_int64, dp]),
    ("iskra_circuit_create", c_int, [CTX, c_double, c_double, c_double, c_double, c_double, c_double, c_int, u8p,
                                     u8p, c_double, c_double]),
    ("iskra_circuit_advance", c_int, [CTX, c_double]),
    ("iskra_circuit_state", c_int, [CTX, dp]),
    ("iskra_step", c_int, [CTX, c_double, c_int, c_uint64, c_double]),
    ("iskra_set_sort_every", c_int, [CTX, c_int]),
    ("iskra_autotune_sort", c_int, [CTX, c_double, c_int, c_uint64, c_double, dp, dp]),
    ("iskra_set_tile", c_int, [CTX, c_int]),
    ("iskra_get_tile", c_int, [CTX, ip]),
    ("iskra_autotune", c_int, [CTX, c_double, c_int, c_uint64, c_double, ip, dp, dp, dp, ip]),
    ("iskra_solve_info", c_int, [CTX, ip, dp]),
    ("iskra_poisson_residual", c_int, [CTX, dp, dp, dp]),
    ("iskra_kernel_launches", c_int, [CTX, POINTER(c_uint64)]),
    ("iskra_write_openpmd", c_int, [CTX, c_char_p, c_int64, c_double, c_double, POINTER(c_char_p), c_int]),
    ("iskra_density_noalloc", c_int, [POINTER(Grid), c_void_p, c_int64, c_int64, c_double, c_void_p, c_void_p,
                                      c_uint64]),
    ("iskra_ens_create", c_int, [CTX, c_int, c_int64, POINTER(c_void_p)]),
    ("iskra_ens_destroy", c_int, [c_void_p]),
    ("iskra_ens_last_error", c_char_p, [c_void_p]),
    ("iskra_ens_set_seeds", c_int, [c_void_p, POINTER(c_uint64)]),
    ("iskra_ens_set_drive_amplitude", c_int, [c_void_p, c_int, dp]),
    ("iskra_ens_upload", c_int, [c_void_p, c_int, c_int, dp, dp, u32p, c_int64, c_int64]),
    ("iskra_ens_download", c_int, [c_void_p, c_int, c_int, dp, dp, u32p, c_int64, i64p]),
    ("iskra_ens_count", c_int, [c_void_p, c_int, c_int, i64p]),
    ("iskra_ens_step", c_int, [c_void_p, c_double, c_int]),
    ("iskra_ens_sync", c_int, [c_void_p]),
    ("iskra_ens_mcc_counts", c_int, [c_void_p, c_int, c_int, POINTER(c_uint64)]),
    ("iskra_ens_field", c_int, [c_void_p, c_int, c_int, dp]),
    ("iskra_ens_set_compact_every", c_int, [c_void_p, c_int]),
    ("iskra_lws_create", c_int, [CTX, c_int, c_uint64]),
    ("iskra_lws_destroy", c_int, [CTX]),
    ("iskra_lws_set_mode", c_int, [CTX, c_int, c_int, c_int]),
    ("iskra_lws_info", c_int, [CTX, ip, ip, i64p, i64p, dp, dp]),
    ("iskra_lws_eval", c_int, [CTX, dp, dp]),
    ("iskra_lws_weights", c_int, [CTX, f32p, f32p]),
    ("iskra_lws_forward", c_int, [CTX, f32p, f32p]),
    ("iskra_lws_loss_grad", c_int, [CTX, f32p, f32p, dp, f32p]),
    ("iskra_lws_train", c_int, [CTX, c_int, c_double, c_uint64, dp]),
]

_LIB = None


def load(path: str | None = None):
    """Loads libiskra_gpu.so (building it first if absent) and binds every symbol."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        from . import build as _build
        _build.build()
    lib = ctypes.CDLL(p)
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def check(lib, ctx, rc):
    if rc != ISKRA_OK:
        msg = lib.iskra_last_error(ctx)
        raise IskraError(rc, msg.decode() if msg else "")
    return rc
