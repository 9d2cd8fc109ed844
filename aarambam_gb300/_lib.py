"""ctypes binding of libaarambam_gpu.so (the C ABI declared in include/aarambam.h).

The library is built in-tree by aarambam_gb300.build; loading fails loudly
when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

AAR_OK = 0
AAR_ERR_ARG = 1
AAR_ERR_CUDA = 2
AAR_ERR_OOM = 3
AAR_ERR_STATE = 4
AAR_ERR_NMAX = 200
AAR_ERR_TRANSFER = 1111
AAR_ERR_TRANSFER_DUP = 777
AAR_FUSED_FP32 = 0
AAR_PLAIN_FP64 = 1
AAR_PLAIN_FP64_REGROUPED = 2
AAR_SLAB_FP32 = 3
AAR_VARIANT_BASIS = 0
AAR_VARIANT_RESBASIS = 1

# every symbol include/aarambam.h declares
EXPORTS = [
    "aar_plan_create", "aar_set_tables", "aar_set_transfer", "aar_get_scalars", "aar_set_seed", "aar_run",
    "aar_run_glass", "aar_run_host", "aar_run_glass_host", "aar_run_glass_host_async", "aar_run_lattice", "aar_wait_host_copies",
    "aar_plan_prepare", "aar_plan_device_bytes", "aar_modal_partition", "aar_set_modal_partition", "aar_seedtable", "aar_stage_noise", "aar_stage_modal", "aar_stage_lpt",
    "aar_stage_readout", "aar_stage_readout_glass", "aar_copy_spectrum", "aar_copy_field", "aar_gaussian_spectrum_noalloc", "aar_c2r", "aar_r2c", "aar_last_launch_count", "aar_profile_enable", "aar_profile_report",
    "aar_last_error", "aar_plan_destroy", "aar_version",
    "aar_batch_create", "aar_batch_run", "aar_batch_launch_count", "aar_batch_last_error", "aar_batch_destroy",
    "aar_set_spectrum", "aar_adj_spectral", "aar_adj_source", "aar_adj_products", "aar_set_jit", "aar_jit_status",
    "aar_tetra_covariance_scratch_bytes", "aar_tetra_covariance", "aar_tetra_QS", "aar_tetra_residual",
    "aar_tetra_modes_ld", "aar_tetra_modes", "aar_modes_covariance_scratch_bytes", "aar_modes_covariance",
    "aar_modes_project", "aar_modes_residual",
    "aar_bordered_cond", "aar_autotune", "aar_profile_modal_rows",
]
AAR_ADJ_OP_ONE, AAR_ADJ_OP_GAUSS, AAR_ADJ_OP_Q, AAR_ADJ_OP_RHO = 0, 1, 2, 3
AAR_ADJ_OP_HESS, AAR_ADJ_OP_PSI1, AAR_ADJ_OP_PSI2 = 4, 5, 6


class Params(C.Structure):
    _fields_ = [("nmesh", C.c_int32), ("nsample", C.c_int32), ("nmax", C.c_int32), ("seed", C.c_int32),
                ("box", C.c_double), ("omega", C.c_double), ("omega_lambda", C.c_double),
                ("hubble_param", C.c_double), ("sigma8", C.c_double), ("primordial_index", C.c_double),
                ("redshift", C.c_double), ("fnl", C.c_double), ("unit_length_in_cm", C.c_double),
                ("unit_mass_in_g", C.c_double), ("unit_velocity_in_cm_per_s", C.c_double),
                ("input_spectrum_unit_length_in_cm", C.c_double), ("fixed_amplitude", C.c_int32),
                ("phase_flip", C.c_int32), ("sphere_mode", C.c_int32), ("precision", C.c_int32),
                ("mem_limit_bytes", C.c_int64), ("variant", C.c_int32), ("which_spectrum", C.c_int32),
                ("a_res", C.c_double), ("w_res", C.c_double), ("phi_res", C.c_double),
                ("noise_fp64", C.c_int32), ("nslab", C.c_int32)]


class Scalars(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("norm", "anorm", "d0", "dplus", "init_time", "hubble", "beta",
                                          "vel_prefac", "vel_prefac2")]


class AarError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the library (optionally building it first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise RuntimeError(f"{_build.LIB} is not built; run aarambam_gb300.build.build() "
                               "(the CUDA extension is required, there is no CPU path)")
        _build.build()
    L = C.CDLL(_build.LIB)
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    dp = C.POINTER(C.c_double)
    L.aar_plan_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    L.aar_set_tables.argtypes = [vp, dp, dp, i32]
    L.aar_set_transfer.argtypes = [vp, dp, dp, i32]
    L.aar_get_scalars.argtypes = [vp, C.POINTER(Scalars)]
    L.aar_set_seed.argtypes = [vp, i32]
    L.aar_run.argtypes = [vp, vp, i64, vp, vp, vp]
    L.aar_run_glass.argtypes = [vp, vp, i64, C.c_double, i32, vp, vp, vp, vp]
    L.aar_run_host.argtypes = [vp, vp, i64, vp, vp, vp]
    L.aar_run_glass_host.argtypes = [vp, vp, i64, C.c_double, i32, vp, vp, vp, vp]
    L.aar_run_lattice.argtypes = [vp, i32, C.c_double, i32, vp, vp, vp, vp]
    L.aar_run_glass_host_async.argtypes = [vp, vp, i64, C.c_double, i32, vp, vp, vp, vp]
    L.aar_wait_host_copies.argtypes = [vp]
    L.aar_plan_prepare.argtypes = [vp]
    L.aar_modal_partition.argtypes = [dp, i32, i32, C.POINTER(i32)]
    L.aar_set_modal_partition.argtypes = [vp, i32, i32]
    L.aar_profile_modal_rows.argtypes = [vp, vp, i64, vp]
    L.aar_plan_device_bytes.argtypes = [vp]
    L.aar_plan_device_bytes.restype = i64
    L.aar_seedtable.argtypes = [vp, vp, vp]
    for n in ("aar_stage_noise", "aar_stage_modal", "aar_stage_lpt"):
        getattr(L, n).argtypes = [vp, vp]
    L.aar_stage_readout.argtypes = [vp, vp, i64, vp, vp, vp]
    L.aar_stage_readout_glass.argtypes = [vp, vp, i64, C.c_double, i32, vp, vp, vp, vp]
    L.aar_copy_spectrum.argtypes = [vp, vp, vp]
    L.aar_copy_field.argtypes = [vp, i32, vp, vp]
    L.aar_gaussian_spectrum_noalloc.argtypes = [vp, vp, vp]
    L.aar_c2r.argtypes = [vp, vp, vp, vp]
    L.aar_r2c.argtypes = [vp, vp, vp, vp]
    L.aar_last_launch_count.argtypes = [vp]
    L.aar_profile_enable.argtypes = [vp, i32]
    L.aar_profile_report.argtypes = [vp, C.c_char_p, i32]
    L.aar_batch_create.argtypes = [C.POINTER(vp), i32, C.POINTER(vp)]
    L.aar_batch_run.argtypes = [vp, C.POINTER(vp), C.POINTER(i64), C.POINTER(vp), C.POINTER(vp), vp]
    L.aar_batch_launch_count.argtypes = [vp]
    L.aar_batch_last_error.argtypes = [vp]
    L.aar_batch_last_error.restype = C.c_char_p
    L.aar_batch_destroy.argtypes = [vp]
    L.aar_batch_destroy.restype = None
    L.aar_set_jit.argtypes = [vp, i32]
    L.aar_autotune.argtypes = [vp, C.c_char_p, i32, vp]
    L.aar_jit_status.argtypes = [vp]
    L.aar_jit_status.restype = C.c_char_p
    L.aar_set_spectrum.argtypes = [vp, vp, vp]
    L.aar_adj_spectral.argtypes = [vp, i32, i32, i32, vp, vp, i32, vp]
    L.aar_adj_source.argtypes = [vp, vp, vp, vp, vp]
    L.aar_adj_products.argtypes = [vp, vp, vp, vp, vp, vp]
    # Decomposer (device pointers; tetrapyd arguments as tetrapyd.c's)
    tetra = [vp, vp, vp, vp, i32, vp, vp, vp, i32, vp, i32, i32]
    L.aar_tetra_covariance_scratch_bytes.argtypes = [i32, i32]
    L.aar_tetra_covariance_scratch_bytes.restype = C.c_size_t
    L.aar_tetra_covariance.argtypes = [vp] + tetra + [vp, C.c_size_t, vp]
    L.aar_tetra_QS.argtypes = [vp, vp, i32] + tetra + [vp]
    L.aar_tetra_residual.argtypes = [vp, vp, vp, vp, i32] + tetra + [vp]
    L.aar_tetra_modes_ld.argtypes = [i32]
    L.aar_tetra_modes_ld.restype = i64
    L.aar_tetra_modes.argtypes = [vp, i64, vp, vp, vp, i32, vp, vp, vp, i32, vp, i32, i32, vp]
    L.aar_modes_covariance_scratch_bytes.argtypes = [i32, i32]
    L.aar_modes_covariance_scratch_bytes.restype = C.c_size_t
    L.aar_modes_covariance.argtypes = [vp, vp, i64, vp, i32, i32, vp, C.c_size_t, vp]
    L.aar_modes_project.argtypes = [vp, vp, i32, vp, vp, i64, i32, i32, vp]
    L.aar_modes_residual.argtypes = [vp, vp, vp, vp, i32, vp, i64, i32, vp]
    L.aar_bordered_cond.argtypes = [vp, vp, i32, vp, vp, i32, vp]
    L.aar_last_error.argtypes = [vp]
    L.aar_last_error.restype = C.c_char_p
    L.aar_plan_destroy.argtypes = [vp]
    L.aar_plan_destroy.restype = None
    _lib = L
    return L


def check(L, plan, rc: int) -> None:
    if rc != AAR_OK:
        msg = L.aar_last_error(plan)
        raise AarError(rc, msg.decode() if msg else "")
