"""ctypes mirror of include/hexed_gpu.h and the loader of the CUDA library.

The structures here must match the C header field for field; tests check their sizes
against the header's declarations through the compiled library.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libhexed_gpu.so")

c_int, c_double = ctypes.c_int, ctypes.c_double
P_double = ctypes.POINTER(ctypes.c_double)
P_int = ctypes.POINTER(ctypes.c_int)

HEXED_OK = 0
STATUS_NAMES = {0: "HEXED_OK", -1: "HEXED_ERR_INVALID", -2: "HEXED_ERR_CUDA", -3: "HEXED_ERR_NUMERICAL",
                -4: "HEXED_ERR_NO_DEVICE", -5: "HEXED_ERR_ALLOC", -6: "HEXED_ERR_PRECONDITION"}

BC_FREESTREAM, BC_RIEMANN, BC_NONPENETRATION, BC_COPY, BC_OUTFLOW, BC_PRESSURE_OUTFLOW, BC_NO_SLIP = range(7)
THERMAL_HEAT_FLUX, THERMAL_ENERGY, THERMAL_EQUILIBRIUM = range(3)
ARRAY_ELEM, ARRAY_RCACHE, ARRAY_FACE, ARRAY_BC_CACHE, ARRAY_NOM_SIZE, ARRAY_VERT_TSS, ARRAY_BC_NRML, \
    ARRAY_REF_STATE, ARRAY_JAC, ARRAY_FACE_NRML, ARRAY_DEF_CON_NRML, ARRAY_SAV_AUX, ARRAY_SAV_FACE = range(13)
INT_CAR_CON, INT_BC_CON = 0, 1
FP64, MIXED = 0, 1


class BcSpec(ctypes.Structure):
    _fields_ = [("kind", c_int), ("thermal_kind", c_int), ("freestream", c_double * 5),
                ("pressure", c_double), ("coercion", c_double), ("thermal_value", c_double),
                ("emissivity", c_double), ("heat_transfer_coef", c_double), ("temperature", c_double)]


class Transport(ctypes.Structure):
    _fields_ = [("const_val", c_double), ("ref_val", c_double), ("ref_temp", c_double),
                ("temp_offset", c_double), ("is_viscous", c_int)]


class MeshDesc(ctypes.Structure):
    _fields_ = [("n_dim", c_int), ("row_size", c_int), ("n_car_elem", c_int), ("n_def_elem", c_int),
                ("n_slot", c_int), ("n_car_con", c_int), ("n_def_con", c_int), ("n_bc_con", c_int),
                ("n_ref_face", c_int), ("n_bc_spec", c_int),
                ("elem", P_double), ("rcache", P_double), ("face", P_double),
                ("nom_size", P_double), ("vert_tss", P_double), ("jac", P_double), ("face_nrml", P_double),
                ("car_con", P_int), ("def_con", P_int), ("def_con_nrml", P_double),
                ("bc_con", P_int), ("bc_nrml", P_double), ("bc_cache", P_double),
                ("ref_face", P_int), ("bc_spec", ctypes.POINTER(BcSpec)),
                ("n_vert", c_int), ("vert_id", P_int)]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("launches", c_int), ("total_ms", c_double)]


class UpdateParams(ctypes.Structure):
    _fields_ = [("max_safety", c_double), ("max_time_step", c_double), ("n_cheby_flow", c_int),
                ("flow_iters", c_int), ("local_time", c_int), ("use_filter", c_int), ("use_ldg", c_int),
                ("visc", Transport), ("cond", Transport), ("av_admis_char_speed", c_double),
                ("fix_admis", c_int), ("fix_admis_max_safety", c_double)]


class SavParams(ctypes.Structure):
    """hexed_sav_params: the settings of Solver::update_art_visc_smoothness."""
    _fields_ = [("advect_length", c_double), ("advect_iters", c_int), ("diff_iters", c_int), ("n_cheby", c_int),
                ("av_row_size", c_int), ("advect_safety", c_double), ("diff_safety", c_double),
                ("diff_ratio", c_double), ("visc_mult", c_double), ("unscaled_max", c_double),
                ("freestream_mass", c_double), ("freestream_energy", c_double)]


def sav_params(advect_length, row_size, freestream_mass, freestream_energy, advect_iters=1, diff_iters=1,
               n_cheby=1, av_row_size=None, advect_safety=0.7, diff_safety=0.7, diff_ratio=0.3, visc_mult=1e2,
               unscaled_max=5.):
    """Settings of Solver::update_art_visc_smoothness; defaults of the Solver namespace
    (src/Solver.cpp:154-163), av_row_size defaulting to the row size."""
    return SavParams(advect_length, advect_iters, diff_iters, n_cheby, av_row_size or row_size, advect_safety,
                     diff_safety, diff_ratio, visc_mult, unscaled_max, freestream_mass, freestream_energy)


def transport_inviscid():
    """Transport_model::inviscid (include/Transport_model.hpp:41)."""
    return Transport(0., 0., 1., 1., 0)


def transport_constant(value):
    """Transport_model::constant (include/Transport_model.hpp:43)."""
    return Transport(value, 0., 1., 1., 1)


def transport_sutherland(ref_value, ref_temp, offset):
    """Transport_model::sutherland (include/Transport_model.hpp:48-51)."""
    return Transport(0., ref_value, ref_temp, offset, 1)


def update_params(max_safety=0.7, max_time_step=1.7976931348623157e308, n_cheby_flow=1, flow_iters=1,
                  local_time=False, use_filter=False, visc=None, cond=None, use_ldg=None, av_admis_char_speed=0.,
                  fix_admis=False, fix_admis_max_safety=0.7):
    """Defaults of the Solver namespace (src/Solver.cpp:151-174). use_ldg follows
    Solver::use_ldg (src/Solver.cpp:117-120): viscous transport or artificial viscosity.
    fix_admis: Solver::fix_admissibility after every stage (Solver::set_fix_admissibility)."""
    visc = visc or transport_inviscid()
    cond = cond or transport_inviscid()
    if use_ldg is None:
        use_ldg = bool(visc.is_viscous or cond.is_viscous or av_admis_char_speed > 0)
    return UpdateParams(max_safety, max_time_step, n_cheby_flow, flow_iters, int(local_time),
                        int(use_filter), int(use_ldg), visc, cond, av_admis_char_speed, int(fix_admis),
                        fix_admis_max_safety)


class HexedError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_LIB = None


def load_library(path=LIB_PATH):
    """Load libhexed_gpu.so; raises if it has not been built (there is no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise ImportError(f"hexed_gb300 CUDA library not built: {path} missing "
                          "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    sig = {
        "hexed_gpu_last_error": ([], ctypes.c_char_p),
        "hexed_gpu_version": ([], ctypes.c_char_p),
        "hexed_gpu_create": ([ctypes.POINTER(MeshDesc), c_int, ctypes.POINTER(vp)], c_int),
        "hexed_gpu_destroy": ([vp], c_int),
        "hexed_gpu_upload": ([vp, c_int, P_double], c_int),
        "hexed_gpu_download": ([vp, c_int, P_double], c_int),
        "hexed_gpu_synchronize": ([vp], c_int),
        "hexed_gpu_compute_euler": ([vp, c_double, c_int, c_int, c_int], c_int),
        "hexed_gpu_compute_navier_stokes": ([vp, c_double, c_int, c_int, c_int, ctypes.POINTER(Transport),
                                             ctypes.POINTER(Transport)], c_int),
        "hexed_gpu_max_dt": ([vp, c_double, c_double, c_int, c_int, c_int, ctypes.POINTER(Transport),
                              ctypes.POINTER(Transport), P_double], c_int),
        "hexed_gpu_compute_prolong": ([vp, c_int, c_int], c_int),
        "hexed_gpu_compute_restrict": ([vp, c_int, c_int], c_int),
        "hexed_gpu_compute_write_face": ([vp], c_int),
        "hexed_gpu_apply_state_bcs": ([vp], c_int),
        "hexed_gpu_set_art_visc_admis": ([vp, c_double], c_int),
        "hexed_gpu_apply_flux_bcs": ([vp], c_int),
        "hexed_gpu_update": ([vp, ctypes.POINTER(UpdateParams), P_double], c_int),
        "hexed_gpu_compute_residual": ([vp, ctypes.POINTER(UpdateParams)], c_int),
        "hexed_gpu_residual_norm": ([vp, c_double * 3], c_int),
        "hexed_gpu_profile_enable": ([vp, c_int], c_int),
        "hexed_gpu_profile_read": ([vp, ctypes.POINTER(KernelTime), c_int, ctypes.POINTER(c_int)], c_int),
        "hexed_gpu_stream": ([vp], vp),
        "hexed_gpu_fp64_peak": ([P_double], c_int),
        "hexed_gpu_write_face_range": ([vp, c_int, c_int], c_int),
        "hexed_gpu_set_reference_state": ([vp, P_double], c_int),
        "hexed_gpu_set_launch_shape": ([vp, c_int, c_int], c_int),
        "hexed_gpu_check_conversions": ([P_double, ctypes.c_long, ctypes.POINTER(ctypes.c_long)], c_int),
        "hexed_gpu_is_admissible": ([vp, P_int, P_int], c_int),
        "hexed_gpu_fix_admissibility": ([vp, ctypes.POINTER(UpdateParams), c_double, P_int], c_int),
        "hexed_gpu_device_flags": ([vp, P_int], c_int),
        "hexed_gpu_compute_jacobian": ([vp, P_double], c_int),
        "hexed_gpu_write_state": ([vp, P_double], c_int),
        "hexed_gpu_read_state": ([vp, P_double], c_int),
        "hexed_gpu_launch_shape": ([vp, P_int, P_int], c_int),
        "hexed_gpu_write_range": ([vp, c_int, ctypes.c_long, ctypes.c_long, P_double], c_int),
        "hexed_gpu_read_range": ([vp, c_int, ctypes.c_long, ctypes.c_long, P_double], c_int),
        "hexed_gpu_write_int_range": ([vp, c_int, ctypes.c_long, ctypes.c_long, ctypes.POINTER(c_int)], c_int),
        "hexed_gpu_write_bc_spec": ([vp, c_int, ctypes.POINTER(BcSpec)], c_int),
        "hexed_gpu_set_active": ([vp, c_int, c_int, c_int], c_int),
        "hexed_gpu_segment_residual_norms": ([vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int), P_double],
                                             c_int),
        "hexed_gpu_update_n": ([vp, ctypes.POINTER(UpdateParams), c_int, c_int], c_int),
        "hexed_gpu_segment_residual_norms_static": ([vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                                     P_double], c_int),
        "hexed_gpu_update_art_visc_smoothness": ([vp, ctypes.POINTER(SavParams), P_double], c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _LIB = lib
    return lib


def check(status):
    if status != HEXED_OK:
        lib = load_library()
        raise HexedError(status, lib.hexed_gpu_last_error().decode())
    return status
