"""ctypes binding of libkpt.so (include/kpt.h).

The library is the product: there is no Python or CPU implementation behind
this module, and loading fails loudly when libkpt.so has not been built.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkpt.so")

KPT_OK = 0
STAGES = ("camera", "shade", "shadow", "extend", "sky", "accumulate", "post")   # KPT_STAGE_* order
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "invalid state", -4: "out of device memory",
          -5: "traversal stack overflow"}


class KptError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Material(C.Structure):
    _fields_ = [("albedo", C.c_float * 3), ("metallic", C.c_float), ("roughness", C.c_float),
                ("transmission", C.c_float), ("ior", C.c_float), ("emission", C.c_float * 3),
                ("emission_scale", C.c_float), ("normal_scale", C.c_float), ("albedo_tex", C.c_int32),
                ("orm_tex", C.c_int32), ("transmission_tex", C.c_int32), ("emission_tex", C.c_int32),
                ("normal_tex", C.c_int32), ("pad", C.c_int32)]


class Environment(C.Structure):
    _fields_ = [("sun_angular_diameter", C.c_float), ("sun_phi", C.c_float), ("sun_theta", C.c_float),
                ("sun_emission_factor", C.c_float), ("rayleigh", C.c_float * 3), ("mie", C.c_float),
                ("mie_absorption", C.c_float), ("rayleigh_height", C.c_float), ("mie_height", C.c_float),
                ("pad", C.c_float)]


class Settings(C.Structure):
    _fields_ = [("max_depth", C.c_int32), ("bloom", C.c_int32), ("karis", C.c_int32),
                ("auto_exposure", C.c_int32), ("bloom_final_blend", C.c_float),
                ("bloom_internal_blend", C.c_float), ("frame_delta_ms", C.c_float), ("rng_order", C.c_int32),
                ("temporal_accumulation", C.c_int32), ("postprocess_effects", C.c_int32), ("upscale", C.c_int32),
                ("sky_arith", C.c_int32), ("temporal_arith", C.c_int32)]


class Exposure(C.Structure):
    _fields_ = [("aperture", C.c_float), ("iso", C.c_float), ("shutter", C.c_float), ("ev_comp", C.c_float),
                ("white_ev", C.c_float), ("black_ev", C.c_float), ("max_iso", C.c_float), ("min_iso", C.c_float),
                ("max_shutter", C.c_float), ("min_shutter", C.c_float), ("pad0", C.c_float), ("pad1", C.c_float)]


class Stats(C.Structure):
    _fields_ = [("box_tests", C.c_uint64), ("tri_tests", C.c_uint64), ("inst_xforms", C.c_uint64),
                ("overflows", C.c_uint64), ("path_box_tests", C.c_uint64), ("path_tri_tests", C.c_uint64),
                ("path_inst_xforms", C.c_uint64), ("shadow_box_tests", C.c_uint64),
                ("shadow_tri_tests", C.c_uint64), ("shadow_inst_xforms", C.c_uint64),
                ("path_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("camera_rays", C.c_uint64),
                ("avg_luminance", C.c_float), ("adapted_luminance", C.c_float),
                ("exposure_scalar", C.c_float), ("iso", C.c_float), ("shutter", C.c_float),
                ("avg_bin", C.c_float), ("frame_index", C.c_int32), ("pad", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [("grid_scale", C.c_float), ("wave_cap", C.c_int32), ("shade_block", C.c_int32),
                ("sort_rays", C.c_int32), ("fetch_batch", C.c_int32), ("group_lobes", C.c_int32)]


assert C.sizeof(Material) == 72 and C.sizeof(Environment) == 48
assert C.sizeof(Settings) == 52 and C.sizeof(Exposure) == 48

_P = C.c_void_p
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)
_S = C.c_int

SIGNATURES = {
    "kpt_last_error": (C.c_char_p, []),
    "kpt_environment_default": (None, [C.POINTER(Environment)]),
    "kpt_settings_default": (None, [C.POINTER(Settings)]),
    "kpt_exposure_default": (None, [C.POINTER(Exposure)]),
    "kpt_create": (_S, [C.c_int, C.POINTER(_P)]),
    "kpt_destroy": (_S, [_P]),
    "kpt_resize": (_S, [_P, C.c_int, C.c_int]),
    "kpt_get_render_size": (_S, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "kpt_set_materials": (_S, [_P, C.c_int, C.POINTER(Material)]),
    "kpt_set_textures": (_S, [_P, C.c_int, _I, C.c_size_t, C.POINTER(C.c_uint8)]),
    "kpt_upload_mesh": (_S, [_P, C.c_int, _F, _F, _F, _I, C.POINTER(C.c_int)]),
    "kpt_add_instance": (_S, [_P, C.c_int, _F, C.c_int, C.POINTER(C.c_int)]),
    "kpt_set_blas_build": (_S, [_P, C.c_int]),
    "kpt_refit_mesh": (_S, [_P, C.c_int, _F, _F]),
    "kpt_get_blas": (_S, [_P, C.c_int, _I, _F, _I, _F]),
    "kpt_commit_scene": (_S, [_P]),
    "kpt_clear_scene": (_S, [_P]),
    "kpt_counts": (_S, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "kpt_set_material": (_S, [_P, C.c_int, C.POINTER(Material)]),
    "kpt_get_material": (_S, [_P, C.c_int, C.POINTER(Material)]),
    "kpt_set_instance_transform": (_S, [_P, C.c_int, _F]),
    "kpt_get_instance_transform": (_S, [_P, C.c_int, _F]),
    "kpt_set_view": (_S, [_P, _F, _F]),
    "kpt_set_camera_inverse": (_S, [_P, _F, _F]),
    "kpt_set_environment": (_S, [_P, C.POINTER(Environment)]),
    "kpt_get_environment": (_S, [_P, C.POINTER(Environment)]),
    "kpt_set_settings": (_S, [_P, C.POINTER(Settings)]),
    "kpt_get_settings": (_S, [_P, C.POINTER(Settings)]),
    "kpt_set_exposure": (_S, [_P, C.POINTER(Exposure)]),
    "kpt_get_exposure": (_S, [_P, C.POINTER(Exposure)]),
    "kpt_reset_accumulation": (_S, [_P]),
    "kpt_render_frame": (_S, [_P, C.c_int, C.c_float]),
    "kpt_synchronize": (_S, [_P]),
    "kpt_read_image": (_S, [_P, _F]),
    "kpt_read_render": (_S, [_P, _F]),
    "kpt_read_accumulation": (_S, [_P, _F]),
    "kpt_read_albedo": (_S, [_P, _F]),
    "kpt_read_history": (_S, [_P, _F]),
    "kpt_read_histogram": (_S, [_P, C.POINTER(C.c_uint64)]),
    "kpt_get_stats": (_S, [_P, C.POINTER(Stats)]),
    "kpt_get_level_counts": (_S, [_P, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "kpt_render_samples_device": (_S, [_P, C.c_int, C.c_int, _P, _P, _P]),
    "kpt_trace_device": (_S, [_P, C.c_int, _P, _P, C.c_float, C.c_float, _P, _P, _P, _P]),
    "kpt_occluded_device": (_S, [_P, C.c_int, _P, _P, C.c_float, _P, _P]),
    "kpt_trace_bounces_device": (_S, [_P, C.c_int, _P, _P, C.c_int, _P, _P, _P]),
    "kpt_trace_bounces": (_S, [_P, C.c_int, _F, _F, C.c_int, _I, _I, _F]),
    "kpt_trace_bounces_noalloc": (_S, [_P, C.c_int, _F, _F, C.c_int, _I, _I, _F]),
    "kpt_sky_device": (_S, [_P, C.c_int, _P, _P]),
    "kpt_enable_timing": (_S, [_P, C.c_int]),
    "kpt_stage_ms": (_S, [_P, C.c_int, C.POINTER(C.c_float)]),
    "kpt_path_kernel_ms": (_S, [_P, C.c_int, C.POINTER(C.c_float)]),
    "kpt_get_stream": (_S, [_P, C.POINTER(_P)]),
    "kpt_launch_count": (_S, [_P, C.POINTER(C.c_uint64)]),
    "kpt_tuning_default": (None, [C.POINTER(Tuning)]),
    "kpt_set_tuning": (_S, [_P, C.POINTER(Tuning)]),
    "kpt_get_tuning": (_S, [_P, C.POINTER(Tuning)]),
    "kpt_batch_create": (_S, [C.c_int, C.POINTER(_P)]),
    "kpt_batch_destroy": (_S, [_P]),
    "kpt_submit_batch": (_S, [_P, C.c_int, C.POINTER(_P), _I, C.c_int]),
    "kpt_batch_set_shared": (_S, [_P, C.c_int]),
    "kpt_batch_get_shared": (_S, [_P, _I]),
    "kpt_wait_batch": (_S, [_P, _F, _F]),
    "kpt_autotune_batch": (_S, [_P, C.c_int, C.POINTER(_P), _I, C.c_int, C.POINTER(Tuning), _I, _F]),
    "kpt_adjoint_param_count": (_S, [_P, C.POINTER(C.c_int)]),
    "kpt_adjoint_device": (_S, [_P, C.c_int, C.c_int, _P, _P, _P]),
    "kpt_adjoint": (_S, [_P, C.c_int, C.c_int, _F, C.POINTER(C.c_double), _F]),
    "kpt_adjoint_forward_device": (_S, [_P, C.c_int, C.c_int, _P]),
    "kpt_adjoint_backward_device": (_S, [_P, _P, _P]),
    "kpt_adjoint_record_size": (C.c_int, []),
    "kpt_sky_grad_device": (_S, [_P, C.c_int, _P, _P]),
    "kpt_adjoint_records_device": (_S, [_P, C.c_int, C.c_int, _P, _P, _P, C.c_int, C.POINTER(C.c_int)]),
}

_lib = None


def load():
    """Load libkpt.so and bind every entry point; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError(f"{LIB_PATH} is not built; run kittlespt_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != KPT_OK:
        raise KptError(status, load().kpt_last_error().decode())


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_F)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_I)
