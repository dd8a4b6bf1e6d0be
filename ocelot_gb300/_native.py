"""ctypes binding of libocelot_sc.so (the C ABI declared in include/ocelot_sc.h).

The library is the only compute path of this package: there is no CPU
fallback.  If it has not been built, every call raises ``NativeLibraryError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libocelot_sc.so")

SC_ABI_VERSION = 1

SC_FP64 = 0
SC_FP32 = 1
SC_FP32_SORTED_DEPOSIT = 0x10
SC_FP32_EXACT_IGF = 0x20
SC_FP32_SPECTRAL_FIELDS = 0x40

SC_OK = 0
SC_ERR_ARG = 1
SC_ERR_CUDA = 2
SC_ERR_WORKSPACE = 3
SC_ERR_DEGENERATE = 4
SC_ERR_NONFINITE = 5
SC_ERR_UNSUPPORTED = 6
SC_ERR_TIMEOUT = 7
SC_ERR_OOM = 8

SC_NSTAGES = 11

# launch-shape parameters of a plan (sc_plan_set_param)
SC_PARAM_KICK_VARIANT = 0
SC_PARAM_RECORD_FIELD = 1
SC_PARAM_FFT_PLANE_FWD = 2
SC_PARAM_FFT_PLANE_INV = 3
SC_PARAM_FFT_COLS_X = 4
SC_PARAM_FFT_COLS_Y = 5
SC_KICK_NVARIANTS = 21

# the kernels whose bulk-copy waits sc_plan_set_wait_limit bounds
SC_WAIT_FRAME = 0
SC_WAIT_EXTENT = 1
SC_WAIT_KICK = 2

# largest mesh (in corners) of the workspace-free sc_sym_kernel_static
SC_SYM_KERNEL_STATIC_MAX_CORNERS = 524288

# transport records: doubles per packed second-order map (R[36], B[6], the
# combined coefficients Tc[6][21]) and the slice kinds of sc_slices_apply
SC_MAP2_DOUBLES = 36 + 6 + 6 * 21
SC_SLICE_MAP = 0
SC_SLICE_CAVITY = 1
SC_SLICE_MAP_PLANAR = 2
SC_SLICE_MAP_DRIFT = 3
SC_SLICE_MAP_LINEAR = 4

# doubles per set of beam moments written by sc_moments
SC_MOMENTS = 21

REGIONS = {"qgrid": 0, "phi": 1, "ex": 2, "ey": 3, "ez": 4, "keys": 5, "status": 6, "first_error": 7, "field": 8,
           "igf": 9}

ERROR_TEXT = {
    SC_ERR_DEGENERATE: "degenerate beam: zero or non-finite extent or total charge (mesh step would be 0)",
    SC_ERR_NONFINITE: "non-finite particle coordinates or momenta (or a particle outside the mesh)",
    SC_ERR_TIMEOUT: "a device-side wait for a bulk copy gave up after its iteration limit",
}

vp = C.c_void_p
i64 = C.c_int64
dbl = C.c_double

class ScBeam(C.Structure):
    """struct sc_beam of include/ocelot_sc.h."""
    _fields_ = [("plan", vp), ("ws", vp), ("ws_bytes", C.c_size_t), ("rparticles", vp), ("ld", i64), ("q", vp),
                ("n", i64), ("energy_gev", dbl), ("zstep", dbl), ("mesh_scale", dbl), ("mesh_shift", dbl),
                ("tmap", C.POINTER(dbl))]


# name -> (restype, argtypes); the same list as include/ocelot_sc.h
SIGNATURES = {
    "sc_plan_create": (C.c_int, [C.POINTER(vp), C.c_int, C.c_int, C.c_int, C.c_int]),
    "sc_plan_destroy": (None, [vp]),
    "sc_plan_fft_shape": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sc_workspace_bytes": (i64, [vp, i64]),
    "sc_workspace_init": (C.c_int, [vp, vp, C.c_size_t, vp]),
    "sc_workspace_region": (C.c_int, [vp, i64, C.c_int, C.POINTER(i64), C.POINTER(i64)]),
    "sc_read_status": (C.c_int, [vp, vp, vp]),
    "sc_kick": (C.c_int, [vp, vp, C.c_size_t, vp, i64, vp, i64, dbl, dbl, dbl, dbl, vp]),
    "sc_el_field": (C.c_int, [vp, vp, C.c_size_t, vp, vp, i64, dbl, dbl, dbl, vp, vp]),
    "sc_potential": (C.c_int, [vp, vp, C.c_size_t, vp, dbl, dbl, dbl, vp, vp]),
    "sc_sym_kernel": (C.c_int, [vp, vp, C.c_size_t, dbl, dbl, dbl, vp, vp]),
    "sc_sym_kernel_static": (C.c_int, [C.c_int, C.c_int, C.c_int, dbl, dbl, dbl, vp, vp]),
    "sc_sort_workspace_bytes": (i64, [i64, C.c_int]),
    "sc_sort_keys": (C.c_int, [vp, i64, C.c_int, vp, vp, vp, C.c_size_t, vp]),
    "sc_tmap_apply": (C.c_int, [C.POINTER(dbl), C.POINTER(dbl), vp, i64, i64, vp]),
    "sc_tmap_apply_indexed": (C.c_int, [vp, vp, C.c_int, vp, i64, i64, vp]),
    "sc_tmap2_apply": (C.c_int, [vp, C.c_int, vp, i64, i64, vp]),
    "sc_tmap2_apply_step": (C.c_int, [vp, vp, vp, C.c_int, vp, i64, i64, vp]),
    "sc_slices_apply": (C.c_int, [vp, vp, C.c_int, vp, i64, i64, vp]),
    "sc_moments_scratch_bytes": (i64, []),
    "sc_moments": (C.c_int, [vp, i64, i64, vp, C.c_int, C.c_int, dbl, dbl, vp, vp, vp]),
    "sc_slices_apply_step": (C.c_int, [vp, vp, vp, vp, C.c_int, vp, i64, i64, vp]),
    "sc_batch_create": (C.c_int, [C.POINTER(vp), C.c_int]),
    "sc_batch_destroy": (None, [vp]),
    "sc_batch_set": (C.c_int, [vp, C.POINTER(ScBeam), C.c_int, vp]),
    "sc_kick_batched": (C.c_int, [vp, vp]),
    "sc_batch_launches": (C.c_int, [vp]),
    "sc_batch_profile_enable": (C.c_int, [vp, C.c_int]),
    "sc_batch_profile_read": (C.c_int, [vp, C.POINTER(C.c_float)]),
    "sc_tmap_batched": (C.c_int, [vp, vp]),
    "sc_profile_enable": (C.c_int, [vp, C.c_int]),
    "sc_profile_read": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_int)]),
    "sc_profile_stage_name": (C.c_char_p, [C.c_int]),
    "sc_kick_launches": (C.c_int, [vp]),
    "sc_plan_set_wait_limit": (C.c_int, [vp, C.c_int, C.c_longlong]),
    "sc_plan_set_param": (C.c_int, [vp, C.c_int, C.c_int]),
    "sc_plan_get_param": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int)]),
    "sc_kick_variant": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int)]),
    "sc_last_error": (C.c_char_p, []),
    "sc_abi_version": (C.c_int, []),
}


class NativeLibraryError(RuntimeError):
    pass


class ScError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[sc error {code}] {message}")
        self.code = code


_lib = None
_lock = threading.Lock()


def lib():
    """Load libocelot_sc.so once; raise loudly if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise NativeLibraryError(
                    f"{LIB_PATH} is not built; build it with ocelot_gb300.build.build() "
                    "(the sm_103a library is the only compute path of ocelot_gb300)")
            h = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(h, name)
                f.restype = res
                f.argtypes = args
            _lib = h
    return _lib


def last_error() -> str:
    m = lib().sc_last_error()
    return m.decode() if m else ""


def check(code: int) -> None:
    if code != SC_OK:
        msg = last_error()
        if code in (SC_ERR_ARG, SC_ERR_DEGENERATE, SC_ERR_NONFINITE, SC_ERR_UNSUPPORTED):
            raise ValueError(f"[sc error {code}] {msg}")
        if code == SC_ERR_OOM:
            raise MemoryError(f"[sc error {code}] {msg}")
        raise ScError(code, msg)
