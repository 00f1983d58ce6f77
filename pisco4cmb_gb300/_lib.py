"""ctypes binding of libpisco_gb300.so (declared in include/pisco_gb300.h).

The library is the only compute path: there is no CPU fallback.  If it is
missing or cannot be loaded, every entry point raises ``PiscoUnavailable``.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

PISCO_OK = 0
PISCO_ERR_INVALID_ARGUMENT = 1
PISCO_ERR_INVALID_CONFIG = 2
PISCO_ERR_NOT_READY = 3
PISCO_ERR_CUDA = 4
PISCO_ERR_OUT_OF_MEMORY = 5
PISCO_ERR_UNSUPPORTED = 6
PISCO_ERR_DEVICE_CHECK = 7

FLOAT32 = 0
FLOAT64 = 1
FORM_PLAIN = 0
FORM_TUNED = 1
FORM_FP64 = 2
BEAM_NEAREST = 0
BEAM_BILINEAR = 1

FORMS = {"plain": FORM_PLAIN, "tuned": FORM_TUNED, "fp64": FORM_FP64}


class PiscoError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


class PiscoInvalidArgument(PiscoError, ValueError):
    """Raised where the reference throws std::invalid_argument."""


class PiscoUnavailable(PiscoError):
    pass


class RunConfig(ctypes.Structure):
    """Mirrors CUDACONV::RunConfig (src/GpuConvolver/cuda/cudaConv2.h:13-26)."""

    _fields_ = [("nStreams", ctypes.c_int), ("maxMemUsage", ctypes.c_size_t),
                ("deviceId", ctypes.c_int), ("gridSizeX", ctypes.c_int),
                ("gridSizeY", ctypes.c_int), ("blockSizeX", ctypes.c_int),
                ("blockSizeY", ctypes.c_int), ("ptgPerConv", ctypes.c_int),
                ("pixelsPerDisc", ctypes.c_int)]

    def __init__(self, nStreams=1, maxMemUsage=0, deviceId=0, gridSizeX=0, gridSizeY=0,
                 blockSizeX=0, blockSizeY=0, ptgPerConv=1 << 20, pixelsPerDisc=0):
        super().__init__(nStreams, maxMemUsage, deviceId, gridSizeX, gridSizeY, blockSizeX,
                         blockSizeY, ptgPerConv, pixelsPerDisc)


PISCO_DET_SKY_ORDER = 1


class DetDesc(ctypes.Structure):
    """pisco_det_desc: one detector pair of a batched forward (device pointers)."""

    _fields_ = [("beam_slot", ctypes.c_int), ("flags", ctypes.c_int),
                ("nsamples", ctypes.c_longlong), ("ra", ctypes.c_void_p),
                ("dec", ctypes.c_void_p), ("pa", ctypes.c_void_p),
                ("tod_a", ctypes.c_void_p), ("tod_b", ctypes.c_void_p)]


class NoallocDet(ctypes.Structure):
    """pisco_noalloc_det: one detector pair of the allocation-free batched forward."""

    _fields_ = [("nside_beam", ctypes.c_int), ("npix_beam", ctypes.c_long),
                ("beam_ab", ctypes.c_void_p), ("nsamples", ctypes.c_longlong),
                ("ra", ctypes.c_void_p), ("dec", ctypes.c_void_p), ("pa", ctypes.c_void_p),
                ("tod_a", ctypes.c_void_p), ("tod_b", ctypes.c_void_p)]


class PairDump(ctypes.Structure):
    """pisco_pair_dump: host arrays receiving a form's per-pair decisions."""

    _fields_ = [("capacity", ctypes.c_longlong), ("sample", ctypes.c_void_p),
                ("sky_pix", ctypes.c_void_p), ("beam_pix", ctypes.c_void_p),
                ("c2chi", ctypes.c_void_p), ("s2chi", ctypes.c_void_p), ("chi", ctypes.c_void_p),
                ("flags", ctypes.c_void_p), ("stencil_pix", ctypes.c_void_p),
                ("stencil_w", ctypes.c_void_p)]


PAIR_REDONE = 1
PAIR_OUTSIDE_BEAM = 2

NOALLOC_MAX_DETS = 128
NOALLOC_MAX_ITEMS = 32768


# every symbol the header declares: (name, restype, argtypes)
_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long
_D = ctypes.c_double
_S = ctypes.c_int  # pisco_status
_PP = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = [
    ("pisco_create", _S, [ctypes.POINTER(RunConfig), ctypes.POINTER(_P)]),
    ("pisco_destroy", _S, [_P]),
    ("pisco_last_error", ctypes.c_char_p, [_P]),
    ("pisco_status_string", ctypes.c_char_p, [_S]),
    ("pisco_abi_version", _I, []),
    ("pisco_set_sky", _S, [_P, _I, _P, _P, _P, _P, _I]),
    ("pisco_set_sky_device", _S, [_P, _I, _P, _I, _P]),
    ("pisco_set_beam", _S, [_P, _I, _L, _PP, _PP, _I]),
    ("pisco_set_scan", _S, [_P, _L, _P, _P, _P, _I]),
    ("pisco_set_scan_device", _S, [_P, _L, _P, _P, _P, _P]),
    ("pisco_set_interp", _S, [_P, _I]),
    ("pisco_set_sample_order", _S, [_P, _I]),
    ("pisco_forward", _S, [_P, ctypes.c_char, _P, _P, _I, _I]),
    ("pisco_forward_device", _S, [_P, _I, _L, _L, _P, _P, _I, _P]),
    ("pisco_sync", _S, [_P]),
    ("pisco_memory_used", _S, [_P, ctypes.POINTER(ctypes.c_size_t)]),
    ("pisco_count_pairs", _S, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    ("pisco_last_fallbacks", _S, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    ("pisco_tuned_calibrate", _S, [_P, _L, _L, ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(ctypes.c_longlong)]),
    ("pisco_debug_pairs", _S, [_P, _I, _L, _L, ctypes.POINTER(PairDump),
                               ctypes.POINTER(ctypes.c_longlong)]),
    ("pisco_hpx_pix2ang_device", _S, [_I, ctypes.c_longlong, _P, _P, _P, _P]),
    ("pisco_hpx_ang2pix_device", _S, [_I, ctypes.c_longlong, _P, _P, _P, _P]),
    ("pisco_hpx_get_interpol_device", _S, [_I, ctypes.c_longlong, _P, _P, _P, _P, _P]),
    ("pisco_set_beam_slot", _S, [_P, _I, _I, _L, _PP, _PP, _I]),
    ("pisco_forward_batched", _S, [_P, ctypes.POINTER(DetDesc), _I, _I, _I, _P]),
    ("pisco_autotune_batched", _S, [_P, ctypes.POINTER(DetDesc), _I, _I, ctypes.c_char_p,
                                    ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]),
    ("pisco_batched_config", _S, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    ("pisco_set_batched_config", _S, [_P, _I, _I]),
    ("pisco_forward_batched_noalloc", _S, [_I, _I, _P, ctypes.POINTER(NoallocDet), _I, _I, _P]),
    ("pisco_set_beam_device", _S, [_P, _I, _L, _P, _I, _P]),
    ("pisco_adjoint_device", _S, [_P, _L, _L, _P, _P, _I, _P, _P, _I, _I, _P]),
    ("pisco_adjoint", _S, [_P, _P, _P, _I, _P, _P, _P, _P, _I, _I]),
    ("pisco_adjoint_gaussian_device", _S, [_P, _L, _L, _P, _P, _I, _P, _I, _I, _D, _I, _D, _D,
                                           _D, _D, _D, _P, _P]),
    ("pisco_focal_plane_to_sky", _S, [_I, _P, _P, _P, _L, _P, _P, _P, _I, _P, _P, _P]),
    ("pisco_focal_plane_to_sky_device", _S, [_I, _P, _P, _P, _L, _P, _P, _P, _I, _P, _P, _P, _P]),
    ("pisco_hpx_pix2ang", _S, [_I, _L, _P, _P, _P]),
    ("pisco_hpx_ang2pix", _S, [_I, _L, _P, _P, _P]),
    ("pisco_beam_npix_for_radius", _L, [_I, _D]),
    ("pisco_beam_rho_max", _D, [_I, _L]),
    ("pisco_beam_gaussian_fields", _S, [_I, _L, _D, _D, _D, _P, _P, _P, _P]),
    ("pisco_beam_from_fields", _S, [_L, _P, _P, _P, _P, _P, _P, _P, _P]),
    ("pisco_beam_build", _S, [_I, _L, _D, ctypes.c_char, _I, _PP, _PP, _PP, _PP]),
    ("pisco_beam_gaussian_param_grad", _S, [_I, _L, _D, _I, _D, _D, _D, _D, _D, _P, _P]),
    ("pisco_beam_build_device", _S, [_P, _I, _L, _D, ctypes.c_char, _I, _P, _P, _P, _I, _P]),
    ("pisco_beam_gaussian_device", _S, [_P, _I, _L, _D, _I, _D, _D, _D, _D, _D, _P, _I, _P]),
    ("pisco_beam_gaussian_param_grad_device", _S,
     [_P, _I, _L, _D, _I, _D, _D, _D, _D, _D, _P, _I, _P, _P]),
    ("pisco_map_create", _S, [_I, _I, ctypes.POINTER(_P)]),
    ("pisco_map_destroy", None, [_P]),
    ("pisco_map_last_error", ctypes.c_char_p, [_P]),
    ("pisco_map_reset", _S, [_P]),
    ("pisco_map_accumulate", _S, [_P, _L, _P, _P, _P, _I, _P, _P, _I]),
    ("pisco_map_accumulate_device", _S, [_P, _L, _P, _P, _P, _I, _P, _P, _I, _P]),
    ("pisco_map_solve", _S, [_P]),
    ("pisco_map_get", _S, [_P, _P, _P, _P, _P]),
    ("pisco_map_get_normal", _S, [_P, _P, _P]),
    ("pisco_map_device_arrays", _S, [_P, ctypes.POINTER(_P), ctypes.POINTER(_P),
                                     ctypes.POINTER(_P)]),
]

_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load the library (building it first when nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if build_if_missing and not _build.up_to_date():
        try:
            _build.build()
        except Exception as e:  # noqa: BLE001 -- reported below
            if not os.path.exists(path):
                raise PiscoUnavailable(-1, "libpisco_gb300.so is not built and the build "
                                           "failed: %s" % e) from e
    if not os.path.exists(path):
        raise PiscoUnavailable(-1, "libpisco_gb300.so not found at %s; run "
                                   "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    L = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int, ctx=None, what: str = "") -> None:
    if status == PISCO_OK:
        return
    L = load()
    msg = L.pisco_last_error(ctx).decode()
    text = "%s: %s (%s)" % (what, msg or L.pisco_status_string(status).decode(),
                            L.pisco_status_string(status).decode())
    if status == PISCO_ERR_INVALID_ARGUMENT:
        raise PiscoInvalidArgument(status, text)
    raise PiscoError(status, text)


def ptr_array(ptrs) -> ctypes.Array:
    arr = (ctypes.c_void_p * len(ptrs))()
    for i, p in enumerate(ptrs):
        arr[i] = p
    return arr
