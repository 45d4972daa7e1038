"""ctypes bindings of ``libporescale_gpu.so`` (declarations: include/porescale.h)."""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBNAME = "libporescale_gpu.so"

PREC_F64, PREC_F32, PREC_F16, PREC_BF16 = 0, 1, 2, 3
PREC_NAMES = {PREC_F64: "f64", PREC_F32: "f32", PREC_F16: "f16", PREC_BF16: "bf16"}

PS_OK = 0
ERRORS = {1: "PS_ERR_ARG", 2: "PS_ERR_CUDA", 3: "PS_ERR_NOMEM", 4: "PS_ERR_TIMEOUT", 5: "PS_ERR_NOTCONV",
          6: "PS_ERR_NODEVICE", 7: "PS_ERR_STATE"}


class PorescaleError(RuntimeError):
    """A PS_ERR_* code returned by the library, with its message."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class LbmParams(C.Structure):
    """ps_lbm_params: INPUT_PARAMETERS of the LBM (S1:435-469)."""
    _fields_ = [("cr2", C.c_double), ("rr0", C.c_double), ("rb0", C.c_double), ("B", C.c_double),
                ("sig", C.c_double), ("vir", C.c_double), ("vib", C.c_double), ("wet", C.c_double),
                ("ee", C.c_double), ("dt", C.c_double), ("bfr", C.c_double * 3), ("bfb", C.c_double * 3),
                ("idir", C.c_int32), ("iipore", C.c_int32)]


class LbmInfo(C.Structure):
    _fields_ = [("nl", C.c_int64), ("nps", C.c_int64), ("npb2", C.c_int64), ("npb4", C.c_int64),
                ("ns", C.c_int64), ("nvox", C.c_int64), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("precision", C.c_int32), ("tile_x", C.c_int32), ("tile_y", C.c_int32), ("occupancy", C.c_int32),
                ("schedule", C.c_int32), ("wave", C.c_int32), ("march", C.c_int32),
                ("device_bytes", C.c_int64)]


class LbmObs(C.Structure):
    _fields_ = [("tmr", C.c_double), ("tmb", C.c_double), ("tm", C.c_double), ("Cpr", C.c_double),
                ("Cpb", C.c_double), ("nr_cf", C.c_double), ("nb_cf", C.c_double), ("nr", C.c_double),
                ("nb", C.c_double), ("Qr", C.c_double * 3), ("Qb", C.c_double * 3), ("um", C.c_double * 3),
                ("umr", C.c_double * 3), ("umb", C.c_double * 3), ("tfr", C.c_double * 3), ("tfb", C.c_double * 3),
                ("bmt", C.c_double * 3), ("rmt", C.c_double * 3), ("permr", C.c_double), ("permb", C.c_double),
                ("sat_r", C.c_double), ("sat_b", C.c_double), ("isneg", C.c_int32), ("nneg_rr", C.c_int32),
                ("nneg_rb", C.c_int32), ("reserved", C.c_int32)]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)

# name -> (restype, argtypes); every symbol declared in include/porescale.h
SIGNATURES = {
    "ps_lbm_create": (C.c_int, [C.POINTER(LbmParams), _IP, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                C.POINTER(C.c_void_p)]),
    "ps_lbm_destroy": (C.c_int, [_P]),
    "ps_lbm_get_info": (C.c_int, [_P, C.POINTER(LbmInfo)]),
    "ps_lbm_tables": (C.c_int, [_P, _IP, _IP, _IP, _IP]),
    "ps_lbm_set_state": (C.c_int, [_P, _DP, _DP]),
    "ps_lbm_get_state": (C.c_int, [_P, _DP, _DP]),
    "ps_lbm_init_random": (C.c_int, [_P, C.c_double]),
    "ps_lbm_step": (C.c_int, [_P, C.c_int32]),
    "ps_lbm_observables": (C.c_int, [_P, C.POINTER(LbmObs)]),
    "ps_lbm_fields": (C.c_int, [_P, _DP, _DP, _DP]),
    "ps_lbm_wall_load": (C.c_int, [_P, C.c_double, _DP]),
    "ps_lbm_stream": (C.c_void_p, [_P]),
    "ps_lbm_sync": (C.c_int, [_P]),
    "ps_lbm_set_tile": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "ps_lbm_autotune": (C.c_int, [_P, C.c_int32, _IP, _IP, _IP]),
    "ps_lbm_set_fused": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "ps_lbm_set_wait_limit": (C.c_int, [_P, C.c_int32]),
    "ps_lbm_set_sort": (C.c_int, [_P, C.c_int32]),
    "ps_lbm_set_rounding_seed": (C.c_int, [_P, C.c_uint32]),
    "ps_lbm_set_march": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "ps_lbm_set_wave": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "ps_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]),
    "ps_batch_destroy": (C.c_int, [_P]),
    "ps_batch_step": (C.c_int, [_P, C.c_int32]),
    "ps_batch_set_tile": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "ps_batch_autotune": (C.c_int, [_P, C.c_int32, _IP, _IP, _IP]),
    "ps_batch_stream": (C.c_void_p, [_P]),
    "ps_last_error": (C.c_int, [C.c_char_p, C.c_int32]),
    "ps_version": (C.c_char_p, []),
}

_lib = None


def library_path() -> str:
    return os.path.join(_HERE, _LIBNAME)


def library() -> C.CDLL:
    """Loads the CUDA library (raises ImportError when it has not been built)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise ImportError(f"{path} is missing: build it with __graft_entry__.build() "
                              "(porescale_gb300 has no CPU fallback)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    library().ps_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(rc: int) -> None:
    if rc != PS_OK:
        raise PorescaleError(rc, last_error())


def dptr(a):
    """double* of a C-contiguous float64 numpy array."""
    assert a.dtype.name == "float64" and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_DP)


def iptr(a):
    assert a.dtype.name == "int32" and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_IP)
