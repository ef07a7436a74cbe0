"""ctypes binding of libfsgb300.so (the C ABI declared in include/fsgb300.h).

The library is loaded from ``fastsimus_gb300/_lib/libfsgb300.so`` (built in-tree by
``fastsimus_gb300.build``).  There is no fallback: if the library or a CUDA device is missing,
every entry point raises.
"""

from __future__ import annotations

import ctypes
import math
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfsgb300.so"

FSG_OK, FSG_EINVAL, FSG_ECUDA, FSG_ETIMEOUT, FSG_EUNSUPPORTED, FSG_EWORKSPACE = range(6)
FSG_BAFFLE_SOFT, FSG_BAFFLE_RIGID, FSG_BAFFLE_IMPEDANCE = range(3)
FSG_OUT_SELECTED_RAW, FSG_OUT_FULL_CORRECTED = range(2)
ABI_VERSION = 4


class FsgError(RuntimeError):
    """A libfsgb300 call failed; ``status`` is the FsgStatus code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[fsg status {status}] {message}")
        self.status = status


class FsgProbe(ctypes.Structure):
    _fields_ = [("n_elements", ctypes.c_int32), ("n_sub", ctypes.c_int32), ("pitch", ctypes.c_double),
                ("element_width", ctypes.c_double), ("radius", ctypes.c_double), ("freq_center", ctypes.c_double),
                ("baffle", ctypes.c_int32), ("reserved0", ctypes.c_int32), ("baffle_impedance", ctypes.c_double)]


class FsgMedium(ctypes.Structure):
    _fields_ = [("speed_of_sound", ctypes.c_double), ("attenuation", ctypes.c_double)]


class FsgFreqPlan(ctypes.Structure):
    _fields_ = [("n_freq", ctypes.c_int32), ("n_freq_full", ctypes.c_int32), ("freq_idx_start", ctypes.c_int32),
                ("reserved0", ctypes.c_int32), ("freq_start", ctypes.c_double), ("freq_step", ctypes.c_double),
                ("seg_length", ctypes.c_double), ("correction_factor", ctypes.c_double),
                ("pulse_spectrum", ctypes.c_void_p), ("probe_spectrum", ctypes.c_void_p)]


class FsgPhantom(ctypes.Structure):
    _fields_ = [("scat_xz", ctypes.c_void_p), ("rc", ctypes.c_void_p), ("n_scat", ctypes.c_int64),
                ("plan", FsgFreqPlan), ("out", ctypes.c_void_p)]


class FsgMlpWeights(ctypes.Structure):
    _fields_ = [("packed", ctypes.c_void_p * 4), ("bias", ctypes.c_void_p * 4), ("w_head", ctypes.c_void_p),
                ("b_head", ctypes.c_void_p), ("bmat", ctypes.c_void_p), ("n_out", ctypes.c_int32),
                ("reserved0", ctypes.c_int32)]


class FsgSurrogateDomain(ctypes.Structure):
    _fields_ = [("x_lo", ctypes.c_double), ("x_hi", ctypes.c_double), ("z_lo", ctypes.c_double),
                ("z_hi", ctypes.c_double), ("f_lo", ctypes.c_double), ("f_hi", ctypes.c_double),
                ("max_angle", ctypes.c_double), ("pitch", ctypes.c_double), ("speed_of_sound", ctypes.c_double),
                ("n_elements", ctypes.c_int32), ("n_carriers", ctypes.c_int32)]


_V4 = ctypes.c_void_p * 4


class FsgMlpTrain(ctypes.Structure):
    _fields_ = [("u", ctypes.c_void_p), ("aux", ctypes.c_void_p), ("n_data", ctypes.c_int64),
                ("seed", ctypes.c_uint64), ("bmat", ctypes.c_void_p),
                ("w", _V4), ("m_w", _V4), ("v_w", _V4), ("packed_fwd", _V4), ("packed_bwd", _V4),
                ("b", _V4), ("m_b", _V4), ("v_b", _V4),
                ("w_head", ctypes.c_void_p), ("m_w_head", ctypes.c_void_p), ("v_w_head", ctypes.c_void_p),
                ("b_head", ctypes.c_void_p), ("m_b_head", ctypes.c_void_p), ("v_b_head", ctypes.c_void_p),
                ("packed_head", ctypes.c_void_p), ("n_out", ctypes.c_int32), ("n_tiles", ctypes.c_int32), ("n_split", ctypes.c_int32),
                ("total_steps", ctypes.c_int32), ("warmup_steps", ctypes.c_int32),
                ("lr", ctypes.c_float), ("lr_min", ctypes.c_float), ("beta1", ctypes.c_float),
                ("beta2", ctypes.c_float), ("eps", ctypes.c_float),
                ("step", ctypes.c_void_p), ("loss_hist", ctypes.c_void_p), ("loss_hist_len", ctypes.c_int32),
                ("status", ctypes.c_void_p), ("workspace", ctypes.c_void_p), ("workspace_bytes", ctypes.c_size_t)]


class FsgBatchTuning(ctypes.Structure):
    _fields_ = [("freqs_per_item", ctypes.c_int32), ("chunk_scatterers", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("tile_scatterers", ctypes.c_int32), ("packed", ctypes.c_int32),
                ("threads_per_cta", ctypes.c_int32), ("reserved", ctypes.c_int32 * 2)]


FSG_DAS_LINEAR, FSG_DAS_NEAREST = range(2)


class FsgDasParams(ctypes.Structure):
    _fields_ = [("speed_of_sound", ctypes.c_double), ("fs", ctypes.c_double), ("fc", ctypes.c_double),
                ("t0", ctypes.c_double), ("fnumber", ctypes.c_double), ("method", ctypes.c_int32),
                ("iq", ctypes.c_int32)]


_P = ctypes.c_void_p
_DP = ctypes.POINTER(ctypes.c_double)
_SIGNATURES = {
    "fsg_abi_version": (ctypes.c_int32, []),
    "fsg_last_error_string": (ctypes.c_char_p, []),
    "fsg_simus_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgFreqPlan),
                                                   ctypes.c_int64]),
    "fsg_simus_launches": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgFreqPlan), ctypes.c_int64,
                                            ctypes.c_int32]),
    "fsg_simus": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgMedium), ctypes.POINTER(FsgFreqPlan),
                                   _P, _P, ctypes.c_int64, _P, _P, ctypes.c_int32, ctypes.c_int32, _P, _P,
                                   ctypes.c_size_t, _P]),
    "fsg_pfield_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgFreqPlan),
                                                    ctypes.c_int64]),
    "fsg_pfield": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgMedium), ctypes.POINTER(FsgFreqPlan),
                                    _P, ctypes.c_int64, _P, _P, ctypes.c_int32, _P, _P, ctypes.c_size_t, _P]),
    "fsg_simus_batched_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgPhantom),
                                                           ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                           ctypes.POINTER(FsgBatchTuning)]),
    "fsg_simus_batched": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgMedium),
                                           ctypes.POINTER(FsgPhantom), ctypes.c_int32, _P, _P, ctypes.c_int32,
                                           ctypes.c_int32, ctypes.POINTER(FsgBatchTuning), _P, ctypes.c_size_t,
                                           _P]),
    "fsg_simus_batched_tc_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgPhantom),
                                                              ctypes.c_int32, ctypes.c_int32,
                                                              ctypes.POINTER(FsgBatchTuning)]),
    "fsg_simus_batched_tc": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgMedium),
                                              ctypes.POINTER(FsgPhantom), ctypes.c_int32, _P, _P, ctypes.c_int32,
                                              ctypes.POINTER(FsgBatchTuning), _P, ctypes.c_size_t, _P]),
    "fsg_simus_batched_tc_status": (ctypes.c_int32, [_P, ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgPhantom),
                                                     ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(FsgBatchTuning),
                                                     ctypes.POINTER(ctypes.c_int32), _P]),
    "fsg_simus_batched_rx": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgMedium),
                                              ctypes.POINTER(FsgPhantom), _P, ctypes.c_int32, _P,
                                              ctypes.POINTER(FsgBatchTuning), _P, ctypes.c_size_t, _P]),
    "fsg_txfield": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgMedium), ctypes.c_double,
                                     ctypes.c_double, _P, ctypes.c_int64, _P, _P, ctypes.c_size_t, _P]),
    "fsg_surrogate_inputs": (ctypes.c_int32, [ctypes.POINTER(FsgSurrogateDomain), _P, ctypes.c_int64, _P,
                                              ctypes.c_double, _P, _P, _P]),
    "fsg_surrogate_combine": (ctypes.c_int32, [ctypes.POINTER(FsgSurrogateDomain), _P, ctypes.c_int64, _P,
                                               ctypes.c_double, _P, _P]),
    "fsg_mlp_train_workspace_size": (ctypes.c_size_t, [ctypes.c_int32, ctypes.c_int32]),
    "fsg_mlp_train_n_params": (ctypes.c_int64, [ctypes.c_int32]),
    "fsg_mlp_train_init": (ctypes.c_int32, [ctypes.POINTER(FsgMlpTrain), _P]),
    "fsg_mlp_train_steps": (ctypes.c_int32, [ctypes.POINTER(FsgMlpTrain), ctypes.c_int32, _P]),
    "fsg_mlp_train_gradients": (ctypes.c_int32, [ctypes.POINTER(FsgMlpTrain), _P, _P, _P]),
    "fsg_tc_selftest": (ctypes.c_int32, [_P, _P, _P, ctypes.c_int32, ctypes.c_int32, _P, _P]),
    "fsg_simus_noalloc": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgMedium),
                                           ctypes.POINTER(FsgFreqPlan), _P, _P, ctypes.c_int64, _P, _P, ctypes.c_int32,
                                           ctypes.c_int32, _P, _P]),
    "fsg_simus_noalloc_scratch_bytes": (ctypes.c_size_t, []),
    "fsg_fp32_fma_probe": (ctypes.c_int32, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                            _P]),
    "fsg_rf_workspace_size": (ctypes.c_size_t, [ctypes.c_int32, ctypes.c_int32]),
    "fsg_mlp_tc_packed_bytes": (ctypes.c_size_t, [ctypes.c_int32]),
    "fsg_mlp_tc_pack": (ctypes.c_int32, [_P, ctypes.c_int32, ctypes.c_int32, _P, _P]),
    "fsg_mlp_tc_forward": (ctypes.c_int32, [ctypes.POINTER(FsgMlpWeights), _P, ctypes.c_int64, _P, _P, _P]),
    "fsg_irfft_gate": (ctypes.c_int32, [_P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _P, _P,
                                        ctypes.c_size_t, _P]),
    "fsg_rf2iq": (ctypes.c_int32, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_int32, _DP, _DP, ctypes.c_int32, _P,
                                   _P]),
    "fsg_das": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgDasParams), _P, ctypes.c_int32,
                                 ctypes.c_int32, _P, _P, ctypes.c_int64, _P, _P]),
    "fsg_dasmtx_nnz_per_row": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32]),
    "fsg_wait_selftest": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32, _P, _P]),
    "fsg_dasmtx": (ctypes.c_int32, [ctypes.POINTER(FsgProbe), ctypes.POINTER(FsgDasParams), ctypes.c_int32, _P, _P,
                                    ctypes.c_int64, _P, _P, _P, _P]),
}

_lib = None
_lock = threading.Lock()


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def load(path: Path | str | None = None):
    """Load (once) and return the ctypes handle of libfsgb300.so."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise FsgError(FSG_EINVAL, f"native library {p} not found: run `python -m fastsimus_gb300.build` "
                                       "(or __graft_entry__.build()) first")
        lib = ctypes.CDLL(str(p))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        v = lib.fsg_abi_version()
        if v != ABI_VERSION:
            raise FsgError(FSG_EINVAL, f"libfsgb300 ABI version {v} != expected {ABI_VERSION}")
        _lib = lib
        return lib


def check(status: int):
    if status != FSG_OK:
        msg = load().fsg_last_error_string().decode(errors="replace")
        if status == FSG_EUNSUPPORTED:
            raise NotImplementedError(f"[fsg status {status}] {msg}")
        if status in (FSG_EINVAL, FSG_EWORKSPACE):
            raise ValueError(f"[fsg status {status}] {msg}")
        raise FsgError(status, msg)


def make_probe(params, n_sub: int) -> FsgProbe:
    from fastsimus_gb300.params import BaffleType

    b = params.baffle
    if isinstance(b, BaffleType) or isinstance(b, str):
        kind = FSG_BAFFLE_SOFT if str(b) == "soft" else FSG_BAFFLE_RIGID
        imp = 0.0
    else:
        kind = FSG_BAFFLE_IMPEDANCE
        imp = float(b)
    radius = float(params.radius)
    return FsgProbe(n_elements=int(params.n_elements), n_sub=int(n_sub), pitch=float(params.pitch),
                    element_width=float(params.element_width), radius=radius if math.isfinite(radius) else math.inf,
                    freq_center=float(params.freq_center), baffle=kind, reserved0=0, baffle_impedance=imp)


def make_medium(medium) -> FsgMedium:
    return FsgMedium(speed_of_sound=float(medium.speed_of_sound), attenuation=float(medium.attenuation))
