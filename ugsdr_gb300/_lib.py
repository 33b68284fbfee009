"""ctypes binding of include/ugsdr_cuda.h (libugsdr_cuda.so).

Loading fails loudly: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libugsdr_cuda.so"

ABI_VERSION = 9  # UGSDR_CUDA_ABI_VERSION the structs below mirror

OK = 0
E_INVALID = -1
E_CUDA = -2
E_NOMEM = -3
E_UNSUPPORTED = -4
E_NOT_FOUND = -5
E_QUEUE_FULL = -6
E_TIMEOUT = -7

GPS_L1CA, GPS_L2CM, GPS_L5I, GPS_L5Q, GLONASS_L1OF, GLONASS_L2OF, GALILEO_E1B, GALILEO_E1C = range(8)
SAMPLES_CF32, SAMPLES_CI8, SAMPLES_CI16, SAMPLES_RI8 = range(4)
SAMPLES_BBP_DDC, SAMPLES_NT1065_1, SAMPLES_NT1065_2, SAMPLES_NT1065_3, SAMPLES_NT1065_4 = range(4, 9)
SPECTRUM_ONE_SIDED, SPECTRUM_TWO_SIDED = 0, 1
STAT_ABS, STAT_ABS2 = 0, 1


class AcqJob(C.Structure):
    _fields_ = [
        ("samples", C.c_void_p),
        ("sample_type", C.c_int),
        ("samples_on_device", C.c_int),
        ("n_samples", C.c_size_t),
        ("sampling_rate", C.c_double),
        ("intermediate_frequency", C.c_double),
        ("frontend_frequency", C.c_double),
        ("code_offset_ratio", C.c_double),
        ("block_samples", C.c_size_t),
        ("n_blocks", C.c_size_t),
        ("fold_samples", C.c_size_t),
        ("fold_coherent", C.c_int),
        ("doppler_range", C.c_double),
        ("doppler_step", C.c_double),
        ("codes", C.POINTER(C.c_int)),
        ("n_codes", C.c_int),
        ("statistic", C.c_int),
        ("spectrum_mode", C.c_int),
        ("input_sampling_rate", C.c_double),
    ]


class AcqResult(C.Structure):
    _fields_ = [
        ("code", C.c_int),
        ("doppler_bin", C.c_int),
        ("index", C.c_uint32),
        ("n_doppler", C.c_uint32),
        ("doppler", C.c_double),
        ("code_offset", C.c_double),
        ("level", C.c_double),
        ("sigma", C.c_double),
        ("mean", C.c_double),
        ("std", C.c_double),
        ("snr", C.c_double),
    ]


class AcqCell(C.Structure):
    _fields_ = [("level", C.c_float), ("index", C.c_uint32), ("mean", C.c_float), ("std", C.c_float)]


class TileShape(C.Structure):
    _fields_ = [("n1", C.c_int), ("cols", C.c_int), ("rows", C.c_int), ("warp_cols", C.c_int), ("warp_rows", C.c_int),
                ("block_samples", C.c_int),
                ("ms", C.c_double)]


class TrackChannel(C.Structure):
    _fields_ = [
        ("code", C.c_int),
        ("sampling_rate", C.c_double),
        ("code_frequency", C.c_double),
        ("code_length", C.c_double),
        ("code_phase", C.c_double),
        ("carrier_frequency", C.c_double),
        ("carrier_phase", C.c_double),
        ("boc", C.c_int),
    ]


class TrackConfig(C.Structure):
    _fields_ = [
        ("early_late_spacing", C.c_double),
        ("very_early_late_spacing", C.c_double),
        ("pll_bandwidth", C.c_double),
        ("dll_bandwidth", C.c_double),
        ("fll_bandwidth", C.c_double),
        ("integration_time", C.c_double),
        ("nco_mode", C.c_int),
    ]


class TrackOutput(C.Structure):
    _fields_ = [
        ("taps", (C.c_float * 2) * 5),
        ("carrier_frequency", C.c_double),
        ("carrier_phase", C.c_double),
        ("code_phase", C.c_double),
        ("code_frequency", C.c_double),
        ("phase_error", C.c_double),
        ("code_error", C.c_double),
    ]


NAV_GPS_LNAV, NAV_GLONASS = 0, 1


class ObservableChannel(C.Structure):
    _fields_ = [("sampling_rate", C.c_double), ("intermediate_frequency", C.c_double),
                ("carrier_frequency", C.c_double), ("carrier_phase", C.c_double),
                ("preamble_position", C.c_longlong), ("range_correction_ms", C.c_double)]


class Observable(C.Structure):
    _fields_ = [("pseudorange", C.c_double), ("pseudophase", C.c_double), ("doppler", C.c_double),
                ("snr", C.c_double)]


SERVE_FIFO, SERVE_RESPONSE_RATIO = 0, 1

INTERFERENCE_NONE, INTERFERENCE_NARROWBAND, INTERFERENCE_WIDEBAND = 0, 1, 2


class JammingDetection(C.Structure):
    _fields_ = [("type", C.c_int), ("frequency_bin", C.c_int), ("frequency", C.c_double),
                ("jammer_to_noise", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("max_inflight", C.c_int), ("memory_budget", C.c_size_t), ("queue_capacity", C.c_int),
                ("policy", C.c_int)]


# exported symbols and their signatures (restype, argtypes)
_vp, _sz, _i, _d, _u32, _u64 = C.c_void_p, C.c_size_t, C.c_int, C.c_double, C.c_uint32, C.c_uint64
_fp = C.POINTER(C.c_float)
SIGNATURES = {
    "ugsdr_ctx_create": (_i, [_i, C.POINTER(_vp)]),
    "ugsdr_ctx_destroy": (_i, [_vp]),
    "ugsdr_ctx_set_stream": (_i, [_vp, _vp]),
    "ugsdr_ctx_synchronize": (_i, [_vp]),
    "ugsdr_last_error": (C.c_char_p, [_vp]),
    "ugsdr_ctx_launch_count": (_i, [_vp, C.POINTER(_u64)]),
    "ugsdr_abi_version": (_i, []),
    "ugsdr_ctx_enable_timing": (_i, [_vp, _i]),
    "ugsdr_ctx_kernel_time": (_i, [_vp, C.c_char_p, C.POINTER(_u64), C.POINTER(_d)]),
    "ugsdr_ctx_reset_timing": (_i, [_vp]),
    "ugsdr_prn_code": (_i, [_i, _i, _vp, _sz, C.POINTER(_sz)]),
    "ugsdr_repeat_upsample": (_i, [_vp, _sz, _sz, _vp, _sz]),
    "ugsdr_code_put": (_i, [_vp, _vp, _sz, _sz, _sz, _u32, _sz, _i, C.POINTER(_i)]),
    "ugsdr_code_release": (_i, [_vp, _i]),
    "ugsdr_acquire": (_i, [_vp, C.POINTER(AcqJob), C.POINTER(AcqResult), C.POINTER(AcqCell)]),
    "ugsdr_acquire_batch": (_i, [_vp, C.POINTER(AcqJob), _i, C.POINTER(C.POINTER(AcqResult))]),
    "ugsdr_doppler_bins": (_i, [_d, _d, C.POINTER(_u32)]),
    "ugsdr_dft25_batch": (_i, [_vp, _vp, _vp, _sz, _i, C.POINTER(C.c_float)]),
    "ugsdr_tile_get": (_i, [_vp, _sz, C.POINTER(TileShape)]),
    "ugsdr_tile_set": (_i, [_vp, _sz, C.POINTER(TileShape)]),
    "ugsdr_autotune": (_i, [_vp, C.POINTER(AcqJob), _i, C.POINTER(TileShape), _i, C.POINTER(_i)]),
    "ugsdr_mix": (_i, [_vp, _vp, _sz, _d, _d, _d]),
    "ugsdr_dft": (_i, [_vp, _vp, _vp, _sz, _i]),
    "ugsdr_matched_filter_prepare": (_i, [_vp, _vp, _sz, _i, _vp]),
    "ugsdr_matched_filter": (_i, [_vp, _vp, _sz, _vp, _i]),
    "ugsdr_abs": (_i, [_vp, _vp, _sz, _vp]),
    "ugsdr_reshape_sum": (_i, [_vp, _vp, _sz, _sz, _i, _vp]),
    "ugsdr_max_index": (_i, [_vp, _vp, _sz, _fp, C.POINTER(_sz)]),
    "ugsdr_mean_stddev": (_i, [_vp, _vp, _sz, _fp, _fp]),
    "ugsdr_upsample": (_i, [_vp, _vp, _sz, _i, _vp, _sz]),
    "ugsdr_resample": (_i, [_vp, _vp, _sz, _u64, _u64, _vp, _sz, C.POINTER(_sz)]),
    "ugsdr_correlate": (_i, [_vp, _vp, _vp, _sz, _vp]),
    "ugsdr_convert_samples": (_i, [_vp, _vp, _i, _sz, _vp]),
    "ugsdr_sample_bytes": (_i, [_i, _d, _sz, C.POINTER(_sz)]),
    "ugsdr_unpack_samples": (_i, [_vp, _vp, _sz, _i, _d, _sz, _vp]),
    "ugsdr_track_create": (_i, [_vp, C.POINTER(TrackConfig), C.POINTER(TrackChannel), _i, _vp, C.POINTER(_i), _i, _i,
                                C.POINTER(_vp)]),
    "ugsdr_track_run": (_i, [_vp, _vp, _i, _i, _sz, _i, C.POINTER(TrackOutput)]),
    "ugsdr_track_run_device": (_i, [_vp, _vp, _i, _sz, _i, _vp]),
    "ugsdr_track_destroy": (_i, [_vp]),
    "ugsdr_track_refine": (_i, [_vp, C.POINTER(TrackChannel), _i, _vp, C.POINTER(_i), _i, _i, _vp, _i, _i, _sz,
                                C.POINTER(_i), C.POINTER(_i)]),
    "ugsdr_preamble_search": (_i, [_vp, _vp, _i, _i, _i, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), _i]),
    "ugsdr_observables": (_i, [_vp, _vp, _i, _i, _i, C.POINTER(ObservableChannel), _vp]),
    "ugsdr_stft": (_i, [_vp, _vp, _sz, _i, _i, _vp, C.POINTER(_sz)]),
    "ugsdr_istft": (_i, [_vp, _vp, _sz, _i, _i, _vp]),
    "ugsdr_jamming_detect": (_i, [_vp, _vp, _sz, _d, _i, C.POINTER(JammingDetection), _i, C.POINTER(_i)]),
    "ugsdr_jamming_suppress": (_i, [_vp, _vp, _sz, _d, _i, C.POINTER(JammingDetection), _i, C.POINTER(_i)]),
    "ugsdr_server_create": (_i, [_vp, C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "ugsdr_server_submit": (_i, [_vp, C.POINTER(AcqJob), C.POINTER(_u64)]),
    "ugsdr_server_submit_track": (_i, [_vp, _vp, _vp, _i, C.c_size_t, _i, _vp, C.POINTER(_u64)]),
    "ugsdr_server_poll": (_i, [_vp, _u64, C.POINTER(AcqResult), C.POINTER(_i)]),
    "ugsdr_server_drain": (_i, [_vp]),
    "ugsdr_server_destroy": (_i, [_vp]),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libugsdr_cuda.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path or os.environ.get("UGSDR_CUDA_LIB", LIB_PATH))
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                           "(the CUDA extension is required; there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.ugsdr_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{p} has ABI {lib.ugsdr_abi_version()}, these bindings expect {ABI_VERSION}: rebuild it")
    if path is None:
        _lib = lib
    return lib


class UgsdrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


def check(status: int, ctx=None) -> None:
    if status != OK:
        msg = load().ugsdr_last_error(ctx).decode() if ctx else "error"
        raise UgsdrError(status, msg)


class StaticJob(C.Structure):
    """ugsdr_static_job (allocation-free entry point; device pointers)."""
    _fields_ = [
        ("samples", C.c_void_p),
        ("sample_type", C.c_int),
        ("n_samples", C.c_size_t),
        ("sampling_rate", C.c_double),
        ("frontend_frequency", C.c_double),
        ("block_samples", C.c_size_t),
        ("n_blocks", C.c_size_t),
        ("fold_samples", C.c_size_t),
        ("fold_coherent", C.c_int),
        ("doppler_range", C.c_double),
        ("doppler_step", C.c_double),
        ("code_samples", C.c_void_p),
        ("n_codes", C.c_int),
        ("statistic", C.c_int),
        ("spectrum_mode", C.c_int),
    ]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64), ("inflight", C.c_int),
                ("max_inflight_seen", C.c_int), ("device_bytes", C.c_size_t), ("busy_seconds", C.c_double)]


SIGNATURES["ugsdr_server_get_stats"] = (C.c_int, [C.c_void_p, C.POINTER(ServerStats)])

STATIC_SCRATCH_BYTES = 16 << 20
SIGNATURES["ugsdr_acquire_static"] = (C.c_int, [C.c_void_p, C.POINTER(StaticJob), C.c_void_p, C.POINTER(C.c_size_t)])
