"""Python host layer over the C ABI.

Mirrors the reference's policy vocabulary (ugsdr::Mixer<Impl>::Translate,
MatchedFilter::PrepareCodeSpectrum / FilterOptimized, Abs, ReshapeAndSum,
MaxIndex, MeanStdDev, Upsampler, Resampler, Correlator, Codegen) with numpy
arrays in place of std::vector, and the batched FastSearchEngine entry
(src/acquisition/fse.hpp:242-276) as `Context.acquire`.  Every call runs on
the GPU through libugsdr_cuda.so; errors surface as UgsdrError the way the
reference policies throw std::runtime_error.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Context:
    """One device context (stream, plan cache, code-spectrum cache, scratch)."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        h = C.c_void_p()
        st = self.lib.ugsdr_ctx_create(device, C.byref(h))
        if st != L.OK:
            raise L.UgsdrError(st, f"ugsdr_ctx_create({device}) failed")
        self.h = h
        self._codes: dict[int, tuple] = {}

    def close(self) -> None:
        if self.h:
            self.lib.ugsdr_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int) -> None:
        L.check(st, self.h)

    def set_stream(self, stream_ptr: int | None) -> None:
        self._check(self.lib.ugsdr_ctx_set_stream(self.h, C.c_void_p(stream_ptr or 0)))

    def synchronize(self) -> None:
        self._check(self.lib.ugsdr_ctx_synchronize(self.h))

    def launch_count(self) -> int:
        n = C.c_uint64()
        self._check(self.lib.ugsdr_ctx_launch_count(self.h, C.byref(n)))
        return n.value

    def enable_timing(self, on: bool = True) -> None:
        self._check(self.lib.ugsdr_ctx_enable_timing(self.h, 1 if on else 0))

    def reset_timing(self) -> None:
        self._check(self.lib.ugsdr_ctx_reset_timing(self.h))

    def kernel_time(self, kernel: str) -> tuple[int, float]:
        """(launches, total ms) of `kernel` measured with CUDA events on its stream."""
        n, ms = C.c_uint64(), C.c_double()
        self._check(self.lib.ugsdr_ctx_kernel_time(self.h, kernel.encode(), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    # -------------------------------------------------------------- codes
    def code_put(self, chips: np.ndarray, samples: int, repeats: int = 1, spectrum_mode: int = L.SPECTRUM_ONE_SIDED,
                 sign_mask: int = 0, sign_segment: int = 0) -> int:
        chips = np.ascontiguousarray(chips, np.float32)
        h = C.c_int()
        self._check(self.lib.ugsdr_code_put(self.h, _ptr(chips), chips.size, repeats, samples, sign_mask, sign_segment,
                                            spectrum_mode, C.byref(h)))
        return h.value

    def code_release(self, handle: int) -> None:
        self._check(self.lib.ugsdr_code_release(self.h, handle))

    # -------------------------------------------------------- acquisition
    def make_job(self, samples, sample_type: int, fs: float, block_samples: int, n_blocks: int, codes,
                 doppler_range: float, doppler_step: float, *, n_samples: int | None = None, on_device: bool = False,
                 intermediate_frequency: float = 0.0, frontend_frequency: float = 0.0,
                 code_offset_ratio: float = 1.0, fold_samples: int = 0,
                 fold_coherent: bool = True, statistic: int = L.STAT_ABS,
                 spectrum_mode: int = L.SPECTRUM_ONE_SIDED, input_sampling_rate: float = 0.0) -> "Job":
        codes_arr = (C.c_int * len(codes))(*codes)
        if on_device:
            ptr = int(samples)
            assert n_samples is not None
        else:
            arr = np.ascontiguousarray(samples)
            ptr = _ptr(arr)
            if n_samples is None:
                n_samples = self.samples_in(sample_type, input_sampling_rate or fs, arr.nbytes)
            samples = arr
        job = L.AcqJob(ptr, sample_type, 1 if on_device else 0, n_samples, fs, intermediate_frequency, frontend_frequency,
                       code_offset_ratio,
                       block_samples, n_blocks, fold_samples, 1 if fold_coherent else 0, doppler_range, doppler_step,
                       codes_arr, len(codes), statistic, spectrum_mode, input_sampling_rate)
        return Job(job, codes_arr, samples)

    def acquire(self, job: "Job", cells: bool = False):
        n = job.c.n_codes
        res = (L.AcqResult * n)()
        cell_arr = None
        if cells:
            nd = C.c_uint32()
            self._check(self.lib.ugsdr_doppler_bins(job.c.doppler_range, job.c.doppler_step, C.byref(nd)))
            cell_arr = (L.AcqCell * (n * nd.value))()
        self._check(self.lib.ugsdr_acquire(self.h, C.byref(job.c), res, cell_arr))
        out = [AcqResult.from_c(r) for r in res]
        if cells:
            c = np.frombuffer(cell_arr, dtype=np.dtype([("level", "<f4"), ("index", "<u4"), ("mean", "<f4"), ("std", "<f4")]))
            return out, c.reshape(n, -1).copy()
        return out

    def acquire_batch(self, jobs: list["Job"]):
        arr = (L.AcqJob * len(jobs))(*[j.c for j in jobs])
        res = [(L.AcqResult * j.c.n_codes)() for j in jobs]
        ptrs = (C.POINTER(L.AcqResult) * len(jobs))(*[C.cast(r, C.POINTER(L.AcqResult)) for r in res])
        self._check(self.lib.ugsdr_acquire_batch(self.h, arr, len(jobs), ptrs))
        return [[AcqResult.from_c(x) for x in r] for r in res]

    # ----------------------------------------------- four-step tile shapes
    @staticmethod
    def _shape_dict(t: L.TileShape) -> dict:
        return dict(block_samples=t.block_samples, n1=t.n1, cols=t.cols, rows=t.rows, warp_cols=t.warp_cols,
                    warp_rows=t.warp_rows, ms=t.ms)

    def tile_shape(self, block_samples: int) -> dict:
        """The four-step shape block_samples runs with (ugsdr_tile_get)."""
        t = L.TileShape()
        self._check(self.lib.ugsdr_tile_get(self.h, block_samples, C.byref(t)))
        return self._shape_dict(t)

    def set_tile_shape(self, block_samples: int, shape: dict | None) -> None:
        """Pins a shape (a dict as tile_shape / autotune return; None: the rule)."""
        if shape is None:
            self._check(self.lib.ugsdr_tile_set(self.h, block_samples, None))
            return
        t = L.TileShape(shape.get("n1", 0), shape.get("cols", 0), shape.get("rows", 0), shape.get("warp_cols", -1),
                        shape.get("warp_rows", -1), block_samples, 0.0)
        self._check(self.lib.ugsdr_tile_set(self.h, block_samples, C.byref(t)))

    def autotune(self, jobs: list["Job"], max_tried: int = 64) -> list[dict]:
        """ugsdr_autotune over the jobs' large block sizes; returns every
        measured shape with its block size and device time."""
        arr = (L.AcqJob * len(jobs))(*[j.c for j in jobs])
        tried = (L.TileShape * max_tried)()
        n = C.c_int()
        self._check(self.lib.ugsdr_autotune(self.h, arr, len(jobs), tried, max_tried, C.byref(n)))
        return [self._shape_dict(t) for t in tried[:min(n.value, max_tried)]]

    def samples_in(self, sample_type: int, fs: float, nbytes: int) -> int:
        """Samples held by `nbytes` bytes of a capture (BBP DDC: whole epochs)."""
        if sample_type == L.SAMPLES_BBP_DDC:
            one = C.c_size_t()
            self._check(self.lib.ugsdr_sample_bytes(sample_type, fs, int(fs // 1000), C.byref(one)))
            return nbytes // one.value * int(fs // 1000)
        per = {L.SAMPLES_CF32: 8, L.SAMPLES_CI8: 2, L.SAMPLES_CI16: 4}.get(sample_type, 1)
        return nbytes // per

    # ------------------------------------------------------------ per-op
    def unpack_samples(self, raw: np.ndarray, sample_type: int, fs: float, n_samples: int | None = None) -> np.ndarray:
        """SignalParametersBase::GetSeveralMs decoding of any capture format
        (packed BBP DDC / NT1065 included) to complex64."""
        raw = np.ascontiguousarray(raw)
        n = n_samples if n_samples is not None else self.samples_in(sample_type, fs, raw.nbytes)
        out = np.empty(n, np.complex64)
        self._check(self.lib.ugsdr_unpack_samples(self.h, _ptr(raw), raw.nbytes, sample_type, fs, n, _ptr(out)))
        return out

    def mix(self, iq: np.ndarray, fs: float, frequency: float, phase: float = 0.0) -> np.ndarray:
        """Mixer<TableMixer>::Translate(src_dst, fs, f, phase), in place (complex64)."""
        assert iq.dtype == np.complex64 and iq.flags.c_contiguous
        self._check(self.lib.ugsdr_mix(self.h, _ptr(iq), iq.size, fs, frequency, phase))
        return iq

    # ------------------------------------------------ interference stage
    def stft(self, x: np.ndarray, window_length: int = 128, overlap_length: int = 96) -> np.ndarray:
        """ShortTimeFourierTransform<SequentialStft>::Transform(src, window, overlap):
        (columns, window_length) complex64."""
        x = np.ascontiguousarray(x, np.complex64)
        cols = C.c_size_t()
        self._check(self.lib.ugsdr_stft(self.h, _ptr(x), x.size, window_length, overlap_length, None, C.byref(cols)))
        out = np.empty((cols.value, window_length), np.complex64)
        self._check(self.lib.ugsdr_stft(self.h, _ptr(x), x.size, window_length, overlap_length, _ptr(out), C.byref(cols)))
        return out

    def istft(self, columns: np.ndarray, overlap_length: int = 96) -> np.ndarray:
        """The container-of-containers Transform overload (OverlapAndAdd)."""
        columns = np.ascontiguousarray(columns, np.complex64)
        n_cols, w = columns.shape
        out = np.empty(w + (n_cols - 1) * (w - overlap_length), np.complex64)
        self._check(self.lib.ugsdr_istft(self.h, _ptr(columns), n_cols, w, overlap_length, _ptr(out)))
        return out

    @staticmethod
    def _detections(buf, count: int) -> list[dict]:
        return [{"type": buf[i].type, "frequency_bin": buf[i].frequency_bin, "frequency": buf[i].frequency,
                 "jammer_to_noise": buf[i].jammer_to_noise} for i in range(min(count, len(buf)))]

    def jamming_detect(self, x, fs: float, n: int | None = None) -> list[dict]:
        """JammingDetector(fs).Process(src): detection results.  `x`: complex64
        numpy array, or a device pointer (int) to `n` complex samples."""
        buf = (L.JammingDetection * 64)()
        cnt = C.c_int()
        if isinstance(x, int):
            self._check(self.lib.ugsdr_jamming_detect(self.h, C.c_void_p(x), n, fs, 1, buf, 64, C.byref(cnt)))
        else:
            x = np.ascontiguousarray(x, np.complex64)
            self._check(self.lib.ugsdr_jamming_detect(self.h, _ptr(x), x.size, fs, 0, buf, 64, C.byref(cnt)))
        return self._detections(buf, cnt.value)

    def jamming_suppress(self, x, fs: float, n: int | None = None) -> list[dict]:
        """JammingSuppressionEngine<complex<float>>(fs).Process(src_dst), in place
        on a complex64 array (or on `n` samples at a device pointer); returns
        the detections."""
        buf = (L.JammingDetection * 64)()
        cnt = C.c_int()
        if isinstance(x, int):
            self._check(self.lib.ugsdr_jamming_suppress(self.h, C.c_void_p(x), n, fs, 1, buf, 64, C.byref(cnt)))
        else:
            assert x.dtype == np.complex64 and x.flags.c_contiguous
            self._check(self.lib.ugsdr_jamming_suppress(self.h, _ptr(x), x.size, fs, 0, buf, 64, C.byref(cnt)))
        return self._detections(buf, cnt.value)

    def dft(self, x: np.ndarray, inverse: bool = False) -> np.ndarray:
        x = np.ascontiguousarray(x, np.complex64)
        out = np.empty_like(x)
        self._check(self.lib.ugsdr_dft(self.h, _ptr(x), _ptr(out), x.size, 1 if inverse else 0))
        return out

    def prepare_code_spectrum(self, code: np.ndarray, spectrum_mode: int = L.SPECTRUM_ONE_SIDED) -> np.ndarray:
        code = np.ascontiguousarray(code, np.float32)
        out = np.empty(code.size, np.complex64)
        self._check(self.lib.ugsdr_matched_filter_prepare(self.h, _ptr(code), code.size, spectrum_mode, _ptr(out)))
        return out

    def filter_optimized(self, x: np.ndarray, spectrum: np.ndarray, spectrum_mode: int = L.SPECTRUM_ONE_SIDED) -> np.ndarray:
        x = np.array(x, np.complex64, copy=True)
        spectrum = np.ascontiguousarray(spectrum, np.complex64)
        self._check(self.lib.ugsdr_matched_filter(self.h, _ptr(x), x.size, _ptr(spectrum), spectrum_mode))
        return x

    def abs(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.complex64)
        out = np.empty(x.size, np.float32)
        self._check(self.lib.ugsdr_abs(self.h, _ptr(x), x.size, _ptr(out)))
        return out

    def reshape_and_sum(self, x: np.ndarray, block: int) -> np.ndarray:
        cplx = np.iscomplexobj(x)
        x = np.ascontiguousarray(x, np.complex64 if cplx else np.float32)
        out = np.empty(block, x.dtype)
        self._check(self.lib.ugsdr_reshape_sum(self.h, _ptr(x), x.size, block, 1 if cplx else 0, _ptr(out)))
        return out

    def max_index(self, x: np.ndarray) -> tuple[float, int]:
        x = np.ascontiguousarray(x, np.float32)
        v, i = C.c_float(), C.c_size_t()
        self._check(self.lib.ugsdr_max_index(self.h, _ptr(x), x.size, C.byref(v), C.byref(i)))
        return v.value, i.value

    def mean_stddev(self, x: np.ndarray) -> tuple[float, float]:
        x = np.ascontiguousarray(x, np.float32)
        m, s = C.c_float(), C.c_float()
        self._check(self.lib.ugsdr_mean_stddev(self.h, _ptr(x) if x.size else None, x.size, C.byref(m), C.byref(s)))
        return m.value, s.value

    def upsample(self, x: np.ndarray, samples: int) -> np.ndarray:
        cplx = np.iscomplexobj(x)
        x = np.ascontiguousarray(x, np.complex64 if cplx else np.float32)
        out = np.empty(samples, x.dtype)
        self._check(self.lib.ugsdr_upsample(self.h, _ptr(x), x.size, 1 if cplx else 0, _ptr(out), samples))
        return out

    def resample(self, x: np.ndarray, new_fs: int, old_fs: int) -> np.ndarray:
        x = np.ascontiguousarray(x, np.complex64)
        n = C.c_size_t()
        self._check(self.lib.ugsdr_resample(self.h, _ptr(x), x.size, new_fs, old_fs, None, 0, C.byref(n)))
        out = np.empty(n.value, np.complex64)
        self._check(self.lib.ugsdr_resample(self.h, _ptr(x), x.size, new_fs, old_fs, _ptr(out), out.size, C.byref(n)))
        return out

    def correlate(self, x: np.ndarray, code: np.ndarray) -> complex:
        x = np.ascontiguousarray(x, np.complex64)
        code = np.ascontiguousarray(code, np.float32)
        if x.size != code.size:
            raise L.UgsdrError(L.E_INVALID, "Size mismatch")
        out = np.empty(1, np.complex64)
        self._check(self.lib.ugsdr_correlate(self.h, _ptr(x), _ptr(code), x.size, _ptr(out)))
        return complex(out[0])

    def convert_samples(self, raw: np.ndarray, sample_type: int) -> np.ndarray:
        raw = np.ascontiguousarray(raw)
        per = {L.SAMPLES_CF32: 8, L.SAMPLES_CI8: 2, L.SAMPLES_CI16: 4, L.SAMPLES_RI8: 1}[sample_type]
        n = raw.nbytes // per
        out = np.empty(n, np.complex64)
        self._check(self.lib.ugsdr_convert_samples(self.h, _ptr(raw), sample_type, n, _ptr(out)))
        return out


@dataclass
class Job:
    c: L.AcqJob
    codes_arr: object
    keep: object = field(repr=False, default=None)


@dataclass
class AcqResult:
    code: int
    doppler_bin: int
    index: int
    n_doppler: int
    doppler: float
    code_offset: float
    level: float
    sigma: float
    mean: float
    std: float
    snr: float

    @staticmethod
    def from_c(r: L.AcqResult) -> "AcqResult":
        return AcqResult(r.code, r.doppler_bin, r.index, r.n_doppler, r.doppler, r.code_offset, r.level, r.sigma, r.mean,
                         r.std, r.snr)


def prn_code(signal: int, sv: int) -> np.ndarray:
    """Codegen<Impl>::Get<float>(sv): +-1 chips."""
    lib = L.load()
    n = C.c_size_t()
    buf = np.empty(20000, np.float32)
    st = lib.ugsdr_prn_code(signal, sv, _ptr(buf), buf.size, C.byref(n))
    if st != L.OK:
        raise L.UgsdrError(st, f"ugsdr_prn_code({signal}, {sv}) failed")
    return buf[: n.value].copy()


def repeat_upsample(chips: np.ndarray, repeats: int, samples: int) -> np.ndarray:
    lib = L.load()
    chips = np.ascontiguousarray(chips, np.float32)
    out = np.empty(samples, np.float32)
    st = lib.ugsdr_repeat_upsample(_ptr(chips), chips.size, repeats, _ptr(out), samples)
    if st != L.OK:
        raise L.UgsdrError(st, "ugsdr_repeat_upsample failed")
    return out


def doppler_bins(range_hz: float, step_hz: float) -> int:
    n = C.c_uint32()
    st = L.load().ugsdr_doppler_bins(range_hz, step_hz, C.byref(n))
    if st != L.OK:
        raise L.UgsdrError(st, "bad doppler grid")
    return n.value


TRACK_DTYPE = np.dtype([("taps", "<f4", (5, 2)), ("carrier_frequency", "<f8"), ("carrier_phase", "<f8"),
                        ("code_phase", "<f8"), ("code_frequency", "<f8"), ("phase_error", "<f8"), ("code_error", "<f8")])


class TrackBank:
    """Correlator bank (ugsdr_track_create / _run): channels advance together,
    their NCO and loop state stays on the device between run() calls."""

    def __init__(self, ctx: Context, channels: list[dict], codes: list[np.ndarray], *, early_late: float = 0.25,
                 very_early_late: float = 0.5, pll_bw: float = 25.0, dll_bw: float = 0.7, fll_bw: float = 250.0,
                 nco_mode: int = 0):
        self.ctx = ctx
        lens = [len(c) for c in codes]
        lmax = max(lens)
        table = np.zeros((len(codes), lmax), np.float32)
        for i, c in enumerate(codes):
            table[i, : len(c)] = c
        chs = (L.TrackChannel * len(channels))()
        for i, ch in enumerate(channels):
            code_len = lens[ch["code"]] if 0 <= ch["code"] < len(lens) else 0  # the library rejects bad indices
            chs[i] = L.TrackChannel(ch["code"], ch["fs"], ch["code_frequency"], code_len, ch["code_phase"],
                                    ch["carrier_frequency"], ch.get("carrier_phase", 0.0), ch.get("boc", 0))
        cfg = L.TrackConfig(early_late, very_early_late, pll_bw, dll_bw, fll_bw, 1e-3, nco_mode)
        lens_arr = (C.c_int * len(lens))(*lens)
        h = C.c_void_p()
        ctx._check(ctx.lib.ugsdr_track_create(ctx.h, C.byref(cfg), chs, len(channels), _ptr(table), lens_arr, len(codes),
                                              lmax, C.byref(h)))
        self.h = h
        self.n = len(channels)
        self.spm = int(channels[0]["fs"] // 1000)

    def run(self, samples, sample_type: int, n_epochs: int, on_device: bool = False, outputs: bool = True,
            out: np.ndarray | None = None):
        """Advances n_epochs; returns (n_epochs, n_channels) TRACK_DTYPE rows
        (into `out` when given, e.g. a view of pinned memory)."""
        ptr = int(samples) if on_device else _ptr(np.ascontiguousarray(samples))
        keep = samples
        if outputs and out is None:
            out = np.zeros((n_epochs, self.n), TRACK_DTYPE)
        if not outputs:
            out = None
        elif out.dtype != TRACK_DTYPE or out.size != n_epochs * self.n or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous TRACK_DTYPE array of n_epochs x n_channels")
        self.ctx._check(self.ctx.lib.ugsdr_track_run(self.h, C.c_void_p(ptr), sample_type, 1 if on_device else 0, self.spm,
                                                     n_epochs, C.cast(out.ctypes.data, C.POINTER(L.TrackOutput))
                                                     if outputs else None))
        del keep
        return out

    def run_device(self, samples_ptr: int, sample_type: int, n_epochs: int, outputs_ptr: int | None = None) -> None:
        """ugsdr_track_run_device: device samples and (optional) device outputs,
        enqueued on the context stream without waiting."""
        self.ctx._check(self.ctx.lib.ugsdr_track_run_device(self.h, C.c_void_p(int(samples_ptr)), sample_type, self.spm,
                                                            n_epochs, C.c_void_p(int(outputs_ptr or 0))))

    def close(self):
        if self.h:
            self.ctx.lib.ugsdr_track_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def track_refine(ctx: Context, channels: list[dict], codes: list[np.ndarray], samples, sample_type: int):
    """ugsdr_track_refine: TrackingParameters::AddSignalImpl's code-phase
    refinement of acquired channels.  Returns (accepted, offsets, channels
    with refined code_phase)."""
    lens = [len(c) for c in codes]
    lmax = max(lens)
    table = np.zeros((len(codes), lmax), np.float32)
    for i, c in enumerate(codes):
        table[i, : len(c)] = c
    chs = (L.TrackChannel * len(channels))()
    for i, ch in enumerate(channels):
        code_len = lens[ch["code"]] if 0 <= ch["code"] < len(lens) else 0
        chs[i] = L.TrackChannel(ch["code"], ch["fs"], ch["code_frequency"], code_len, ch["code_phase"],
                                ch["carrier_frequency"], ch.get("carrier_phase", 0.0), ch.get("boc", 0))
    raw = np.ascontiguousarray(samples)
    n = ctx.samples_in(sample_type, channels[0]["fs"], raw.nbytes)
    acc = (C.c_int * len(channels))()
    off = (C.c_int * len(channels))()
    lens_arr = (C.c_int * len(lens))(*lens)
    ctx._check(ctx.lib.ugsdr_track_refine(ctx.h, chs, len(channels), _ptr(table), lens_arr, len(codes), lmax, _ptr(raw),
                                          sample_type, 0, n, acc, off))
    out = [dict(ch, code_phase=chs[i].code_phase) for i, ch in enumerate(channels)]
    return list(acc), list(off), out


OBSERVABLE_DTYPE = np.dtype([("pseudorange", "<f8"), ("pseudophase", "<f8"), ("doppler", "<f8"), ("snr", "<f8")])


def _outputs_arg(outputs, shape):
    """(pointer, on_device, n_epochs, n_channels, keep-alive) of tracking-bank
    outputs: a TRACK_DTYPE array (host) or a device pointer with its shape."""
    if isinstance(outputs, np.ndarray):
        if outputs.dtype != TRACK_DTYPE or outputs.ndim != 2 or not outputs.flags.c_contiguous:
            raise ValueError("outputs must be a contiguous (n_epochs, n_channels) TRACK_DTYPE array")
        return outputs.ctypes.data, 0, outputs.shape[0], outputs.shape[1], outputs
    if shape is None:
        raise ValueError("a device pointer needs shape=(n_epochs, n_channels)")
    return int(outputs), 1, int(shape[0]), int(shape[1]), None


def preamble_search(ctx: Context, outputs, messages: list[int], cap: int = 4096, shape=None, as_arrays: bool = False):
    """ugsdr_preamble_search: per channel the epochs where the navigation
    symbols match the message's preamble (FindPreambleGps / Glonass's
    candidates), ascending.  `outputs`: the bank's TRACK_DTYPE rows, or a
    device pointer with shape=(n_epochs, n_channels).  Returns a list of
    lists, or with as_arrays the (counts, indexes[n_channels, cap]) arrays
    as the C call fills them."""
    ptr, dev, n_ep, n_ch, keep = _outputs_arg(outputs, shape)
    if len(messages) != n_ch:
        raise ValueError("one message per channel")
    msg = np.ascontiguousarray(messages, np.int32)
    counts = np.zeros(n_ch, np.int32)
    idx = np.empty((n_ch, max(cap, 1)), np.int32)
    ip = C.POINTER(C.c_int)
    ctx._check(ctx.lib.ugsdr_preamble_search(ctx.h, C.c_void_p(ptr), dev, n_ep, n_ch, msg.ctypes.data_as(ip),
                                             counts.ctypes.data_as(ip), idx.ctypes.data_as(ip), cap))
    del keep
    if counts.max() > cap:
        raise ValueError(f"more than cap={cap} candidates: {counts.max()}")
    if as_arrays:
        return counts, idx
    return [idx[c, :counts[c]].tolist() for c in range(n_ch)]


def observables(ctx: Context, outputs, channels: list[dict], shape=None, out_ptr: int | None = None):
    """ugsdr_observables: pseudorange (ms), pseudophase (cycles), Doppler (Hz)
    and SNR (dB-Hz) per epoch and channel from the bank's outputs.  channels:
    dicts with fs, carrier_frequency, optional intermediate_frequency,
    carrier_phase, preamble_position, range_correction_ms.  Host outputs give
    an (n_epochs, n_channels) OBSERVABLE_DTYPE array; a device pointer (with
    shape) writes to the device pointer out_ptr and returns None."""
    ptr, dev, n_ep, n_ch, keep = _outputs_arg(outputs, shape)
    if len(channels) != n_ch:
        raise ValueError("one channel description per channel")
    chs = (L.ObservableChannel * n_ch)()
    for i, ch in enumerate(channels):
        chs[i] = L.ObservableChannel(ch["fs"], ch.get("intermediate_frequency", 0.0), ch["carrier_frequency"],
                                     ch.get("carrier_phase", 0.0), ch.get("preamble_position", 0),
                                     ch.get("range_correction_ms", 0.0))
    if dev:
        if not out_ptr:
            raise ValueError("device outputs need a device out_ptr")
        ctx._check(ctx.lib.ugsdr_observables(ctx.h, C.c_void_p(ptr), 1, n_ep, n_ch, chs, C.c_void_p(int(out_ptr))))
        return None
    out = np.zeros((n_ep, n_ch), OBSERVABLE_DTYPE)
    ctx._check(ctx.lib.ugsdr_observables(ctx.h, C.c_void_p(ptr), 0, n_ep, n_ch, chs, C.c_void_p(out.ctypes.data)))
    del keep
    return out


class Server:
    """Continuous-batching acquisition and tracking server (ugsdr_server_*)."""

    def __init__(self, ctx: Context, max_inflight: int = 4, memory_budget: int = 0, queue_capacity: int = 1024,
                 policy: int = L.SERVE_FIFO):
        self.ctx = ctx
        cfg = L.ServerConfig(max_inflight, memory_budget, queue_capacity, policy)
        h = C.c_void_p()
        ctx._check(ctx.lib.ugsdr_server_create(ctx.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self._n_codes: dict[int, int] = {}
        self._tracks: dict[int, np.ndarray] = {}

    def submit(self, job: Job) -> int:
        t = C.c_uint64()
        self.ctx._check(self.ctx.lib.ugsdr_server_submit(self.h, C.byref(job.c), C.byref(t)))
        self._n_codes[t.value] = job.c.n_codes
        return t.value

    def submit_track(self, bank: "TrackBank", samples: np.ndarray, sample_type: int, n_epochs: int) -> int:
        """A tracking run of `bank` over n_epochs epochs of host samples; poll
        returns its outputs (n_epochs x n_channels records)."""
        arr = np.ascontiguousarray(samples)
        out = np.zeros((n_epochs, bank.n), dtype=TRACK_DTYPE)
        t = C.c_uint64()
        self.ctx._check(self.ctx.lib.ugsdr_server_submit_track(self.h, bank.h, _ptr(arr), sample_type, bank.spm, n_epochs,
                                                               _ptr(out), C.byref(t)))
        self._tracks[t.value] = out
        return t.value

    def poll(self, ticket: int):
        """None while pending, else the per-code results, or for a tracking
        request its outputs (the ticket is retired)."""
        if ticket in self._tracks:
            done = C.c_int()
            self.ctx._check(self.ctx.lib.ugsdr_server_poll(self.h, ticket, None, C.byref(done)))
            if not done.value:
                return None
            return self._tracks.pop(ticket)
        n = self._n_codes[ticket]
        res = (L.AcqResult * n)()
        done = C.c_int()
        self.ctx._check(self.ctx.lib.ugsdr_server_poll(self.h, ticket, res, C.byref(done)))
        if not done.value:
            return None
        del self._n_codes[ticket]
        return [AcqResult.from_c(r) for r in res]

    def drain(self) -> None:
        self.ctx._check(self.ctx.lib.ugsdr_server_drain(self.h))

    def stats(self) -> dict:
        s = L.ServerStats()
        self.ctx._check(self.ctx.lib.ugsdr_server_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in L.ServerStats._fields_}

    def close(self) -> None:
        if self.h:
            self.ctx.lib.ugsdr_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
