"""Python mirror of psrdada_cpp's gated-spectrometer handler over the C ABI.

``GatedSpectrometer`` keeps the reference's constructor arguments and its
``init(RawBytes&)`` / ``operator()(RawBytes&)`` pair
(``psrdada_cpp/effelsberg/edd/GatedSpectrometer.cuh:292-320``); the work is
done by the CUDA library ``libgspec.so`` (include/gspec.h).  There is no CPU
fallback: constructing a spectrometer without the library raises.

Also here: ``DadaBufferLayout`` (``edd/DadaBufferLayout.hpp``), ``RawBytes``
(``psrdada_cpp/raw_bytes.hpp``), the sinks ``NullSink`` and
``SimpleFileWriter`` (``psrdada_cpp/src/simple_file_writer.cpp:25-42``) and a
``FileInputStream``-style driver (``psrdada_cpp/detail/file_input_stream.cpp:29-66``).
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
# GSPEC_LIB selects another build of the library (tuning variants)
LIB_PATH = Path(os.environ["GSPEC_LIB"]) if os.environ.get("GSPEC_LIB") else _PKG / "libgspec.so"

GSPEC_OK, GSPEC_STOP = 0, 1
SINGLE_POL, DUAL_POL = 0, 1
POWER, FULL_STOKES = 0, 1
INTENDED, REFERENCE = 0, 1
FLAG_SATURATION_RECORD = 1
FLAG_NO_HOST_BUFFERS = 2
FLAG_UNGATED = 4
FORM_FP32, FORM_BF16, FORM_FP16 = 0, 1, 2
TUNE_KEYS = ("tune_units", "tune_n1", "tune_scratch_mb")


class GspecConfig(ctypes.Structure):
    _fields_ = [
        ("buffer_size", ctypes.c_uint64),
        ("heap_size", ctypes.c_uint64),
        ("n_side_channels", ctypes.c_uint64),
        ("selected_side_channel", ctypes.c_uint64),
        ("selected_bit", ctypes.c_uint64),
        ("fft_length", ctypes.c_uint64),
        ("naccumulate", ctypes.c_uint64),
        ("nbits", ctypes.c_uint32),
        ("input_type", ctypes.c_uint32),
        ("output_type", ctypes.c_uint32),
        ("convention", ctypes.c_uint32),
        ("input_level", ctypes.c_float),
        ("output_level", ctypes.c_float),
        ("device", ctypes.c_int32),
        ("flags", ctypes.c_uint32),
        ("tune_units", ctypes.c_uint64),
        ("tune_n1", ctypes.c_uint32),
        ("tune_scratch_mb", ctypes.c_uint32),
        ("stream_priority", ctypes.c_int32),
        ("form", ctypes.c_uint32),
    ]


class GspecInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "nchans", "n_out", "n_blocks", "nsamps_per_pol", "batch", "output_bytes", "record_bytes",
        "device_bytes", "fft_path", "n1", "n2", "kernel_launches")]


class GspecKernelProfile(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_uint64), ("timed_launches", ctypes.c_uint64),
                ("total_ms", ctypes.c_double)]


class GspecOutput(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("size", ctypes.c_size_t), ("ready", ctypes.c_int)]


_LIB = None


def load_library() -> ctypes.CDLL:
    """Load libgspec.so (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with psrdada_cpp_gb300.build.build()")
    lib = ctypes.CDLL(str(LIB_PATH))
    vp, u64, u32, sz = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_size_t
    lib.gspec_create.restype = vp
    lib.gspec_create.argtypes = [ctypes.POINTER(GspecConfig), ctypes.c_char_p, sz]
    lib.gspec_destroy.restype = None
    lib.gspec_destroy.argtypes = [vp]
    lib.gspec_init.argtypes = [vp, ctypes.c_char_p, sz]
    lib.gspec_process.argtypes = [vp, vp, sz, ctypes.POINTER(GspecOutput)]
    lib.gspec_process_device.argtypes = [vp, vp, sz, ctypes.POINTER(GspecOutput)]
    lib.gspec_run_block_device.argtypes = [vp, vp, vp, vp]
    lib.gspec_clear_output_device.argtypes = [vp, vp, vp]
    lib.gspec_get_info.argtypes = [vp, ctypes.POINTER(GspecInfo)]
    lib.gspec_last_error.restype = ctypes.c_char_p
    lib.gspec_last_error.argtypes = [vp]
    lib.gspec_get_baselines.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
    lib.gspec_set_baselines.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
    lib.gspec_get_saturation.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
    lib.gspec_unpack_device.argtypes = [vp, u32, u64, vp, vp]
    lib.gspec_set_profiling.argtypes = [vp, ctypes.c_int]
    lib.gspec_get_profile.argtypes = [vp, ctypes.POINTER(GspecKernelProfile), ctypes.c_int]
    lib.gspec_reset_profile.argtypes = [vp]
    lib.gspec_gate_device.argtypes = [vp, vp, vp, vp]
    lib.gspec_process_block_noalloc.argtypes = [ctypes.POINTER(GspecConfig), vp, vp, vp, vp, ctypes.c_char_p, sz]
    lib.gspec_query.argtypes = [ctypes.POINTER(GspecConfig), ctypes.POINTER(GspecInfo), ctypes.c_char_p, sz]
    lib.gspec_tc_dft1024_device.argtypes = [vp, vp, u32, ctypes.c_int, vp]
    lib.gspec_register_host.argtypes = [vp, sz]
    lib.gspec_unregister_host.argtypes = [vp]
    from . import serving
    serving.declare(lib)
    _LIB = lib
    return lib


class GspecError(RuntimeError):
    pass


# --------------------------------------------------------------------------
# reference-shaped helpers
# --------------------------------------------------------------------------
class DadaBufferLayout:
    """``DadaBufferLayout`` (``edd/src/DadaBufferLayout.cpp:17-80``).  The
    reference reads the buffer size from the ring buffer; here it is passed."""

    def __init__(self, buffer_size: int, heap_size: int, n_side_channels: int):
        self._buffer_size = int(buffer_size)
        self._heap_size = int(heap_size)
        self._nsc = int(n_side_channels)
        total = self._heap_size + 8 * self._nsc
        self._n_heaps = self._buffer_size // total
        self._gap = self._buffer_size - self._n_heaps * total

    def getBufferSize(self): return self._buffer_size
    def getHeapSize(self): return self._heap_size
    def getNSideChannels(self): return self._nsc
    def sizeOfData(self): return self._n_heaps * self._heap_size
    def sizeOfGap(self): return self._gap
    def sizeOfSideChannelData(self): return 8 * self._nsc * self._n_heaps
    def getNHeaps(self): return self._n_heaps


class RawBytes:
    """``RawBytes`` (``psrdada_cpp/raw_bytes.hpp:19-69``): a non-owning view.

    ``buf`` is a writable numpy uint8 array, a ``bytearray`` or, with
    ``on_device=True``, an integer device pointer."""

    def __init__(self, buf, total_bytes: int | None = None, used_bytes: int | None = None,
                 on_device: bool = False):
        self._buf = buf
        self._on_device = on_device
        if on_device:
            self._ptr = int(buf)
            self._total = int(total_bytes)
        else:
            if isinstance(buf, (bytearray, memoryview)):
                arr = np.frombuffer(buf, dtype=np.uint8)
            else:
                arr = np.asarray(buf)
                if arr.dtype != np.uint8:
                    arr = arr.view(np.uint8)
            self._arr = arr
            self._ptr = arr.ctypes.data
            self._total = int(total_bytes if total_bytes is not None else arr.nbytes)
        self._used = int(used_bytes if used_bytes is not None else self._total)

    def total_bytes(self): return self._total
    def used_bytes(self, value: int | None = None):
        if value is None:
            return self._used
        self._used = int(value)
    def ptr(self): return self._ptr
    def on_device(self): return self._on_device

    def numpy(self) -> np.ndarray:
        if self._on_device:
            raise TypeError("device RawBytes has no host view")
        return self._arr[:self._used]


class NullSink:
    """``NullSink`` (``psrdada_cpp/src/dada_null_sink.cpp``)."""
    def init(self, block: RawBytes): pass
    def __call__(self, block: RawBytes): return False


class CollectingSink:
    """Keeps a copy of every header and output block (tests, tools)."""
    def __init__(self):
        self.header = None
        self.blocks = []
    def init(self, block: RawBytes):
        self.header = bytes(block.numpy())
    def __call__(self, block: RawBytes):
        self.blocks.append(block.numpy().copy())
        return False


class SimpleFileWriter:
    """``SimpleFileWriter`` (``psrdada_cpp/src/simple_file_writer.cpp:25-42``):
    the first 4096 header bytes, then every output block."""
    HEADER_SIZE = 4096

    def __init__(self, filename: str):
        self._f = open(filename, "wb")

    def init(self, block: RawBytes):
        h = bytes(block.numpy()[:self.HEADER_SIZE])
        self._f.write(h.ljust(self.HEADER_SIZE, b"\0"))

    def __call__(self, block: RawBytes):
        self._f.write(block.numpy().tobytes())
        return False

    def close(self):
        self._f.close()


# --------------------------------------------------------------------------
# the handler
# --------------------------------------------------------------------------
class GatedSpectrometer:
    """``GatedSpectrometer<Handler, InputType, OutputType>``
    (``edd/GatedSpectrometer.cuh:270-366``) on the GB300 library.

    ``input_type``/``output_type`` select the template instantiation:
    (SINGLE_POL, POWER) or (DUAL_POL, FULL_STOKES)."""

    def __init__(self, layout: DadaBufferLayout, selectedSideChannel: int, selectedBit: int,
                 fft_length: int, naccumulate: int, nbits: int, input_level: float,
                 output_level: float, handler, input_type: int = SINGLE_POL,
                 output_type: int | None = None, convention: int = INTENDED, device: int = 0,
                 flags: int = 0, tune: dict | None = None, form: int = 0):
        self._lib = load_library()
        if output_type is None:
            output_type = FULL_STOKES if input_type == DUAL_POL else POWER
        cfg = GspecConfig(
            buffer_size=layout.getBufferSize(), heap_size=layout.getHeapSize(),
            n_side_channels=layout.getNSideChannels(), selected_side_channel=selectedSideChannel,
            selected_bit=selectedBit, fft_length=fft_length, naccumulate=naccumulate, nbits=nbits,
            input_type=input_type, output_type=output_type, convention=convention,
            input_level=input_level, output_level=output_level, device=device, flags=flags, form=form,
            **{k: int(v) for k, v in (tune or {}).items() if k in TUNE_KEYS})
        err = ctypes.create_string_buffer(512)
        h = self._lib.gspec_create(ctypes.byref(cfg), err, len(err))
        if not h:
            raise GspecError(err.value.decode())
        self._h = ctypes.c_void_p(h)
        self._handler = handler
        self._out = GspecOutput()
        self._views = {}
        self.config = cfg
        self.layout = layout

    # -- lifetime
    def close(self):
        self._views = {}
        if getattr(self, "_h", None):
            self._lib.gspec_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc < 0:
            raise GspecError(self._lib.gspec_last_error(self._h).decode())
        return rc

    # -- reference interface
    def init(self, block: RawBytes):
        """``init(RawBytes&)`` (``edd/detail/GatedSpectrometer.cu:179-215``)."""
        arr = block.numpy()
        buf = (ctypes.c_char * block.total_bytes()).from_address(block.ptr())
        rc = self._lib.gspec_init(self._h, buf, block.total_bytes())
        self._check(rc)
        # the header text may have grown: report the used bytes like a C string
        used = int(np.argmax(arr == 0)) if (arr == 0).any() else block.total_bytes()
        block.used_bytes(max(block.used_bytes(), used))
        self._handler.init(block)

    def __call__(self, block: RawBytes) -> bool:
        """``operator()(RawBytes&)``: returns True to stop the stream."""
        fn = self._lib.gspec_process_device if block.on_device() else self._lib.gspec_process
        rc = self._check(fn(self._h, ctypes.c_void_p(block.ptr()), block.used_bytes(), ctypes.byref(self._out)))
        if rc == GSPEC_STOP:
            return True
        if self._out.ready:
            n = self._out.size
            key = (self._out.data, n)
            view = self._views.get(key)
            if view is None:   # one view per pinned output buffer, made once
                view = np.ctypeslib.as_array((ctypes.c_uint8 * n).from_address(self._out.data))
                self._views[key] = view
            self._handler(RawBytes(view, n, n))
        return False

    # -- extras
    def info(self) -> GspecInfo:
        info = GspecInfo()
        self._check(self._lib.gspec_get_info(self._h, ctypes.byref(info)))
        return info

    def baselines(self) -> np.ndarray:
        out = (ctypes.c_float * 4)()
        self._check(self._lib.gspec_get_baselines(self._h, out))
        return np.frombuffer(out, dtype=np.float32).copy()

    def set_baselines(self, values) -> None:
        v = (ctypes.c_float * 4)(*[float(x) for x in np.asarray(values, np.float32).ravel()[:4]])
        self._check(self._lib.gspec_set_baselines(self._h, v))

    def saturation(self) -> np.ndarray:
        n = self.info().n_out
        out = (ctypes.c_uint64 * (2 * n))()
        self._check(self._lib.gspec_get_saturation(self._h, out))
        return np.frombuffer(out, dtype=np.uint64).reshape(n, 2).copy()

    def clear_output_device(self, d_out: int, stream: int = 0) -> None:
        """Clears a device output buffer for the first block of an output block
        (only the counters when each block holds whole outputs)."""
        self._check(self._lib.gspec_clear_output_device(self._h, ctypes.c_void_p(d_out), ctypes.c_void_p(stream)))

    def run_block_device(self, d_block: int, d_out: int, stream: int = 0) -> None:
        self._check(self._lib.gspec_run_block_device(self._h, ctypes.c_void_p(d_block), ctypes.c_void_p(d_out),
                                                     ctypes.c_void_p(stream)))

    def gate_device(self, d_block: int, d_gated: int, stream: int = 0) -> None:
        self._check(self._lib.gspec_gate_device(self._h, ctypes.c_void_p(d_block), ctypes.c_void_p(d_gated),
                                                ctypes.c_void_p(stream)))

    def set_profiling(self, enable: bool) -> None:
        self._check(self._lib.gspec_set_profiling(self._h, 1 if enable else 0))

    def profile(self) -> dict:
        """{kernel name: (launches, timed launches, total device ms)}."""
        arr = (GspecKernelProfile * 8)()
        n = self._check(self._lib.gspec_get_profile(self._h, arr, 8))
        return {arr[i].name.decode(): (arr[i].launches, arr[i].timed_launches, arr[i].total_ms) for i in range(n)}

    def reset_profile(self) -> None:
        self._check(self._lib.gspec_reset_profile(self._h))

    def last_error(self) -> str:
        return self._lib.gspec_last_error(self._h).decode()


class FftSpectrometer(GatedSpectrometer):
    """``FftSpectrometer<Handler>`` (``edd/FftSpectrometer.cuh:19-85``,
    ``edd/detail/FftSpectrometer.cu:13-179``): the ungated spectrometer on
    the same library (``GSPEC_FLAG_UNGATED``).  The block holds only packed
    samples; every ``fft_length`` of them is one R2C frame; ``naccumulate``
    frames add up to one power spectrum of ``fft_length/2 + 1`` float32
    channels; an output block is ``n_out`` such spectra, handed to the handler
    with the reference's pipeline delay (block n's spectra at call n + 3).
    ``init`` forwards the header unchanged.

    Three defects of the reference are not reproduced: its in-place R2C plan
    reads each frame from ``fft_length`` floats apart but writes
    ``fft_length/2 + 1`` complex values apart (``:54-56,103-107``), so frames
    overwrite their successors' input; its power buffers are never zeroed, so
    an output block also holds every second earlier block (``:133-147``); and
    it derives the frame count from the float count divided by
    ``2 * nchans`` (``:107``), dropping frames."""

    def __init__(self, buffer_bytes: int, fft_length: int, naccumulate: int, nbits: int, input_level: float,
                 output_level: float, handler, device: int = 0, flags: int = 0, tune: dict | None = None,
                 form: int = 0):
        layout = DadaBufferLayout(buffer_bytes, buffer_bytes, 0)
        super().__init__(layout, 0, 0, fft_length, naccumulate, nbits, input_level, output_level, handler,
                         input_type=SINGLE_POL, output_type=POWER, device=device, flags=flags | FLAG_UNGATED,
                         tune=tune, form=form)


def query(config: GspecConfig) -> GspecInfo:
    """Sizes of a handle for ``config`` (``gspec_query``) without creating it."""
    lib = load_library()
    info = GspecInfo()
    err = ctypes.create_string_buffer(512)
    if lib.gspec_query(ctypes.byref(config), ctypes.byref(info), err, len(err)) != GSPEC_OK:
        raise GspecError(err.value.decode())
    return info


def process_block_noalloc(config: GspecConfig, d_block: int, d_baselines: int, d_out: int, stream: int = 0) -> None:
    """gspec_process_block_noalloc: one device-resident block through the
    chain without any device allocation, for callers whose device memory is
    all reserved up front (see include/gspec.h).  d_baselines (4 float32) is
    read and updated; d_out accumulates.  Calls that overlap on the GPU race
    on the library's shared working array."""
    err = ctypes.create_string_buffer(256)
    rc = load_library().gspec_process_block_noalloc(ctypes.byref(config), ctypes.c_void_p(d_block),
                                                    ctypes.c_void_p(d_baselines), ctypes.c_void_p(d_out),
                                                    ctypes.c_void_p(stream), err, len(err))
    if rc != GSPEC_OK:
        raise GspecError(err.value.decode())


def tc_dft1024_device(d_in: int, d_out: int, ntransforms: int, form: int = FORM_BF16, stream: int = 0) -> None:
    """Tensor-core split-precision DFT-1024 of ntransforms (a multiple of 4)
    contiguous complex64 sequences in device memory (``gspec_tc_dft1024_device``)."""
    lib = load_library()
    rc = lib.gspec_tc_dft1024_device(ctypes.c_void_p(d_in), ctypes.c_void_p(d_out), ntransforms, form,
                                     ctypes.c_void_p(stream))
    if rc != GSPEC_OK:
        raise GspecError(f"gspec_tc_dft1024_device returned {rc}")


def unpack_device(d_raw: int, nbits: int, nsamples: int, d_out: int, stream: int = 0) -> None:
    """``Unpacker::unpack<nbits>`` on device memory."""
    rc = load_library().gspec_unpack_device(ctypes.c_void_p(d_raw), nbits, nsamples, ctypes.c_void_p(d_out),
                                            ctypes.c_void_p(stream))
    if rc != GSPEC_OK:
        raise GspecError(f"gspec_unpack_device failed ({rc})")


def file_input_stream(path: str, handler, header_size: int = 4096, block_size: int | None = None) -> int:
    """Drive a handler from a DADA file (``FileInputStream``,
    ``psrdada_cpp/detail/file_input_stream.cpp:29-66``): a ``header_size``
    header then data blocks of ``block_size`` bytes.  Returns blocks read."""
    n = 0
    with open(path, "rb") as f:
        header = bytearray(f.read(header_size))
        handler.init(RawBytes(header, header_size, header_size))
        while True:
            data = f.read(block_size)
            if not data:
                break
            buf = np.frombuffer(bytearray(data), dtype=np.uint8)
            n += 1
            if handler(RawBytes(buf, block_size, len(data))):
                break
    return n
