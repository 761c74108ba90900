"""VLBI: EDD samples to 2-bit VDIF frames on the GPU (Python mirror of
``VLBI<Handler>``, ``psrdada_cpp/effelsberg/edd/VLBI.cuh:91-170``, over
``gspec_vlbi_*`` of include/gspec.h) and the VDIF header
(``VDIFHeaderView`` / ``VDIFHeader``, ``edd/VLBI.cuh:20-84``, field layout of
the VDIF specification 1.1.1 as the reference's accessors in
``edd/src/VLBI.cu:20-170``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from .gated_spectrometer import RawBytes, GspecError, GspecOutput, GSPEC_OK, GSPEC_STOP, load_library


def _bits(w: int, first: int, last: int) -> int:
    return (w >> first) & ((1 << (last - first + 1)) - 1)


def _set(w: int, first: int, last: int, v: int) -> int:
    mask = ((1 << (last - first + 1)) - 1) << first
    if v >= (1 << (last - first + 1)):
        raise ValueError("Value does not fit into bitrange")
    return (w & ~mask & 0xFFFFFFFF) | ((v << first) & mask)


class VDIFHeaderView:
    """Reads the fields of a 32-byte VDIF header (eight little-endian words)."""

    def __init__(self, words):
        self.words = np.asarray(words, np.uint32).copy() if words is not None else np.zeros(8, np.uint32)

    def _w(self, i):
        return int(self.words[i])

    def isValid(self): return _bits(self._w(0), 31, 31) == 0
    def getSecondsFromReferenceEpoch(self): return _bits(self._w(0), 0, 29)
    def getReferenceEpoch(self): return _bits(self._w(1), 24, 29)
    def getDataFrameNumber(self): return _bits(self._w(1), 0, 23)
    def getDataFrameLength(self): return _bits(self._w(2), 0, 23)
    def getVersionNumber(self): return _bits(self._w(2), 29, 31)
    def getNumberOfChannels(self): return _bits(self._w(2), 24, 28)
    def isRealDataType(self): return _bits(self._w(3), 31, 31) == 0
    def isComplexDataType(self): return _bits(self._w(3), 31, 31) == 1
    def getBitsPerSample(self): return _bits(self._w(3), 26, 30)
    def getThreadId(self): return _bits(self._w(3), 16, 25)
    def getStationId(self): return _bits(self._w(3), 0, 15)

    def getTimestamp(self) -> int:
        """POSIX seconds of the header's epoch and second."""
        import datetime
        ep = self.getReferenceEpoch()
        start = datetime.datetime(2000 + ep // 2, 7 if ep % 2 else 1, 1, tzinfo=datetime.timezone.utc)
        return int(start.timestamp()) + self.getSecondsFromReferenceEpoch()


class VDIFHeader(VDIFHeaderView):
    """A VDIF header with setters; a new header has version 1, as the reference's."""

    def __init__(self, words=None):
        super().__init__(words)
        if words is None:
            self.words[2] = _set(int(self.words[2]), 29, 31, 1)

    def _put(self, i, first, last, v):
        self.words[i] = _set(int(self.words[i]), first, last, int(v))

    def setInvalid(self): self._put(0, 31, 31, 1)
    def setValid(self): self._put(0, 31, 31, 0)
    def setSecondsFromReferenceEpoch(self, v): self._put(0, 0, 29, v)
    def setReferenceEpoch(self, v): self._put(1, 24, 29, v)
    def setDataFrameNumber(self, v): self._put(1, 0, 23, v)
    def setDataFrameLength(self, v): self._put(2, 0, 23, v)
    def setNumberOfChannels(self, v): self._put(2, 24, 28, v)
    def setComplexDataType(self): self._put(3, 31, 31, 1)
    def setRealDataType(self): self._put(3, 31, 31, 0)
    def setBitsPerSample(self, v): self._put(3, 26, 30, v)
    def setThreadId(self, v): self._put(3, 16, 25, v)
    def setStationId(self, v): self._put(3, 0, 15, v)

    def setTimeReferencesFromTimestamp(self, posix_seconds: int):
        arr = (ctypes.c_uint32 * 8)(*[int(w) for w in self.words])
        if _lib().gspec_vdif_set_time(arr, int(posix_seconds)) != GSPEC_OK:
            raise ValueError("Cannot encode time before 1 Jan 2000")
        self.words = np.array(list(arr), np.uint32)

    def getData(self) -> np.ndarray:
        return self.words


class GspecVlbiConfig(ctypes.Structure):
    _fields_ = [("buffer_size", ctypes.c_uint64), ("nbits", ctypes.c_uint32), ("device", ctypes.c_int32),
                ("spead_heap_size", ctypes.c_uint64), ("sample_rate", ctypes.c_double),
                ("digitizer_threshold", ctypes.c_double), ("vdif_header", ctypes.c_uint32 * 8)]


class GspecVlbiInfo(ctypes.Structure):
    _fields_ = [("frame_bytes", ctypes.c_uint64), ("frames_per_output", ctypes.c_uint64),
                ("output_bytes", ctypes.c_uint64), ("frames_per_second", ctypes.c_uint64),
                ("bytes_to_skip", ctypes.c_uint64), ("spill_bytes", ctypes.c_uint64),
                ("header", ctypes.c_uint32 * 8), ("last_sum", ctypes.c_int64), ("last_sum_sq", ctypes.c_uint64)]


def _lib():
    lib = load_library()
    vp, sz = ctypes.c_void_p, ctypes.c_size_t
    lib.gspec_vlbi_create.restype = vp
    lib.gspec_vlbi_create.argtypes = [ctypes.POINTER(GspecVlbiConfig), ctypes.c_char_p, sz]
    lib.gspec_vlbi_init.argtypes = [vp, ctypes.c_char_p, sz]
    lib.gspec_vlbi_process.argtypes = [vp, vp, sz, ctypes.POINTER(GspecOutput)]
    lib.gspec_vlbi_get_info.argtypes = [vp, ctypes.POINTER(GspecVlbiInfo)]
    lib.gspec_vlbi_last_error.restype = ctypes.c_char_p
    lib.gspec_vlbi_last_error.argtypes = [vp]
    lib.gspec_vlbi_destroy.restype = None
    lib.gspec_vlbi_destroy.argtypes = [vp]
    lib.gspec_vdif_set_time.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint64]
    return lib


class VLBI:
    """``VLBI<Handler>(buffer_bytes, input_bitDepth, speadHeapSize, sampleRate,
    digitizer_threshold, vdifHeader, handler)`` (``edd/VLBI.cuh:106-110``)."""

    def __init__(self, buffer_bytes: int, input_bitDepth: int, speadHeapSize: int, sampleRate: float,
                 digitizer_threshold: float, vdifHeader: VDIFHeader, handler, device: int = 0):
        self._lib = _lib()
        cfg = GspecVlbiConfig(buffer_size=buffer_bytes, nbits=input_bitDepth, device=device,
                              spead_heap_size=speadHeapSize, sample_rate=sampleRate,
                              digitizer_threshold=digitizer_threshold)
        for i in range(8):
            cfg.vdif_header[i] = int(vdifHeader.words[i])
        err = ctypes.create_string_buffer(512)
        h = self._lib.gspec_vlbi_create(ctypes.byref(cfg), err, len(err))
        if not h:
            raise GspecError(err.value.decode())
        self._h = ctypes.c_void_p(h)
        self._handler = handler
        self._out = GspecOutput()

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gspec_vlbi_destroy(self._h)
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

    def init(self, block: RawBytes):
        buf = (ctypes.c_char * block.total_bytes()).from_address(block.ptr())
        rc = self._lib.gspec_vlbi_init(self._h, buf, block.total_bytes())
        if rc < 0:
            raise GspecError(self._lib.gspec_vlbi_last_error(self._h).decode())
        # no time reference (GSPEC_STOP): a warning in the reference, the header goes on unchanged
        arr = block.numpy() if not block.on_device() else None
        if arr is not None and (arr == 0).any():
            block.used_bytes(max(block.used_bytes(), int(np.argmax(arr == 0))))
        self._handler.init(block)

    def __call__(self, block: RawBytes) -> bool:
        rc = self._lib.gspec_vlbi_process(self._h, ctypes.c_void_p(block.ptr()), block.used_bytes(),
                                          ctypes.byref(self._out))
        if rc == GSPEC_STOP:
            return True
        if rc < 0:
            raise GspecError(self._lib.gspec_vlbi_last_error(self._h).decode())
        if self._out.ready:
            n = self._out.size
            view = np.ctypeslib.as_array((ctypes.c_uint8 * n).from_address(self._out.data))
            self._handler(RawBytes(view, n, n))
        return False

    def info(self) -> GspecVlbiInfo:
        info = GspecVlbiInfo()
        if self._lib.gspec_vlbi_get_info(self._h, ctypes.byref(info)) != GSPEC_OK:
            raise GspecError("gspec_vlbi_get_info failed")
        return info
