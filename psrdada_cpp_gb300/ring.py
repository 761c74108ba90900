"""Ring-buffer sources and sinks around the gated spectrometer (Python mirror
of ``include/psrdada_cpp_gb300/ring.hpp``).

* :class:`MemoryRing` - an in-process ring of data blocks and a header block
  with psrdada's reader/writer protocol: the reader's ``header_stream()`` /
  ``data_stream()`` give ``next()`` / ``release()`` / ``at_end()`` as
  ``DadaReadClient::HeaderStream`` / ``DataStream``
  (``psrdada_cpp/src/dada_read_client.cpp:73-190``); the writer's give
  ``next()`` / ``release()`` and ``end_of_data()``.  With ``page_lock`` the
  ring is registered with CUDA (``gspec_register_host``), as
  ``dada_cuda_dbregister`` registers a psrdada ring's blocks on attach
  (``psrdada_cpp/src/dada_client_base.cpp:78-88``), so a block's host-to-device
  copy runs at the host link's full rate.
* :class:`FileReader` - the reader interface over a DADA file.
* :class:`DadaInputStream` - the handler loop of
  ``psrdada_cpp/detail/dada_input_stream.cpp:21-52`` over one reader.
* :class:`DadaOutputStream` - a handler copying its header and blocks into a
  ring writer (``psrdada_cpp/src/dada_output_stream.cpp:19-35``).
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from .gated_spectrometer import RawBytes, GSPEC_OK, GspecError, load_library


class _Stream:
    def __init__(self):
        self._cur = None

    def _take(self, rb):
        if self._cur is not None:
            raise RuntimeError(f"Previous {self._kind} block not released")
        self._cur = rb
        return rb

    def _drop(self):
        if self._cur is None:
            raise RuntimeError(f"No {self._kind} block to be released")
        rb, self._cur = self._cur, None
        return rb


class MemoryRing:
    """``nbufs`` data blocks of ``block_bytes`` and one header block."""

    def __init__(self, block_bytes: int, nbufs: int, header_bytes: int = 4096, page_lock: bool = False):
        if nbufs <= 0 or block_bytes <= 0:
            raise ValueError("MemoryRing: empty ring")
        self.block_bytes, self.nbufs, self.header_bytes = int(block_bytes), int(nbufs), int(header_bytes)
        stride = (self.block_bytes + 4095) // 4096 * 4096
        hstride = (self.header_bytes + 4095) // 4096 * 4096
        raw = np.zeros(hstride + stride * self.nbufs + 4096, np.uint8)
        off = (-raw.ctypes.data) % 4096                 # 4096-byte aligned blocks
        self._mem = raw[off:off + hstride + stride * self.nbufs]
        self._raw = raw
        self._header = self._mem[:self.header_bytes]
        self._blocks = [self._mem[hstride + i * stride:hstride + i * stride + self.block_bytes]
                        for i in range(self.nbufs)]
        self._used = [0] * self.nbufs
        self._cv = threading.Condition()
        self._wpos = self._rpos = self._nfull = self._written = 0
        self._eod = False
        self._header_full = False
        self._header_used = 0
        self.page_locked = False
        if page_lock:
            rc = load_library().gspec_register_host(ctypes.c_void_p(self._mem.ctypes.data), self._mem.nbytes)
            if rc != GSPEC_OK:
                raise GspecError("MemoryRing: page-locking the ring failed")
            self.page_locked = True

    def close(self):
        if self.page_locked:
            load_library().gspec_unregister_host(ctypes.c_void_p(self._mem.ctypes.data))
            self.page_locked = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def data_buffer_size(self):
        return self.block_bytes

    def header_buffer_size(self):
        return self.header_bytes

    @property
    def blocks_written(self):
        return self._written

    # ---------------------------------------------------------- writer
    class _HeaderWrite(_Stream):
        _kind = "header"

        def __init__(self, r):
            super().__init__()
            self._r = r

        def next(self):
            r = self._r
            with r._cv:
                r._cv.wait_for(lambda: not r._header_full)
                return self._take(RawBytes(r._header, r.header_bytes, 0))

        def release(self):
            r = self._r
            with r._cv:
                rb = self._drop()
                r._header_used = rb.used_bytes()
                r._header_full = True
                r._cv.notify_all()

    class _DataWrite(_Stream):
        _kind = "data"

        def __init__(self, r):
            super().__init__()
            self._r = r

        def next(self):
            r = self._r
            with r._cv:
                if r._eod:
                    raise RuntimeError("Data block requested after the end of data")
                r._cv.wait_for(lambda: r._nfull < r.nbufs)
                return self._take(RawBytes(r._blocks[r._wpos], r.block_bytes, 0))

        def release(self):
            r = self._r
            with r._cv:
                rb = self._drop()
                r._used[r._wpos] = rb.used_bytes()
                r._wpos = (r._wpos + 1) % r.nbufs
                r._nfull += 1
                r._written += 1
                r._cv.notify_all()

        def end_of_data(self):
            r = self._r
            with r._cv:
                r._eod = True
                r._cv.notify_all()

    class Writer:
        def __init__(self, ring):
            self._h = MemoryRing._HeaderWrite(ring)
            self._d = MemoryRing._DataWrite(ring)

        def header_stream(self):
            return self._h

        def data_stream(self):
            return self._d

    # ---------------------------------------------------------- reader
    class _HeaderRead(_Stream):
        _kind = "header"

        def __init__(self, r):
            super().__init__()
            self._r = r

        def next(self):
            r = self._r
            with r._cv:
                r._cv.wait_for(lambda: r._header_full)
                return self._take(RawBytes(r._header, r.header_bytes, r._header_used))

        def release(self):
            r = self._r
            with r._cv:
                self._drop()
                r._header_full = False
                r._cv.notify_all()

        def at_end(self):
            return False

    class _DataRead(_Stream):
        _kind = "data"

        def __init__(self, r):
            super().__init__()
            self._r = r

        def next(self):
            r = self._r
            with r._cv:
                r._cv.wait_for(lambda: r._nfull > 0 or r._eod)
                if r._nfull == 0:
                    raise RuntimeError("Could not open block to read: end of data")
                return self._take(RawBytes(r._blocks[r._rpos], r.block_bytes, r._used[r._rpos]))

        def release(self):
            r = self._r
            with r._cv:
                self._drop()
                r._rpos = (r._rpos + 1) % r.nbufs
                r._nfull -= 1
                r._cv.notify_all()

        def at_end(self):
            """Every block written before the end-of-data mark was read; waits
            while the writer has neither written more nor marked the end."""
            r = self._r
            with r._cv:
                r._cv.wait_for(lambda: r._nfull > 0 or r._eod)
                return r._eod and r._nfull == 0

    class Reader:
        def __init__(self, ring):
            self._ring = ring
            self._h = MemoryRing._HeaderRead(ring)
            self._d = MemoryRing._DataRead(ring)

        def header_stream(self):
            return self._h

        def data_stream(self):
            return self._d

        def data_buffer_size(self):
            return self._ring.block_bytes

    def writer(self):
        return MemoryRing.Writer(self)

    def reader(self):
        return MemoryRing.Reader(self)


class FileReader:
    """A DADA file (``header_bytes`` of header, then whole data blocks of
    ``block_bytes``) with the reader interface; a block is valid until
    ``release()``."""

    def __init__(self, path: str, block_bytes: int, header_bytes: int = 4096):
        self._f = open(path, "rb")
        self.block_bytes, self.header_bytes = int(block_bytes), int(header_bytes)
        self._size = os.path.getsize(path)
        self._buf = np.zeros(self.block_bytes, np.uint8)
        self._idx = 0
        reader = self

        class _H(_Stream):
            _kind = "header"

            def next(self):
                reader._f.seek(0)
                h = np.frombuffer(bytearray(reader._f.read(reader.header_bytes)), np.uint8)
                if h.size != reader.header_bytes:
                    raise RuntimeError("Could not get header")
                return self._take(RawBytes(h, reader.header_bytes, reader.header_bytes))

            def release(self):
                self._drop()

            def at_end(self):
                return False

        class _D(_Stream):
            _kind = "data"

            def next(self):
                if self.at_end():
                    raise RuntimeError("Could not open block to read: end of data")
                reader._f.seek(reader.header_bytes + reader._idx * reader.block_bytes)
                n = reader._f.readinto(memoryview(reader._buf))
                if n != reader.block_bytes:
                    raise RuntimeError("Could not read data block")
                return self._take(RawBytes(reader._buf, reader.block_bytes, reader.block_bytes))

            def release(self):
                self._drop()
                reader._idx += 1

            def at_end(self):
                return reader.header_bytes + (reader._idx + 1) * reader.block_bytes > reader._size

        self._h, self._d = _H(), _D()

    def header_stream(self):
        return self._h

    def data_stream(self):
        return self._d

    def data_buffer_size(self):
        return self.block_bytes

    def close(self):
        self._f.close()


class DadaInputStream:
    """``DadaInputStream<Handler>::start`` (``detail/dada_input_stream.cpp:21-52``)
    over one reader: the header block to ``handler.init``, then each data
    block to ``handler(...)`` until it returns True or the data ends.
    ``start()`` returns the number of data blocks handed out."""

    def __init__(self, reader, handler):
        self._reader, self._handler = reader, handler
        self._stop = False

    def start(self) -> int:
        hs = self._reader.header_stream()
        self._handler.init(hs.next())
        hs.release()
        ds = self._reader.data_stream()
        n, handler_stop = 0, False
        while not self._stop and not handler_stop:
            handler_stop = bool(self._handler(ds.next()))
            ds.release()
            n += 1
            if ds.at_end():
                break
        return n

    def stop(self):
        self._stop = True


class DadaOutputStream:
    """``DadaOutputStream`` (``psrdada_cpp/src/dada_output_stream.cpp:19-35``):
    copies the header and every block it is handed into a ring writer."""

    def __init__(self, writer):
        self._writer = writer

    def init(self, block: RawBytes):
        s = self._writer.header_stream()
        out = s.next()
        if block.used_bytes() > out.total_bytes():
            raise RuntimeError("header larger than the header block")
        _copy(out, block)
        s.release()

    def __call__(self, block: RawBytes) -> bool:
        s = self._writer.data_stream()
        out = s.next()
        if block.used_bytes() > out.total_bytes():
            raise RuntimeError("output larger than the ring's blocks")
        _copy(out, block)
        s.release()
        return False


def _copy(dst: RawBytes, src: RawBytes):
    n = src.used_bytes()
    ctypes.memmove(dst.ptr(), src.ptr(), n)
    dst.used_bytes(n)
