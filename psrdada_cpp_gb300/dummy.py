"""Synthetic DADA block producer on the GPU (``gspec_dummy_block*`` of
include/gspec.h), replacing psrdada_cpp's ``dummy_data_generator``
(``psrdada_cpp/effelsberg/edd/src/dummy_data_generator.cu``).

:func:`dummy_data_generator` is that program's loop: a fixed DADA header,
then the same two-tone 8-bit block written ``nblocks`` times (0: forever)
with ``delay_ms`` between blocks, into any ring writer with the
``header_stream()`` / ``data_stream()`` interface (:class:`ring.MemoryRing`
writer, a psrdada write client) through :class:`ring.DadaOutputStream`.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from .gated_spectrometer import RawBytes, GspecError, GSPEC_OK, load_library
from . import ring

TWO_TONE, STREAM = 0, 1

# the header the reference program writes (dummy_data_generator.cu:120-124)
REFERENCE_HEADER = (b"HEADER       DADA\nHDR_VERSION  1.0\nHDR_SIZE     4096\nDADA_VERSION 1.0\n"
                    b"FILE_SIZE    2013265920\nNBIT           32\nNDIM         2\nNPOL         1\nNCHAN     4096\n"
                    b"RESOLUTION   1\nDSB 1\nSYNC_TIME    1234567890\nSAMPLE_CLOCK_START 175671842316288\n")


class DummyConfig(ctypes.Structure):
    _fields_ = [("buffer_size", ctypes.c_uint64), ("heap_size", ctypes.c_uint64),
                ("n_side_channels", ctypes.c_uint64), ("nbits", ctypes.c_uint32), ("dual_pol", ctypes.c_uint32),
                ("mode", ctypes.c_uint32), ("reserved", ctypes.c_uint32), ("block_index", ctypes.c_uint64),
                ("seed", ctypes.c_uint64), ("selected_side_channel", ctypes.c_uint64),
                ("selected_bit", ctypes.c_uint64), ("diode_period_heaps", ctypes.c_uint64),
                ("tone_period", ctypes.c_uint64), ("sigma", ctypes.c_float), ("tone_amplitude", ctypes.c_float),
                ("lost_fraction", ctypes.c_float), ("reserved2", ctypes.c_float)]


def _lib():
    lib = load_library()
    lib.gspec_dummy_block.argtypes = [ctypes.POINTER(DummyConfig), ctypes.c_void_p]
    lib.gspec_dummy_block_device.argtypes = [ctypes.POINTER(DummyConfig), ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p]
    return lib


def make_config(buffer_size: int, heap_size: int, n_side_channels: int, nbits: int = 8, mode: int = TWO_TONE,
                dual_pol: bool = False, **kw) -> DummyConfig:
    return DummyConfig(buffer_size=buffer_size, heap_size=heap_size, n_side_channels=n_side_channels, nbits=nbits,
                       dual_pol=1 if dual_pol else 0, mode=mode, **kw)


def block(cfg: DummyConfig) -> np.ndarray:
    """One block generated on the current GPU, in host memory."""
    out = np.zeros(cfg.buffer_size, np.uint8)
    rc = _lib().gspec_dummy_block(ctypes.byref(cfg), ctypes.c_void_p(out.ctypes.data))
    if rc != GSPEC_OK:
        raise GspecError(f"gspec_dummy_block failed ({rc})")
    return out


def block_device(cfg: DummyConfig, d_block: int, d_work: int, stream: int = 0) -> None:
    """One block generated into device memory (d_work: 8 bytes, two-tone mode)."""
    rc = _lib().gspec_dummy_block_device(ctypes.byref(cfg), ctypes.c_void_p(d_block), ctypes.c_void_p(d_work),
                                         ctypes.c_void_p(stream))
    if rc != GSPEC_OK:
        raise GspecError(f"gspec_dummy_block_device failed ({rc})")


def dummy_data_generator(writer, buffer_size: int, input_bit_depth: int = 8, delay_ms: float = 0.0,
                         nblocks: int = 0, speadheap_size: int = 4096, nsidechannelitems: int = 1) -> int:
    """The reference program's loop (``dummy_data_generator.cu:108-190``):
    header, then the two-tone block every ``delay_ms`` until ``nblocks``
    blocks are written (0: no limit).  Only 8-bit output, as the reference.
    Returns the number of blocks written."""
    if input_bit_depth != 8:
        raise ValueError("Currently only 8 bit supported")
    out = ring.DadaOutputStream(writer)
    hdr = np.zeros(4096, np.uint8)
    hdr[:len(REFERENCE_HEADER)] = np.frombuffer(REFERENCE_HEADER, np.uint8)
    out.init(RawBytes(hdr, 4096, 4096))
    data = block(make_config(buffer_size, speadheap_size, nsidechannelitems, 8, TWO_TONE))
    counter = 0
    while True:
        counter += 1
        out(RawBytes(data))
        if counter == nblocks:
            break
        if delay_ms:
            time.sleep(delay_ms / 1e3)
    return counter
