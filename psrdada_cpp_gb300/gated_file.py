"""Reader of the gated spectrometer's output file (the file a
``SimpleFileWriter`` handler writes: a 4096-byte DADA header with the
spectrometer's parameters appended, then the output blocks).

Follows ``tools/plot_gatedfiles.py:40-143`` of psrdada_cpp: the parameters
come from the header keys ``fft_length``, ``naccumulate``,
``output_bit_depth`` and ``full_stokes_output``; a power row is
``[G0 C][G1 C][nG0 u64][nG1 u64]`` and a Stokes row
``[I0][I1][Q0][Q1][U0][U1][V0][V1]`` spectra then ``[nG0, nG1] x 4`` u64
(``edd/src/GatedSpectrometer.cu:346-384,430-527``).  G0 is the noise diode
off (bit not set), G1 on.  Two defects of that script are not reproduced:
its power-mode counters are read at a fixed offset from the start of the
data instead of the row's, and nG1 from the same 8 bytes as nG0.

With ``records_per_block`` the file's blocks may carry this library's
saturation extension record (``n_out x [sat0, sat1]`` u64 after each block's
rows, ``GSPEC_FLAG_SATURATION_RECORD``).
"""
from __future__ import annotations

import dataclasses
import warnings

import numpy as np

HEADER_SIZE = 4096
KEYS = ("fft_length", "naccumulate", "output_bit_depth", "full_stokes_output", "nchannels",
        "selected_side_channel", "selected_bit")


def parse_header(header: bytes) -> dict:
    """``key value`` lines of a DADA header (text up to the first NUL;
    ``#`` starts a comment)."""
    text = header.split(b"\0", 1)[0].decode("ascii", errors="replace")
    out = {}
    for line in text.split("\n"):
        line = line.split("#")[0].strip()
        if not line:
            continue
        parts = line.split(None, 1)
        if len(parts) == 2:
            out[parts[0]] = parts[1].strip()
    return out


@dataclasses.dataclass
class GatedFile:
    header: dict
    fft_length: int
    nchans: int
    naccumulate: int
    bit_depth: int
    stokes: bool
    spectra: np.ndarray      # power: [rows, 2 (G0, G1), C]; Stokes: [rows, 4 (I, Q, U, V), 2 (G0, G1), C]
    n0: np.ndarray           # [rows] samples in gate 0 (diode off)
    n1: np.ndarray           # [rows] samples in gate 1 (diode on)
    saturation: np.ndarray | None = None   # [rows, 2] with records_per_block and a saturation record
    trailing_bytes: int = 0

    @property
    def rows(self) -> int:
        return self.spectra.shape[0]

    def stokes_product(self, name: str, gate: int) -> np.ndarray:
        """[rows, C] of product ``I``, ``Q``, ``U`` or ``V`` for gate 0/1."""
        if not self.stokes:
            raise ValueError("power-mode file")
        return self.spectra[:, "IQUV".index(name), gate]


def row_bytes(nchans: int, bit_depth: int, stokes: bool) -> int:
    """Bytes per output spectrum row (``tools/plot_gatedfiles.py:64-67``)."""
    return (8 if stokes else 2) * (nchans * bit_depth // 8 + 8)


def parse_rows(data: bytes, nchans: int, bit_depth: int, stokes: bool):
    """(spectra, n0, n1) of whole rows; Stokes rows must repeat their
    counter pair four times."""
    rb = row_bytes(nchans, bit_depth, stokes)
    nrows = len(data) // rb
    raw = np.frombuffer(data[:nrows * rb], np.uint8).reshape(nrows, rb)
    nspec = 8 if stokes else 2
    sbytes = nchans * bit_depth // 8
    dtype = "<f4" if bit_depth == 32 else np.int8
    spec = raw[:, :nspec * sbytes].copy().view(dtype).astype(np.float64).reshape(nrows, nspec, nchans)
    cnt = raw[:, nspec * sbytes:].copy().view("<u8")
    if stokes:
        spec = spec.reshape(nrows, 4, 2, nchans)
        if not (cnt == np.tile(cnt[:, :2], 4)).all():
            raise ValueError("Stokes row counters are not four copies of (nG0, nG1)")
    return spec, cnt[:, 0].copy(), cnt[:, 1].copy()


def read_gated_file(path: str, records_per_block: int | None = None, saturation_record: bool = False) -> GatedFile:
    """Reads a gated spectrometer output file.  ``records_per_block`` (the
    handle's n_out) is needed only to skip the saturation extension record of
    each block when ``saturation_record`` is set."""
    with open(path, "rb") as f:
        header = f.read(HEADER_SIZE)
        data = f.read()
    h = parse_header(header)
    for k in ("fft_length", "naccumulate", "output_bit_depth", "full_stokes_output"):
        if k not in h:
            raise ValueError(f"header has no {k}")
    fft = int(h["fft_length"])
    nchans = fft // 2 + 1
    bits = int(h["output_bit_depth"])
    if bits not in (8, 32):
        raise ValueError(f"unsupported output bit depth {bits}")
    stokes = h["full_stokes_output"].lower() == "yes"
    sat = None
    if saturation_record:
        if not records_per_block:
            raise ValueError("records_per_block is needed to skip the saturation record")
        rb = row_bytes(nchans, bits, stokes)
        blk = records_per_block * (rb + 16)
        nblk = len(data) // blk
        body, sats = [], []
        for b in range(nblk):
            chunk = data[b * blk:(b + 1) * blk]
            body.append(chunk[:records_per_block * rb])
            sats.append(np.frombuffer(chunk[records_per_block * rb:], "<u8").reshape(records_per_block, 2))
        trailing = len(data) - nblk * blk
        data = b"".join(body)
        sat = np.concatenate(sats) if sats else np.zeros((0, 2), np.uint64)
    else:
        trailing = len(data) % row_bytes(nchans, bits, stokes)
    if trailing:
        warnings.warn(f"{trailing} bytes remaining in datafile")
    spec, n0, n1 = parse_rows(data, nchans, bits, stokes)
    return GatedFile(h, fft, nchans, int(h["naccumulate"]), bits, stokes, spec, n0, n1, sat, trailing)
