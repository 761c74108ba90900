"""CPU oracle of the EDD gated-spectrometer chain (FP64 numpy restatement).

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it.  The product path (the CUDA library behind
``include/gspec.h``) never calls into it.

Every function restates one step of psrdada_cpp's ``GatedSpectrometer`` and
cites the reference file:line it follows (paths relative to the psrdada_cpp
source tree; ``edd/`` abbreviates ``psrdada_cpp/effelsberg/edd/``).

Parity anchors (what pins this oracle):
  * unpack 8/10/12 bit  -> the reference's own C unpackers
    (``edd/test/src/UnpackerTester.cu:41-201``), compiled from the reference
    sources by ``oracle/build_ref.sh`` and compared in ``tests/test_oracle_pin.py``;
  * detect              -> ``edd/test/src/DetectorAccumulatorTester.cu:33-62``
    (same build);
  * Stokes IQUV         -> ``stokes_IQUV`` (``edd/src/GatedSpectrometer.cu:125-131``)
    compiled from the reference, plus the seven polarisation states of
    ``edd/test/src/GatedSpectrometerTest.cu:26-78``;
  * gating              -> the all-G0 / all-G1 known answers of
    ``edd/test/src/GatedSpectrometerTest.cu:142-240``;
  * R2C FFT             -> the DFT definition (cuFFT's unnormalised forward
    transform); no reference test pins FFT output, so the FFT stage is pinned
    only to the mathematics (numpy pocketfft in FP64).

Two gating conventions are implemented:
  * ``"intended"``  - the side-channel item of a sample is the item of the heap
    that holds the sample's first bit; dual-pol items are merged by bitwise OR;
    baselines divide each pol's sum by that pol's own count.
  * ``"reference"`` - the reference's literal index arithmetic where it stays in
    bounds: per output chunk ``j`` the item is
    ``j*step + (t // heapBytes)*nSC + sel`` (``edd/src/GatedSpectrometer.cu:46``,
    ``edd/detail/GatedSpectrometer.cu:239-247``), dual-pol items are merged by
    *logical* OR (``edd/src/GatedSpectrometer.cu:15``) and baseline denominators
    are the cumulative output counters (``edd/src/GatedSpectrometer.cu:105-115``
    called after each pol, ``edd/detail/GatedSpectrometer.cu:401-402``).
Deviations shared by both conventions (documented reference defects):
  * baseline sums are exact integers and the baseline is
    ``float32(sum / count)`` computed in FP64 (the reference sums float atomics
    in a nondeterministic order, ``edd/src/GatedSpectrometer.cu:79-88``);
  * a gate with zero samples gets baseline 0 (the reference divides by zero,
    ``edd/src/GatedSpectrometer.cu:114-115``);
  * power spectrum ``k`` of a block is accumulated into output slot ``k`` (the
    reference's detect kernel writes slot ``2k``, ``edd/DetectorAccumulator.cuh:57-59``,
    and overruns its buffer; ``data2Host`` reads slot ``k``,
    ``edd/src/GatedSpectrometer.cu:361,367``).
"""
from __future__ import annotations

import dataclasses
import numpy as np

HEADER_PARAM_FMT = (
    "\n"
    "# Gated spectrometer parameters: \n"
    "fft_length               {fft}\n"
    "nchannels                {nchans}\n"
    "naccumulate              {nacc}\n"
    "selected_side_channel    {sel}\n"
    "selected_bit             {bit}\n"
    "output_bit_depth         32\n"
    "full_stokes_output       {stokes}\n"
)


# --------------------------------------------------------------------------
# R4 / R4b: unpack
# --------------------------------------------------------------------------
def unpack(raw: np.ndarray, nbits: int) -> np.ndarray:
    """Big-endian packed two's-complement samples -> int32.

    The stream is a big-endian bit stream of ``nbits``-bit samples (MSB first),
    which is what the reference's word-wise code computes on 64-bit words after
    ``be64toh`` (``edd/test/src/UnpackerTester.cu:41-89`` 12 bit,
    ``:91-174`` 10 bit, ``:176-201`` 8 bit; GPU ``edd/src/Unpacker.cu:24-108``).
    """
    b = np.asarray(raw, dtype=np.uint8).astype(np.int32)
    if nbits == 8:
        return np.asarray(raw, dtype=np.uint8).view(np.int8).astype(np.int32)
    if nbits == 12:
        b = b.reshape(-1, 3)
        s0 = (b[:, 0] << 4) | (b[:, 1] >> 4)
        s1 = ((b[:, 1] & 0xF) << 8) | b[:, 2]
        s = np.stack([s0, s1], axis=1).reshape(-1)
        return s - ((s & 0x800) << 1)
    if nbits == 10:
        b = b.reshape(-1, 5)
        s0 = (b[:, 0] << 2) | (b[:, 1] >> 6)
        s1 = ((b[:, 1] & 0x3F) << 4) | (b[:, 2] >> 4)
        s2 = ((b[:, 2] & 0xF) << 6) | (b[:, 3] >> 2)
        s3 = ((b[:, 3] & 0x3) << 8) | b[:, 4]
        s = np.stack([s0, s1, s2, s3], axis=1).reshape(-1)
        return s - ((s & 0x200) << 1)
    raise ValueError(f"unsupported nbits {nbits}")


def pack(samples: np.ndarray, nbits: int) -> np.ndarray:
    """Inverse of :func:`unpack` (used by the synthetic-block generators)."""
    s = np.asarray(samples, dtype=np.int64) & ((1 << nbits) - 1)
    if nbits == 8:
        return s.astype(np.uint8)
    if nbits == 12:
        s = s.reshape(-1, 2)
        out = np.empty((s.shape[0], 3), dtype=np.uint8)
        out[:, 0] = s[:, 0] >> 4
        out[:, 1] = ((s[:, 0] & 0xF) << 4) | (s[:, 1] >> 8)
        out[:, 2] = s[:, 1] & 0xFF
        return out.reshape(-1)
    if nbits == 10:
        s = s.reshape(-1, 4)
        out = np.empty((s.shape[0], 5), dtype=np.uint8)
        out[:, 0] = s[:, 0] >> 2
        out[:, 1] = ((s[:, 0] & 0x3) << 6) | (s[:, 1] >> 4)
        out[:, 2] = ((s[:, 1] & 0xF) << 4) | (s[:, 2] >> 6)
        out[:, 3] = ((s[:, 2] & 0x3F) << 2) | (s[:, 3] >> 8)
        out[:, 4] = s[:, 3] & 0xFF
        return out.reshape(-1)
    raise ValueError(f"unsupported nbits {nbits}")


# --------------------------------------------------------------------------
# R1: block layout
# --------------------------------------------------------------------------
@dataclasses.dataclass(frozen=True)
class BufferLayout:
    """``DadaBufferLayout`` (``edd/src/DadaBufferLayout.cpp:17-39,41-80``)."""
    buffer_size: int
    heap_size: int
    n_side_channels: int

    @property
    def side_channel_size(self) -> int:
        return self.n_side_channels * 8

    @property
    def n_heaps(self) -> int:
        return self.buffer_size // (self.heap_size + self.side_channel_size)

    @property
    def gap(self) -> int:
        return self.buffer_size - self.n_heaps * (self.heap_size + self.side_channel_size)

    @property
    def data_bytes(self) -> int:
        return self.n_heaps * self.heap_size

    @property
    def side_channel_bytes(self) -> int:
        return self.side_channel_size * self.n_heaps

    @property
    def side_channel_offset(self) -> int:
        return self.data_bytes + self.gap


# --------------------------------------------------------------------------
# R11: configuration derived in the constructor
# --------------------------------------------------------------------------
@dataclasses.dataclass
class Config:
    layout: BufferLayout
    selected_side_channel: int
    selected_bit: int
    fft_length: int
    naccumulate: int
    nbits: int
    dual_pol: bool            # DualPolarizationInput + GatedFullStokesOutput
    convention: str = "intended"   # or "reference"

    def __post_init__(self):
        if self.nbits not in (8, 10, 12):
            raise ValueError("nbits must be 8, 10 or 12")
        if self.naccumulate <= 0 or self.fft_length <= 0:
            raise ValueError("fft_length and naccumulate must be positive")
        if self.selected_bit >= 64:
            raise ValueError("selected_bit must be < 64")
        if self.layout.n_side_channels and self.selected_side_channel >= self.layout.n_side_channels:
            raise ValueError("selected_side_channel out of range")
        if self.layout.n_side_channels == 0:
            raise ValueError("at least one side-channel item per heap is required")
        if self.convention not in ("intended", "reference"):
            raise ValueError("convention must be 'intended' or 'reference'")
        if self.dual_pol and self.layout.n_heaps % 2:
            raise ValueError("dual-pol blocks need an even number of heaps")
        n = self.nsamps_per_pol
        if (self.layout.data_bytes // (2 if self.dual_pol else 1) * 8) % self.nbits:
            raise ValueError("pol data is not a whole number of samples")
        per_out = self.fft_length * self.naccumulate
        # edd/detail/GatedSpectrometer.cu:114-130 (asserts there; errors here)
        if per_out <= n:
            if n % per_out:
                raise ValueError("samples per pol not a multiple of fft_length*naccumulate")
            self.n_blocks = 1
        else:
            if per_out % n:
                raise ValueError("fft_length*naccumulate not a multiple of samples per pol")
            self.n_blocks = per_out // n
            if self.naccumulate % self.n_blocks or n % self.fft_length:
                raise ValueError("block does not hold whole spectra")
        self.batch = n // self.fft_length
        self.nacc_per_block = self.naccumulate // self.n_blocks
        self.n_out = self.batch // self.nacc_per_block
        if self.convention == "reference":
            self._check_reference_indexing()

    # derived sizes --------------------------------------------------------
    @property
    def nchans(self) -> int:
        return self.fft_length // 2 + 1

    @property
    def nsamps_per_pol(self) -> int:
        # SinglePolarizationInput / DualPolarizationInput::getSamplesPerInputPolarization
        # (edd/src/GatedSpectrometer.cu:199-202,255-258)
        d = self.layout.data_bytes * 8 // self.nbits
        return d // 2 if self.dual_pol else d

    @property
    def items_per_pol(self) -> int:
        n = self.layout.n_heaps * self.layout.n_side_channels
        return n // 2 if self.dual_pol else n

    @property
    def output_bytes(self) -> int:
        # edd/src/GatedSpectrometer.cu:333 (power), :417 (Stokes)
        per = (8 if self.dual_pol else 2) * (self.nchans * 4 + 8)
        return per * self.n_out

    @property
    def chunk_len(self) -> int:
        return self.nsamps_per_pol // self.n_out

    @property
    def step(self) -> int:
        # edd/detail/GatedSpectrometer.cu:239
        return self.items_per_pol // self.n_out

    def _check_reference_indexing(self):
        """The literal gating index is only defined where chunks tile the
        block and every index stays inside the item array."""
        L, step = self.chunk_len, self.step
        if step * 4096 != L:
            raise ValueError("reference gating: chunk offset step*4096 does not tile the block")
        last = (self.n_out - 1) * step + ((L - 1) // self.layout.heap_size) * \
            self.layout.n_side_channels + self.selected_side_channel
        if last >= self.items_per_pol:
            raise ValueError("reference gating: side-channel index runs past the item array")


# --------------------------------------------------------------------------
# R2 / R3: split a block into per-pol raw streams and items
# --------------------------------------------------------------------------
def split_block(block: np.ndarray, cfg: Config):
    """Single: ``edd/src/GatedSpectrometer.cu:212-230``; dual (heaps P0P1P0P1,
    items de-interleaved item-wise with pitch 16 B): ``:261-306``."""
    L = cfg.layout
    block = np.asarray(block, dtype=np.uint8)
    data = block[:L.data_bytes]
    items = block[L.side_channel_offset:L.side_channel_offset + L.side_channel_bytes].view("<u8")
    if not cfg.dual_pol:
        return [data], [items.copy()]
    H = L.heap_size
    nrows = L.data_bytes // H // 2
    heaps = data[:nrows * 2 * H].reshape(nrows, 2, H)
    nitems = L.side_channel_bytes // 2 // 8
    raws = [heaps[:, 0, :].reshape(-1).copy(), heaps[:, 1, :].reshape(-1).copy()]
    its = [items[0::2][:nitems].copy(), items[1::2][:nitems].copy()]
    return raws, its


def merge_side_channels(a: np.ndarray, b: np.ndarray, convention: str):
    """``mergeSideChannels`` (``edd/src/GatedSpectrometer.cu:9-19``): the
    reference's ``A || B`` is a logical OR (0/1); the intended merge, "if one
    item is lost both are lost" (``edd/detail/GatedSpectrometer.cu:36-37``), is
    a bitwise OR."""
    if convention == "reference":
        v = ((a != 0) | (b != 0)).astype(np.uint64)
    else:
        v = a | b
    return v, v.copy()


# --------------------------------------------------------------------------
# R5: gate assignment
# --------------------------------------------------------------------------
def sample_item_index(cfg: Config) -> np.ndarray:
    """Side-channel item index for every sample of one pol."""
    n = cfg.nsamps_per_pol
    s = np.arange(n, dtype=np.int64)
    nsc, sel = cfg.layout.n_side_channels, cfg.selected_side_channel
    if cfg.convention == "reference":
        # edd/src/GatedSpectrometer.cu:46-47 with the per-chunk offsets of
        # edd/detail/GatedSpectrometer.cu:243-246 (heapSize in BYTES)
        L = cfg.chunk_len
        j, t = s // L, s % L
        return j * cfg.step + (t // cfg.layout.heap_size) * nsc + sel
    heap = (s * cfg.nbits) // (8 * cfg.layout.heap_size)
    return heap * nsc + sel


def gate(v: np.ndarray, items: np.ndarray, bitpos: int, b0: np.float32, b1: np.float32):
    """``gating`` (``edd/src/GatedSpectrometer.cu:22-59``) per sample.

    Returns float32 G0/G1 with the reference's exact float formula
    ``(v - b) * m + b`` and the 0/1 masks m0 (gate 0: bit clear, heap not lost)
    and m1 (gate 1: bit set, heap not lost)."""
    items = np.asarray(items, dtype=np.uint64)
    bit = ((items >> np.uint64(bitpos)) & np.uint64(1)).astype(bool)
    lost = (items >> np.uint64(63)).astype(bool)
    m1 = bit & ~lost
    m0 = ~bit & ~lost
    vf = v.astype(np.float32)
    b0 = np.float32(b0)
    b1 = np.float32(b1)
    g1 = np.where(m1, (vf - b1) + b1, b1).astype(np.float32)
    g0 = np.where(m0, (vf - b0) + b0, b0).astype(np.float32)
    return g0, g1, m0, m1


def baseline(total: int, count: int) -> np.float32:
    """``update_baselines`` (``edd/src/GatedSpectrometer.cu:98-118``) with an
    exact integer sum, an FP64 division and a zero-count guard."""
    if count == 0:
        return np.float32(0.0)
    return np.float32(np.float64(total) / np.float64(count))


# --------------------------------------------------------------------------
# R9 / R10: detect and Stokes
# --------------------------------------------------------------------------
def stokes_iquv(p1: np.ndarray, p2: np.ndarray):
    """``stokes_IQUV`` (``edd/src/GatedSpectrometer.cu:125-131``)."""
    a1 = p1.real ** 2 + p1.imag ** 2
    a2 = p2.real ** 2 + p2.imag ** 2
    I = a1 + a2
    Q = a1 - a2
    U = 2.0 * (p1.real * p2.real + p1.imag * p2.imag)
    V = -2.0 * (p1.imag * p2.real - p1.real * p2.imag)
    return I, Q, U, V


def rfft64(frames_f32: np.ndarray) -> np.ndarray:
    """cuFFT R2C (unnormalised forward, ``edd/detail/GatedSpectrometer.cu:144-145,281-288``)
    evaluated in FP64."""
    return np.fft.rfft(frames_f32.astype(np.float64), axis=-1)


# --------------------------------------------------------------------------
# One block through the chain
# --------------------------------------------------------------------------
@dataclasses.dataclass
class PolState:
    b0: np.float32 = np.float32(0.0)
    b1: np.float32 = np.float32(0.0)


@dataclasses.dataclass
class BlockResult:
    """Per-block contribution to an output buffer."""
    spectra: np.ndarray        # power: [n_out, 2, C]; stokes: [n_out, 4, 2, C] (I,Q,U,V x G0,G1)
    n0: np.ndarray             # [n_out] uint64
    n1: np.ndarray
    sat0: np.ndarray           # [n_out] saturation counts (extension record)
    sat1: np.ndarray
    gated: list                # per pol (g0, g1) float32 (for bit-exact checks)
    pol_counts: list           # per pol (c0, c1) this block
    pol_sums: list             # per pol (s0, s1) exact integer sums


def process_block(block: np.ndarray, cfg: Config, states: list, period_counts=(0, 0),
                  keep_gated: bool = False) -> BlockResult:
    """``process`` for one block (``edd/detail/GatedSpectrometer.cu:369-441``).

    ``states`` holds the per-pol baselines and is updated in place exactly as
    ``update_baselines`` runs after each pol's ``gated_fft``.
    ``period_counts`` are the G0/G1 counter totals already in the output buffer
    (non-zero only when several input blocks integrate into one output); they
    enter the baseline denominators in the ``reference`` convention."""
    raws, items = split_block(block, cfg)
    if cfg.dual_pol:
        items = list(merge_side_channels(items[0], items[1], cfg.convention))
    idx = sample_item_index(cfg)
    N, C, n_out, nacc = cfg.fft_length, cfg.nchans, cfg.n_out, cfg.nacc_per_block
    L = cfg.chunk_len
    lo, hi = -(1 << (cfg.nbits - 1)), (1 << (cfg.nbits - 1)) - 1
    n0 = np.zeros(n_out, np.uint64)
    n1 = np.zeros(n_out, np.uint64)
    sat0 = np.zeros(n_out, np.uint64)
    sat1 = np.zeros(n_out, np.uint64)
    spectra_pol = []
    gated = []
    pol_counts, pol_sums = [], []
    cum0, cum1 = period_counts
    for p, (raw, it) in enumerate(zip(raws, items)):
        v = unpack(raw, cfg.nbits)[:cfg.nsamps_per_pol]
        st = states[p]
        g0, g1, m0, m1 = gate(v, it[idx], cfg.selected_bit, st.b0, st.b1)
        c0 = m0.reshape(n_out, L).sum(axis=1).astype(np.uint64)
        c1 = m1.reshape(n_out, L).sum(axis=1).astype(np.uint64)
        sat = (v == lo) | (v == hi)
        sat0 += (sat & m0).reshape(n_out, L).sum(axis=1).astype(np.uint64)
        sat1 += (sat & m1).reshape(n_out, L).sum(axis=1).astype(np.uint64)
        n0 += c0
        n1 += c1
        s0 = int(np.sum(v.astype(np.int64) * m0))
        s1 = int(np.sum(v.astype(np.int64) * m1))
        tc0, tc1 = int(c0.sum()), int(c1.sum())
        pol_counts.append((tc0, tc1))
        pol_sums.append((s0, s1))
        # baseline update for the next block (edd/detail/GatedSpectrometer.cu:263-271)
        if cfg.convention == "reference":
            cum0 += tc0
            cum1 += tc1
            st.b0, st.b1 = baseline(s0, cum0), baseline(s1, cum1)
        else:
            st.b0, st.b1 = baseline(s0, tc0), baseline(s1, tc1)
        X0 = rfft64(g0.reshape(-1, N))       # [batch, C]
        X1 = rfft64(g1.reshape(-1, N))
        spectra_pol.append((X0, X1))
        if keep_gated:
            gated.append((g0, g1))
    if not cfg.dual_pol:
        X0, X1 = spectra_pol[0]
        P0 = (np.abs(X0) ** 2).reshape(n_out, nacc, C).sum(axis=1)
        P1 = (np.abs(X1) ** 2).reshape(n_out, nacc, C).sum(axis=1)
        spectra = np.stack([P0, P1], axis=1)
    else:
        out = np.zeros((n_out, 4, 2, C))
        for g in range(2):
            I, Q, U, V = stokes_iquv(spectra_pol[0][g], spectra_pol[1][g])
            for si, S in enumerate((I, Q, U, V)):
                out[:, si, g, :] = S.reshape(n_out, nacc, C).sum(axis=1)
        spectra = out
    return BlockResult(spectra, n0, n1, sat0, sat1, gated, pol_counts, pol_sums)


def _item_index_range(cfg: Config, s0: int, s1: int) -> np.ndarray:
    """:func:`sample_item_index` for pol samples ``[s0, s1)`` only."""
    s = np.arange(s0, s1, dtype=np.int64)
    nsc, sel = cfg.layout.n_side_channels, cfg.selected_side_channel
    if cfg.convention == "reference":
        L = cfg.chunk_len
        j, t = s // L, s % L
        return j * cfg.step + (t // cfg.layout.heap_size) * nsc + sel
    return ((s * cfg.nbits) // (8 * cfg.layout.heap_size)) * nsc + sel


def process_block_chunked(block: np.ndarray, cfg: Config, states: list, period_counts=(0, 0),
                          outputs_per_chunk: int = 1) -> BlockResult:
    """:func:`process_block` evaluated ``outputs_per_chunk`` output spectra
    at a time, so that a full-size block (2^28 samples per pol) fits in a
    few GB of host memory.  Same arithmetic, same FP64 FFT, same baseline
    update (after both pols, ``edd/detail/GatedSpectrometer.cu:263-271``):
    every quantity of the chain is a sum over samples of one output spectrum
    or an exact integer sum over the block, so the chunking changes no
    value."""
    raws, items = split_block(block, cfg)
    if cfg.dual_pol:
        items = list(merge_side_channels(items[0], items[1], cfg.convention))
    N, C, n_out, nacc = cfg.fft_length, cfg.nchans, cfg.n_out, cfg.nacc_per_block
    L = cfg.chunk_len
    lo, hi = -(1 << (cfg.nbits - 1)), (1 << (cfg.nbits - 1)) - 1
    npol = len(raws)
    n0 = np.zeros(n_out, np.uint64)
    n1 = np.zeros(n_out, np.uint64)
    sat0 = np.zeros(n_out, np.uint64)
    sat1 = np.zeros(n_out, np.uint64)
    spectra = np.zeros((n_out, 4, 2, C)) if cfg.dual_pol else np.zeros((n_out, 2, C))
    tot = [[0, 0] for _ in range(npol)]
    sums = [[0, 0] for _ in range(npol)]
    b = [(np.float32(st.b0), np.float32(st.b1)) for st in states]
    for k0 in range(0, n_out, outputs_per_chunk):
        k1 = min(n_out, k0 + outputs_per_chunk)
        s0, s1 = k0 * L, k1 * L
        idx = _item_index_range(cfg, s0, s1)
        X = []
        for p in range(npol):
            raw = raws[p][s0 * cfg.nbits // 8:s1 * cfg.nbits // 8]
            v = unpack(raw, cfg.nbits)
            g0, g1, m0, m1 = gate(v, items[p][idx], cfg.selected_bit, b[p][0], b[p][1])
            c0 = m0.reshape(k1 - k0, L).sum(axis=1).astype(np.uint64)
            c1 = m1.reshape(k1 - k0, L).sum(axis=1).astype(np.uint64)
            sat = (v == lo) | (v == hi)
            sat0[k0:k1] += (sat & m0).reshape(k1 - k0, L).sum(axis=1).astype(np.uint64)
            sat1[k0:k1] += (sat & m1).reshape(k1 - k0, L).sum(axis=1).astype(np.uint64)
            n0[k0:k1] += c0
            n1[k0:k1] += c1
            tot[p][0] += int(c0.sum())
            tot[p][1] += int(c1.sum())
            sums[p][0] += int(np.sum(v.astype(np.int64) * m0))
            sums[p][1] += int(np.sum(v.astype(np.int64) * m1))
            X.append((rfft64(g0.reshape(-1, N)), rfft64(g1.reshape(-1, N))))
        if not cfg.dual_pol:
            for g in range(2):
                spectra[k0:k1, g] = (np.abs(X[0][g]) ** 2).reshape(k1 - k0, nacc, C).sum(axis=1)
        else:
            for g in range(2):
                for si, S in enumerate(stokes_iquv(X[0][g], X[1][g])):
                    spectra[k0:k1, si, g] = S.reshape(k1 - k0, nacc, C).sum(axis=1)
    cum0, cum1 = period_counts
    for p in range(npol):
        st = states[p]
        if cfg.convention == "reference":
            cum0 += tot[p][0]
            cum1 += tot[p][1]
            st.b0, st.b1 = baseline(sums[p][0], cum0), baseline(sums[p][1], cum1)
        else:
            st.b0, st.b1 = baseline(sums[p][0], tot[p][0]), baseline(sums[p][1], tot[p][1])
    return BlockResult(spectra, n0, n1, sat0, sat1, [], [tuple(t) for t in tot], [tuple(s) for s in sums])


# --------------------------------------------------------------------------
# The ungated FftSpectrometer (edd/detail/FftSpectrometer.cu:13-179)
# --------------------------------------------------------------------------
def fft_spectrometer_block(block: np.ndarray, nbits: int, fft_length: int, naccumulate: int) -> np.ndarray:
    """One block of ``FftSpectrometer::process``: unpack the whole block
    (``edd/detail/FftSpectrometer.cu:93-99``), R2C every ``fft_length``
    samples (``:101-107``) and sum ``|X|^2`` over groups of ``naccumulate``
    frames (``detect_and_accumulate<float>``, ``edd/DetectorAccumulator.cuh:40-61``).
    The intended frame count (all frames of the block) and a fresh sum per
    block are used; the reference's in-place stride overlap, frame-count
    rounding and never-cleared output buffers are defects.  Returns
    [n_out, fft_length/2 + 1] power spectra in FP64."""
    v = unpack(np.asarray(block, np.uint8), nbits)
    n = v.size // fft_length
    if n % naccumulate:
        raise ValueError("frames per block not a multiple of naccumulate")
    X = rfft64(v[:n * fft_length].astype(np.float32).reshape(n, fft_length))
    C = fft_length // 2 + 1
    return (np.abs(X) ** 2).reshape(n // naccumulate, naccumulate, C).sum(axis=1)


# --------------------------------------------------------------------------
# Synthetic producer (edd/src/dummy_data_generator.cu)
# --------------------------------------------------------------------------
def dummy_two_tone_block(n: int) -> np.ndarray:
    """The reference generator's data: the C2R (unnormalised) of 50 at bin
    nFreqs/3 and 20 at bin nFreqs/2, nFreqs = n/2 + 1
    (``dummy_data_generator.cu:130-137``), as float32; quantised between its
    own minimum and maximum to 0..255 by ``packNbit<8>``
    (``edd/Packer.cuh:32-41``: (x - min) / level, level = (max - min) / 255,
    clamped, truncated) and shifted by -128 (``:150-156``).  int8 samples."""
    t = np.arange(n, dtype=np.int64)
    nf = n // 2 + 1
    x = np.zeros(n)
    for k, amp in ((nf // 3, 50.0), (nf // 2, 20.0)):
        w = amp if (k == 0 or 2 * k == n) else 2.0 * amp
        x += w * np.cos(2.0 * np.pi * ((k * t) % n) / n)
    x = x.astype(np.float32)
    lo, hi = x.min(), x.max()
    level = np.float32((hi - lo) / np.float32(255.0))
    v = np.clip((x - lo) / level, np.float32(0), np.float32(255)).astype(np.uint32)
    return (v.astype(np.int32) - 128).astype(np.int8)


def _mix64(z):
    z = (z + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def dummy_stream_samples(seed: int, pol: int, s0: int, n: int, sigma: float, tone_amplitude: float,
                         tone_period: int, nbits: int) -> np.ndarray:
    """Samples s0 .. s0+n-1 of one pol of the device generator's stream mode:
    the centred sum of twelve 16-bit uniforms of a splitmix64 counter hash
    times sigma / 65536, plus tone_amplitude cos(2 pi (s mod tone_period) /
    tone_period), rounded half to even and clipped to nbits."""
    with np.errstate(over="ignore"):
        s = np.arange(s0, s0 + n, dtype=np.uint64)
        key = _mix64(np.uint64(seed) ^ np.uint64(0x51ED27 * (pol + 1))) ^ s
        tot = np.zeros(n, np.int64)
        for j in range(3):
            h = _mix64(key * np.uint64(3) + np.uint64(j))
            for i in range(4):
                tot += ((h >> np.uint64(16 * i)) & np.uint64(0xFFFF)).astype(np.int64)
    noise = (tot - 393210).astype(np.float64) * float(np.float32(sigma)) / 65536.0
    tone = 0.0
    if tone_period > 0 and tone_amplitude != 0:
        tone = float(np.float32(tone_amplitude)) * np.cos(2.0 * np.pi * (s.astype(np.int64) % tone_period) / tone_period)
    lo, hi = -(1 << (nbits - 1)), (1 << (nbits - 1)) - 1
    return np.clip(np.rint(noise + tone), lo, hi).astype(np.int64)


# --------------------------------------------------------------------------
# VLBI: 2-bit VDIF (edd/detail/VLBI.cu, edd/src/VLBI.cu)
# --------------------------------------------------------------------------
def vdif_time_fields(posix_seconds: int):
    """(reference epoch, seconds since the epoch) of a POSIX time: epochs are
    half-years since 2000-01-01 UTC (``VDIFHeader::setTimeReferencesFromTimestamp``,
    ``edd/src/VLBI.cu:143-170``)."""
    import datetime
    t = datetime.datetime.fromtimestamp(posix_seconds, tz=datetime.timezone.utc)
    half = 1 if t.month >= 7 else 0
    start = datetime.datetime(t.year, 7 if half else 1, 1, tzinfo=datetime.timezone.utc)
    return (t.year - 2000) * 2 + half, int((t - start).total_seconds())


def vlbi_pack2bit(samples: np.ndarray, v: float) -> np.ndarray:
    """``pack2bit_nonLinear`` (``edd/src/VLBI.cu:183-237``) with the block
    statistics of ``edd/detail/VLBI.cu:216-237`` (mean, then the mean square
    residual): level = (x - mean >= -v sigma) + (x - mean >= 0) +
    (x - mean >= v sigma), four samples per byte, sample j in bits 2j..2j+1.
    The sums are exact integers here (the reference adds floats in a
    nondeterministic order); mean and sigma^2 in FP64, rounded to float."""
    x = np.asarray(samples, np.int64)
    n = x.size
    mean_d = float(x.sum()) / n
    var = float((x * x).sum()) / n - mean_d * mean_d
    mean = np.float32(mean_d)
    vsig = np.float32(np.float32(v) * np.sqrt(np.float32(max(var, 0.0))))
    inp = x.astype(np.float32) - mean
    lev = ((inp >= -vsig).astype(np.uint8) + (inp >= 0).astype(np.uint8) + (inp >= vsig).astype(np.uint8))
    lev = lev.reshape(-1, 4)
    return (lev[:, 0] | (lev[:, 1] << 2) | (lev[:, 2] << 4) | (lev[:, 3] << 6)).astype(np.uint8)


class OracleVLBI:
    """``VLBI<Handler>`` (``edd/detail/VLBI.cu:22-354``) on the CPU: block n's
    frames are handed out at call n + 3; the 2-bit stream of a block is
    [spill of the previous block | the block's bytes after the first-second
    skip]; every output holds ``frames_per_output`` frames, those without
    data invalid (the reference marks the validity one frame late, a defect
    not reproduced)."""

    def __init__(self, buffer_size, nbits, sample_rate, v, header_words):
        self.buffer_size, self.nbits, self.rate, self.v = buffer_size, nbits, sample_rate, v
        self.hdr = [int(w) & 0xFFFFFFFF for w in header_words]
        self.hdr[3] = (self.hdr[3] & ~(0x1F << 26)) | (1 << 26)
        self.hdr[3] &= ~(1 << 31)
        self.frame_bytes = (self.hdr[2] & 0xFFFFFF) * 8
        self.payload = self.frame_bytes - 32
        self.nsamples = buffer_size * 8 // nbits
        self.packed = self.nsamples // 4
        self.nframes = self.packed // self.payload + 1
        self.fps = int(sample_rate / (self.payload * 4))
        self.skip = 0
        self.spill = b""
        self.pending = []        # outputs awaiting hand-out
        self.calls = 0
        self.last = None

    def init(self, sync_time, sample_clock_start):
        frac = sync_time + sample_clock_start / self.rate
        ts = int(frac) + 1
        self.skip = int((ts - frac) * self.rate) * 2 // 8
        ep, sec = vdif_time_fields(ts)
        self.hdr[1] = (self.hdr[1] & ~(0x3F << 24)) | (ep << 24)
        self.hdr[0] = (self.hdr[0] & ~0x3FFFFFFF) | sec

    def _frames(self, block):
        packed = vlbi_pack2bit(unpack(np.asarray(block, np.uint8), self.nbits), self.v).tobytes()
        stream = self.spill + packed[self.skip:]
        self.skip = 0
        nvalid = len(stream) // self.payload
        out = bytearray(self.nframes * self.frame_bytes)
        num0, sec0 = self.hdr[1] & 0xFFFFFF, self.hdr[0] & 0x3FFFFFFF
        for f in range(self.nframes):
            num = num0 + f
            w = list(self.hdr)
            w[0] = (w[0] & ~0x3FFFFFFF) | ((sec0 + num // self.fps) & 0x3FFFFFFF)
            w[0] = (w[0] & ~(1 << 31)) | ((0 if f < nvalid else 1) << 31)
            w[1] = (w[1] & ~0xFFFFFF) | (num % self.fps)
            o = f * self.frame_bytes
            out[o:o + 32] = np.array(w, "<u4").tobytes()
            if f < nvalid:
                out[o + 32:o + self.frame_bytes] = stream[f * self.payload:(f + 1) * self.payload]
        self.spill = stream[nvalid * self.payload:]
        num = num0 + nvalid
        self.hdr[1] = (self.hdr[1] & ~0xFFFFFF) | (num % self.fps)
        self.hdr[0] = (self.hdr[0] & ~0x3FFFFFFF) | ((sec0 + num // self.fps) & 0x3FFFFFFF)
        return bytes(out)

    def __call__(self, block):
        """(stop, frames handed out or None)."""
        if self.skip > self.packed:
            self.skip -= self.packed
            return False, None
        if len(block) != self.buffer_size:
            return True, None
        self.calls += 1
        self.pending.append(self._frames(block))
        # handed out three calls after the block arrived
        if self.calls >= 4:
            return False, self.pending.pop(0)
        return False, None


# --------------------------------------------------------------------------
# R13 / R14: output block layout
# --------------------------------------------------------------------------
def output_bytes(spectra: np.ndarray, n0: np.ndarray, n1: np.ndarray, dual_pol: bool) -> bytes:
    """Power: per spectrum ``[G0 f32*C][G1 f32*C][nG0 u64][nG1 u64]``
    (``edd/src/GatedSpectrometer.cu:346-384``).  Stokes: per spectrum
    ``[I0][I1][Q0][Q1][U0][U1][V0][V1]`` f32*C then ``[nG0,nG1]*4`` u64
    (``:430-527``)."""
    n_out = spectra.shape[0]
    parts = []
    for k in range(n_out):
        if not dual_pol:
            parts.append(spectra[k].astype("<f4").tobytes())
            parts.append(np.array([n0[k], n1[k]], "<u8").tobytes())
        else:
            parts.append(spectra[k].astype("<f4").tobytes())   # [4][2][C]
            parts.append(np.array([n0[k], n1[k]] * 4, "<u8").tobytes())
    return b"".join(parts)


def parse_output(buf: bytes, cfg: Config):
    """Inverse of :func:`output_bytes` -> (spectra float32, n0, n1)."""
    C, n_out = cfg.nchans, cfg.n_out
    a = np.frombuffer(buf, dtype=np.uint8)
    if not cfg.dual_pol:
        rec = 2 * C * 4 + 16
        a = a[:rec * n_out].reshape(n_out, rec)
        spec = a[:, :2 * C * 4].copy().view("<f4").reshape(n_out, 2, C)
        cnt = a[:, 2 * C * 4:].copy().view("<u8").reshape(n_out, 2)
        return spec, cnt[:, 0], cnt[:, 1]
    rec = 8 * C * 4 + 64
    a = a[:rec * n_out].reshape(n_out, rec)
    spec = a[:, :8 * C * 4].copy().view("<f4").reshape(n_out, 4, 2, C)
    cnt = a[:, 8 * C * 4:].copy().view("<u8").reshape(n_out, 8)
    return spec, cnt[:, 0], cnt[:, 1]


# --------------------------------------------------------------------------
# R12 / R15: the handler (init + operator()) state machine
# --------------------------------------------------------------------------
def header_append(header: bytearray, cfg: Config) -> bool:
    """``init`` header append (``edd/detail/GatedSpectrometer.cu:179-215``)."""
    text = HEADER_PARAM_FMT.format(
        fft=cfg.fft_length, nchans=cfg.nchans, nacc=cfg.naccumulate,
        sel=cfg.selected_side_channel, bit=cfg.selected_bit,
        stokes="yes" if cfg.dual_pol else "no").encode()
    end = header.find(b"\0")
    if end < 0:
        end = len(header)
    if end + len(text) < len(header):
        header[end:end + len(text) + 1] = text + b"\0"
        return True
    return False


class OracleSpectrometer:
    """``GatedSpectrometer::operator()`` (``edd/detail/GatedSpectrometer.cu:299-365``).

    Mirrors the double buffers: block n is copied at call n, processed at call
    n+1, copied to the host at the next output swap and handed to the handler
    one swap later.  ``__call__`` returns ``(stop, payload_or_None)``."""

    def __init__(self, cfg: Config, keep_results: bool = False):
        self.cfg = cfg
        self.call_count = 0
        self.states = [PolState() for _ in range(2 if cfg.dual_pol else 1)]
        self.in_a = None
        self.in_b = None
        shape = (cfg.n_out, 4, 2, cfg.nchans) if cfg.dual_pol else (cfg.n_out, 2, cfg.nchans)
        self._shape = shape
        self.out_a = self._zero_out()
        self.out_b = self._zero_out()
        self.host_a = None
        self.host_b = None
        self.keep_results = keep_results
        self.results = []

    def _zero_out(self):
        c = self.cfg
        return {"spec": np.zeros(self._shape), "n0": np.zeros(c.n_out, np.uint64),
                "n1": np.zeros(c.n_out, np.uint64), "sat0": np.zeros(c.n_out, np.uint64),
                "sat1": np.zeros(c.n_out, np.uint64)}

    def _process(self, block):
        o = self.out_a
        r = process_block(block, self.cfg, self.states,
                          period_counts=(int(o["n0"].sum()), int(o["n1"].sum())))
        o["spec"] = o["spec"] + r.spectra
        o["n0"] = o["n0"] + r.n0
        o["n1"] = o["n1"] + r.n1
        o["sat0"] = o["sat0"] + r.sat0
        o["sat1"] = o["sat1"] + r.sat1
        if self.keep_results:
            self.results.append(r)

    def __call__(self, block):
        cfg = self.cfg
        self.call_count += 1
        block = np.asarray(block, dtype=np.uint8)
        if block.size != cfg.layout.buffer_size:
            return True, None
        self.in_a, self.in_b = block.copy(), self.in_a
        if self.call_count == 1:
            return False, None
        new_block = ((self.call_count - 1) % cfg.n_blocks) == 0
        if new_block:
            self.out_a, self.out_b = self.out_b, self.out_a
            self.out_a = self._zero_out()
            self.host_a, self.host_b = self.host_b, self.host_a
        self._process(self.in_b)
        if self.call_count == 2 or not new_block:
            return False, None
        ob = self.out_b
        self.host_a = {"bytes": output_bytes(ob["spec"], ob["n0"], ob["n1"], cfg.dual_pol),
                       "spec": ob["spec"].copy(), "n0": ob["n0"].copy(), "n1": ob["n1"].copy(),
                       "sat0": ob["sat0"].copy(), "sat1": ob["sat1"].copy()}
        if self.call_count == 3:
            return False, None
        # the reference hands out a never-written pinned buffer here when
        # n_blocks >= 3 (first output swap at call n_blocks + 1); skipped
        return False, self.host_b


# --------------------------------------------------------------------------
# tolerance helper shared by the parity tests
# --------------------------------------------------------------------------
def rel_err(got: np.ndarray, ref: np.ndarray, floor_frac: float = 1e-2, rms: bool = False) -> float:
    """Maximum (``rms=True``: root-mean-square) relative spectral error
    against the FP64 reference.

    Power spectra ([n_out, gate, C]): |got - ref| / |ref| per bin.
    Stokes spectra ([n_out, IQUV, gate, C]): every product is normalised by
    the total intensity I of the same bin (|Q|, |U|, |V| <= I), so signed
    products near zero are measured on the scale their FP32 error lives on.
    Denominators are floored at floor_frac times the spectrum's MEAN power
    (default 1 %): an FP32 FFT's absolute error in |X|^2 scales with the
    spectrum's RMS amplitude, so bins far below the mean cannot carry a
    fixed relative error; empty spectra fall back to the peak."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    if ref.ndim == 4:
        base = np.abs(ref[:, 0:1])
    else:
        base = np.abs(ref)
    scale = np.mean(base, axis=-1, keepdims=True)
    denom = np.maximum(base, floor_frac * scale)
    denom = np.where(denom == 0, 1.0, denom)
    e = np.abs(got - ref) / denom
    return float(np.sqrt(np.mean(e * e))) if rms else float(np.max(e))


def rel_err_by_product(got: np.ndarray, ref: np.ndarray, floor_frac: float = 1e-2, rms: bool = False) -> dict:
    """:func:`rel_err` per Stokes product (I, Q, U, V) or per gate (power)."""
    if np.asarray(ref).ndim == 4:
        out = {}
        g_all = np.asarray(got, np.float64)
        r_all = np.asarray(ref, np.float64)
        base = np.abs(r_all[:, 0:1])
        denom = np.maximum(base, floor_frac * np.mean(base, axis=-1, keepdims=True))
        denom = np.where(denom == 0, 1.0, denom)
        for i, name in enumerate("IQUV"):
            e = np.abs(g_all[:, i] - r_all[:, i]) / denom[:, 0]
            out[name] = float(np.sqrt(np.mean(e * e))) if rms else float(np.max(e))
        return out
    return {f"G{g}": rel_err(np.asarray(got)[:, g:g + 1], np.asarray(ref)[:, g:g + 1], floor_frac, rms)
            for g in range(np.asarray(ref).shape[1])}
