"""Seeded synthetic EDD blocks for the gated spectrometer.

Builds DADA data blocks in the layout ``DadaBufferLayout`` describes
(``edd/src/DadaBufferLayout.cpp:17-39``): ``n_heaps`` heaps of packed
big-endian two's-complement samples (dual-pol heaps alternate P0 P1 P0 P1),
then a gap, then ``n_heaps * nSC`` little-endian uint64 side-channel items
(dual-pol items alternate P0 P1 like the heaps,
``edd/src/GatedSpectrometer.cu:285-300``).  Bit 0 of the selected item is the
noise-diode state; bit 63 marks a lost heap.

There is no public dataset for this path: the workloads below are seeded
synthetic stand-ins with the shapes, sizes and value distributions of the
benchmark configurations.
"""
from __future__ import annotations

import dataclasses
import numpy as np


def pack_samples(samples: np.ndarray, nbits: int) -> np.ndarray:
    """int samples -> big-endian bit stream of ``nbits``-bit two's complement."""
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


@dataclasses.dataclass
class StreamSpec:
    """One gated-spectrometer stream configuration."""
    name: str
    nbits: int
    dual_pol: bool
    heap_size: int            # bytes of sample data per heap
    n_side_channels: int
    samples_per_pol: int      # per block
    fft_length: int
    naccumulate: int
    selected_side_channel: int = 0
    selected_bit: int = 0
    diode_period_heaps: int = 32   # diode bit toggles every this many heaps (per pol)
    gap_bytes: int = 0
    sigma: float = 0.0             # Gaussian sigma of the "default" samples (0: 15 % of full scale)

    @property
    def heaps_per_pol(self) -> int:
        return self.samples_per_pol * self.nbits // (8 * self.heap_size)

    @property
    def n_heaps(self) -> int:
        return self.heaps_per_pol * (2 if self.dual_pol else 1)

    @property
    def buffer_size(self) -> int:
        return self.n_heaps * (self.heap_size + 8 * self.n_side_channels) + self.gap_bytes

    @property
    def npol(self) -> int:
        return 2 if self.dual_pol else 1


# Benchmark-shaped workloads -------------------------------------------------
def config1() -> StreamSpec:
    """Single-pol 8-bit, 4096-B heaps, 1 item/heap, diode every 32 heaps,
    2^24 samples/block, fft 1024, naccumulate 64."""
    return StreamSpec("single_pol_8bit_fft1024_nacc64", 8, False, 4096, 1, 1 << 24, 1024, 64,
                      diode_period_heaps=32)


def config2() -> StreamSpec:
    """Dual-pol 12-bit Stokes, 6144-B heaps (4096 samples), diode every 64
    heaps, 2^26 samples/pol/block, fft 2^16, naccumulate 32."""
    return StreamSpec("dual_pol_12bit_fft65536_nacc32", 12, True, 6144, 1, 1 << 26, 1 << 16, 32,
                      diode_period_heaps=64)


def config3() -> StreamSpec:
    """Dual-pol 12-bit Stokes at fft 2^20, naccumulate 8, 2^28 samples/pol."""
    return StreamSpec("dual_pol_12bit_fft1048576_nacc8", 12, True, 6144, 1, 1 << 28, 1 << 20, 8,
                      diode_period_heaps=64)


def uneven_streams(n: int = 16, seed: int = 3, min_log_block: int = 22, max_log_block: int = 26,
                   max_log_fft: int = 18) -> list:
    """Independent streams of mixed shapes (batched-streams workload): fft
    log-uniform in 2^10..2^max_log_fft, nbits from {8, 10, 12}, naccumulate a
    power of two in 8..256, block 2^min_log_block..2^max_log_block samples per
    pol (at least one fft), diode period 16..128 heaps, sigma 10..400 (clipped
    to the bit depth), single or dual pol.  Heaps hold 4096 samples."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nbits = int(rng.choice([8, 10, 12]))
        log_fft = int(rng.integers(10, max_log_fft + 1))
        log_block = int(rng.integers(max(min_log_block, log_fft), max(max_log_block, log_fft) + 1))
        nacc = int(1 << rng.integers(3, 9))
        dual = bool(rng.integers(0, 2))
        period = int(rng.integers(16, 129))
        sigma = float(min(rng.uniform(10.0, 400.0), 0.3 * (1 << (nbits - 1))))
        heap = 4096 * nbits // 8
        name = f"s{i}_{'dual' if dual else 'single'}_{nbits}bit_fft{1 << log_fft}_nacc{nacc}_blk{1 << log_block}"
        out.append(StreamSpec(name, nbits, dual, heap, 1, 1 << log_block, 1 << log_fft, nacc,
                              diode_period_heaps=period, sigma=sigma))
    return out


def _clip(x, nbits):
    lo, hi = -(1 << (nbits - 1)), (1 << (nbits - 1)) - 1
    return np.clip(np.rint(x), lo, hi).astype(np.int32)


def config_samples(spec: StreamSpec, rng: np.random.Generator, kind: str = "default"):
    """Per-pol integer samples for one block.

    ``kind``:
      * ``"c1"``: round(N(0,20) + 8 cos(2 pi 137 n / fft)), clipped (config 1);
      * ``"c2"``: A = N(0,300), B = 0.6 A + 0.8 N(0,300) plus a tone at bin
        4097 of amplitude 75 in phase in both pols (25 % of sigma, linear
        polarisation at +45 deg), clipped (config 2);
      * ``"c3"``: N(0,500) clipped, 0.1 % outliers at +-2047 (config 3);
      * ``"default"``: N(0, 0.15 * full scale) per pol, clipped.
    """
    n = spec.samples_per_pol
    t = np.arange(n, dtype=np.float64)
    nb = spec.nbits
    if kind == "c1":
        x = rng.normal(0.0, 20.0, n) + 8.0 * np.cos(2 * np.pi * 137 * (t % spec.fft_length) / spec.fft_length)
        return [_clip(x, nb)]
    if kind == "c2":
        a = rng.normal(0.0, 300.0, n)
        b = 0.6 * a + 0.8 * rng.normal(0.0, 300.0, n)
        tone = 75.0 * np.cos(2 * np.pi * 4097 * (t % spec.fft_length) / spec.fft_length)
        return [_clip(a + tone, nb), _clip(b + tone, nb)]
    if kind == "c3":
        pols = []
        for _ in range(spec.npol):
            x = rng.normal(0.0, 500.0, n)
            out = rng.random(n) < 1e-3
            x[out] = np.where(rng.random(int(out.sum())) < 0.5, -2047.0, 2047.0)
            pols.append(_clip(x, nb))
        return pols
    sigma = spec.sigma if spec.sigma > 0 else 0.15 * (1 << (nb - 1))
    return [_clip(rng.normal(0.0, sigma, n), nb) for _ in range(spec.npol)]


def diode_items(spec: StreamSpec, block_index: int = 0, lost_frac: float = 0.0,
                rng: np.random.Generator | None = None, extra_bits: bool = False) -> list:
    """Per-pol uint64 side-channel items (``heaps_per_pol * nSC`` each).

    The selected item of heap h carries the diode state
    ``((h + block_index*heaps_per_pol) // period) & 1`` in ``selected_bit``;
    ``lost_frac`` of the heaps get bit 63 set; ``extra_bits`` fills the other
    bits and the unselected items with random noise."""
    hp = spec.heaps_per_pol
    h = np.arange(hp, dtype=np.int64) + block_index * hp
    state = ((h // spec.diode_period_heaps) & 1).astype(np.uint64)
    pols = []
    for p in range(spec.npol):
        it = np.zeros((hp, spec.n_side_channels), np.uint64)
        if extra_bits and rng is not None:
            it[:] = rng.integers(0, 1 << 62, size=it.shape, dtype=np.uint64)
            it[:, spec.selected_side_channel] &= ~np.uint64(1 << spec.selected_bit)
        it[:, spec.selected_side_channel] |= state << np.uint64(spec.selected_bit)
        if lost_frac > 0 and rng is not None:
            lost = rng.random(hp) < lost_frac
            it[lost, spec.selected_side_channel] |= np.uint64(1) << np.uint64(63)
        pols.append(it.reshape(-1))
    return pols


def build_block(spec: StreamSpec, pol_samples: list, pol_items: list) -> np.ndarray:
    """Assemble one DADA data block (uint8, ``spec.buffer_size`` bytes)."""
    H = spec.heap_size
    hp = spec.heaps_per_pol
    block = np.zeros(spec.buffer_size, dtype=np.uint8)
    data_bytes = spec.n_heaps * H
    packed = [pack_samples(s, spec.nbits).reshape(hp, H) for s in pol_samples]
    if spec.dual_pol:
        d = block[:data_bytes].reshape(hp, 2, H)
        d[:, 0, :] = packed[0]
        d[:, 1, :] = packed[1]
        items = np.stack([pol_items[0].reshape(hp, spec.n_side_channels),
                          pol_items[1].reshape(hp, spec.n_side_channels)], axis=1)
        # item-wise interleave with pitch 16 B: P0 item i, P1 item i, ...
        items = np.stack([pol_items[0], pol_items[1]], axis=1).reshape(-1)
    else:
        block[:data_bytes] = packed[0].reshape(-1)
        items = pol_items[0]
    off = data_bytes + spec.gap_bytes
    block[off:off + items.size * 8] = items.astype("<u8").view(np.uint8)
    return block


def make_block(spec: StreamSpec, seed: int, block_index: int = 0, kind: str = "default",
               lost_frac: float = 0.0, extra_bits: bool = False) -> np.ndarray:
    rng = np.random.default_rng([seed, block_index])
    samples = config_samples(spec, rng, kind)
    items = diode_items(spec, block_index, lost_frac, rng, extra_bits)
    return build_block(spec, samples, items)
