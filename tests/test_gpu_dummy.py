"""The GPU synthetic DADA producer (gspec_dummy_block*, replacing
edd/src/dummy_data_generator.cu) against the oracle's restatement: the
reference's two-tone 8-bit block; the seeded gated stream (samples, diode
and lost-heap items, block continuation); the reference program's ring loop;
and stream blocks through the gated spectrometer against the oracle."""
import threading

import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import dummy, ring, synth
import psrdada_cpp_gb300 as G
from tests.gpu_helpers import oracle_config, SPEC_TOL

pytestmark = pytest.mark.gpu


def _unpack_pol(blk, cfg, pol):
    H = cfg.heap_size
    nheaps = cfg.buffer_size // (H + 8 * cfg.n_side_channels)
    data = blk[:nheaps * H]
    if cfg.dual_pol:
        data = data.reshape(nheaps // 2, 2, H)[:, pol].reshape(-1)
    return O.unpack(data, cfg.nbits)


def test_two_tone_block_matches_reference_restatement():
    n_heaps, heap, nsc = 512, 4096, 1
    cfg = dummy.make_config(n_heaps * (heap + 8 * nsc), heap, nsc, 8, dummy.TWO_TONE)
    blk = dummy.block(cfg)
    n = n_heaps * heap
    got = blk[:n].view(np.int8).astype(np.int32)
    ref = O.dummy_two_tone_block(n).astype(np.int32)
    diff = np.abs(got - ref)
    assert diff.max() <= 1 and np.count_nonzero(diff) <= max(1, n // 100000), np.count_nonzero(diff)
    assert not blk[n:].any()                       # the items are zero
    assert got.min() == -128 and got.max() in (126, 127)   # packNbit's min/max scaling, truncated


@pytest.mark.parametrize("nbits,dual", [(8, False), (12, True), (10, True)])
def test_stream_block_matches_oracle(nbits, dual):
    heap = 4096 * nbits // 8
    heaps_per_pol, nsc = 64, 2
    npol = 2 if dual else 1
    cfg = dummy.make_config(heaps_per_pol * npol * (heap + 8 * nsc), heap, nsc, nbits, dummy.STREAM, dual,
                            seed=77, selected_side_channel=1, selected_bit=3, diode_period_heaps=5, sigma=60.0,
                            lost_fraction=0.1, block_index=3)
    blk = dummy.block(cfg)
    spp = heaps_per_pol * 4096
    for p in range(npol):
        got = _unpack_pol(blk, cfg, p)
        ref = O.dummy_stream_samples(77, p, 3 * spp, spp, 60.0, 0.0, 0, nbits)
        assert np.array_equal(got, ref), (p, np.count_nonzero(got != ref))
    items = blk[heaps_per_pol * npol * heap:].view("<u8").reshape(heaps_per_pol, nsc, npol)
    gh = np.arange(heaps_per_pol) + 3 * heaps_per_pol
    assert not items[:, 0].any()
    for p in range(npol):
        with np.errstate(over="ignore"):
            u = (O._mix64(np.uint64(77) ^ np.uint64(0x10575EED) ^ (gh.astype(np.uint64) * np.uint64(2)
                                                                   + np.uint64(p))) >> np.uint64(11)) * 2.0 ** -53
        expect = (((gh // 5) & 1).astype(np.uint64) << np.uint64(3)) | \
            np.where(u < np.float32(0.1), np.uint64(1) << np.uint64(63), np.uint64(0))
        assert np.array_equal(items[:, 1, p], expect)
    assert (items[:, 1, 0] >> np.uint64(63)).any()


def test_stream_tone_and_continuation():
    """A tone; block k+1 continues block k (one long stream cut in two)."""
    heap, hp = 4096, 32
    mk = lambda idx: dummy.make_config(hp * (heap + 8), heap, 1, 8, dummy.STREAM, False, seed=5, sigma=10.0,
                                       tone_amplitude=30.0, tone_period=1000, block_index=idx)
    a, b = dummy.block(mk(0)), dummy.block(mk(1))
    spp = hp * heap
    got = np.concatenate([a[:spp].view(np.int8), b[:spp].view(np.int8)]).astype(np.int64)
    ref = O.dummy_stream_samples(5, 0, 0, 2 * spp, 10.0, 30.0, 1000, 8)
    diff = np.abs(got - ref)
    assert diff.max() <= 1 and np.count_nonzero(diff) <= 2


def test_generator_loop_into_ring():
    """The reference program's loop: its header, then nblocks identical
    two-tone blocks into a ring, read back through DadaInputStream."""
    buf = 64 * 4104
    rg = ring.MemoryRing(buf, 2)
    got = G.CollectingSink()
    t = threading.Thread(target=lambda: ring.DadaInputStream(rg.reader(), got).start())
    t.start()
    n = dummy.dummy_data_generator(rg.writer(), buf, nblocks=5, delay_ms=1.0)
    rg.writer().data_stream().end_of_data()
    t.join(timeout=60)
    assert n == 5 and len(got.blocks) == 5
    assert got.header.startswith(b"HEADER       DADA\n") and b"SYNC_TIME    1234567890" in got.header
    for blk in got.blocks[1:]:
        assert np.array_equal(blk, got.blocks[0])


def test_stream_blocks_through_the_gated_spectrometer():
    """Generated blocks are valid gated-spectrometer input: the chain on
    them matches the oracle (counters bit-exact)."""
    spec = synth.StreamSpec("dummy_d12", 12, True, 6144, 1, 1 << 16, 2048, 4, diode_period_heaps=2)
    mk = lambda idx: dummy.make_config(spec.buffer_size, spec.heap_size, 1, 12, dummy.STREAM, True, seed=9,
                                       sigma=300.0, diode_period_heaps=2, lost_fraction=0.05, block_index=idx)
    blocks = [dummy.block(mk(i)) for i in range(6)]
    cfg = oracle_config(spec, "intended")
    orc = O.OracleSpectrometer(cfg)
    refs = [p for p in (orc(b)[1] for b in blocks) if p is not None]
    sink = G.CollectingSink()
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, 1)
    with G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, 12, 1.0, 1.0, sink,
                             input_type=G.DUAL_POL) as gs:
        for b in blocks:
            gs(G.RawBytes(b))
    assert len(sink.blocks) == len(refs) == 3
    for got, ref in zip(sink.blocks, refs):
        sf, n0, n1 = O.parse_output(bytes(got), cfg)
        assert np.array_equal(n0, ref["n0"]) and np.array_equal(n1, ref["n1"])
        assert O.rel_err(sf, ref["spec"]) <= SPEC_TOL
