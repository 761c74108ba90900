"""Host-side logic of the chain in the oracle: layout, configuration,
conventions, handler pipeline and the regression fixtures."""
import os

import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cfg_of(spec, convention="intended"):
    lay = O.BufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    return O.Config(lay, spec.selected_side_channel, spec.selected_bit, spec.fft_length, spec.naccumulate,
                    spec.nbits, spec.dual_pol, convention)


def test_layout_config1():
    spec = synth.config1()
    assert spec.buffer_size == 16_809_984
    c = cfg_of(spec)
    assert c.layout.n_heaps == 4096 and c.layout.gap == 0
    assert c.nsamps_per_pol == 1 << 24 and c.n_out == 256 and c.n_blocks == 1
    assert c.output_bytes == 256 * (2 * 513 * 4 + 16) == 1_054_720


def test_layout_config2_config3():
    c2 = cfg_of(synth.config2())
    assert c2.layout.data_bytes == 201_326_592 and c2.n_out == 32 and c2.nchans == 32769
    assert c2.output_bytes == 32 * 1_048_672
    c3 = cfg_of(synth.config3())
    assert c3.layout.data_bytes == 805_306_368 and c3.n_out == 32 and c3.nchans == 524_289
    assert c3.output_bytes == 536_873_984


def test_layout_with_gap():
    spec = synth.StreamSpec("g", 8, False, 4096, 2, 1 << 16, 256, 4, gap_bytes=100)
    lay = O.BufferLayout(spec.buffer_size, 4096, 2)
    assert lay.n_heaps == 16 and lay.gap == 100
    assert lay.side_channel_offset == 16 * 4096 + 100


def test_nblocks_gt1():
    spec = synth.StreamSpec("m", 8, False, 4096, 1, 1 << 14, 1024, 64)
    c = cfg_of(spec)
    assert c.n_blocks == 4 and c.n_out == 1 and c.nacc_per_block == 16


def test_invalid_configs():
    spec = synth.StreamSpec("bad", 8, False, 4096, 1, 1 << 14, 1024, 3)
    with pytest.raises(ValueError):
        cfg_of(spec)
    spec = synth.StreamSpec("bad2", 8, False, 8192, 1, 1 << 16, 1024, 16)
    with pytest.raises(ValueError):        # reference indexing does not tile 8192-B heaps
        cfg_of(spec, "reference")


def test_conventions_agree_on_config1_geometry():
    """8-bit, 4096-B heaps, one item: the reference's literal index equals the
    intended one, so both conventions give identical outputs (single block)."""
    spec = synth.StreamSpec("c1s", 8, False, 4096, 1, 1 << 15, 1024, 8, diode_period_heaps=1)
    blk = synth.make_block(spec, seed=1, kind="c1")
    a = O.process_block(blk, cfg_of(spec, "intended"), [O.PolState()])
    b = O.process_block(blk, cfg_of(spec, "reference"), [O.PolState()])
    assert np.array_equal(a.n0, b.n0) and np.array_equal(a.n1, b.n1)
    assert np.array_equal(a.spectra, b.spectra)


def test_reference_indexing_differs_for_12bit():
    """12-bit 6144-B heaps: the literal index divides sample offsets by the
    heap size in bytes, so gate assignment differs from the intended one."""
    spec = synth.StreamSpec("r12", 12, False, 6144, 1, 1 << 14, 512, 16, diode_period_heaps=1)
    ci, cr = cfg_of(spec, "intended"), cfg_of(spec, "reference")
    assert not np.array_equal(O.sample_item_index(ci), O.sample_item_index(cr))
    assert O.sample_item_index(cr).max() < ci.items_per_pol


def test_dual_merge():
    a = np.array([0, 1, 0, 1 << 63, 6], np.uint64)
    b = np.array([0, 0, 2, 0, 1], np.uint64)
    m, _ = O.merge_side_channels(a, b, "reference")
    assert list(m) == [0, 1, 1, 1, 1]
    m, _ = O.merge_side_channels(a, b, "intended")
    assert list(m) == [0, 1, 2, 1 << 63, 7]


def test_pipeline_schedule_nblocks1():
    """The output of block n reaches the handler at call n+3."""
    spec = synth.StreamSpec("p1", 8, False, 4096, 1, 1 << 13, 256, 8, diode_period_heaps=1)
    c = cfg_of(spec)
    orc = O.OracleSpectrometer(c)
    blocks = [synth.make_block(spec, seed=5, block_index=i) for i in range(6)]
    emitted = []
    for i, blk in enumerate(blocks):
        stop, out = orc(blk)
        assert not stop
        emitted.append(out)
    assert emitted[:3] == [None, None, None]
    st = [O.PolState()]
    r0 = O.process_block(blocks[0], c, st)
    assert np.array_equal(emitted[3]["n0"], r0.n0)
    np.testing.assert_allclose(emitted[3]["spec"], r0.spectra)


def test_pipeline_schedule_nblocks2():
    """Two blocks per output: the first handed output integrates block 0 only
    (the reference's first period), then blocks (1, 2)."""
    spec = synth.StreamSpec("p2", 8, False, 4096, 1, 1 << 13, 256, 64, diode_period_heaps=1)
    c = cfg_of(spec)
    assert c.n_blocks == 2
    orc = O.OracleSpectrometer(c)
    blocks = [synth.make_block(spec, seed=6, block_index=i) for i in range(7)]
    outs = [orc(b)[1] for b in blocks]
    assert [o is not None for o in outs] == [False, False, False, False, True, False, True]
    st = [O.PolState()]
    r0 = O.process_block(blocks[0], c, st)
    np.testing.assert_allclose(outs[4]["spec"], r0.spectra)
    r1 = O.process_block(blocks[1], c, st, period_counts=(0, 0))
    r2 = O.process_block(blocks[2], c, st, period_counts=(int(r1.n0.sum()), int(r1.n1.sum())))
    np.testing.assert_allclose(outs[6]["spec"], r1.spectra + r2.spectra)


def test_wrong_size_stops():
    spec = synth.StreamSpec("w", 8, False, 4096, 1, 1 << 13, 256, 8)
    orc = O.OracleSpectrometer(cfg_of(spec))
    stop, _ = orc(np.zeros(spec.buffer_size - 1, np.uint8))
    assert stop


def test_header_append():
    spec = synth.config1()
    c = cfg_of(spec)
    h = bytearray(4096)
    h[:10] = b"HDR_VERSION"[:10]
    assert O.header_append(h, c)
    text = bytes(h).split(b"\0")[0].decode()
    assert "fft_length               1024\n" in text and "full_stokes_output       no\n" in text
    small = bytearray(b"X" * 60 + b"\0" * 40)
    assert not O.header_append(small, c)


def test_output_bytes_roundtrip():
    spec = synth.StreamSpec("o", 12, True, 6144, 1, 1 << 13, 256, 8, diode_period_heaps=1)
    c = cfg_of(spec)
    r = O.process_block(synth.make_block(spec, 2), c, [O.PolState(), O.PolState()])
    b = O.output_bytes(r.spectra, r.n0, r.n1, True)
    assert len(b) == c.output_bytes
    spec_f, n0, n1 = O.parse_output(b, c)
    np.testing.assert_allclose(spec_f, r.spectra.astype(np.float32))
    assert np.array_equal(n0, r.n0)


@pytest.mark.parametrize("name", ["chain_single8", "chain_dual12", "chain_single8_reference"])
def test_chain_fixtures(name):
    """Regression: the oracle reproduces its committed end-to-end fixtures."""
    from tests.golden.make_golden import CHAIN_CASES, chain_config
    case = CHAIN_CASES[name]
    g = np.load(os.path.join(GOLD, name + ".npz"))
    orc = O.OracleSpectrometer(chain_config(case["spec"], case["convention"]))
    outs = [orc(b)[1] for b in g["blocks"]]
    outs = [np.frombuffer(o["bytes"], np.uint8) for o in outs if o is not None]
    assert len(outs) == len(g["outputs"])
    for got, ref in zip(outs, g["outputs"]):
        assert np.array_equal(got, ref)


def test_synth_diode_and_lost():
    spec = synth.StreamSpec("s", 8, True, 4096, 2, 1 << 14, 256, 4, selected_side_channel=1, selected_bit=5,
                            diode_period_heaps=2)
    rng = np.random.default_rng(0)
    items = synth.diode_items(spec, 0, lost_frac=0.5, rng=rng, extra_bits=True)
    it = items[0].reshape(-1, 2)
    state = (it[:, 1] >> np.uint64(5)) & np.uint64(1)
    assert list(state[:4]) == [0, 0, 1, 1]
    assert ((it[:, 1] >> np.uint64(63)) != 0).any()


@pytest.mark.parametrize("name,spec,convention", [
    ("s8", synth.StreamSpec("ck_s8", 8, False, 4096, 1, 1 << 15, 512, 8, diode_period_heaps=3), "intended"),
    ("s8_ref", synth.StreamSpec("ck_s8r", 8, False, 4096, 1, 1 << 15, 512, 8, diode_period_heaps=3), "reference"),
    ("d12", synth.StreamSpec("ck_d12", 12, True, 6144, 1, 1 << 15, 1024, 4, diode_period_heaps=1), "intended"),
    ("d10_ref", synth.StreamSpec("ck_d10", 10, True, 5120, 1, 1 << 15, 512, 8, diode_period_heaps=2),
     "intended"),
])
def test_chunked_oracle_equals_whole_block(name, spec, convention):
    """The output-chunked evaluation used for full-size blocks gives the same
    spectra, counters and next-block baselines as the whole-block one."""
    cfg = cfg_of(spec, convention)
    start = [O.PolState(np.float32(1.5), np.float32(-2.25)) for _ in range(spec.npol)]
    for b in range(2):
        blk = synth.make_block(spec, seed=9, block_index=b, lost_frac=0.1, extra_bits=True)
        sa = [O.PolState(s.b0, s.b1) for s in start]
        sb = [O.PolState(s.b0, s.b1) for s in start]
        ra = O.process_block(blk, cfg, sa, period_counts=(3, 5))
        rb = O.process_block_chunked(blk, cfg, sb, period_counts=(3, 5), outputs_per_chunk=3)
        assert np.allclose(ra.spectra, rb.spectra, rtol=1e-12, atol=1e-9)
        for f in ("n0", "n1", "sat0", "sat1"):
            assert np.array_equal(getattr(ra, f), getattr(rb, f)), f
        assert ra.pol_counts == rb.pol_counts and ra.pol_sums == rb.pol_sums
        assert [(s.b0, s.b1) for s in sa] == [(s.b0, s.b1) for s in sb]
        start = sa
