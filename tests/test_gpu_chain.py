"""End-to-end parity of the handler (R11-R16) on the GPU through the C ABI:
every output block handed to the handler is compared with the oracle's
(counters and baselines bit-exact, spectra within SPEC_TOL of FP64)."""
import numpy as np
import pytest

from psrdada_cpp_gb300 import synth
import psrdada_cpp_gb300 as G
from tests.gpu_helpers import run_both, SPEC_TOL

pytestmark = pytest.mark.gpu

S = synth.StreamSpec

CHAIN_CASES = [
    # shared-memory FFT path, single pol power
    ("s8_n32", S("s8_n32", 8, False, 4096, 1, 1 << 15, 32, 64, diode_period_heaps=1), "intended", 0.1),
    ("s8_n256", S("s8_n256", 8, False, 4096, 1, 1 << 16, 256, 16, diode_period_heaps=3), "intended", 0.1),
    ("s8_n1024_c1", S("s8_n1024", 8, False, 4096, 1, 1 << 17, 1024, 64, diode_period_heaps=32), "intended", 0.0),
    ("s12_n4096", S("s12_n4096", 12, False, 6144, 2, 1 << 17, 4096, 4, selected_side_channel=1,
                    diode_period_heaps=2), "intended", 0.05),
    ("s10_n512", S("s10_n512", 10, False, 5120, 1, 1 << 16, 512, 8, diode_period_heaps=2), "intended", 0.1),
    # dual pol Stokes
    ("d12_n1024", S("d12_n1024", 12, True, 6144, 1, 1 << 16, 1024, 8, diode_period_heaps=2), "intended", 0.1),
    ("d8_n64", S("d8_n64", 8, True, 4096, 1, 1 << 15, 64, 32, diode_period_heaps=1), "intended", 0.1),
    ("d10_n2048", S("d10_n2048", 10, True, 5120, 1, 1 << 16, 2048, 4, diode_period_heaps=1), "intended", 0.0),
    # four-step FFT path
    ("s8_n8192", S("s8_n8192", 8, False, 4096, 1, 1 << 17, 8192, 4, diode_period_heaps=1), "intended", 0.1),
    ("d12_n16384", S("d12_n16384", 12, True, 6144, 1, 1 << 17, 16384, 4, diode_period_heaps=2), "intended", 0.1),
    ("d12_n65536", S("d12_n65536", 12, True, 6144, 1, 1 << 18, 65536, 2, diode_period_heaps=8), "intended", 0.05),
    # several input blocks per output spectrum
    ("s8_nblocks4", S("s8_nb", 8, False, 4096, 1, 1 << 14, 1024, 64, diode_period_heaps=1), "intended", 0.1),
    ("d12_nblocks2", S("d12_nb", 12, True, 6144, 1, 1 << 15, 8192, 8, diode_period_heaps=1), "intended", 0.1),
    # the reference's literal gate indexing and dual-pol logical-OR merge
    ("s8_reference", S("s8_ref", 8, False, 4096, 1, 1 << 16, 1024, 16, diode_period_heaps=3), "reference", 0.2),
    ("s12_reference", S("s12_ref", 12, False, 6144, 1, 1 << 16, 1024, 8, diode_period_heaps=1), "reference", 0.0),
    ("d8_reference", S("d8_ref", 8, True, 4096, 1, 1 << 16, 512, 16, diode_period_heaps=2), "reference", 0.1),
    ("d12_reference_nb2", S("d12_refnb", 12, True, 6144, 1, 1 << 14, 1024, 32, diode_period_heaps=1), "reference",
     0.0),
]


@pytest.mark.parametrize("name,spec,convention,lost", CHAIN_CASES, ids=[c[0] for c in CHAIN_CASES])
def test_chain_parity(name, spec, convention, lost):
    nblocks = 11 if "nblocks" in name else 7
    blocks, payloads, err = run_both(spec, convention, nblocks=nblocks, lost=lost, extra_bits=True)
    assert len(blocks) >= 1
    assert err <= SPEC_TOL, f"{name}: max rel err {err:.3g}"


def test_config1_shape_with_tone():
    """Config-1 statistics (N(0,20) + tone at bin 137) at a reduced block."""
    spec = S("c1", 8, False, 4096, 1, 1 << 18, 1024, 64, diode_period_heaps=32)
    blocks, payloads, err = run_both(spec, "intended", nblocks=5, kind="c1")
    assert err <= SPEC_TOL
    spec_f = np.frombuffer(bytes(blocks[0]), np.uint8)
    assert spec_f.size == payloads[0]["spec"].shape[0] * (2 * 513 * 4 + 16)


def test_saturation_record():
    spec = S("sat", 12, True, 6144, 1, 1 << 16, 1024, 8, diode_period_heaps=2)
    blocks, payloads, err = run_both(spec, "intended", nblocks=5, kind="c3", flags=G.FLAG_SATURATION_RECORD)
    assert err <= SPEC_TOL
    assert any(int(p["sat0"].sum()) > 0 for p in payloads)


def test_all_heaps_lost():
    """Every heap lost: no sample in either gate, zero counters, zero
    baselines (the reference would divide by zero)."""
    spec = S("lost", 8, False, 4096, 1, 1 << 15, 512, 8, diode_period_heaps=1)
    blocks, payloads, err = run_both(spec, "intended", nblocks=5, lost=1.0)
    for p in payloads:
        assert int(p["n0"].sum()) == 0 and int(p["n1"].sum()) == 0


def test_wrong_block_size_stops():
    spec = S("w", 8, False, 4096, 1, 1 << 14, 256, 8)
    sink = G.CollectingSink()
    lay = G.DadaBufferLayout(spec.buffer_size, 4096, 1)
    with G.GatedSpectrometer(lay, 0, 0, 256, 8, 8, 1.0, 1.0, sink) as gs:
        blk = np.zeros(spec.buffer_size, np.uint8)
        assert gs(G.RawBytes(blk, spec.buffer_size, spec.buffer_size - 8)) is True
        assert "Unexpected Buffer Size" in gs.last_error()
        assert gs(G.RawBytes(blk)) is False


def test_init_header():
    spec = S("h", 12, True, 6144, 1, 1 << 14, 256, 8)
    sink = G.CollectingSink()
    lay = G.DadaBufferLayout(spec.buffer_size, 6144, 1)
    with G.GatedSpectrometer(lay, 0, 0, 256, 8, 12, 1.0, 1.0, sink, input_type=G.DUAL_POL) as gs:
        hdr = np.zeros(4096, np.uint8)
        hdr[:11] = np.frombuffer(b"HEADER 1.0\n", np.uint8)
        gs.init(G.RawBytes(hdr))
        text = bytes(sink.header).split(b"\0")[0].decode()
        assert text.startswith("HEADER 1.0\n")
        assert "full_stokes_output       yes\n" in text and "nchannels                129\n" in text


def test_invalid_configs_rejected():
    lay = G.DadaBufferLayout(16 * 4104, 4096, 1)
    with pytest.raises(G.GspecError, match="not implemented"):
        G.GatedSpectrometer(lay, 0, 0, 256, 8, 8, 1.0, 1.0, G.NullSink(), input_type=G.DUAL_POL,
                            output_type=G.POWER)
    with pytest.raises(G.GspecError, match="nbits"):
        G.GatedSpectrometer(lay, 0, 0, 256, 8, 16, 1.0, 1.0, G.NullSink())
    with pytest.raises(G.GspecError, match="multiple"):
        G.GatedSpectrometer(lay, 0, 0, 256, 3, 8, 1.0, 1.0, G.NullSink())


def test_device_block_input():
    """RawBytes with on_device() == true: same outputs as host blocks."""
    torch = pytest.importorskip("torch")
    spec = S("dev", 8, False, 4096, 1, 1 << 15, 512, 8, diode_period_heaps=1)
    lay = G.DadaBufferLayout(spec.buffer_size, 4096, 1)
    a, b = G.CollectingSink(), G.CollectingSink()
    with G.GatedSpectrometer(lay, 0, 0, 512, 8, 8, 1.0, 1.0, a) as ga, \
            G.GatedSpectrometer(lay, 0, 0, 512, 8, 8, 1.0, 1.0, b) as gb:
        for i in range(6):
            blk = synth.make_block(spec, seed=4, block_index=i, lost_frac=0.1)
            ga(G.RawBytes(blk))
            d = torch.from_numpy(blk).cuda()
            gb(G.RawBytes(d.data_ptr(), spec.buffer_size, spec.buffer_size, on_device=True))
    assert len(a.blocks) == len(b.blocks) == 3
    for x, y in zip(a.blocks, b.blocks):
        assert np.array_equal(x, y)
