"""Single stages on the GPU against the oracle, bit-exact: unpack (R4/R4b)
and gate assignment with baseline fill (R5/R6)."""
import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth
import psrdada_cpp_gb300 as G

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("nbits", [8, 10, 12])
def test_unpack_bit_exact(nbits):
    rng = np.random.default_rng(nbits)
    nsamp = 32 * 4096
    raw = rng.integers(0, 256, size=nsamp * nbits // 8, dtype=np.uint8)
    raw[:16] = [0x80, 0x00, 0x7F, 0xFF, 0xFF, 0xFF, 0x80, 0x08, 0x00, 0x7F, 0xF8, 0x01, 0, 0, 0xFF, 0x80]
    d_raw = torch.from_numpy(raw).cuda()
    d_out = torch.empty(nsamp, dtype=torch.float32, device="cuda")
    G.unpack_device(d_raw.data_ptr(), nbits, nsamp, d_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    ref = O.unpack(raw, nbits).astype(np.float32)
    assert np.array_equal(d_out.cpu().numpy(), ref)


GATE_CASES = [
    # (spec, convention, lost, extra_bits)
    (synth.StreamSpec("s8", 8, False, 4096, 1, 1 << 16, 1024, 4, diode_period_heaps=3), "intended", 0.2, False),
    (synth.StreamSpec("s12", 12, False, 6144, 3, 1 << 16, 512, 8, selected_side_channel=2, selected_bit=7,
                      diode_period_heaps=2), "intended", 0.1, True),
    (synth.StreamSpec("s12b", 12, False, 3072, 1, 1 << 15, 256, 8, diode_period_heaps=1), "intended", 0.1, False),
    (synth.StreamSpec("d12", 12, True, 6144, 1, 1 << 16, 1024, 8, diode_period_heaps=2), "intended", 0.2, True),
    (synth.StreamSpec("d10", 10, True, 5120, 2, 1 << 16, 1024, 8, selected_side_channel=1,
                      diode_period_heaps=1), "intended", 0.1, True),
    (synth.StreamSpec("s8r", 8, False, 4096, 1, 1 << 16, 1024, 16, diode_period_heaps=3), "reference", 0.2, True),
    (synth.StreamSpec("s12r", 12, False, 6144, 1, 1 << 16, 1024, 8, diode_period_heaps=1), "reference", 0.0, False),
    (synth.StreamSpec("d8r", 8, True, 4096, 1, 1 << 16, 1024, 16, diode_period_heaps=2), "reference", 0.2, True),
]


@pytest.mark.parametrize("case", GATE_CASES, ids=[c[0].name + "-" + c[1] for c in GATE_CASES])
def test_gate_bit_exact(case):
    spec, convention, lost, extra = case
    cfg = O.Config(O.BufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels),
                   spec.selected_side_channel, spec.selected_bit, spec.fft_length, spec.naccumulate, spec.nbits,
                   spec.dual_pol, convention)
    blk = synth.make_block(spec, seed=3, kind="default", lost_frac=lost, extra_bits=extra)
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    gpu = G.GatedSpectrometer(lay, spec.selected_side_channel, spec.selected_bit, spec.fft_length,
                              spec.naccumulate, spec.nbits, 1.0, 1.0, G.NullSink(),
                              input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL,
                              convention=G.REFERENCE if convention == "reference" else G.INTENDED)
    try:
        bl = np.array([0.37, -1.25, 2.5e-3, 17.0625], np.float32)
        gpu.set_baselines(bl)
        d_blk = torch.from_numpy(blk).cuda()
        n = cfg.nsamps_per_pol
        d_g = torch.empty(spec.npol * 2 * n, dtype=torch.float32, device="cuda")
        gpu.gate_device(d_blk.data_ptr(), d_g.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        got = d_g.cpu().numpy().reshape(spec.npol, 2, n)
        raws, items = O.split_block(blk, cfg)
        if cfg.dual_pol:
            items = list(O.merge_side_channels(items[0], items[1], convention))
        idx = O.sample_item_index(cfg)
        for p in range(spec.npol):
            v = O.unpack(raws[p], spec.nbits)[:n]
            g0, g1, _, _ = O.gate(v, items[p][idx], spec.selected_bit, bl[2 * p], bl[2 * p + 1])
            assert np.array_equal(got[p, 0].view(np.uint32), g0.view(np.uint32)), f"pol {p} G0"
            assert np.array_equal(got[p, 1].view(np.uint32), g1.view(np.uint32)), f"pol {p} G1"
    finally:
        gpu.close()
