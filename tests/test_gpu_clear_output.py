"""gspec_clear_output_device: with one block per output the chain stores every
spectrum value, so clearing only the counters of a buffer that holds garbage
(or nothing, where the chain stores the counters as well) gives the same bytes
as a fully zeroed buffer; with several blocks per output the whole buffer is
cleared.  Shared-memory and four-step paths, single and
dual pol, FP32 and the tensor-core form."""
import numpy as np
import pytest

from psrdada_cpp_gb300 import synth
import psrdada_cpp_gb300 as G

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CASES = [
    # (spec, form): n_blocks = 1 unless the block holds less than fft * naccumulate
    (synth.StreamSpec("s8_small", 8, False, 4096, 1, 1 << 18, 1024, 64, diode_period_heaps=3), G.FORM_FP32),
    # 256 spectra: one warp-chain CTA per spectrum stores its counters too (clearing is a no-op)
    (synth.StreamSpec("s8_whole", 8, False, 4096, 1, 1 << 24, 1024, 64, diode_period_heaps=3), G.FORM_FP32),
    (synth.StreamSpec("d12_small_slices", 12, True, 6144, 1, 1 << 16, 2048, 8, diode_period_heaps=2), G.FORM_FP32),
    (synth.StreamSpec("d12_fs", 12, True, 6144, 1, 1 << 18, 1 << 16, 4, diode_period_heaps=2), G.FORM_FP32),
    (synth.StreamSpec("d12_fs_bf16", 12, True, 6144, 1, 1 << 18, 1 << 16, 4, diode_period_heaps=2), G.FORM_BF16),
    (synth.StreamSpec("s8_fs_nb2", 8, False, 4096, 1, 1 << 16, 1 << 14, 8, diode_period_heaps=3), G.FORM_FP32),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0].name for c in CASES])
def test_clear_output_matches_zeroed(case):
    spec, form = case
    dev = torch.device("cuda", 0)
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    blocks = [synth.make_block(spec, seed=21, block_index=i, kind="default", lost_frac=0.05) for i in range(4)]
    outs = {}
    for mode in ("zeroed", "cleared"):
        with G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 1.0, 1.0, G.NullSink(),
                                 input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL,
                                 flags=G.FLAG_NO_HOST_BUFFERS, form=form) as gs:
            info = gs.info()
            nb = int(info.n_blocks)
            d_out = torch.full((int(info.output_bytes),), 0x5A, dtype=torch.uint8, device=dev)
            s = torch.cuda.current_stream(dev).cuda_stream
            got = []
            for i, blk in enumerate(blocks):
                if i % nb == 0:
                    if mode == "zeroed":
                        d_out.zero_()
                    else:
                        gs.clear_output_device(d_out.data_ptr(), s)
                d_blk = torch.from_numpy(blk).to(dev)
                gs.run_block_device(d_blk.data_ptr(), d_out.data_ptr(), s)
                if (i + 1) % nb == 0:
                    got.append(d_out.cpu().numpy().copy())
            outs[mode] = got
    assert len(outs["zeroed"]) == len(outs["cleared"]) > 0
    for a, b in zip(outs["zeroed"], outs["cleared"]):
        assert np.array_equal(a, b)
