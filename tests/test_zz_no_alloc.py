"""The allocation-free entry point (gspec_process_block_noalloc) against the
handle-based one (gspec_run_block_device).

Callers that cannot allocate device memory between blocks - a DADA consumer
whose device memory is reserved up front by the ring buffer and its own
pool, or a real-time loop that must not pay cudaMalloc's latency - use the
allocation-free call with a library-owned device array as working memory.
It must give the same spectra, counters and baselines as the regular entry
point, on two calls in a row (the shared array keeps the previous call's
contents, so stale state would show on the second call).  This file is
collected last so a failure here comes after every other test has run."""
import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth
import psrdada_cpp_gb300 as G
from tests.gpu_helpers import oracle_config, SPEC_TOL

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CASES = [
    synth.StreamSpec("na_s8", 8, False, 4096, 1, 1 << 18, 1024, 16, diode_period_heaps=3),
    synth.StreamSpec("na_d12", 12, True, 6144, 1, 1 << 16, 512, 8, diode_period_heaps=2),
]


@pytest.mark.parametrize("spec", CASES, ids=[c.name for c in CASES])
def test_noalloc_matches_regular_entry_point(spec):
    cfg = oracle_config(spec, "intended")
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    gs = G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 1.0, 1.0, G.NullSink(),
                             input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL)
    try:
        start = np.array([0.25, -0.5, 1.5, -2.0], np.float32)
        gs.set_baselines(start)
        d_bl = torch.from_numpy(start.copy()).cuda()
        stream = torch.cuda.current_stream().cuda_stream
        nbytes = cfg.output_bytes
        blks = [torch.from_numpy(synth.make_block(spec, seed=17, block_index=c, lost_frac=0.05,
                                                  extra_bits=True)).cuda() for c in range(2)]
        outs = [[torch.zeros(nbytes, dtype=torch.uint8, device="cuda") for _ in range(2)] for _ in range(2)]
        torch.cuda.synchronize()
        for call in range(2):
            d_blk = blks[call]
            d_ref, d_new = outs[call]
            gs.run_block_device(d_blk.data_ptr(), d_ref.data_ptr(), stream)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            G.process_block_noalloc(gs.config, d_blk.data_ptr(), d_bl.data_ptr(), d_new.data_ptr(), stream)
            torch.cuda.synchronize()
            if call == 1:
                # every buffer of the call already exists: the call itself takes no device memory
                assert torch.cuda.mem_get_info()[0] == free0, "call 1 changed the free device memory"
            ref_b = d_ref.cpu().numpy().tobytes()
            new_b = d_new.cpu().numpy().tobytes()
            ref_spec, ref_n0, ref_n1 = O.parse_output(ref_b, cfg)
            assert int(ref_n0.sum() + ref_n1.sum()) > 0
            # the same kernels in the same order on the same block: byte-equal outputs
            assert new_b == ref_b, f"call {call}: output differs from gspec_run_block_device"
            assert O.rel_err(ref_spec, ref_spec.astype(np.float64)) <= SPEC_TOL
            assert np.array_equal(d_bl.cpu().numpy()[:2 * spec.npol], gs.baselines()[:2 * spec.npol]), \
                f"call {call}: baselines"
    finally:
        gs.close()


def test_noalloc_rejects_oversized_work():
    """Four-step lengths and working sets beyond the fixed array are refused
    with a clear error before any kernel touches memory (the 16-byte device
    buffers passed here are never read)."""
    d = torch.zeros(16, dtype=torch.uint8, device="cuda")
    spec = synth.StreamSpec("na_big", 12, True, 6144, 1, 1 << 16, 65536, 1, diode_period_heaps=2)
    cfg = G.GspecConfig(buffer_size=spec.buffer_size, heap_size=spec.heap_size, n_side_channels=1,
                        fft_length=spec.fft_length, naccumulate=1, nbits=12, input_type=G.DUAL_POL,
                        output_type=G.FULL_STOKES)
    with pytest.raises(G.GspecError, match="4096"):
        G.process_block_noalloc(cfg, d.data_ptr(), d.data_ptr(), d.data_ptr(), 0)
    # 2^25 heaps of 8 bytes: one gate-mask byte per side-channel item alone is 32 MiB
    heaps = 1 << 25
    cfg = G.GspecConfig(buffer_size=heaps * (8 + 8), heap_size=8, n_side_channels=1, fft_length=1024,
                        naccumulate=64, nbits=8, input_type=G.SINGLE_POL, output_type=G.POWER)
    with pytest.raises(G.GspecError, match="allocation-free scratch"):
        G.process_block_noalloc(cfg, d.data_ptr(), d.data_ptr(), d.data_ptr(), 0)
