"""Four-step FFT path at 2^17..2^20 and the benchmark configurations at their
own full geometry, on the GPU through the C ABI, against the FP64 oracle.

The handler-level cases cover every pass instantiation the four-step split
picks above 2^16 (N1 x N2 = 256x512, 512x512, 512x1024, 1024x1024): the
column pass at 512 and 1024 points (the 1024-point one held to 64 registers
for 8- and 12-bit samples, unbounded for 10-bit) and the row pass at 512 and
1024 points, single-pol power and dual-pol Stokes.  The full-geometry cases
run one whole block of the dual-pol 12-bit workloads (2^26 samples/pol at fft
2^16 and 2^28 samples/pol at fft 2^20: 32 output spectra, several scratch
chunks per block) in the FP32 form and the two tensor-core forms."""
import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth
import psrdada_cpp_gb300 as G
from tests.gpu_helpers import run_both, oracle_config, SPEC_TOL, FLOOR

pytestmark = pytest.mark.gpu

S = synth.StreamSpec

FOURSTEP_CASES = [
    # N1 = 256, N2 = 512: fourstep_a<256>, fourstep_b<512> (single pol)
    ("s8_n2p17", S("fs_s8_n2p17", 8, False, 4096, 1, 1 << 18, 1 << 17, 2, diode_period_heaps=5), 0.05),
    # N1 = N2 = 512 (dual pol, 12 bit)
    ("d12_n2p18", S("fs_d12_n2p18", 12, True, 6144, 1, 1 << 19, 1 << 18, 2, diode_period_heaps=7), 0.05),
    # N1 = 512, N2 = 1024: fourstep_b<1024> single pol, 10 bit
    ("s10_n2p19", S("fs_s10_n2p19", 10, False, 5120, 1, 1 << 20, 1 << 19, 2, diode_period_heaps=9), 0.05),
    # N1 = 512, N2 = 1024, dual pol, 8 bit
    ("d8_n2p19", S("fs_d8_n2p19", 8, True, 4096, 1, 1 << 19, 1 << 19, 1, diode_period_heaps=11), 0.0),
    # N1 = N2 = 1024: the two-CTA column pass (12 bit), fourstep_b<1024> dual pol
    ("d12_n2p20", S("fs_d12_n2p20", 12, True, 6144, 1, 1 << 21, 1 << 20, 2, diode_period_heaps=64), 0.02),
    # N1 = N2 = 1024: the two-CTA column pass (8 bit), single pol, frames with one gate paired
    ("s8_n2p20", S("fs_s8_n2p20", 8, False, 4096, 1, 1 << 21, 1 << 20, 2, diode_period_heaps=256), 0.02),
    # N1 = N2 = 1024: the unbounded column pass (10 bit), dual pol, 2 blocks per output spectrum
    ("d10_n2p20_nb2", S("fs_d10_n2p20", 10, True, 5120, 1, 1 << 20, 1 << 20, 2, diode_period_heaps=100), 0.0),
]


@pytest.mark.parametrize("name,spec,lost", FOURSTEP_CASES, ids=[c[0] for c in FOURSTEP_CASES])
def test_fourstep_fp32_parity(name, spec, lost):
    nblocks = 9 if "nb2" in name else 6
    prod = {}
    blocks, payloads, err = run_both(spec, "intended", nblocks=nblocks, lost=lost, extra_bits=True,
                                     kind="c3" if spec.nbits == 12 else "default", by_product=prod)
    assert len(blocks) >= 1
    print(f"{name}: max rel err {err:.3e} {prod}")
    assert err <= SPEC_TOL, f"{name}: max rel err {err:.3g}"


# ------------------------------------------------------------ full geometry
# form -> (max, rms) bound on the per-bin relative error with the 1 % floor
FULL_TOL = {G.FORM_FP32: (SPEC_TOL, 1e-6), G.FORM_FP16: (1e-4, 1e-5), G.FORM_BF16: (1e-4, 1e-5)}
# fractional baselines carried in from a previous block: half of every frame's
# samples per gate is this fill value
START_BASELINES = np.array([0.3718, -0.2093, 0.5807, -0.4411], np.float32)
_ORACLE = {}


def _full_case(name):
    if name in _ORACLE:
        return _ORACLE[name]
    spec = synth.config3() if name == "c3" else synth.config2()
    blk = synth.make_block(spec, seed=2 if name == "c3" else 1, block_index=0, kind=name)
    cfg = oracle_config(spec, "intended")
    states = [O.PolState(START_BASELINES[2 * p], START_BASELINES[2 * p + 1]) for p in range(spec.npol)]
    res = O.process_block_chunked(blk, cfg, states, outputs_per_chunk=2)
    _ORACLE.clear()                      # one full-size case in host memory at a time
    _ORACLE[name] = (spec, blk, cfg, res, states)
    return _ORACLE[name]


def _run_device(spec, blk, form):
    torch = pytest.importorskip("torch")
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    gs = G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 1.0, 1.0, G.NullSink(),
                             input_type=G.DUAL_POL, form=form)
    try:
        info = gs.info()
        d_blk = torch.from_numpy(blk).cuda()
        d_out = torch.zeros(int(info.output_bytes), dtype=torch.uint8, device="cuda")
        gs.set_baselines(START_BASELINES)
        gs.set_profiling(True)
        gs.run_block_device(d_blk.data_ptr(), d_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        prof = gs.profile()
        out = d_out.cpu().numpy().tobytes()
        return out, gs.baselines()[:2 * spec.npol].copy(), prof, info
    finally:
        gs.close()


@pytest.mark.parametrize("form", [G.FORM_FP32, G.FORM_FP16, G.FORM_BF16], ids=["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("name", ["c2", "c3"])
def test_full_geometry_block(name, form):
    """One whole benchmark block (both gates in every frame, 32 output
    spectra, several four-step scratch chunks per block) against the FP64
    oracle: counters and next-block baselines bit-exact, the spectra within
    the form's bound.  The error is reported per Stokes product with the 1 %
    floor and without it (pure per-bin, normalised by the bin's own I)."""
    # (at fft 2^16 the tensor-core forms split 64 x 1024: only the row pass
    # runs on the tensor cores)
    spec, blk, cfg, res, states = _full_case(name)
    out, bl, prof, info = _run_device(spec, blk, form)
    # several scratch chunks per block: the chunk loop is exercised
    assert prof["fourstep_a"][0] > 1, prof["fourstep_a"]
    spec_f, n0, n1 = O.parse_output(out, cfg)
    assert np.array_equal(n0, res.n0) and np.array_equal(n1, res.n1)
    cnt = np.frombuffer(out, np.uint8).reshape(cfg.n_out, -1)[:, 8 * cfg.nchans * 4:].copy().view("<u8")
    assert np.array_equal(cnt, np.tile(np.stack([res.n0, res.n1], 1), 4))
    ref_bl = np.array([[s.b0, s.b1] for s in states], np.float32).ravel()
    assert np.array_equal(bl, ref_bl), (bl, ref_bl)
    mx = O.rel_err(spec_f, res.spectra, FLOOR)
    rms = O.rel_err(spec_f, res.spectra, FLOOR, rms=True)
    by = O.rel_err_by_product(spec_f, res.spectra, FLOOR)
    by_rms = O.rel_err_by_product(spec_f, res.spectra, FLOOR, rms=True)
    by_nofloor = O.rel_err_by_product(spec_f, res.spectra, 0.0)
    print(f"{name} form={form} n1={info.n1} n2={info.n2}: max {mx:.3e} rms {rms:.3e}; per product max {by}, "
          f"rms {by_rms}, max without floor {by_nofloor}")
    tmax, trms = FULL_TOL[form]
    assert mx <= tmax, (mx, by)
    assert rms <= trms, (rms, by_rms)
