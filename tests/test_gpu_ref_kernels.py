"""The reference's own GPU kernels, run beside this library's stages on the
same seeded inputs (tests/ref_kernels.py): unpack bit-exact against
gspec_unpack_device, gate assignment and fill bit-exact against
gspec_gate_device with the reference's counters, and stokes_accumulate
against the oracle's Stokes restatement.  Every launch keeps the reference
kernels' reads in bounds: word counts are multiples of 512 (8-bit) and 1536
(12-bit) 64-bit words, as the reference's one-pass unpack grids need, and each
block is one output chunk (nOut = 1), where the reference's literal item index
stays inside the side-channel array."""
import ctypes

import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth
import psrdada_cpp_gb300 as G
from tests import ref_kernels as R

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

if not R.available():
    pytest.skip("the reference kernels were not built here (oracle/build_ref.sh with PSRDADA_CPP_TREE)",
                allow_module_level=True)


@pytest.fixture(scope="module")
def ref():
    torch.cuda.init()
    torch.zeros(1, device="cuda")
    k = R.RefKernels()
    yield k
    k.close()


def ref_unpack(ref, raw_u8: np.ndarray, nbits: int):
    """Unpacker::unpack<nbits> (edd/src/Unpacker.cu:124-140): nblocks = words / 512, 512 threads."""
    words = raw_u8.view(np.uint64)
    n = words.size
    assert n % (1536 if nbits == 12 else 512) == 0
    d_in = torch.from_numpy(words.view(np.int64).copy()).cuda()
    d_out = torch.zeros(n * 64 // nbits, dtype=torch.float32, device="cuda")
    ref.launch("unpack12" if nbits == 12 else "unpack8", n // 512, 512, [R.ptr(d_in), R.ptr(d_out), ctypes.c_int(n)])
    torch.cuda.synchronize()
    return d_out


@pytest.mark.parametrize("nbits", [8, 12])
def test_reference_unpack_kernel(ref, nbits):
    rng = np.random.default_rng(100 + nbits)
    nwords = 1536 * 24
    raw = rng.integers(0, 256, size=nwords * 8, dtype=np.uint8)
    raw[:16] = [0x80, 0x00, 0x7F, 0xFF, 0xFF, 0xFF, 0x80, 0x08, 0x00, 0x7F, 0xF8, 0x01, 0, 0, 0xFF, 0x80]
    want = ref_unpack(ref, raw, nbits).cpu().numpy()
    nsamp = want.size
    d_raw = torch.from_numpy(raw).cuda()
    d_out = torch.empty(nsamp, dtype=torch.float32, device="cuda")
    G.unpack_device(d_raw.data_ptr(), nbits, nsamp, d_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy().view(np.uint32), want.view(np.uint32))


GATE_CASES = [
    # one output chunk per block (nOut = 1): fft * naccumulate = samples per pol
    (synth.StreamSpec("s8", 8, False, 4096, 1, 1 << 18, 1 << 12, 64, diode_period_heaps=3), "intended"),
    # two side channels: the reference convention is refused there (its literal index does
    # not tile the block); at 8 bits the intended index equals the reference kernel's
    (synth.StreamSpec("s8_sc2", 8, False, 4096, 2, 1 << 18, 1 << 12, 64, selected_side_channel=1, selected_bit=5,
                      diode_period_heaps=2), "intended"),
    (synth.StreamSpec("s12r", 12, False, 6144, 1, 1 << 18, 1 << 12, 64, diode_period_heaps=1), "reference"),
    (synth.StreamSpec("d8r", 8, True, 4096, 1, 1 << 18, 1 << 12, 64, diode_period_heaps=2), "reference"),
    (synth.StreamSpec("d12r", 12, True, 6144, 1, 1 << 18, 1 << 12, 64, diode_period_heaps=3), "reference"),
]


@pytest.mark.parametrize("case", GATE_CASES, ids=[c[0].name for c in GATE_CASES])
def test_reference_gating_kernel(ref, case):
    spec, convention = case
    cfg = O.Config(O.BufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels),
                   spec.selected_side_channel, spec.selected_bit, spec.fft_length, spec.naccumulate, spec.nbits,
                   spec.dual_pol, convention)
    assert cfg.nsamps_per_pol == spec.fft_length * spec.naccumulate, "one output chunk per block"
    blk = synth.make_block(spec, seed=11, kind="default", lost_frac=0.15, extra_bits=True)
    bl = np.array([0.37, -1.25, 2.5e-3, 17.0625], np.float32)
    n = cfg.nsamps_per_pol
    # this library: the gate stage of a handle with these baselines
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    gpu = G.GatedSpectrometer(lay, spec.selected_side_channel, spec.selected_bit, spec.fft_length,
                              spec.naccumulate, spec.nbits, 1.0, 1.0, G.NullSink(),
                              input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL,
                              convention=G.REFERENCE if convention == "reference" else G.INTENDED)
    try:
        gpu.set_baselines(bl)
        d_blk = torch.from_numpy(blk).cuda()
        d_g = torch.empty(spec.npol * 2 * n, dtype=torch.float32, device="cuda")
        gpu.gate_device(d_blk.data_ptr(), d_g.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        got = d_g.cpu().numpy().reshape(spec.npol, 2, n)
    finally:
        gpu.close()
    # the reference: each pol's heaps and items (the block layout of getFromBlock), the
    # dual-pol merge kernel, then unpack and gating with the reference's launch shapes
    raws, items = O.split_block(blk, cfg)
    d_items = [torch.from_numpy(np.ascontiguousarray(it).view(np.int64)).cuda() for it in items]
    if spec.dual_pol:
        ref.launch("merge", 1024, 1024, [R.ptr(d_items[0]), R.ptr(d_items[1]), R.size(d_items[0].numel())])
    for p in range(spec.npol):
        d_g0 = ref_unpack(ref, np.ascontiguousarray(raws[p]), spec.nbits)
        assert d_g0.numel() == n
        d_g1 = torch.zeros(n, dtype=torch.float32, device="cuda")
        d_b = torch.tensor([bl[2 * p], bl[2 * p + 1], 0.0, 0.0], dtype=torch.float32, device="cuda")
        d_st = torch.zeros(2, dtype=torch.int64, device="cuda")
        fb = d_b.data_ptr()
        ref.launch("gating", 1024, 1024,
                   [R.ptr(d_g0), R.ptr(d_g1), R.ptr(d_items[p]), R.size(n), R.size(spec.heap_size),
                    R.size(spec.selected_bit), R.size(spec.n_side_channels), R.size(spec.selected_side_channel),
                    ctypes.c_void_p(fb), ctypes.c_void_p(fb + 4), ctypes.c_void_p(fb + 8), ctypes.c_void_p(fb + 12),
                    ctypes.c_void_p(d_st.data_ptr()), ctypes.c_void_p(d_st.data_ptr() + 8)])
        torch.cuda.synchronize()
        g0, g1 = d_g0.cpu().numpy(), d_g1.cpu().numpy()
        assert np.array_equal(got[p, 0].view(np.uint32), g0.view(np.uint32)), f"pol {p} G0"
        assert np.array_equal(got[p, 1].view(np.uint32), g1.view(np.uint32)), f"pol {p} G1"
        # the reference's counters: samples per gate (exact) and the baseline sums
        # (float atomics in an unordered sum: within float rounding of the exact sums)
        it_merged = d_items[p].cpu().numpy().view(np.uint64)
        idx = O.sample_item_index(cfg)
        v = O.unpack(raws[p], spec.nbits)[:n].astype(np.float64)
        _, _, m0, m1 = O.gate(v.astype(np.float32), it_merged[idx], spec.selected_bit, bl[2 * p], bl[2 * p + 1])
        st = d_st.cpu().numpy()
        assert int(st[0]) == int(m0.sum()) and int(st[1]) == int(m1.sum()), (st, m0.sum(), m1.sum())
        sums = d_b.cpu().numpy()[2:]
        want = np.array([v[m0].sum(), v[m1].sum()])
        assert np.all(np.abs(sums - want) <= 1e-5 * np.abs(v).sum() + 1.0), (sums, want)


def test_reference_stokes_kernel(ref):
    rng = np.random.default_rng(7)
    nchans, nacc = 4097, 16
    p1 = (rng.normal(size=(nacc, nchans)) + 1j * rng.normal(size=(nacc, nchans))).astype(np.complex64) * 300
    p2 = (rng.normal(size=(nacc, nchans)) + 1j * rng.normal(size=(nacc, nchans))).astype(np.complex64) * 300
    d1 = torch.from_numpy(p1.view(np.float32).reshape(-1).copy()).cuda()
    d2 = torch.from_numpy(p2.view(np.float32).reshape(-1).copy()).cuda()
    out = torch.zeros(4, nchans, dtype=torch.float32, device="cuda")
    base = out.data_ptr()
    ref.launch("stokes", 1024, 1024, [R.ptr(d1), R.ptr(d2)] + [ctypes.c_void_p(base + 4 * nchans * i) for i in range(4)]
               + [ctypes.c_int(nchans), ctypes.c_int(nacc)])
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.float64)
    want = np.zeros((4, nchans))
    for k in range(nacc):
        want += np.array(O.stokes_iquv(p1[k].astype(np.complex128), p2[k].astype(np.complex128)))
    # FP32 accumulation of 16 spectra against FP64: relative to I of the bin
    assert np.max(np.abs(got - want) / want[0]) < 1e-5
