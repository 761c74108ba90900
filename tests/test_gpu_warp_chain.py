"""Single-pol 1024-point blocks that hold at least one output spectrum per SM:
the warp chain runs with one CTA per spectrum, stores every word of its
records (the output is never cleared between blocks), and its last CTA
finalises the block.  Several blocks through the handler against the
oracle: counters and the next block's baselines bit-exact after every
block, spectra within SPEC_TOL of FP64.  8, 10 and 12 bits, lost heaps,
extra side-channel bits, two side channels and the reference's item
convention."""
import pytest

from psrdada_cpp_gb300 import synth
from tests.gpu_helpers import run_both, SPEC_TOL

pytestmark = pytest.mark.gpu

S = synth.StreamSpec

# (name, spec, convention, lost, kind, calls); 2^24 samples and naccumulate 64: 256 spectra;
# the handler hands out a block's output three calls later
WHOLE_CASES = [
    ("c1_full", synth.config1(), "intended", 0.0, "c1", 6),
    ("s8_lost_bits", S("s8w", 8, False, 4096, 1, 1 << 24, 1024, 64, diode_period_heaps=5), "intended", 0.05,
     "default", 5),
    ("s12_nsc2", S("s12w", 12, False, 6144, 2, 1 << 24, 1024, 64, selected_side_channel=1, diode_period_heaps=3),
     "intended", 0.02, "default", 5),
    ("s10", S("s10w", 10, False, 5120, 1, 1 << 24, 1024, 64, diode_period_heaps=7), "intended", 0.0, "default", 5),
    ("s8_reference", S("s8wr", 8, False, 4096, 1, 1 << 24, 1024, 64, diode_period_heaps=9), "reference", 0.03,
     "default", 5),
]


@pytest.mark.parametrize("name,spec,convention,lost,kind,nblocks", WHOLE_CASES, ids=[c[0] for c in WHOLE_CASES])
def test_warp_chain_whole_spectra(name, spec, convention, lost, kind, nblocks):
    blocks, payloads, err = run_both(spec, convention, nblocks=nblocks, lost=lost, kind=kind,
                                     extra_bits=(kind == "default"))
    assert len(blocks) >= 1
    print(f"{name}: max rel err {err:.3e}")
    assert err <= SPEC_TOL, f"{name}: max rel err {err:.3g}"
