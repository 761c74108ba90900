"""The C/OpenMP restatement (the timed CPU baseline) against the numpy oracle:
counters and baselines bit-exact, spectra within the FP32 tolerance."""
import numpy as np
import pytest

from oracle import gspec_oracle as O
from oracle import gspec_cpu
from psrdada_cpp_gb300 import synth
from tests.gpu_helpers import oracle_config

S = synth.StreamSpec
CASES = [
    (S("c8", 8, False, 4096, 1, 1 << 15, 1024, 8, diode_period_heaps=3), "intended"),
    (S("c12", 12, False, 6144, 2, 1 << 15, 512, 8, selected_side_channel=1, diode_period_heaps=1), "intended"),
    (S("c10d", 10, True, 5120, 1, 1 << 14, 256, 8, diode_period_heaps=1), "intended"),
    (S("c12d", 12, True, 6144, 1, 1 << 15, 2048, 4, diode_period_heaps=2), "intended"),
    (S("c8r", 8, True, 4096, 1, 1 << 15, 512, 16, diode_period_heaps=2), "reference"),
]


@pytest.mark.parametrize("spec,convention", CASES, ids=[c[0].name for c in CASES])
def test_cpu_port_matches_oracle(spec, convention):
    cfg = oracle_config(spec, convention)
    cpu = gspec_cpu.CpuChain(spec, convention, nthreads=4)
    states = [O.PolState() for _ in range(spec.npol)]
    for b in range(3):
        blk = synth.make_block(spec, seed=21, block_index=b, lost_frac=0.1, extra_bits=True)
        cpu.zero()
        cpu.run_block(blk)
        r = O.process_block(blk, cfg, states)
        spec_f, n0, n1 = O.parse_output(cpu.out.tobytes(), cfg)
        assert np.array_equal(n0, r.n0) and np.array_equal(n1, r.n1)
        assert np.array_equal(cpu.sat.reshape(-1, 2)[:, 0], r.sat0)
        assert O.rel_err(spec_f, r.spectra) < 1e-5
        ref_b = np.array([[s.b0, s.b1] for s in states], np.float32).ravel()
        assert np.array_equal(cpu.baselines[:2 * spec.npol], ref_b)
