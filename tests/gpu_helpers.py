"""Shared driver of the GPU parity tests: runs the same seeded blocks through
the CUDA library (psrdada_cpp_gb300.GatedSpectrometer over the C ABI) and the
oracle, and compares every handed-out output block."""
from __future__ import annotations

import numpy as np

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth
import psrdada_cpp_gb300 as G

# FP32 chain vs FP64 oracle: oracle.rel_err, the per-bin relative error
# (Stokes products normalised by I of the same bin; denominators floored at
# FLOOR times the spectrum's mean power) must stay within SPEC_TOL;
# counters, gate assignment and baselines are bit-exact.
SPEC_TOL = 1e-5
FLOOR = 1e-2


def oracle_config(spec, convention):
    lay = O.BufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    return O.Config(lay, spec.selected_side_channel, spec.selected_bit, spec.fft_length, spec.naccumulate,
                    spec.nbits, spec.dual_pol, convention)


def make_gpu(spec, convention, sink, flags=0, form=0):
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    return G.GatedSpectrometer(lay, spec.selected_side_channel, spec.selected_bit, spec.fft_length,
                               spec.naccumulate, spec.nbits, 100.0, 100.0, sink,
                               input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL,
                               convention=G.REFERENCE if convention == "reference" else G.INTENDED,
                               flags=flags, form=form)


def run_both(spec, convention="intended", nblocks=6, kind="default", lost=0.0, seed=11, extra_bits=False,
             flags=0, check_baselines=True, form=0, by_product=None):
    """Feeds nblocks blocks to both implementations; returns
    (gpu_blocks, oracle_payloads, max_rel_err).  by_product (a dict) collects
    the worst error per Stokes product / gate."""
    cfg = oracle_config(spec, convention)
    sink = G.CollectingSink()
    gpu = make_gpu(spec, convention, sink, flags, form)
    orc = O.OracleSpectrometer(cfg)
    payloads = []
    try:
        for b in range(nblocks):
            blk = synth.make_block(spec, seed=seed, block_index=b, kind=kind, lost_frac=lost, extra_bits=extra_bits)
            stop = gpu(G.RawBytes(blk))
            assert not stop
            _, p = orc(blk)
            if p is not None:
                payloads.append(p)
            if check_baselines:
                got = gpu.baselines()[:2 * spec.npol]
                # the GPU processes block b-1 at call b like the reference
                ref = np.array([[s.b0, s.b1] for s in orc.states], np.float32).ravel()
                assert np.array_equal(got, ref), (b, got, ref)
        assert len(sink.blocks) == len(payloads)
        worst = 0.0
        for got, ref in zip(sink.blocks, payloads):
            base = bytes(got[:cfg.output_bytes])
            spec_f, n0, n1 = O.parse_output(base, cfg)
            assert np.array_equal(n0, ref["n0"]), "G0 counters differ"
            assert np.array_equal(n1, ref["n1"]), "G1 counters differ"
            if cfg.dual_pol:
                cnt = np.frombuffer(base, np.uint8).reshape(cfg.n_out, -1)[:, 8 * cfg.nchans * 4:].copy().view("<u8")
                assert np.array_equal(cnt, np.tile(np.stack([ref["n0"], ref["n1"]], 1), 4))
            err = O.rel_err(spec_f, ref["spec"], FLOOR)
            worst = max(worst, err)
            if by_product is not None:
                for key, v in O.rel_err_by_product(spec_f, ref["spec"], FLOOR).items():
                    by_product[key] = max(by_product.get(key, 0.0), v)
            if flags & G.FLAG_SATURATION_RECORD:
                sat = np.frombuffer(bytes(got[cfg.output_bytes:]), "<u8").reshape(cfg.n_out, 2)
                assert np.array_equal(sat[:, 0], ref["sat0"]) and np.array_equal(sat[:, 1], ref["sat1"])
        return sink.blocks, payloads, worst
    finally:
        gpu.close()
