"""Host-side checks of the serving / batching / autotuning layer (no GPU):
the ctypes mirrors of the C structs match the compiler's layout, the
uneven-stream generator only makes configurations the chain accepts, the
autotuner's candidate schedules are valid splits, and the server and query
entry points fail loudly without a device."""
import ctypes
import subprocess

import numpy as np
import pytest

import psrdada_cpp_gb300 as G
from psrdada_cpp_gb300 import synth, autotune, serving
from psrdada_cpp_gb300.gated_spectrometer import GspecConfig, GspecInfo
from oracle import gspec_oracle as O
from tests.gpu_helpers import oracle_config

ROOT = __import__("pathlib").Path(__file__).resolve().parents[1]

STRUCTS = {
    "gspec_config": (GspecConfig, ["buffer_size", "naccumulate", "nbits", "device", "flags", "tune_units",
                                   "tune_n1", "tune_scratch_mb", "stream_priority", "form"]),
    "gspec_info": (GspecInfo, ["nchans", "device_bytes", "kernel_launches"]),
    "gspec_server_config": (serving.GspecServerConfig, ["memory_budget", "device", "max_inflight",
                                                        "output_buffers", "inflight_bytes"]),
    "gspec_result": (serving.GspecResult, ["stream", "status", "tag", "block_index", "data", "size", "buffer",
                                           "t_submit", "t_start", "t_done", "h2d_ms", "wait_ms", "chain_ms", "d2h_ms",
                                           "issue_ms", "observe_ms"]),
}


def test_ctypes_layout_matches_header(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gspec.h"', "int main(void) {"]
    for name, (_, fields) in STRUCTS.items():
        lines.append(f'  printf("{name} __sizeof__ %zu\\n", sizeof({name}));')
        for f in fields:
            lines.append(f'  printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines.append("  return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            s, f, v = line.split()
            got[(s, f)] = int(v)
    for name, (cls, fields) in STRUCTS.items():
        assert got[(name, "__sizeof__")] == ctypes.sizeof(cls), name
        for f in fields:
            assert got[(name, f)] == getattr(cls, f).offset, (name, f)


def test_uneven_streams_are_valid_configs():
    specs = synth.uneven_streams()
    assert len(specs) == 16
    assert [s.name for s in specs] == [s.name for s in synth.uneven_streams()]      # seeded
    for s in specs:
        cfg = oracle_config(s, "intended")             # raises on an invalid shape
        assert 2 ** 10 <= s.fft_length <= 2 ** 18 and s.nbits in (8, 10, 12)
        assert 8 <= s.naccumulate <= 256 and 16 <= s.diode_period_heaps <= 128
        assert s.samples_per_pol >= s.fft_length and cfg.n_out >= 1
        assert s.sigma <= 0.3 * (1 << (s.nbits - 1))
    assert len({s.fft_length for s in specs}) > 3 and len({s.nbits for s in specs}) == 3
    assert {s.dual_pol for s in specs} == {True, False}


def test_autotune_candidates_are_valid_splits():
    for N in (1 << 13, 1 << 16, 1 << 18, 1 << 20):
        spec = synth.StreamSpec("x", 12, True, 6144, 1, max(N, 1 << 20), N, 8)
        cands = autotune.candidates(spec, 152)
        assert cands[0] == {}
        for c in cands[1:]:
            n1 = c["tune_n1"]
            assert 64 <= n1 <= 1024 and 128 <= N // n1 <= 1024 and n1 * (N // n1) == N
    small = autotune.candidates(synth.config1(), 152)
    assert {c.get("tune_units") for c in small[1:]} == {152, 304, 1216}
    assert autotune.shape_key(synth.config1(), "GPU") != autotune.shape_key(synth.config2(), "GPU")


def test_span_priorities_favour_short_blocks():
    from psrdada_cpp_gb300 import loadgen
    p = loadgen.span_priorities([synth.config1(), synth.config3(), synth.config2()])
    assert p[synth.config1().name] < 0 and p[synth.config3().name] == 0
    assert p[synth.config1().name] <= p[synth.config2().name] <= p[synth.config3().name]


def test_make_config_carries_tune_and_layout():
    c = G.make_config(synth.config2(), tune={"tune_n1": 512, "tune_scratch_mb": 256, "bogus": 1})
    assert (c.tune_n1, c.tune_scratch_mb, c.tune_units) == (512, 256, 0)
    assert c.buffer_size == synth.config2().buffer_size and c.input_type == G.DUAL_POL
    assert c.output_type == G.FULL_STOKES


def test_entry_points_fail_loudly_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(G.GspecError):
        G.Server(1 << 30)
    with pytest.raises(G.GspecError):
        G.query(G.make_config(synth.config1()))
    with pytest.raises(G.GspecError):
        G.Batch([G.make_config(synth.config1())])


def test_poisson_plan_rates_and_order():
    from psrdada_cpp_gb300 import loadgen
    specs = [synth.config1()] * 3 + [synth.config3()] * 2
    rate = 1e9                                            # samples/s per stream
    plan = loadgen.poisson_plan(specs, rate, 3000, seed=4)
    assert len(plan) == 3000
    t = [e[0] for e in plan]
    assert t == sorted(t) and t[0] >= 0
    # per-stream block counts follow 1 / block span (config 3 blocks are 32x longer)
    counts = [sum(1 for _, i in plan if i == k) for k in range(len(specs))]
    span1 = loadgen.block_samples(synth.config1()) / rate
    horizon = t[-1]
    for k in range(3):
        assert abs(counts[k] - horizon / span1) < 5 * (horizon / span1) ** 0.5
    assert sum(counts[3:]) < sum(counts[:3]) / 10
    assert loadgen.poisson_plan(specs, rate, 3000, seed=4) == plan                 # seeded


def test_burst_plan_interleaves_streams():
    from psrdada_cpp_gb300 import loadgen
    plan = loadgen.burst_plan([synth.config1(), synth.config2()], [3, 2])
    assert [i for _, i in plan] == [0, 1, 0, 1, 0] and all(t == 0.0 for t, _ in plan)


def test_latency_summary_splits_stages():
    """Per-shape percentiles of the block latency and of each recorded stage,
    and p99 over the block span, from synthetic records."""
    from psrdada_cpp_gb300 import loadgen
    specs = [synth.config1(), synth.config3()]
    rows = []
    for k in range(100):
        for i in (0, 1):
            t_sub = 0.01 * k
            lat = (1.0 + (k % 10)) * 1e-3 * (1 + 9 * i)        # long blocks take 10x as long
            # stream, block, t_submit, t_start, t_done, h2d, wait, chain, d2h, issue, observe (ms)
            rows.append((i, k, t_sub, t_sub + 1e-4, t_sub + lat, 0.1, 0.0, 0.2 * (1 + i), 0.05, 0.02, 0.01))
    res = {"records": np.array(rows)}
    rate = 1e9
    out = loadgen.latency_summary(res, specs, rate)
    assert out["blocks"] == 200
    short, long_ = out["by_shape"][specs[0].name], out["by_shape"][specs[1].name]
    assert short["blocks"] == long_["blocks"] == 100
    assert abs(short["p50_ms"] - np.percentile([(1.0 + k % 10) for k in range(100)], 50)) < 1e-9
    assert abs(long_["p99_ms"] / short["p99_ms"] - 10.0) < 1e-9
    assert short["chain_p50_ms"] == pytest.approx(0.2) and long_["chain_p50_ms"] == pytest.approx(0.4)
    assert short["issue_p99_ms"] == pytest.approx(0.02) and short["observe_p50_ms"] == pytest.approx(0.01)
    assert short["queue_p50_ms"] == pytest.approx(0.1)
    span_ms = loadgen.block_samples(specs[0]) / rate * 1e3
    assert short["block_span_ms"] == pytest.approx(span_ms)
    assert short["p99_over_span"] == pytest.approx(short["p99_ms"] / span_ms)
