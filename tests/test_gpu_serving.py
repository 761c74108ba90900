"""Serving loop, graph-batched streams and the autotuner on the GPU.

* every result of a stream served next to other streams equals, byte for
  byte, the result of the same stream served alone, and both agree with the
  FP64 oracle (counters bit-exact, spectra within SPEC_TOL);
* admission by device-memory budget: a stream that does not fit waits until
  memory is freed, then produces the same results;
* a batch of uneven streams in one CUDA graph equals the streams run one by
  one through gspec_run_block_device;
* gspec_query predicts gspec_create's device memory exactly;
* tuned schedules stay within the oracle tolerance.
"""
import numpy as np
import pytest

import psrdada_cpp_gb300 as G
from psrdada_cpp_gb300 import synth
from oracle import gspec_oracle as O
from tests.gpu_helpers import SPEC_TOL, FLOOR, oracle_config

pytestmark = pytest.mark.gpu

S = synth.StreamSpec
# uneven streams: both FFT paths, 8/10/12 bit, single/dual pol, n_blocks 1 and 2
STREAMS = [
    S("a_s8_n1024", 8, False, 4096, 1, 1 << 16, 1024, 16, diode_period_heaps=1),
    S("b_d12_n8192", 12, True, 6144, 1, 1 << 17, 8192, 4, diode_period_heaps=2),
    S("c_s10_n256", 10, False, 5120, 1, 1 << 15, 256, 64, diode_period_heaps=1),
    S("d_d8_n2048_nb2", 8, True, 4096, 1, 1 << 15, 2048, 32, diode_period_heaps=1),
    S("e_s12_n16384_nb2", 12, False, 6144, 1, 1 << 16, 16384, 8, diode_period_heaps=1),
    S("f_d10_n512", 10, True, 5120, 1, 1 << 16, 512, 8, diode_period_heaps=3),
]
NBLK = 4


def blocks_of(spec, seed):
    return [synth.make_block(spec, seed=seed, block_index=b, lost_frac=0.05, extra_bits=True)
            for b in range(NBLK)]


def oracle_direct(spec, blocks):
    """Output blocks of the chain without the reference's pipeline delay:
    one output every n_blocks blocks."""
    cfg = oracle_config(spec, "intended")
    states = [O.PolState() for _ in range(spec.npol)]
    outs, acc = [], None
    for i, blk in enumerate(blocks):
        prev = (0, 0) if acc is None else (int(acc["n0"].sum()), int(acc["n1"].sum()))
        r = O.process_block(blk, cfg, states, period_counts=prev)
        if acc is None:
            acc = {"spec": r.spectra.copy(), "n0": r.n0.copy(), "n1": r.n1.copy()}
        else:
            acc["spec"] = acc["spec"] + r.spectra
            acc["n0"] = acc["n0"] + r.n0
            acc["n1"] = acc["n1"] + r.n1
        if (i + 1) % cfg.n_blocks == 0:
            outs.append(acc)
            acc = None
    return cfg, outs


def check_vs_oracle(spec, cfg, got: bytes, ref):
    spec_f, n0, n1 = O.parse_output(got[:cfg.output_bytes], cfg)
    assert np.array_equal(n0, ref["n0"]) and np.array_equal(n1, ref["n1"]), spec.name
    err = O.rel_err(spec_f, ref["spec"], FLOOR)
    assert err <= SPEC_TOL, (spec.name, err)


def serve(streams_blocks, budget=64 << 30, order="interleaved", pinned=False, **server_args):
    """Runs the streams through one Server; returns {stream index: [output bytes]}.
    ``pinned`` submits page-locked copies of the blocks (read by SM loads)."""
    if pinned:
        import torch
        streams_blocks = [(spec, [torch.from_numpy(b).pin_memory() for b in blocks])
                          for spec, blocks in streams_blocks]
    outs = {i: [] for i in range(len(streams_blocks))}
    with G.Server(budget, **server_args) as srv:
        ids = [srv.open(G.make_config(spec)) for spec, _ in streams_blocks]
        jobs = []
        for i, (_, blocks) in enumerate(streams_blocks):
            for b, blk in enumerate(blocks):
                jobs.append((b, i, blk))
        if order == "interleaved":
            jobs.sort(key=lambda j: (j[0], j[1]))
        for b, i, blk in jobs:
            srv.submit(ids[i], blk, tag=1000 * i + b)
        want = sum(len(bl) for _, bl in streams_blocks)
        got = 0
        while got < want:
            for r in srv.poll(64, 200000):
                assert r["status"] == 0, srv.last_error()
                i = ids.index(r["stream"])
                assert r["tag"] == 1000 * i + r["block_index"]
                if r["data"] is not None:
                    outs[i].append(r["data"].tobytes())
                got += 1
        assert srv.kernel_launches() > 0
    return outs


@pytest.fixture(scope="module")
def stream_blocks():
    return [(spec, blocks_of(spec, 40 + i)) for i, spec in enumerate(STREAMS)]


def test_query_matches_create():
    for spec in STREAMS + [synth.config2()]:
        q = G.query(G.make_config(spec, flags=G.FLAG_NO_HOST_BUFFERS))
        lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
        with G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 1.0, 1.0, G.NullSink(),
                                 input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL,
                                 flags=G.FLAG_NO_HOST_BUFFERS) as gs:
            info = gs.info()
        assert q.device_bytes == info.device_bytes, spec.name
        assert (q.n_out, q.n_blocks, q.output_bytes, q.fft_path) == \
            (info.n_out, info.n_blocks, info.output_bytes, info.fft_path)


def test_serving_alone_equals_mix(stream_blocks):
    alone = {}
    for i, sb in enumerate(stream_blocks):
        alone[i] = serve([sb])[0]
    mix = serve(stream_blocks)
    for i, (spec, blocks) in enumerate(stream_blocks):
        cfg, ref = oracle_direct(spec, blocks)
        assert len(alone[i]) == len(ref) == len(mix[i]), spec.name
        for a, m, r in zip(alone[i], mix[i], ref):
            assert a == m, f"{spec.name}: result differs between alone and mix"
            check_vs_oracle(spec, cfg, a, r)


def test_serving_pinned_inputs_equal_pageable(stream_blocks):
    """Page-locked blocks (SM loads on the compute stream) give the same bytes
    as pageable blocks (copy engine on the copy stream)."""
    assert serve(stream_blocks, pinned=True) == serve(stream_blocks)


def test_serving_inflight_cap_equals_default(stream_blocks):
    """A cap on the long blocks in flight gives the same bytes as the
    default server."""
    big = S("g_d12_n65536_long", 12, True, 6144, 1, 1 << 25, 1 << 16, 4, diode_period_heaps=5)
    blocks = [synth.make_block(big, seed=60 + b, block_index=b) for b in range(2)]
    assert blocks[0].nbytes > 64 << 20
    mix = [(big, blocks), (big, blocks[::-1])] + stream_blocks[:2]
    ref = serve(mix)
    assert serve(mix, inflight_bytes=blocks[0].nbytes) == ref


def test_serving_admission_by_budget(stream_blocks):
    big = stream_blocks[1]          # four-step dual-pol stream
    small = stream_blocks[0]
    qb = G.query(G.make_config(big[0], flags=G.FLAG_NO_HOST_BUFFERS)).device_bytes
    qs = G.query(G.make_config(small[0], flags=G.FLAG_NO_HOST_BUFFERS)).device_bytes
    budget = max(qb, qs) + min(qb, qs) // 2          # room for one of them at a time
    with G.Server(budget) as srv:
        a = srv.open(G.make_config(big[0]))
        b = srv.open(G.make_config(small[0]))
        for k, blk in enumerate(big[1]):
            srv.submit(a, blk, tag=k)
        for k, blk in enumerate(small[1]):
            srv.submit(b, blk, tag=100 + k)
        res_a, res_b = [], []
        while len(res_a) < len(big[1]):
            for r in srv.poll(16, 200000):
                assert r["status"] == 0, srv.last_error()
                (res_a if r["stream"] == a else res_b).append(r)
            assert srv.memory_in_use() <= budget
        assert res_b == [] and srv.state(b) == 0, "the second stream must wait for memory"
        srv.close_stream(a)
        while len(res_b) < len(small[1]):
            for r in srv.poll(16, 200000):
                assert r["status"] == 0, srv.last_error()
                res_b.append(r)
            assert srv.memory_in_use() <= budget
        assert srv.state(a) == 3 and srv.state(b) == 1
    for spec_blocks, res in ((big, res_a), (small, res_b)):
        spec, blocks = spec_blocks
        cfg, ref = oracle_direct(spec, blocks)
        outs = [r["data"].tobytes() for r in res if r["data"] is not None]
        assert len(outs) == len(ref)
        for o, r in zip(outs, ref):
            check_vs_oracle(spec, cfg, o, r)


def test_serving_rejects_wrong_size_and_oversized(stream_blocks):
    spec, blocks = stream_blocks[0]
    with G.Server(1 << 30) as srv:
        sid = srv.open(G.make_config(spec))
        with pytest.raises(G.GspecError):
            srv.submit(sid, blocks[0][:-8], tag=0)
        with pytest.raises(G.GspecError):
            G.Server(1 << 20).open(G.make_config(synth.config2()))


def run_alone_device(spec, blocks):
    """The stream through gspec_run_block_device, one output per n_blocks."""
    import torch
    dev = torch.device("cuda", 0)
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    outs = []
    with G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 1.0, 1.0, G.NullSink(),
                             input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL,
                             flags=G.FLAG_NO_HOST_BUFFERS) as gs:
        info = gs.info()
        # garbage first: the caller's clear (counters only when a block holds whole outputs)
        # must be all the buffer needs
        d_out = torch.full((int(info.output_bytes),), 0x5A, dtype=torch.uint8, device=dev)
        s = torch.cuda.current_stream(dev).cuda_stream
        for i, blk in enumerate(blocks):
            if i % int(info.n_blocks) == 0:
                gs.clear_output_device(d_out.data_ptr(), s)
            d_blk = torch.from_numpy(blk).to(dev)
            gs.run_block_device(d_blk.data_ptr(), d_out.data_ptr(), s)
            if (i + 1) % int(info.n_blocks) == 0:
                outs.append(d_out.cpu().numpy().tobytes())
    return outs


def test_batch_graph_equals_alone(stream_blocks):
    import torch
    torch.cuda.init()
    alone = [run_alone_device(spec, blocks) for spec, blocks in stream_blocks]
    outs = [[] for _ in stream_blocks]
    with G.Batch([G.make_config(spec) for spec, _ in stream_blocks]) as bt:
        for step in range(NBLK):
            for i, (_, blocks) in enumerate(stream_blocks):
                bt.set_input(i, blocks[step])
            bt.run()
            for i in range(bt.n):
                _, _, complete = bt.output(i)
                if complete:
                    outs[i].append(bt.read_output(i).tobytes())
        assert bt.kernels_per_step() >= 3 * bt.n
        assert bt.steps() == NBLK
    for i, (spec, blocks) in enumerate(stream_blocks):
        assert len(outs[i]) == len(alone[i]) == NBLK // max(1, (spec.fft_length * spec.naccumulate) //
                                                             spec.samples_per_pol), spec.name
        for a, b in zip(alone[i], outs[i]):
            assert a == b, f"{spec.name}: batched result differs from the stream run alone"
        cfg, ref = oracle_direct(spec, blocks)
        for o, r in zip(outs[i], ref):
            check_vs_oracle(spec, cfg, o, r)


def test_autotune_schedules_stay_in_tolerance(tmp_path, stream_blocks):
    from psrdada_cpp_gb300 import autotune
    for idx in (0, 1):
        spec, blocks = stream_blocks[idx]
        best = autotune.tune(spec, cache_path=tmp_path / "cache.json", steps=3)
        assert set(best) <= set(G.gated_spectrometer.TUNE_KEYS)
        cache = autotune.load_cache(tmp_path / "cache.json")
        assert any(v["tune"] == best for v in cache.values())
        # every candidate schedule is a correct chain
        cfg, ref = oracle_direct(spec, blocks)
        import torch
        props = torch.cuda.get_device_properties(0)
        for cand in autotune.candidates(spec, props.multi_processor_count)[:4]:
            with G.Server(8 << 30) as srv:
                sid = srv.open(G.make_config(spec, tune=cand))
                for k, blk in enumerate(blocks):
                    srv.submit(sid, blk, tag=k)
                outs = []
                while len(outs) < len(blocks):
                    outs += srv.poll(16, 200000)
                data = [r["data"].tobytes() for r in outs if r["data"] is not None]
            for o, r in zip(data, ref):
                check_vs_oracle(spec, cfg, o, r)


def test_batch_inputs_copied_one_step_ahead(stream_blocks):
    """The next step's blocks go in on a copy stream while the current step
    runs (two input buffers per member); results equal the serial loop."""
    import torch
    dev = torch.device("cuda", 0)
    alone = [run_alone_device(spec, blocks) for spec, blocks in stream_blocks]
    outs = [[] for _ in stream_blocks]
    compute = torch.cuda.current_stream(dev)
    copy = torch.cuda.Stream(dev)
    pinned = [[torch.from_numpy(b).pin_memory() for b in blocks] for _, blocks in stream_blocks]
    with G.Batch([G.make_config(spec) for spec, _ in stream_blocks]) as bt:
        copied = [torch.cuda.Event() for _ in range(NBLK)]
        ran = [torch.cuda.Event() for _ in range(NBLK)]

        def put(k):
            if k >= 2:
                copy.wait_event(ran[k - 2])
            for i in range(bt.n):
                bt.set_input(i, pinned[i][k], copy.cuda_stream)
            copied[k].record(copy)

        put(0)
        for k in range(NBLK):
            compute.wait_event(copied[k])
            bt.run(compute.cuda_stream)
            ran[k].record(compute)
            if k + 1 < NBLK:
                put(k + 1)
            for i in range(bt.n):
                _, n, complete = bt.output(i)
                if complete:
                    dst = torch.empty(n, dtype=torch.uint8, pin_memory=True)
                    bt.copy_output(i, dst, compute.cuda_stream)
                    outs[i].append(dst)
        torch.cuda.synchronize(dev)
    for i, (spec, _) in enumerate(stream_blocks):
        got = [o.numpy().tobytes() for o in outs[i]]
        assert got == alone[i], spec.name


def test_closing_a_waiting_stream_answers_its_blocks(stream_blocks):
    """A stream closed before it was admitted frees its queue: each queued block
    comes back with an error status, and the admitted stream is unaffected."""
    big, small = stream_blocks[1], stream_blocks[0]
    qb = G.query(G.make_config(big[0], flags=G.FLAG_NO_HOST_BUFFERS)).device_bytes
    qs = G.query(G.make_config(small[0], flags=G.FLAG_NO_HOST_BUFFERS)).device_bytes
    with G.Server(max(qb, qs) + min(qb, qs) // 2) as srv:
        a = srv.open(G.make_config(big[0]))
        b = srv.open(G.make_config(small[0]))
        for k, blk in enumerate(small[1][:2]):
            srv.submit(b, blk, tag=k)
        assert srv.state(b) == 0
        srv.close_stream(b)
        srv.submit(a, big[1][0], tag=7)
        res = []
        while len(res) < 3:
            res += srv.poll(8, 200000)
        by = {(r["stream"], r["tag"]): r for r in res}
        assert by[(b, 0)]["status"] < 0 and by[(b, 1)]["status"] < 0
        assert by[(a, 7)]["status"] == 0
        assert srv.state(b) == 3
        with pytest.raises(G.GspecError):
            srv.submit(b, small[1][0], tag=9)
