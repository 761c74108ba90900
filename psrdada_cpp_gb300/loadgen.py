"""Load generator for the serving loop: open-loop (Poisson) and as-fast-as-possible
arrivals of blocks from many virtual streams, with block-to-spectrum latency.

A virtual stream emits blocks of its own shape.  With a sample rate r its
block spans ``samples_per_block / r`` seconds of sky; Poisson arrivals draw
the gaps between its blocks from an exponential distribution with that mean.
Every block is submitted to a ``Server`` at its arrival time (host blocks are
shared read-only buffers, one set per stream shape) and its latency is the
server-clock time from ``gspec_submit`` to the output on the host.
"""
from __future__ import annotations

import threading
import time

import numpy as np

from .serving import Server, make_config


def block_samples(spec) -> int:
    return spec.samples_per_pol * spec.npol


def poisson_plan(specs: list, rate_per_stream: float, total_blocks: int, seed: int = 4) -> list:
    """[(t_arrival_s, stream_index)] sorted by time: each stream a Poisson
    process with mean gap block_samples / rate_per_stream, cut at the time by
    which total_blocks blocks have arrived."""
    rng = np.random.default_rng(seed)
    spans = np.array([block_samples(s) / rate_per_stream for s in specs])
    # expected blocks per second over all streams -> horizon for total_blocks
    horizon = total_blocks / float(np.sum(1.0 / spans)) * 1.2 + spans.max()
    ev = []
    for i, span in enumerate(spans):
        t = rng.exponential(span)
        while t < horizon:
            ev.append((t, i))
            t += rng.exponential(span)
    ev.sort()
    return ev[:total_blocks]


def burst_plan(specs: list, blocks_per_stream: list) -> list:
    """Every block arrives at t = 0 (the server's peak rate), interleaved
    across streams."""
    ev = []
    for i, n in enumerate(blocks_per_stream):
        ev += [(0.0, i, k) for k in range(n)]
    ev.sort(key=lambda e: (e[2], e[1]))
    return [(t, i) for t, i, _ in ev]


def span_priorities(specs: list, levels: int = 2) -> dict:
    """CUDA stream priority per stream shape: the shapes with the shortest
    blocks get the highest priority (most negative), so their kernels are
    dispatched ahead of queued work of long blocks."""
    sizes = sorted({block_samples(s) for s in specs})
    out = {}
    for s in specs:
        rank = sizes.index(block_samples(s))          # 0 = shortest block
        out[s.name] = -max(0, (levels - 1) - rank * (levels - 1) // max(1, len(sizes) - 1))
    return out


def run(specs: list, host_blocks: dict, plan: list, memory_budget: int, device: int = 0,
        tunes: dict | None = None, flags: int = 0, keep_outputs: bool = False,
        priorities: dict | None = None, inflight_bytes: int = 0) -> dict:
    """Serves ``plan`` and returns the per-block records and totals.

    ``host_blocks[name]`` is the list of (pinned) host blocks a stream of that
    shape cycles through; ``tunes[name]`` its schedule overrides and
    ``priorities[name]`` its CUDA stream priority."""
    srv = Server(memory_budget, device=device, inflight_bytes=inflight_bytes)
    try:
        ids = [srv.open(make_config(s, device=device, flags=flags, tune=(tunes or {}).get(s.name),
                                    priority=(priorities or {}).get(s.name, 0))) for s in specs]
        sid_index = {sid: i for i, sid in enumerate(ids)}
        counts = [0] * len(specs)
        # admission and one warm-up block per stream before the clock starts
        deadline = time.time() + 120.0
        while any(srv.state(sid) == 0 for sid in ids) and time.time() < deadline:
            time.sleep(0.005)
        for i, sid in enumerate(ids):
            srv.submit(sid, host_blocks[specs[i].name][0], tag=counts[i])
            counts[i] += 1
        warm = 0
        while warm < len(ids):
            for r in srv.poll(256, 100000):
                if r["status"] != 0:
                    raise RuntimeError(srv.last_error())
                warm += 1
        records = []
        outputs = {} if keep_outputs else None
        n_expected = len(plan)
        done = threading.Event()
        err = []
        launches0 = srv.kernel_launches()

        def poller():
            got = 0
            while got < n_expected:
                for r in srv.poll(256, 100000, copy=keep_outputs):
                    got += 1
                    if r["data"] is not None and not keep_outputs:
                        srv.release(r["stream"], r["buffer"])     # the spectrum is not kept
                    i = sid_index[r["stream"]]
                    records.append((i, r["block_index"], r["t_submit"], r["t_start"], r["t_done"], r["status"],
                                    r["data"] is not None, r["h2d_ms"], r["wait_ms"], r["chain_ms"], r["d2h_ms"],
                                    r["issue_ms"], r["observe_ms"]))
                    if r["status"] != 0:
                        err.append(srv.last_error())
                    if keep_outputs and r["data"] is not None:
                        outputs.setdefault(i, []).append(r["data"])
            done.set()

        th = threading.Thread(target=poller, daemon=True)
        th.start()
        t0 = srv.now()
        for t_arr, i in plan:
            wait = t0 + t_arr - srv.now()
            if wait > 0:
                time.sleep(wait)
            blocks = host_blocks[specs[i].name]
            k = counts[i]
            counts[i] += 1
            srv.submit(ids[i], blocks[k % len(blocks)], tag=k)
        done.wait()
        t1 = max(r[4] for r in records)
        launches = srv.kernel_launches() - launches0
        for sid in ids:
            srv.close_stream(sid)
    finally:
        srv.close()
    if err:
        raise RuntimeError(f"serving errors: {err[:3]}")
    rec = np.array([(r[0], r[1], r[2], r[3], r[4], r[7], r[8], r[9], r[10], r[11], r[12]) for r in records])
    samples = sum(block_samples(specs[int(i)]) for i in rec[:, 0])
    return {"records": rec, "elapsed_s": t1 - t0, "samples": samples,
            "gsamples_per_s": samples / (t1 - t0) / 1e9, "launches": launches, "outputs": outputs}


def latency_summary(res: dict, specs: list, rate_per_stream: float | None = None) -> dict:
    """p50/p95/p99 of block-to-spectrum latency in ms, overall and per stream
    shape, and p99 over the block span when the rate is given."""
    rec = res["records"]
    lat = (rec[:, 4] - rec[:, 2]) * 1e3
    out = {"blocks": int(len(rec)), "p50_ms": float(np.percentile(lat, 50)),
           "p95_ms": float(np.percentile(lat, 95)), "p99_ms": float(np.percentile(lat, 99)), "by_shape": {}}
    names = sorted({s.name for s in specs})
    for name in names:
        sel = np.array([specs[int(i)].name == name for i in rec[:, 0]])
        if not sel.any():
            continue
        l = lat[sel]
        q = (rec[sel, 3] - rec[sel, 2]) * 1e3         # submit -> first copy issued (host queue)
        g = (rec[sel, 4] - rec[sel, 3]) * 1e3         # issued -> spectrum on the host (GPU side)
        d = {"blocks": int(sel.sum()), "p50_ms": float(np.percentile(l, 50)), "p95_ms": float(np.percentile(l, 95)),
             "p99_ms": float(np.percentile(l, 99)),
             "queue_p50_ms": float(np.percentile(q, 50)), "queue_p99_ms": float(np.percentile(q, 99)),
             "gpu_p50_ms": float(np.percentile(g, 50)), "gpu_p99_ms": float(np.percentile(g, 99))}
        for k, name_ in ((5, "h2d"), (6, "wait"), (7, "chain"), (8, "d2h"), (9, "issue"), (10, "observe")):
            v = rec[sel, k]
            d[f"{name_}_p50_ms"] = float(np.percentile(v, 50))
            d[f"{name_}_p99_ms"] = float(np.percentile(v, 99))
        if rate_per_stream:
            spec = next(s for s in specs if s.name == name)
            span_ms = block_samples(spec) / rate_per_stream * 1e3
            d["block_span_ms"] = span_ms
            d["p99_over_span"] = d["p99_ms"] / span_ms
        out["by_shape"][name] = d
    return out
