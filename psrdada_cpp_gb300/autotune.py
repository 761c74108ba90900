"""Project-written autotuner of the chain's schedule per stream shape.

For one stream shape it times the candidate schedules of the chain on
synthetic blocks of that shape on the GPU and keeps the fastest:

* shared-memory path (fft_length <= 4096): the number of work units a block
  is split into (``tune_units``: output spectra x slices), 1-8 per SM;
* four-step path: the split N = N1 x N2 (``tune_n1``; every power of two with
  N1 in [64, 1024] and N2 in [128, 1024]) and the scratch budget of one chunk
  of output spectra (``tune_scratch_mb``).

Each candidate is an ordinary handle (``gspec_create`` with the overrides);
its time is the mean of CUDA-event timed ``gspec_run_block_device`` passes
over device-resident blocks after warm-up.  Results are cached in a JSON file
keyed by device name and stream shape (``GSPEC_TUNE_CACHE``, default
``psrdada_cpp_gb300/_tune_cache.json``).  Every candidate computes the same
chain; only the order of floating-point sums changes between schedules, so a
tuned stream stays within the FP32 tolerance of the FP64 oracle.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

from . import synth
from .gated_spectrometer import FLAG_NO_HOST_BUFFERS, GatedSpectrometer, DadaBufferLayout, DUAL_POL, SINGLE_POL

CACHE = Path(os.environ.get("GSPEC_TUNE_CACHE", Path(__file__).resolve().parent / "_tune_cache.json"))


def shape_key(spec, device_name: str) -> str:
    return (f"{device_name}|nbits={spec.nbits}|dual={int(spec.dual_pol)}|fft={spec.fft_length}|"
            f"nacc={spec.naccumulate}|samples={spec.samples_per_pol}|heap={spec.heap_size}|"
            f"nsc={spec.n_side_channels}")


def candidates(spec, sm_count: int) -> list:
    """Schedules to try for one stream shape ({} is the built-in choice)."""
    N = spec.fft_length
    out = [{}]
    if N <= 4096:
        for per_sm in (1, 2, 8):
            out.append({"tune_units": per_sm * sm_count})
        return out
    for l1 in range(6, 11):
        n1 = 1 << l1
        if N % n1 == 0 and 128 <= N // n1 <= 1024:
            for mb in (256, 512, 1024):
                out.append({"tune_n1": n1, "tune_scratch_mb": mb})
    return out


def _make(spec, tune, device):
    lay = DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    from .gated_spectrometer import NullSink
    return GatedSpectrometer(lay, spec.selected_side_channel, spec.selected_bit, spec.fft_length, spec.naccumulate,
                             spec.nbits, 100.0, 100.0, NullSink(),
                             input_type=DUAL_POL if spec.dual_pol else SINGLE_POL, device=device,
                             flags=FLAG_NO_HOST_BUFFERS, tune=tune)


def time_schedule(spec, tune: dict, d_blocks: list, device: int = 0, steps: int = 8, warmup: int = 3) -> float:
    """Mean device ms per block of one schedule (CUDA events on one stream)."""
    import torch
    dev = torch.device("cuda", device)
    gs = _make(spec, tune, device)
    try:
        info = gs.info()
        d_out = torch.zeros(int(info.output_bytes), dtype=torch.uint8, device=dev)
        stream = torch.cuda.current_stream(dev)
        for i in range(warmup):
            gs.run_block_device(d_blocks[i % len(d_blocks)].data_ptr(), d_out.data_ptr(), stream.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(steps):
            gs.run_block_device(d_blocks[i % len(d_blocks)].data_ptr(), d_out.data_ptr(), stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / steps
    finally:
        gs.close()


def load_cache(path: Path = CACHE) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def tune(spec, device: int = 0, steps: int = 8, cache_path: Path = CACHE, force: bool = False,
         kind: str = "default") -> dict:
    """Best schedule of ``spec`` on ``device`` (cached); returns the tune dict."""
    import torch
    props = torch.cuda.get_device_properties(device)
    key = shape_key(spec, props.name)
    cache = load_cache(cache_path)
    if not force and key in cache:
        return dict(cache[key]["tune"])
    dev = torch.device("cuda", device)
    # distinct device blocks, together larger than L2, so every pass reads HBM
    l2 = int(getattr(props, "L2_cache_size", 0)) or (129 << 20)
    nrot = max(2, -(-2 * l2 // spec.buffer_size))
    host = [synth.make_block(spec, seed=5, block_index=i, kind=kind) for i in range(2)]
    d_blocks = [torch.from_numpy(host[i % 2]).to(dev) for i in range(min(nrot, 64))]
    results = []
    for cand in candidates(spec, props.multi_processor_count):
        try:
            ms = time_schedule(spec, cand, d_blocks, device, steps)
        except Exception as e:                    # a schedule the shape does not allow
            results.append({"tune": cand, "ms": None, "error": str(e)})
            continue
        results.append({"tune": cand, "ms": ms})
    ok = [r for r in results if r["ms"] is not None]
    best = min(ok, key=lambda r: r["ms"])
    cache[key] = {"tune": best["tune"], "ms": best["ms"], "default_ms": next(
        (r["ms"] for r in results if r["tune"] == {}), None), "tried": results}
    tmp = Path(str(cache_path) + ".tmp")
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, cache_path)
    return dict(best["tune"])
