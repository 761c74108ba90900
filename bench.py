"""Throughput benchmark of the GB300 gated spectrometer.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c3|c1|c2|c2m|c4|c5]
                    [--form bf16|fp16|fp32] [--impl gb300|reference]

One step = one DADA block of the workload through the whole chain (unpack,
gate, R2C, Stokes/power accumulate).  Default workload: dual-pol 12-bit gated
Stokes, fft 2^20 (four-step 1024 x 1024), naccumulate 8, 2^28 samples per pol
per block; the BF16 split-precision tensor-core form is ``value`` and the
plain FP32 form is timed on the same blocks in the same run (``forms``,
``tc_over_fp32``, and the two forms' spectral difference
``tc_vs_fp32_spectra``).

* ``value``   device throughput, input Gsamples/s (both pols), inputs resident
              in HBM: K blocks through gspec_run_block_device on the stream
              the kernels run on, timed with CUDA events.  Distinct device
              copies of the block rotate, at least 3x the L2 size per
              rotation, so every step reads its input from HBM.
* ``e2e``     the same metric through the public handler API
              (GatedSpectrometer.__call__ -> gspec_process) with blocks in
              pinned host memory: every step copies its block host->device and
              the pipeline copies one output block device->host.
* ``roofline`` per-kernel CUDA-event times of a profiled pass; the dominant
              kernel's algorithmic bytes per launch over its mean duration.
* ``cpu_baseline`` the C/OpenMP restatement of the chain (oracle/gspec_cpu.c)
              on this host's cores, on a bounded sample of the workload.

``--impl reference`` times that CPU restatement alone (the reference has no
CPU implementation of its own, and its GPU chain needs libpsrdada, Boost and
cuFFT, none of which is installed) on the same metric, each step one output spectrum's worth of
input.  Under torchrun every rank runs its own stream on its own GPU
(replicas, weak scaling); rank 0 prints the line.

``--workload c4`` times 16 uneven streams as one CUDA graph per step (and the
same members without the graph, and end to end from pinned host memory);
``--workload c5`` runs the serving loop: 32 mixed streams, a peak-rate burst,
then Poisson arrivals at 60 % of that rate, with block-to-spectrum latency.
"""
from __future__ import annotations

import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "input Gsamples/s gated Stokes, BF16-TC vs FP32 at ≤1e-4 err; p99 block latency"
UNIT = "Gsamples/s"
FALLBACK_HBM_GBS = 6800.0
L2_FALLBACK = 129 * 2**20                            # GB300 L2 size when the device does not report it


# ------------------------------------------------------------------ helpers
def workload(name: str, frames: int = 0):
    """(stream spec, sample kind) of a one-stream workload; frames > 0 shrinks its block
    to that many fft frames per pol (same kernels and launch shapes per chunk: for
    small ncu captures, never for a bench line)."""
    import dataclasses
    from psrdada_cpp_gb300 import synth
    if name == "c1":
        spec, kind = synth.config1(), "c1"
    elif name == "c3":
        spec, kind = synth.config3(), "c3"
    elif name == "c2m":
        # the diode period (61 heaps of 4096 samples) is not a whole number of 2^16-sample frames:
        # frames straddling a toggle hold data in both gates, the others in one
        c2 = synth.config2()
        spec, kind = dataclasses.replace(c2, name=c2.name + "_diode61", diode_period_heaps=61), "c2"
    else:
        spec, kind = synth.config2(), "c2"
    if frames > 0:
        if frames % spec.naccumulate:
            raise SystemExit(f"--frames must be a multiple of naccumulate ({spec.naccumulate})")
        spec = dataclasses.replace(spec, name=f"{spec.name}_frames{frames}", samples_per_pol=frames * spec.fft_length)
    return spec, kind


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(backend: str):
    import torch.distributed as dist
    ws, rank, _ = dist_env()
    if ws > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29511")
        dist.init_process_group(backend=backend, rank=rank, world_size=ws)
    return ws, rank


def dist_barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def dist_max(x: float, device=None) -> float:
    """Maximum of x over ranks (x itself on a single process)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(x: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            with open(path) as f:
                d = json.load(f)
            for key in ("hbm_gbs", "hbm_GBs", "hbm"):
                if key in d:
                    return float(d[key]), "measured", d
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback", {}


def ncu_traffic(kernel: str, workload_name: str):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith("#"):
                continue
            kv = dict(p.split("=", 1) for p in line.split() if "=" in p)
            if kv.get("kernel") == kernel and kv.get("workload") == workload_name:
                try:
                    return float(kv["dram_bytes_per_launch"])
                except (KeyError, ValueError):
                    return None
    return None


def bind_to_gpu_cpus(index: int, pci_bus_id: str | None = None):
    """Binds this process to the host CPUs NVML reports as local to the GPU
    (nvmlDeviceGetCpuAffinity, a read-only query), so that the page-locked
    blocks and outputs it writes first land on the GPU's NUMA node.  Returns
    the CPU list, or None where NVML or the call is unavailable."""
    import ctypes
    try:
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        ok = bool(pci_bus_id) and lib.nvmlDeviceGetHandleByPciBusId_v2(pci_bus_id.encode(), ctypes.byref(h)) == 0
        if not ok and lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(h)) != 0:
            return None
        words = 64
        mask = (ctypes.c_ulong * words)()
        if lib.nvmlDeviceGetCpuAffinity(h, ctypes.c_uint(words), mask) != 0:
            return None
        bits = ctypes.sizeof(ctypes.c_ulong) * 8
        cpus = {w * bits + b for w in range(words) for b in range(bits) if (mask[w] >> b) & 1}
        cpus &= os.sched_getaffinity(0)
        if not cpus:
            return None
        os.sched_setaffinity(0, cpus)
        return sorted(cpus)
    except (OSError, AttributeError, ValueError):
        return None


class ClockSampler:
    """SM clock, power and clock-event (throttle) reasons sampled while the
    GPU works: read-only NVML queries through ctypes every 20 ms on a host
    thread, or, where NVML cannot be loaded, one-shot nvidia-smi queries.
    Start it before the warm-up and stop it after the last GPU phase so a
    short timed region still has samples on both sides."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # NVML clock-event reason bits (nvml.h: nvmlClocksEventReason*)
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40,
            "hw_power_brake_slowdown": 0x80}

    def __init__(self, index: int, pci_bus_id: str | None = None, period_s: float = 0.02):
        self.index = index
        self.pci = pci_bus_id
        self.period = period_s
        self.samples = []            # (time, sm_mhz, max_mhz, power_w, set of reasons)
        self.source = None
        self._stop = threading.Event()
        self.thread = None

    def _nvml(self):
        import ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        h = ctypes.c_void_p()
        ok = False
        if self.pci:
            ok = lib.nvmlDeviceGetHandleByPciBusId_v2(self.pci.encode(), ctypes.byref(h)) == 0
        if not ok and lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.index), ctypes.byref(h)) != 0:
            raise OSError("no NVML handle")
        try:
            reasons_fn = lib.nvmlDeviceGetCurrentClocksEventReasons
        except AttributeError:
            reasons_fn = lib.nvmlDeviceGetCurrentClocksThrottleReasons
        clk, mx, pw, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))          # NVML_CLOCK_SM = 1

        def read():
            lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk))
            lib.nvmlDeviceGetPowerUsage(h, ctypes.byref(pw))
            reasons_fn(h, ctypes.byref(rs))
            names = {n for n, b in self.BITS.items() if rs.value & b}
            return float(clk.value), float(mx.value), pw.value / 1000.0, names
        read()
        return read

    def _smi(self):
        def read():
            out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                  "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                 timeout=5).stdout
            f = [x.strip() for x in out.strip().split(",")]
            names = {n for n, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                        "sw_power_cap"], f[5:9]) if v.lower() == "active"}
            return float(f[1]), float(f[2]), float(f[3]) if f[3] not in ("", "[N/A]") else 0.0, names
        read()
        return read

    def start(self):
        read = None
        for name, mk in (("nvml", self._nvml), ("nvidia-smi", self._smi)):
            try:
                read = mk()
                self.source = name
                break
            except Exception:
                continue
        if read is None:
            return

        def loop():
            while not self._stop.is_set():
                try:
                    t = time.time()
                    self.samples.append((t,) + read())
                except Exception:
                    pass
                self._stop.wait(self.period)
        self.thread = threading.Thread(target=loop, daemon=True)
        self.thread.start()
        t0 = time.time()
        while not self.samples and time.time() - t0 < 5:
            time.sleep(0.01)

    def stop(self):
        self._stop.set()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0: float, t1: float, busy=None):
        """Median SM clock and the reasons seen in [t0, t1]; when that window
        holds fewer than 3 samples, the busy window (t0', t1') around it
        (warm-up, timed and profiled passes of the same work) is used and
        named."""
        def pick(a, b):
            return [s for s in self.samples if a - 0.03 <= s[0] <= b + 0.03]
        sel, window = pick(t0, t1), "timed"
        if len(sel) < 3 and busy is not None:
            sel, window = pick(*busy), "warm-up + timed + profiled passes of the same work"
        if not sel:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "source": self.source}
        reasons = sorted(set().union(*[s[4] for s in sel]))
        return {"sm_mhz": statistics.median(s[1] for s in sel), "sm_max_mhz": max(s[2] for s in sel),
                "power_w_max": round(max(s[3] for s in sel), 1), "reasons": reasons, "samples": len(sel),
                "window": window, "source": self.source}


def pci_bus_id(dev) -> str | None:
    """NVML-style PCI bus id of a torch CUDA device, when torch reports it."""
    import torch
    p = torch.cuda.get_device_properties(dev)
    if hasattr(p, "pci_bus_id") and hasattr(p, "pci_domain_id"):
        return "%08X:%02X:%02X.0" % (p.pci_domain_id, p.pci_bus_id, getattr(p, "pci_device_id", 0))
    return None


TC_FLOPS_PER_DFT1024 = 2 * 12 * 128 * 64 * 16 * 2 / 4     # 2 stages x 12 MMAs (M128 N64 K16) per 4 transforms
FALLBACK_BF16_TFLOPS = 1900.0


def jobs_per_block(spec) -> int:
    """FFT jobs of one block of a bench workload (no lost heaps): dual pol,
    one per (frame, gate with data); single pol, one per frame with both gates
    plus one per two single-gate frames of the same output spectrum."""
    from psrdada_cpp_gb300 import synth
    items = synth.diode_items(spec, 0)[0]
    state = ((items[spec.selected_side_channel::spec.n_side_channels] >> np.uint64(spec.selected_bit)) & np.uint64(1))
    sph = spec.heap_size * 8 // spec.nbits
    per_sample = np.repeat(state.astype(np.int8), sph)[:spec.samples_per_pol]
    frames = per_sample.reshape(-1, spec.fft_length)
    has1 = frames.max(axis=1) == 1
    has0 = frames.min(axis=1) == 0
    if spec.dual_pol:
        return int(has0.sum() + has1.sum())
    per_out = max(1, (spec.samples_per_pol // spec.fft_length) // max(1, spec.naccumulate))
    mixed = (has0 & has1).reshape(-1, per_out) if frames.shape[0] % per_out == 0 else (has0 & has1)[None]
    single = (has0 ^ has1).reshape(mixed.shape)
    return int(mixed.sum() + np.ceil(single.sum(axis=1) / 2).sum())


def tensor_roofline(spec, info, form, kernels, nprof, G):
    """Tensor-core work of the split-precision forms: MMA flops per block
    over the device time of the passes that run on the tensor cores."""
    if form == G.FORM_FP32 or int(info.fft_path) != 1:
        return None
    n1, n2 = int(info.n1), int(info.n2)
    jobs = jobs_per_block(spec)
    transforms = jobs * ((n2 if n1 == 1024 else 0) + (n1 if n2 == 1024 else 0))
    flops = transforms * TC_FLOPS_PER_DFT1024
    ms = sum(kernels[k][2] for k in ("fourstep_a", "fourstep_b") if k in kernels
             and ((k == "fourstep_a" and n1 == 1024) or (k == "fourstep_b" and n2 == 1024))) / nprof
    ach = flops / (ms / 1e3) / 1e12 if ms > 0 else None
    _, _, peaks = measured_peaks()
    if "bf16_tflops" in peaks:
        peak, source = float(peaks["bf16_tflops"]), "measured dense bf16 (cuBLAS burst)"
    else:
        peak, source = FALLBACK_BF16_TFLOPS, "fallback dense bf16 (no measured peak file)"
    return {"bound": "tensor", "mma_flops_per_block": flops, "dft1024_per_block": transforms,
            "tensor_pass_ms_per_block": round(ms, 4), "achieved_tflops": round(ach, 2) if ach else None,
            "peak_tflops": peak, "peak_source": source, "frac": round(ach / peak, 5) if ach else None}


def cpu_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def sample_spec(spec, n_out: int):
    """A bounded sample of the workload: the same stream with fewer output
    spectra per block."""
    from psrdada_cpp_gb300 import synth
    import dataclasses
    per_out = spec.fft_length * spec.naccumulate
    return dataclasses.replace(spec, name=spec.name + f"_sample{n_out}", samples_per_pol=per_out * n_out)


def cpu_chain_rate(spec, kind: str, seconds: float = 10.0, max_blocks: int = 1 << 20):
    """Times the C restatement on all host cores; returns (Gsamples/s, cores,
    sample description)."""
    from oracle import gspec_cpu
    from psrdada_cpp_gb300 import synth
    cores = cpu_cores()
    n_out = max(1, min(4, spec.samples_per_pol // (spec.fft_length * spec.naccumulate)))
    sub = sample_spec(spec, n_out) if spec.samples_per_pol > spec.fft_length * spec.naccumulate else spec
    chain = gspec_cpu.CpuChain(sub, nthreads=cores)
    blocks = [synth.make_block(sub, seed=1, block_index=i, kind=kind) for i in range(2)]
    chain.run_block(blocks[0])                       # warm-up
    n, t0 = 0, time.perf_counter()
    while n < max_blocks:
        chain.zero()
        chain.run_block(blocks[n % 2])
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    samples = n * sub.samples_per_pol * sub.npol
    desc = (f"{n} blocks of {sub.samples_per_pol} samples/pol ({n_out} output spectra each) of {spec.name}, "
            f"{dt:.1f} s on {cores} threads (parallel over the frames of each output spectrum)")
    return samples / dt / 1e9, cores, desc


# ---------------------------------------------------------------- GPU arm
FORM_DTYPE = {"fp32": "f32",
              "bf16": "bf16 split operands (column pass 2x3 parts, row pass 3x3), f32 accumulate",
              "fp16": "f16 hi+lo operands, f32 accumulate"}


def stokes_rel_err(got: np.ndarray, ref: np.ndarray, dual: bool, floor: float = 1e-2):
    """Per-bin relative difference of two output records' spectra (Stokes
    products normalised by I of the same bin), denominators floored at
    ``floor`` x the spectrum's mean; returns (max, rms, per product max)."""
    got = got.astype(np.float64)
    ref = ref.astype(np.float64)
    base = np.abs(ref[:, 0:1]) if dual else np.abs(ref)
    denom = np.maximum(base, floor * base.mean(axis=-1, keepdims=True))
    denom = np.where(denom == 0, 1.0, denom)
    e = np.abs(got - ref) / denom
    names = "IQUV" if dual else ("G0", "G1")
    by = {n: float(e[:, i].max()) for i, n in enumerate(names)}
    return float(e.max()), float(np.sqrt(np.mean(e * e))), by


def record_spectra(buf: np.ndarray, n_out: int, C: int, dual: bool) -> np.ndarray:
    rec = buf[:n_out * ((8 if dual else 2) * (4 * C + 8))].reshape(n_out, -1)
    f = rec[:, :(8 if dual else 2) * 4 * C].copy().view("<f4")
    return f.reshape(n_out, 4, 2, C) if dual else f.reshape(n_out, 2, C)


def measure_form(args, form_name, spec, kind, host_blocks, d_blocks, dev, clocks):
    """Times one arithmetic form of the chain on the workload: device
    throughput (value), per-kernel roofline, end-to-end through the handler.
    Returns the form's result dict and its first output block (host copy)."""
    import torch
    import psrdada_cpp_gb300 as G
    ws, rank = dist_env()[0], dist_env()[1]
    local = dev.index
    form = {"fp32": G.FORM_FP32, "bf16": G.FORM_BF16, "fp16": G.FORM_FP16}[form_name]
    samples_per_step = spec.samples_per_pol * spec.npol
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    mk = dict(input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL, device=local, form=form)
    gs = G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 100.0, 100.0,
                             G.NullSink(), **mk)
    info = gs.info()
    nrot = len(d_blocks)
    d_out = torch.zeros(int(info.output_bytes), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    def step(i):
        # the caller's part of the contract: clear the output at the start of an output block
        # (the counters only when each block holds whole outputs)
        if i % int(info.n_blocks) == 0:
            gs.clear_output_device(d_out.data_ptr(), sptr)
        gs.run_block_device(d_blocks[i % nrot].data_ptr(), d_out.data_ptr(), sptr)

    # first output block from the zero baselines, kept for the form comparison
    step(0)
    torch.cuda.synchronize(dev)
    first = d_out.cpu().numpy().copy()
    gs.set_baselines(np.zeros(4, np.float32))
    busy0 = time.time()
    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize(dev)

    # ---- device throughput (value)
    launches0 = gs.info().kernel_launches
    dist_barrier()
    torch.cuda.synchronize(dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tw0 = time.time()
    ev0.record(stream)
    for i in range(args.steps):
        step(i)
    ev1.record(stream)
    torch.cuda.synchronize(dev)
    tw1 = time.time()
    dist_barrier()
    launches = gs.info().kernel_launches - launches0
    ms = ev0.elapsed_time(ev1)
    ms_max = dist_max(ms, dev)
    total_samples = dist_sum(samples_per_step * args.steps, dev)
    value = total_samples / (ms_max / 1e3) / 1e9

    # ---- per-kernel profile (roofline): CUDA events on the chain's stream
    gs.reset_profile()
    gs.set_profiling(True)
    nprof = max(4, min(32, args.steps))
    for i in range(nprof):
        step(i)
    prof = gs.profile()
    gs.set_profiling(False)
    torch.cuda.synchronize(dev)
    busy1 = time.time()
    clk = clocks.summary(tw0, tw1, busy=(busy0, busy1))
    kernels = {k: v for k, v in prof.items() if v[1] > 0}
    tot_ms = sum(v[2] for v in kernels.values())
    dom = max(kernels, key=lambda k: kernels[k][2])
    d_launches, d_timed, d_ms = kernels[dom]
    per_launch_ms = d_ms / d_timed
    in_bytes = spec.buffer_size
    out_bytes = int(info.output_bytes)
    launches_per_block = {k: v[1] / nprof for k, v in kernels.items()}
    # engine stage names: "small_chain" is the shared-memory path's chain launch
    # (warp_chain_kernel for single-pol 1024-point frames), reading the block and
    # writing the records
    if dom in ("fourstep_a", "small_chain"):
        alg_bytes_launch = (in_bytes + (out_bytes if dom == "small_chain" else 0)) / launches_per_block[dom]
    elif dom == "fourstep_b":
        alg_bytes_launch = out_bytes / launches_per_block[dom]
    else:
        alg_bytes_launch = (in_bytes + out_bytes) / launches_per_block[dom]
    peak, peak_kind, _ = measured_peaks()
    achieved = alg_bytes_launch / (per_launch_ms / 1e3) / 1e9
    chain_ms = tot_ms / nprof
    chain_gbs = (in_bytes + out_bytes) / (chain_ms / 1e3) / 1e9
    N = spec.fft_length
    seqs = spec.npol                                     # complex FFTs per frame (pair trick)
    fft_flops = 5.0 * N * math.log2(N) * (spec.samples_per_pol // N) * seqs
    roofline = {
        "bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
        "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} copy bandwidth",
        "traffic": ncu_traffic(dom, spec.name if form_name == "fp32" else f"{spec.name}_{form_name}"),
        "algorithmic_bytes_per_launch": int(alg_bytes_launch), "mean_launch_ms": round(per_launch_ms, 4),
        "chain": {"ms_per_block": round(chain_ms, 4), "algorithmic_bytes_per_block": in_bytes + out_bytes,
                  "achieved_GBs": round(chain_gbs, 1), "frac": round(chain_gbs / peak, 4)},
        "kernels": {k: {"launches_per_block": round(launches_per_block[k], 3),
                        "mean_ms": round(v[2] / v[1], 4), "share": round(v[2] / tot_ms, 4)}
                    for k, v in kernels.items()},
        "fp32_fft": {"nominal_flops_per_block": fft_flops,
                     "achieved_tflops": round(fft_flops / (chain_ms / 1e3) / 1e12, 2)},
        "tensor": tensor_roofline(spec, info, form, kernels, nprof, G),
    }
    gs.close()
    del d_out

    # ---- end to end through the handler API, pinned host blocks
    e2e, lat = None, []
    if not args.no_e2e:
        pinned = []
        for b in host_blocks:
            t = torch.empty(b.size, dtype=torch.uint8, pin_memory=True)
            t.numpy()[:] = b
            pinned.append(t)
        ge = G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 100.0, 100.0,
                                 G.NullSink(), **mk)
        raws = [G.RawBytes(p.numpy()) for p in pinned]
        for i in range(max(3, args.warmup)):
            ge(raws[i % len(raws)])
        torch.cuda.synchronize(dev)
        ke = max(8, min(args.steps, 1000))
        dist_barrier()
        gc.disable()     # as timeit does: no collector pauses inside the timed loop
        t0 = time.perf_counter()
        for i in range(ke):
            c0 = time.perf_counter()
            ge(raws[i % len(raws)])
            lat.append((time.perf_counter() - c0) * 1e3)
        torch.cuda.synchronize(dev)
        t1 = time.perf_counter()
        gc.enable()
        dist_barrier()
        e_s = dist_max(t1 - t0, dev)
        e_val = dist_sum(samples_per_step * ke, dev) / e_s / 1e9
        outputs_per_step = 1.0 / int(info.n_blocks)
        e2e = {"value": round(e_val, 3), "unit": UNIT, "h2d_bytes_per_step": spec.buffer_size,
               "d2h_bytes_per_step": int(out_bytes * outputs_per_step), "steps": ke,
               "api": "GatedSpectrometer.__call__ -> gspec_process (pinned host blocks)"}
        ge.close()
        del pinned, raws
    res = {"value": round(value, 3), "ms_per_step": round(ms_max / args.steps, 4), "dtype": FORM_DTYPE[form_name],
           "gpu_launches": int(launches), "clocks": clk, "roofline": roofline, "e2e": e2e,
           "n1": int(info.n1), "n2": int(info.n2)}
    if lat:
        res["latency_ms"] = {"p50": round(float(np.percentile(lat, 50)), 3),
                             "p95": round(float(np.percentile(lat, 95)), 3),
                             "p99": round(float(np.percentile(lat, 99)), 3),
                             "what": "host time of one handler call (H2D of the block, launch of the chain, "
                                     "output D2H issue)"}
    return res, first, info


def run_gpu(args):
    import torch
    ws, rank = dist_init("nccl")
    _, _, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from psrdada_cpp_gb300 import synth

    spec, kind = workload(args.workload, args.frames)
    forms = [args.form] + ([] if args.form == "fp32" or args.no_compare else ["fp32"])
    # host buffers on the GPU's NUMA node: run on the CPUs local to the GPU before any are written
    all_cpus = os.sched_getaffinity(0)
    host_cpus = bind_to_gpu_cpus(local, pci_bus_id(dev))
    # two host blocks where they are cheap to make; one (used twice) at 2^28 samples/pol
    nhost = 1 if spec.samples_per_pol >= (1 << 27) else 2
    host_blocks = [synth.make_block(spec, seed=1 + rank, block_index=i, kind=kind) for i in range(nhost)]
    # distinct device copies rotate so that one rotation is at least 3x the L2 size: every step
    # reads its block from HBM, not from the previous step's L2 lines
    l2_bytes = int(getattr(torch.cuda.get_device_properties(dev), "L2_cache_size", 0)) or L2_FALLBACK
    nrot = max(2, -(-3 * l2_bytes // spec.buffer_size))
    d_blocks = [torch.from_numpy(host_blocks[i % nhost]).to(dev) for i in range(nrot)]
    clocks = ClockSampler(local, pci_bus_id(dev))
    clocks.start()
    results, firsts, info = {}, {}, None
    for f in forms:
        results[f], firsts[f], info = measure_form(args, f, spec, kind, host_blocks, d_blocks, dev, clocks)
    clocks.stop()
    del d_blocks

    cpu = None
    if rank == 0 and not args.no_cpu:
        os.sched_setaffinity(0, all_cpus)   # the CPU baseline uses every host core
        try:
            v, cores, desc = cpu_chain_rate(spec, kind, seconds=args.cpu_seconds)
            cpu = {"value": round(v, 4), "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
        except Exception as exc:  # the CPU leg never hides a GPU result
            cpu = {"value": None, "unit": UNIT, "cores": cpu_cores(), "kind": "port", "sample": f"failed: {exc}"}

    if rank == 0:
        main = results[args.form]
        if args.workload == "c3" and len(forms) > 1:
            metric = METRIC
        else:
            metric = (f"input Gsamples/s gated {'Stokes' if spec.dual_pol else 'power'}, {args.form} form"
                      + (" (fp32 form beside it)" if len(forms) > 1 else ""))
        line = {
            "metric": metric, "value": main["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": main["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": main["dtype"], "data": "synthetic",
            "config": {"workload": spec.name, "fft_length": spec.fft_length, "naccumulate": spec.naccumulate,
                       "nbits": spec.nbits, "pols": spec.npol, "samples_per_pol_per_block": spec.samples_per_pol,
                       "block_bytes": spec.buffer_size, "form": args.form, "n1": main["n1"], "n2": main["n2"],
                       "diode_period_heaps": spec.diode_period_heaps,
                       "host_cpus": ("%d CPUs local to the GPU (NVML affinity)" % len(host_cpus)) if host_cpus
                       else "unbound",
                       "l2": "inputs larger than L2: %d device blocks of %d B rotate (L2 %d B)"
                             % (nrot, spec.buffer_size, l2_bytes),
                       "parallelism": f"replicas x{ws} (one independent stream per GPU)"},
            "e2e": main["e2e"], "gpu_launches": main["gpu_launches"], "clocks": main["clocks"],
            "roofline": main["roofline"], "cpu_baseline": cpu,
        }
        if "latency_ms" in main:
            line["latency_ms"] = main["latency_ms"]
        if len(forms) > 1:
            fp = results["fp32"]
            line["forms"] = {f: {k: r[k] for k in ("value", "ms_per_step", "dtype", "e2e", "roofline", "clocks",
                                                   "gpu_launches")} for f, r in results.items()}
            line["tc_over_fp32"] = {"value": round(main["value"] / fp["value"], 4),
                                    "e2e": (round(main["e2e"]["value"] / fp["e2e"]["value"], 4)
                                            if main["e2e"] and fp["e2e"] else None),
                                    "target": 3.0}
            mx, rms, by = stokes_rel_err(
                record_spectra(firsts[args.form], int(info.n_out), int(info.nchans), spec.dual_pol),
                record_spectra(firsts["fp32"], int(info.n_out), int(info.nchans), spec.dual_pol),
                spec.dual_pol)
            line["tc_vs_fp32_spectra"] = {
                "max_rel": mx, "rms_rel": rms, "by_product_max": by,
                "what": "first output block of the same input through both forms; per-bin |diff| over I of the "
                        "bin (floor 1 % of the mean I). The FP32 form is itself within 1e-5 of the FP64 oracle "
                        "(GPU parity tests), so this bounds the tensor-core form's error to within 1e-5"}
        print(json.dumps(line), flush=True)


# ------------------------------------------------- batched uneven streams
def run_batch(args):
    """16 uneven streams (synth.uneven_streams, seed 3) as one CUDA graph per
    step: every member processes one device-resident block per step.  Also
    times the same members one after another without the graph, and end to
    end with the blocks copied from pinned host memory every step."""
    import torch
    ws, rank = dist_init("nccl")
    _, _, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    bind_to_gpu_cpus(local, pci_bus_id(dev))   # pinned buffers on the GPU's NUMA node
    import psrdada_cpp_gb300 as G
    from psrdada_cpp_gb300 import synth, autotune
    specs = synth.uneven_streams(16, seed=3)
    t_tune = time.time()
    tunes = {s.name: ({} if args.no_tune else autotune.tune(s, device=local, steps=4)) for s in specs}
    t_tune = time.time() - t_tune
    host = [synth.make_block(s, seed=7 + rank, block_index=0) for s in specs]
    samples_per_step = sum(s.samples_per_pol * s.npol for s in specs)
    in_bytes = sum(s.buffer_size for s in specs)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    # the tensor-core forms apply to members with a 1024-point four-step pass
    form = {"fp32": G.FORM_FP32, "bf16": G.FORM_BF16, "fp16": G.FORM_FP16}[args.form]
    forms = {s.name: (form if (1 << 16) <= s.fft_length <= (1 << 20) else G.FORM_FP32) for s in specs}
    if form != G.FORM_FP32:
        tunes = {k: ({} if forms[k] != G.FORM_FP32 else v) for k, v in tunes.items()}
    bt = G.Batch([G.make_config(s, device=local, tune=tunes[s.name], form=forms[s.name]) for s in specs])
    for i, h in enumerate(host):
        bt.set_input(i, h, sp)
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local, pci_bus_id(dev))
    clocks.start()
    busy0 = time.time()
    for _ in range(args.warmup):
        bt.run(sp)
    torch.cuda.synchronize(dev)
    steps = args.steps
    dist_barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tw0 = time.time()
    e0.record(stream)
    for _ in range(steps):
        bt.run(sp)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    tw1 = time.time()
    dist_barrier()
    ms = dist_max(e0.elapsed_time(e1), dev)
    value = dist_sum(samples_per_step * steps, dev) / (ms / 1e3) / 1e9
    kernels = bt.kernels_per_step()

    # the same members one after another, no graph
    seq = []
    d_out = []
    for i, s in enumerate(specs):
        lay = G.DadaBufferLayout(s.buffer_size, s.heap_size, s.n_side_channels)
        g = G.GatedSpectrometer(lay, 0, 0, s.fft_length, s.naccumulate, s.nbits, 1.0, 1.0, G.NullSink(),
                                input_type=G.DUAL_POL if s.dual_pol else G.SINGLE_POL, device=local,
                                flags=G.FLAG_NO_HOST_BUFFERS, tune=tunes[s.name], form=forms[s.name])
        seq.append(g)
        d_out.append(torch.zeros(int(g.info().output_bytes), dtype=torch.uint8, device=dev))
    d_in = [torch.from_numpy(h).to(dev) for h in host]
    ks = max(4, steps // 4)
    for _ in range(2):
        for g, di, do in zip(seq, d_in, d_out):
            g.run_block_device(di.data_ptr(), do.data_ptr(), sp)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(ks):
        for g, di, do in zip(seq, d_in, d_out):
            g.run_block_device(di.data_ptr(), do.data_ptr(), sp)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    busy1 = time.time()
    clocks.stop()
    seq_value = samples_per_step * ks / (e0.elapsed_time(e1) / 1e3) / 1e9
    for g in seq:
        g.close()
    del d_in, d_out

    # end to end: pinned host blocks in, completed outputs out, every step.
    # The blocks of step k + 1 go in on a copy stream while step k runs (the
    # batch alternates two input buffers); outputs leave on the compute stream.
    pinned = []
    for h in host:
        t = torch.empty(h.size, dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = h
        pinned.append(t)
    outs = [torch.empty(int(bt.info(i).output_bytes), dtype=torch.uint8, pin_memory=True) for i in range(bt.n)]
    ke = max(4, min(steps, 64))
    copy_stream = torch.cuda.Stream(dev)
    cs = copy_stream.cuda_stream
    copied = [torch.cuda.Event() for _ in range(ke)]
    ran = [torch.cuda.Event() for _ in range(ke)]
    d2h = 0
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()

    def put(k):
        if k >= 2:
            copy_stream.wait_event(ran[k - 2])          # the buffer was last read by step k - 2
        for i, p_ in enumerate(pinned):
            bt.set_input(i, p_, cs)
        copied[k].record(copy_stream)

    put(0)
    for k in range(ke):
        stream.wait_event(copied[k])
        bt.run(sp)
        ran[k].record(stream)
        if k + 1 < ke:
            put(k + 1)
        for i in range(bt.n):
            _, n, complete = bt.output(i)
            if complete:
                bt.copy_output(i, outs[i], sp)
                d2h += n
    torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t0
    bt.close()
    if rank == 0:
        line = {
            "metric": "batched uneven streams: input Gsamples/s (16 streams, one CUDA graph per step)",
            "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": steps, "warmup": args.warmup,
            "ms_per_step": round(ms / steps, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "uneven_streams_16_seed3", "streams": [s.name for s in specs],
                       "samples_per_step": samples_per_step, "input_bytes_per_step": in_bytes, "form": args.form,
                       "forms": {k: int(v) for k, v in forms.items()},
                       "schedules": tunes, "tune_seconds": round(t_tune, 1),
                       "l2": "inputs larger than L2: the 16 members' blocks total %d B" % in_bytes},
            "sequential_no_graph": {"value": round(seq_value, 3), "unit": UNIT, "steps": ks},
            "e2e": {"value": round(samples_per_step * ke / e2e_s / 1e9, 3), "unit": UNIT,
                    "h2d_bytes_per_step": in_bytes, "d2h_bytes_per_step": int(d2h / ke), "steps": ke,
                    "api": "Batch.set_input (pinned, copy stream, one step ahead) -> gspec_batch_run -> "
                           "gspec_batch_copy_output (pinned)"},
            "gpu_launches": int(kernels * steps), "kernels_per_graph": int(kernels),
            "clocks": clocks.summary(tw0, tw1, busy=(busy0, busy1)),
        }
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------- serving loop
def run_serve(args):
    """32 virtual streams (16 of the 8-bit fft-1024 shape, 16 of the dual-pol
    12-bit fft-2^20 shape) through one Server: first every block of an
    equal-samples-per-stream workload at once (peak aggregate rate), then
    Poisson arrivals at 60 % of that rate until args.serve_blocks blocks."""
    # every served stream drives three CUDA streams; give them their own
    # hardware work queues (the default of 8 shares queues between streams,
    # so a short block can wait behind another stream's long kernels)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", str(args.connections))
    import torch
    ws, rank = dist_init("nccl")
    _, _, local = dist_env()
    torch.cuda.set_device(local)
    bind_to_gpu_cpus(local, pci_bus_id(torch.device("cuda", local)))   # pinned buffers on the GPU's NUMA node
    import psrdada_cpp_gb300 as G
    from psrdada_cpp_gb300 import synth, loadgen, autotune
    c1, c3 = synth.config1(), synth.config3()
    specs = [c1] * 16 + [c3] * 16
    tunes = {} if args.no_tune else {s.name: autotune.tune(s, device=local, steps=4) for s in (c1, c3)}

    def pinned(arr):
        t = torch.empty(arr.size, dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = arr
        return t

    host = {c1.name: [pinned(synth.make_block(c1, seed=4, block_index=i, kind="c1")) for i in range(2)],
            c3.name: [pinned(synth.make_block(c3, seed=4, block_index=0, kind="c3"))]}
    budget = int(args.budget_gb * 2**30)
    ratio = (c3.samples_per_pol * c3.npol) // (c1.samples_per_pol * c1.npol)
    m = args.serve_peak_blocks
    burst = loadgen.burst_plan(specs, [m * ratio] * 16 + [m] * 16)
    prios = {} if args.no_priority else loadgen.span_priorities(specs)
    infl = args.inflight_long * host[c3.name][0].numel()
    peak = loadgen.run(specs, host, burst, budget, device=local, tunes=tunes, priorities=prios, inflight_bytes=infl)
    rate = 0.6 * peak["gsamples_per_s"] * 1e9 / len(specs)
    plan = loadgen.poisson_plan(specs, rate, args.serve_blocks, seed=4)
    clocks = ClockSampler(local, pci_bus_id(torch.device("cuda", local)))
    clocks.start()
    tw0 = time.time()
    res = loadgen.run(specs, host, plan, budget, device=local, tunes=tunes, priorities=prios, inflight_bytes=infl)
    tw1 = time.time()
    clocks.stop()
    lat = loadgen.latency_summary(res, specs, rate)
    if rank == 0:
        worst = max(v["p99_over_span"] for v in lat["by_shape"].values())
        line = {
            "metric": "serving: input Gsamples/s and p50/p95/p99 block-to-spectrum latency (32 mixed streams)",
            "value": round(res["gsamples_per_s"], 3), "unit": UNIT, "n_gpus": ws, "steps": int(lat["blocks"]),
            "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "serving_32_streams_c1x16_c3x16", "arrivals": "Poisson, seed 4",
                       "offered_rate_gsps": round(0.6 * peak["gsamples_per_s"], 3),
                       "peak_gsps": round(peak["gsamples_per_s"], 3), "peak_blocks": len(burst),
                       "memory_budget_bytes": budget, "inflight_bytes": infl, "schedules": tunes,
                       "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                       "stream_priorities": prios,
                       "form": "fp32"},
            "latency_ms": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in lat.items()
                           if k != "by_shape"},
            "latency_by_shape": {k: {kk: round(vv, 4) if isinstance(vv, float) else vv for kk, vv in v.items()}
                                 for k, v in lat["by_shape"].items()},
            "worst_p99_over_block_span": round(worst, 4),
            "elapsed_s": round(res["elapsed_s"], 3), "gpu_launches": int(res["launches"]),
            "e2e": {"value": round(res["gsamples_per_s"], 3), "unit": UNIT,
                    "api": "Server.submit (pinned host blocks) -> gspec_poll (spectra on the host)"},
            "clocks": clocks.summary(tw0, tw1),
        }
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------- reference arm
def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import gspec_cpu
    from psrdada_cpp_gb300 import synth
    spec, kind = workload(args.workload)
    sub = sample_spec(spec, 1)
    cores = cpu_cores()
    chain = gspec_cpu.CpuChain(sub, nthreads=cores)
    blocks = [synth.make_block(sub, seed=1, block_index=i, kind=kind) for i in range(2)]
    for i in range(args.warmup):
        chain.zero()
        chain.run_block(blocks[i % 2])
    times = []
    t0 = time.perf_counter()
    for i in range(args.steps):
        c0 = time.perf_counter()
        chain.zero()
        chain.run_block(blocks[i % 2])
        times.append(time.perf_counter() - c0)
        if time.perf_counter() - t0 > args.ref_budget_s:
            break
    dt = time.perf_counter() - t0
    k = len(times)
    samples = k * sub.samples_per_pol * sub.npol
    v = samples / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": ws, "steps": k,
        "warmup": args.warmup, "ms_per_step": round(dt / k * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": spec.name, "fft_length": spec.fft_length, "naccumulate": spec.naccumulate,
                   "nbits": spec.nbits, "pols": spec.npol, "form": "fp32",
                   "step": f"one output spectrum of input ({sub.samples_per_pol} samples/pol)"},
        "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{k} steps of {sub.samples_per_pol} samples/pol of {spec.name}; the C/OpenMP "
                                   f"restatement of the chain (the reference's own path is CUDA-only)"},
        "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if k < args.steps:
        line["steps_requested"] = args.steps
    print(json.dumps(line), flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["c1", "c2", "c2m", "c3", "c4", "c5"], default="c3",
                    help="c1-c3 one stream (c2m: c2 with a 61-heap diode period); c4 16 uneven streams in one "
                         "CUDA graph; c5 the serving loop")
    ap.add_argument("--form", choices=["fp32", "bf16", "fp16"], default=None,
                    help="FFT arithmetic: FP32 CUDA cores, or tensor-core DFT-32 stages with split BF16/FP16 "
                         "operands (default: bf16 for c3, fp32 otherwise)")
    ap.add_argument("--no-compare", action="store_true",
                    help="time only --form (by default a tensor-core form is timed beside the FP32 form)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--frames", type=int, default=0,
                    help="c1-c3: shrink the block to this many fft frames per pol (small cases for ncu captures; "
                         "its lines are not the workload's bench line)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="wall seconds of the timed CPU sample")
    ap.add_argument("--ref-budget-s", type=float, default=150.0)
    ap.add_argument("--no-tune", action="store_true", help="c4/c5: built-in schedules instead of the autotuner's")
    ap.add_argument("--serve-blocks", type=int, default=10000, help="c5: blocks of the Poisson phase")
    ap.add_argument("--serve-peak-blocks", type=int, default=4, help="c5: fft-2^20 blocks per stream, peak phase")
    ap.add_argument("--budget-gb", type=float, default=120.0, help="c5: device memory budget of the server")
    ap.add_argument("--no-priority", action="store_true", help="c5: equal CUDA stream priorities")
    ap.add_argument("--inflight-long", type=int, default=0,
                    help="c5: fft-2^20 blocks on the GPU at once over all streams (0: no limit)")
    ap.add_argument("--connections", type=int, default=32, help="c5: CUDA_DEVICE_MAX_CONNECTIONS")
    args = ap.parse_args(argv)
    if args.form is None:
        args.form = "bf16" if args.workload == "c3" else "fp32"
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c4":
        run_batch(args)
    elif args.workload == "c5":
        run_serve(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
