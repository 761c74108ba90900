"""Many streams on one GPU: the serving loop and the graph-batched step.

``Server`` wraps ``gspec_server_*`` (include/gspec.h): a native scheduler
thread admits streams by a device-memory budget, keeps each stream's state
resident on the GPU and overlaps the blocks of all admitted streams.
``Batch`` wraps ``gspec_batch_*``: a fixed set of uneven streams whose chains
run as the parallel branches of one CUDA graph, one graph launch per step.
Neither has a counterpart in the reference, which runs one
``GatedSpectrometer`` per process (``psrdada_cpp/effelsberg/edd/src/GatedSpectrometer_cli.cu``).
"""
from __future__ import annotations

import ctypes

import numpy as np

from .gated_spectrometer import (GspecConfig, GspecError, GspecInfo, DUAL_POL, FULL_STOKES, GSPEC_OK,
                                 INTENDED, POWER, SINGLE_POL, TUNE_KEYS, load_library)


class GspecServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget", ctypes.c_uint64), ("device", ctypes.c_int32), ("max_inflight", ctypes.c_int32),
                ("output_buffers", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("inflight_bytes", ctypes.c_uint64)]


class GspecResult(ctypes.Structure):
    _fields_ = [("stream", ctypes.c_int32), ("status", ctypes.c_int32), ("tag", ctypes.c_uint64),
                ("block_index", ctypes.c_uint64), ("data", ctypes.c_void_p), ("size", ctypes.c_uint64),
                ("buffer", ctypes.c_int32), ("reserved", ctypes.c_int32), ("t_submit", ctypes.c_double),
                ("t_start", ctypes.c_double), ("t_done", ctypes.c_double), ("h2d_ms", ctypes.c_float),
                ("wait_ms", ctypes.c_float), ("chain_ms", ctypes.c_float), ("d2h_ms", ctypes.c_float),
                ("issue_ms", ctypes.c_float), ("observe_ms", ctypes.c_float)]


def declare(lib) -> None:
    """ctypes prototypes of the serving and batch entry points."""
    vp, u64, sz, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_int
    cfgp = ctypes.POINTER(GspecConfig)
    lib.gspec_server_create.restype = vp
    lib.gspec_server_create.argtypes = [ctypes.POINTER(GspecServerConfig), ctypes.c_char_p, sz]
    lib.gspec_server_destroy.restype = None
    lib.gspec_server_destroy.argtypes = [vp]
    lib.gspec_stream_open.argtypes = [vp, cfgp, ctypes.POINTER(i32)]
    lib.gspec_stream_state.argtypes = [vp, i32]
    lib.gspec_submit.argtypes = [vp, i32, vp, sz, u64]
    lib.gspec_poll.argtypes = [vp, ctypes.POINTER(GspecResult), i32, i32]
    lib.gspec_server_release.argtypes = [vp, i32, i32]
    lib.gspec_stream_close.argtypes = [vp, i32]
    lib.gspec_server_now.restype = ctypes.c_double
    lib.gspec_server_now.argtypes = [vp]
    lib.gspec_server_memory_in_use.restype = u64
    lib.gspec_server_memory_in_use.argtypes = [vp]
    lib.gspec_server_kernel_launches.restype = u64
    lib.gspec_server_kernel_launches.argtypes = [vp]
    lib.gspec_server_last_error.restype = ctypes.c_char_p
    lib.gspec_server_last_error.argtypes = [vp]
    lib.gspec_batch_create.restype = vp
    lib.gspec_batch_create.argtypes = [cfgp, i32, ctypes.c_char_p, sz]
    lib.gspec_batch_destroy.restype = None
    lib.gspec_batch_destroy.argtypes = [vp]
    lib.gspec_batch_size.argtypes = [vp]
    lib.gspec_batch_get_info.argtypes = [vp, i32, ctypes.POINTER(GspecInfo)]
    lib.gspec_batch_input.restype = vp
    lib.gspec_batch_input.argtypes = [vp, i32]
    lib.gspec_batch_output.argtypes = [vp, i32, ctypes.POINTER(vp), ctypes.POINTER(u64), ctypes.POINTER(i32)]
    lib.gspec_batch_run.argtypes = [vp, vp]
    lib.gspec_batch_set_input.argtypes = [vp, i32, vp, sz, vp]
    lib.gspec_batch_read_output.argtypes = [vp, i32, vp, sz, vp]
    lib.gspec_batch_copy_output.argtypes = [vp, i32, vp, sz, vp]
    lib.gspec_batch_kernels_per_step.restype = u64
    lib.gspec_batch_kernels_per_step.argtypes = [vp]
    lib.gspec_batch_steps.restype = u64
    lib.gspec_batch_steps.argtypes = [vp]
    lib.gspec_batch_last_error.restype = ctypes.c_char_p
    lib.gspec_batch_last_error.argtypes = [vp]


def make_config(spec, device: int = 0, flags: int = 0, tune: dict | None = None,
                convention: int = INTENDED, priority: int = 0, form: int = 0) -> GspecConfig:
    """``GspecConfig`` of a ``synth.StreamSpec`` (selected side channel/bit, layout, shape);
    ``priority`` is the CUDA stream priority (negative = higher)."""
    return GspecConfig(stream_priority=priority, form=form,
        buffer_size=spec.buffer_size, heap_size=spec.heap_size, n_side_channels=spec.n_side_channels,
        selected_side_channel=spec.selected_side_channel, selected_bit=spec.selected_bit,
        fft_length=spec.fft_length, naccumulate=spec.naccumulate, nbits=spec.nbits,
        input_type=DUAL_POL if spec.dual_pol else SINGLE_POL,
        output_type=FULL_STOKES if spec.dual_pol else POWER, convention=convention,
        input_level=100.0, output_level=100.0, device=device, flags=flags,
        **{k: int(v) for k, v in (tune or {}).items() if k in TUNE_KEYS})


class Server:
    """Serving loop over ``gspec_server_*``.

    ``open(config)`` returns a stream id (admitted now or queued for
    admission); ``submit(stream, block, tag)`` queues a host block, which must
    stay alive and unchanged until its result comes back; ``poll()`` returns
    finished results as dicts, copying each output block out and releasing
    its buffer (``copy=False`` keeps the buffer until ``release``)."""

    def __init__(self, memory_budget: int, device: int = 0, max_inflight: int = 2, output_buffers: int = 2,
                 inflight_bytes: int = 0):
        self._lib = load_library()
        cfg = GspecServerConfig(memory_budget=int(memory_budget), device=device, max_inflight=max_inflight,
                                output_buffers=output_buffers, inflight_bytes=int(inflight_bytes))
        err = ctypes.create_string_buffer(512)
        s = self._lib.gspec_server_create(ctypes.byref(cfg), err, len(err))
        if not s:
            raise GspecError(err.value.decode())
        self._s = ctypes.c_void_p(s)
        self._keep = {}      # tag -> block kept alive until its result

    def close(self):
        if getattr(self, "_s", None):
            self._lib.gspec_server_destroy(self._s)
            self._s = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        return self._lib.gspec_server_last_error(self._s).decode()

    def open(self, config: GspecConfig) -> int:
        sid = ctypes.c_int(-1)
        if self._lib.gspec_stream_open(self._s, ctypes.byref(config), ctypes.byref(sid)) != GSPEC_OK:
            raise GspecError(self.last_error())
        return sid.value

    def state(self, stream: int) -> int:
        return self._lib.gspec_stream_state(self._s, stream)

    def submit(self, stream: int, block, tag: int) -> None:
        """``block``: a numpy uint8 array, a torch tensor or a (pointer, size)
        pair; ``tag`` identifies the block in its result.  Page-locked blocks
        (e.g. ``torch.empty(..., pin_memory=True)``) overlap their copy with
        other streams' work, and up to 64 MiB are read by SM loads, never
        queueing behind other streams' copies."""
        if isinstance(block, tuple):
            ptr, size = block
        elif isinstance(block, np.ndarray):
            ptr, size = block.ctypes.data, block.nbytes
            self._keep[(stream, tag)] = block
        else:                                      # a torch tensor (e.g. pinned host memory)
            ptr, size = block.data_ptr(), block.numel() * block.element_size()
            self._keep[(stream, tag)] = block
        rc = self._lib.gspec_submit(self._s, stream, ctypes.c_void_p(ptr), size, tag)
        if rc != GSPEC_OK:
            self._keep.pop((stream, tag), None)
            raise GspecError(self.last_error() or f"submit returned {rc}")

    def poll(self, max_results: int = 64, timeout_us: int = 1000, copy: bool = True) -> list:
        res = (GspecResult * max_results)()
        n = self._lib.gspec_poll(self._s, res, max_results, timeout_us)
        if n < 0:
            raise GspecError(self.last_error())
        out = []
        for r in res[:n]:
            d = {"stream": r.stream, "status": r.status, "tag": r.tag, "block_index": r.block_index,
                 "t_submit": r.t_submit, "t_start": r.t_start, "t_done": r.t_done, "buffer": r.buffer,
                 "h2d_ms": r.h2d_ms, "wait_ms": r.wait_ms, "chain_ms": r.chain_ms, "d2h_ms": r.d2h_ms,
                 "issue_ms": r.issue_ms, "observe_ms": r.observe_ms,
                 "size": r.size, "data": None}
            if r.data and copy:
                d["data"] = np.ctypeslib.as_array((ctypes.c_uint8 * r.size).from_address(r.data)).copy()
                self._lib.gspec_server_release(self._s, r.stream, r.buffer)
            elif r.data:
                d["data"] = np.ctypeslib.as_array((ctypes.c_uint8 * r.size).from_address(r.data))
            self._keep.pop((r.stream, r.tag), None)
            out.append(d)
        return out

    def release(self, stream: int, buffer: int) -> None:
        self._lib.gspec_server_release(self._s, stream, buffer)

    def close_stream(self, stream: int) -> None:
        self._lib.gspec_stream_close(self._s, stream)

    def now(self) -> float:
        return self._lib.gspec_server_now(self._s)

    def memory_in_use(self) -> int:
        return int(self._lib.gspec_server_memory_in_use(self._s))

    def kernel_launches(self) -> int:
        return int(self._lib.gspec_server_kernel_launches(self._s))


class Batch:
    """Uneven streams as the parallel branches of one CUDA graph (``gspec_batch_*``)."""

    def __init__(self, configs: list):
        self._lib = load_library()
        arr = (GspecConfig * len(configs))(*configs)
        err = ctypes.create_string_buffer(512)
        b = self._lib.gspec_batch_create(arr, len(configs), err, len(err))
        if not b:
            raise GspecError(err.value.decode())
        self._b = ctypes.c_void_p(b)
        self.n = len(configs)

    def close(self):
        if getattr(self, "_b", None):
            self._lib.gspec_batch_destroy(self._b)
            self._b = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self, i: int) -> GspecInfo:
        info = GspecInfo()
        if self._lib.gspec_batch_get_info(self._b, i, ctypes.byref(info)) != GSPEC_OK:
            raise GspecError("bad member index")
        return info

    def input_ptr(self, i: int) -> int:
        return int(self._lib.gspec_batch_input(self._b, i))

    def output(self, i: int):
        """(device pointer, bytes, complete) of member i's accumulator."""
        p, n, c = ctypes.c_void_p(), ctypes.c_uint64(), ctypes.c_int()
        self._lib.gspec_batch_output(self._b, i, ctypes.byref(p), ctypes.byref(n), ctypes.byref(c))
        return int(p.value or 0), int(n.value), bool(c.value)

    def set_input(self, i: int, block, stream: int = 0) -> None:
        """Copies a block (numpy array, torch tensor or (pointer, size)) into member i's input."""
        if isinstance(block, tuple):
            ptr, size = block
        elif isinstance(block, np.ndarray):
            ptr, size = block.ctypes.data, block.nbytes
        else:
            ptr, size = block.data_ptr(), block.numel() * block.element_size()
        rc = self._lib.gspec_batch_set_input(self._b, i, ctypes.c_void_p(ptr), size, ctypes.c_void_p(stream))
        if rc != GSPEC_OK:
            raise GspecError(self._lib.gspec_batch_last_error(self._b).decode())

    def read_output(self, i: int, stream: int = 0) -> np.ndarray:
        """Member i's output accumulator copied to the host (waits for the stream)."""
        _, n, _ = self.output(i)
        out = np.empty(n, np.uint8)
        rc = self._lib.gspec_batch_read_output(self._b, i, ctypes.c_void_p(out.ctypes.data), n,
                                               ctypes.c_void_p(stream))
        if rc != GSPEC_OK:
            raise GspecError(self._lib.gspec_batch_last_error(self._b).decode())
        return out

    def copy_output(self, i: int, dst, stream: int = 0) -> None:
        """Enqueues the copy of member i's accumulator into dst (a pinned torch
        tensor or (pointer, size)) on ``stream`` without waiting."""
        if isinstance(dst, tuple):
            ptr, size = dst
        else:
            ptr, size = dst.data_ptr(), dst.numel() * dst.element_size()
        rc = self._lib.gspec_batch_copy_output(self._b, i, ctypes.c_void_p(ptr), size, ctypes.c_void_p(stream))
        if rc != GSPEC_OK:
            raise GspecError(self._lib.gspec_batch_last_error(self._b).decode())

    def run(self, stream: int = 0) -> None:
        if self._lib.gspec_batch_run(self._b, ctypes.c_void_p(stream)) != GSPEC_OK:
            raise GspecError(self._lib.gspec_batch_last_error(self._b).decode())

    def kernels_per_step(self) -> int:
        return int(self._lib.gspec_batch_kernels_per_step(self._b))

    def steps(self) -> int:
        return int(self._lib.gspec_batch_steps(self._b))
