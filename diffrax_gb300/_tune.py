"""Launch-shape autotuner and CUDA-graph replay of repeated solves.

The fused kernels take their launch shape from the problem descriptor
(``block_threads``: trajectories per CTA of the analytic-field kernels;
``ctas_per_sm``: resident CTAs, i.e. row tiles of the MLP kernels, per SM);
0 selects the built-in heuristic.  ``autotune_launch`` times a small set of shapes
on the actual problem and batch with CUDA events and keeps the fastest, per
problem and batch size class, for the life of the process.  The analytic-field
kernels give bit-identical results for every shape (every trajectory runs the
same arithmetic in one thread); the MLP kernels sum each row's error norm with
shared-memory atomics, whose order, and so the last bit of a norm, may change
with the shape.

With ``GBDX_AUTOTUNE_CACHE`` set to a file path, the choices also persist
across processes: they are read from that JSON file on first use and every
new choice is written back, keyed by the GPU's name, the problem and the
batch class.

``GraphedSolve`` captures one forward solve in a CUDA graph and replays it on
new inputs of the same shapes, so a solve repeated inside a training or
serving loop costs one graph launch.
"""
from __future__ import annotations

import json
import math
import os
import tempfile

import torch

from . import _lib
from ._core import RESULT_MESSAGES, RESULTS, SaveAt, Solution
from ._integrate import Lowered, _raise_on_failure

_LAUNCH_KEYS = ("block_threads", "ctas_per_sm")
_TUNED: dict = {}


def _key(fields: dict, batch: int):
    """The problem minus its launch shape, and the batch's power-of-two class."""
    items = []
    for k, v in sorted(fields.items()):
        if k in _LAUNCH_KEYS:
            continue
        items.append((k, tuple(v) if isinstance(v, (list, tuple)) else v))
    return tuple(items), 1 << max(0, math.ceil(math.log2(max(batch, 1))))


def tc_eligible(fields: dict) -> bool:
    """Whether the tcgen05 forward (kernel "tc") serves this problem: BF16
    forward solves of 64 -> 128 -> 128 -> 64 MLP ODE fields with Tsit5 or
    Dopri5."""
    return (fields.get("field") == 3 and fields.get("solver") in (2, 3) and
            tuple(fields.get("mlp_widths", ())) == (64, 128, 128, 64) and
            fields.get("mlp_precision", 0) == 0 and fields.get("adjoint", 0) == 0 and
            fields.get("diffusion", 0) == 0 and not fields.get("save_steps") and
            not fields.get("save_dense") and not fields.get("n_event") and
            not fields.get("n_step_ts") and not fields.get("n_jump_ts"))


def candidates(fields: dict, batch: int) -> list:
    """(kernel, block_threads, ctas_per_sm) shapes worth timing for this
    problem: the launch shape of the fused kernels and, for the MLP fields,
    the tile shape (32-row mma.sync tiles, or 128-row tcgen05 tiles)."""
    kernel = fields.get("kernel", 0)
    if fields.get("field") == 3:  # MLP fields: one row tile per CTA
        out = [("fused", 0, c) for c in (1, 2, 3, 4)]
        if kernel == 0 and tc_eligible(fields):
            out.append(("tc", 0, 1))
        return out
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    out = [("fused", 0, 0)]
    for block in (32, 64, 128, 256):
        for per_sm in (1, 2, 4, 8, 16, 32):
            lanes = block * per_sm * sms
            if lanes > 2 * batch or block * per_sm > 2048:
                continue
            out.append(("fused", block, per_sm))
    return out


_CACHE_ENV = "GBDX_AUTOTUNE_CACHE"
_cache_loaded: set = set()


def _cache_entry_key(device_name: str, key) -> str:
    return json.dumps([device_name, [list(kv) for kv in key[0]], key[1]], sort_keys=True)


def _device_name() -> str:
    try:
        return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:  # no device: the key still separates machines by name
        return "unknown"


def load_cache(path: str, device_name: str) -> int:
    """Merge the choices recorded for `device_name` in the JSON file `path`
    into this process's table; returns how many were read (0 when the file is
    missing or unreadable)."""
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        return 0
    n = 0
    for k, v in data.items():
        try:
            dev, items, cls = json.loads(k)
        except (ValueError, TypeError):
            continue
        if dev != device_name:
            continue
        key = (tuple((a, tuple(b) if isinstance(b, list) else b) for a, b in items), cls)
        _TUNED[key] = (str(v[0]), int(v[1]), int(v[2]))
        n += 1
    return n


def save_cache(path: str, device_name: str) -> None:
    """Write this process's choices for `device_name` into the JSON file
    `path`, keeping the entries it already holds (atomic replace)."""
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        data = {}
    for key, shape in _TUNED.items():
        data[_cache_entry_key(device_name, key)] = list(shape)
    d = os.path.dirname(os.path.abspath(path))
    fd, tmp = tempfile.mkstemp(dir=d, suffix=".tmp")
    with os.fdopen(fd, "w") as f:
        json.dump(data, f, indent=0, sort_keys=True)
    os.replace(tmp, path)


def autotune_launch(low_factory, batch: int, fields: dict, reps: int = 3,
                    verbose: bool = False):
    """Time every candidate shape of the problem and return the fastest
    (kernel, block_threads, ctas_per_sm); cached per problem and batch class
    (and in the GBDX_AUTOTUNE_CACHE file when that is set).

    ``low_factory(kernel, block_threads, ctas_per_sm)`` builds the Lowered
    solve."""
    key = _key(fields, batch)
    path = os.environ.get(_CACHE_ENV)
    if path and path not in _cache_loaded:
        _cache_loaded.add(path)
        load_cache(path, _device_name())
    hit = _TUNED.get(key)
    if hit is not None:
        return hit
    best, best_ms = ("fused", 0, 0), math.inf
    stream = torch.cuda.current_stream()
    for shape in candidates(fields, batch):
        low = low_factory(*shape)
        low.run_forward()  # warm-up (and first-use set-up)
        ms = math.inf
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            low.run_forward()
            e1.record(stream)
            e1.synchronize()
            ms = min(ms, e0.elapsed_time(e1))
        if verbose:
            print(f"autotune {shape}: {ms:.4f} ms")
        if ms < best_ms:
            best, best_ms = shape, ms
    _TUNED[key] = best
    if path:
        save_cache(path, _device_name())
    return best


def tuned_shapes() -> dict:
    """The shapes chosen so far (problem key -> (kernel, block_threads,
    ctas_per_sm))."""
    return dict(_TUNED)


class GraphedSolve:
    """A forward solve captured once as a CUDA graph and replayed on new inputs.

    The constructor takes the arguments of ``diffeqsolve`` (forward solves: no
    gradient); ``y0``, ``args`` and per-trajectory ``t0`` / ``t1`` / ``dt0``
    fix the shapes.  ``__call__(y0=None, args=None, t0=None, t1=None,
    dt0=None)`` copies the given inputs into the captured buffers, replays the
    graph and returns a Solution whose tensors are the graph's output buffers:
    the next call overwrites them (clone what must be kept).  ``autotune=True``
    picks the launch shape before capture.  Inputs in page-locked host memory
    are copied asynchronously: keep them unmodified until the outputs are read.

    ``host_io=True`` serves a host-side caller with one graph launch per solve:
    the inputs given as page-locked host tensors become the solve's staging
    buffers and the outputs (ys, ts, result, stats, and the event index) are
    page-locked host tensors.  Where the GPU maps them (every page-locked
    buffer on a system with unified addressing; NVLink-C2C on Grace), the
    solve's kernels read the inputs and write the outputs in place, with no
    copy before or after them (``zero_copy`` is True); otherwise, or with
    ``host_io="copy"``, the graph copies the inputs to the device and the
    outputs back.  A call then writes
    any new inputs into the staging buffers (or the caller writes them there
    itself), replays the graph, waits for it, and returns a Solution of host
    tensors (the same object each call when it carries no SaveAt fn or event
    mask; overwritten by the next call).
    """

    def __init__(self, terms, solver, t0, t1, dt0, y0, args=None, *,
                 saveat: SaveAt = SaveAt(t1=True), stepsize_controller=None,
                 max_steps: int = 4096, throw: bool = True, kernel: str = "auto",
                 schedule: str = "auto", autotune: bool = False, event=None,
                 host_io=False):
        from ._core import ConstantStepSize
        if stepsize_controller is None:
            stepsize_controller = ConstantStepSize()
        self._fn = getattr(saveat, "fn", None)
        if saveat.dense:
            raise NotImplementedError("GraphedSolve replays solves without dense output")
        dev = torch.device("cuda", torch.cuda.current_device())

        def own(x, dtype=None):
            if x is None:
                return None
            t = torch.as_tensor(x)
            t = t.to(device=dev, dtype=dtype or t.dtype)
            return t.clone().contiguous()  # the graph reads these buffers

        # host_io: the page-locked host inputs stay bound as staging buffers
        self._host_in = {}
        if host_io:
            for name, v in (("y0", y0), ("args", args), ("t0", t0), ("t1", t1), ("dt0", dt0)):
                if isinstance(v, torch.Tensor) and v.device.type == "cpu":
                    if not v.is_pinned():
                        raise ValueError(f"host_io needs page-locked host tensors ({name}: "
                                         "use Tensor.pin_memory())")
                    if not v.is_contiguous():
                        # the graph reads the staging buffer itself: a strided
                        # view would be gathered once, at capture
                        raise ValueError(f"host_io needs contiguous host tensors ({name})")
                    self._host_in[name] = v
        y0 = own(y0)
        if y0.dtype not in (torch.float32, torch.float64):
            y0 = y0.to(torch.float64)
        # every time becomes a buffer of this solve (a Python number too: the
        # calls overwrite the captured times in place)
        t0 = own(torch.tensor([float(t0)]) if not isinstance(t0, torch.Tensor) else t0,
                 torch.float64)
        t1 = own(torch.tensor([float(t1)]) if not isinstance(t1, torch.Tensor) else t1,
                 torch.float64)
        if dt0 is not None:
            dt0 = own(torch.tensor([float(dt0)]) if not isinstance(dt0, torch.Tensor) else dt0,
                      torch.float64)
        args = own(args, y0.dtype)
        self.throw, self.max_steps = throw, max_steps

        def factory(kern, block_threads, ctas_per_sm):
            return Lowered(terms, solver, t0, t1, dt0, y0, args, saveat, stepsize_controller,
                           None, max_steps, kern, block_threads, ctas_per_sm, schedule,
                           event=event)

        shape = (kernel, 0, 0)
        if autotune:
            base = factory(kernel, 0, 0)
            shape = autotune_launch(factory, base.B, base.fields)
        self.shape = shape
        low = factory(*shape)
        self.low = low
        self._event = event
        run = low.run_forward_ex if event is not None else low.run_forward
        for name, h in self._host_in.items():
            dst = getattr(low, name)
            if h.numel() != dst.numel() or h.dtype != dst.dtype:
                raise ValueError(f"host_io: {name} must be a {dst.dtype} tensor of "
                                 f"{dst.numel()} entries")
        warm = run()  # warm-up outside the capture (first-use set-up of the library)
        self.host_io = bool(host_io)
        self._host_out = []
        self._io = None
        if host_io:
            self._host_out = [None if o is None else torch.empty(o.shape, dtype=o.dtype,
                                                                  pin_memory=True)
                              for o in warm]
            if host_io != "copy":
                self._io = self._mapped_io()
        self.zero_copy = self._io is not None
        torch.cuda.synchronize()

        def staged():
            if self._io is not None:
                run(io=self._io)  # the kernels read and write the host buffers in place
                return list(self._host_out)
            for name, h in self._host_in.items():
                dst = getattr(low, name)
                dst.copy_(h.reshape(dst.shape), non_blocking=True)
            outs = run()
            for o, h in zip(outs, self._host_out):
                if h is not None and o is not None and isinstance(o, torch.Tensor):
                    h.copy_(o, non_blocking=True)
            return outs
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._outs = staged()
        torch.cuda.synchronize()
        self._sol = None

    # the solve's outputs in the order run_forward(_ex) returns them
    _OUT_NAMES = ("ys", "ts", "result", "stats", None, "event_index")

    def _mapped_io(self):
        """Device addresses of the page-locked inputs and outputs, or None
        (the copy path) unless every one of them is mapped."""
        io = {}
        pairs = list(self._host_in.items()) + [
            (n, h) for n, h in zip(self._OUT_NAMES, self._host_out) if n and h is not None]
        for name, h in pairs:
            d = _lib.host_device_pointer(h.data_ptr())
            if d is None:
                return None
            io[name] = d
        return io

    def _copy_in(self, name, value):
        dst = getattr(self.low, name)
        if dst is None:
            raise ValueError(f"the captured solve has no {name} input")
        src = torch.as_tensor(value)
        if src.numel() != dst.numel():
            raise ValueError(f"{name} must keep the captured shape {tuple(dst.shape)}")
        # a page-locked host source is copied asynchronously, ahead of the
        # replay on the same stream
        dst.copy_(src.reshape(dst.shape), non_blocking=src.device.type == "cpu" and src.is_pinned())

    def __call__(self, y0=None, args=None, t0=None, t1=None, dt0=None) -> Solution:
        for name, v in (("y0", y0), ("args", args), ("t0", t0), ("t1", t1), ("dt0", dt0)):
            if v is None:
                continue
            h = self._host_in.get(name)
            if h is None:
                self._copy_in(name, v)
            elif v is not h:
                src = torch.as_tensor(v)
                if src.numel() != h.numel():
                    raise ValueError(f"{name} must keep the captured shape {tuple(h.shape)}")
                h.copy_(src.reshape(h.shape))  # into the staging buffer
        self.graph.replay()
        outs = self._outs
        if self.host_io:
            torch.cuda.current_stream().synchronize()
            outs = [h if h is not None else o for o, h in zip(outs, self._host_out)]
        ys, ts, res, stats = outs[:4]
        # a Solution of the same host tensors serves every call when nothing
        # in it is computed per call
        reuse = self.host_io and self._fn is None and self._event is None
        if reuse and self._sol is not None:
            if self.throw:
                _raise_on_failure(res)
            return self._sol
        if self._fn is not None:
            ys = self._fn(ts, ys, self.low.args if args is None else args)
        sol = Solution(t0=self.low.t0, t1=self.low.t1, ts=ts, ys=ys,
                       stats=dict(num_steps=stats[:, 0], num_accepted_steps=stats[:, 1],
                                  num_rejected_steps=stats[:, 2], max_steps=self.max_steps),
                       result=res)
        if reuse:
            self._sol = sol
        if self._event is not None:
            ev = outs[5]
            masks = [ev == i for i in range(len(self._event._conds))]
            sol.event_mask = masks[0] if self._event._single else masks
        if self.throw:
            _raise_on_failure(res)
        return sol


__all__ = ["autotune_launch", "candidates", "tuned_shapes", "GraphedSolve", "RESULTS",
           "RESULT_MESSAGES"]
