"""Continuous-batching inference over the conv/pool kernels.

A stream of requests, each a batch of square 3-channel images, goes through
a residual conv stack laid out like ResNet-18 (``ResidualStack``): a 3x3
stride-2 stem and a 2x2 max pool, four stages of two basic blocks (3x3
convs, 64 to 512 channels, stride-2 downsampling with 1x1 projections), a
global average pool and a 1x1 classifier conv -- 18 weighted layers plus 3
projections (3.4 GFLOP per 224x224 image).
Weights and activations stay on the GPU; the convolutions run through
libowlgpu (BF16 tensor-core MMAs with FP32 accumulation by default).

Serving is continuous batching, not a queue:

  * requests waiting for the same image side are grouped, oldest first,
    into one forward pass of up to ``max_group`` images, padded to a batch
    bucket;
  * each (side, bucket) forward is captured once as a CUDA graph with its
    own input and output buffers (an *instance*); a group is copied into a
    free instance and the graph is replayed on that instance's stream, so
    groups of different sides, and further groups of one side, run
    concurrently on the device;
  * every instance, busy or idle, counts against ``hbm_budget`` bytes of
    device memory; a group reuses an idle instance of its shape, or idle
    instances of other shapes are evicted to make room for a new one, or
    it waits while busy instances hold the memory -- requests that arrive
    while others are on the GPU are admitted as soon as an instance and
    memory free up.

Every image of a group is computed independently (convolutions and pools
never mix batch entries), so a request's result is the same alone and in a
mix; ``tests/test_gpu_serving.py`` checks this.

The scheduler (``Scheduler``) knows nothing of CUDA: it drives an executor
(``estimate``, ``create``, ``destroy``, ``launch``, ``poll``), so its
admission, grouping and eviction logic is tested on the CPU with a
simulated one.
"""

from __future__ import annotations

import bisect
import math
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Any, Callable

import numpy as np

from .dense import NN, SAME, VALID

SIDES = (14, 28, 56, 112, 224)
BUCKETS = (1, 2, 4, 8, 16, 24, 32, 48, 64, 96, 128)

# ---- requests ----------------------------------------------------------------


@dataclass
class Request:
    rid: int
    arrival: float          # seconds from the start of the stream
    batch: int
    side: int
    pixels: Any = None      # host array [batch; side; side; 3] (pinned for speed)
    admitted: float = math.nan
    done: float = math.nan
    output: Any = None      # host array [batch; 10]

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def poisson_stream(n: int, rate: float, seed: int = 0, sides=SIDES, max_batch: int = 64):
    """`n` requests with exponential inter-arrival times of mean 1/rate,
    batch uniform in 1..max_batch, side drawn uniformly from `sides`."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    b = rng.integers(1, max_batch + 1, n)
    s = rng.choice(np.asarray(sides), n)
    return [Request(i, float(t[i]), int(b[i]), int(s[i])) for i in range(n)]


def bucket_for(n: int, buckets=BUCKETS) -> int:
    i = bisect.bisect_left(buckets, n)
    if i == len(buckets):
        raise ValueError(f"group of {n} images exceeds the largest bucket {buckets[-1]}")
    return buckets[i]


# ---- the model ----------------------------------------------------------------

STAGES = ((64, 1), (128, 2), (256, 2), (512, 2))


def stack_layers():
    """(name, kernel shape, stride) of every conv, in order."""
    layers = [("stem", (3, 3, 3, 64), 2)]
    cin = 64
    for si, (cout, stride) in enumerate(STAGES):
        for bi in range(2):
            s = stride if bi == 0 else 1
            layers.append((f"s{si}b{bi}c1", (3, 3, cin, cout), s))
            layers.append((f"s{si}b{bi}c2", (3, 3, cout, cout), 1))
            if s != 1 or cin != cout:
                layers.append((f"s{si}b{bi}proj", (1, 1, cin, cout), s))
            cin = cout
    layers.append(("head", (1, 1, 512, 10), 1))
    return layers


def init_stack(seed: int = 0, dtype=np.float32) -> dict:
    """He-normal weights; the second conv of each block is scaled by 1/2 so
    activations stay of order one through the residual sums."""
    rng = np.random.default_rng(seed)
    w = {}
    for name, shape, _ in stack_layers():
        fan_in = shape[0] * shape[1] * shape[2]
        scale = math.sqrt(2.0 / fan_in) * (0.5 if name.endswith("c2") else 1.0)
        w[name] = (rng.standard_normal(shape) * scale).astype(dtype)
    return w


def _out(n: int, s: int) -> int:
    return -(-n // s)  # SAME: ceil(n / s)


def stack_flops(side: int, batch: int = 1) -> float:
    """Multiply-add FLOPs (2 per MAC) of one forward pass."""
    total = 0.0
    h = side
    for name, (kc, kr, ci, co), s in stack_layers():
        if name == "head":
            total += 2.0 * ci * co
            continue
        if name.startswith("s") and name.endswith("c1"):
            hin = h
        if name.endswith("proj"):
            ho = _out(hin, s)
        else:
            ho = _out(h, s)
            h = ho
        total += 2.0 * ho * ho * kc * kr * ci * co
        if name == "stem":
            h = _out(h, 2)  # 2x2 max pool, stride 2
    return total * batch


class ResidualStack:
    """Forward pass of the stack over one NN function set (GPU or oracle).
    A convolution followed by ReLU runs as one call with the ReLU in the
    convolution's epilogue (owl_gb300.layers); residual sums are plain array
    ops.  On the GPU the stack declares its kernel tensors to the library's
    weight-image cache (they never change), so a forward pass re-lays no
    weights out and a captured one launches only the convolution and pooling
    kernels."""

    def __init__(self, weights: dict, nn: NN):
        from .layers import Layers

        self.w = weights
        self.nn = nn
        self.layers = Layers(nn)
        self._declared = []
        if self.layers.gpu:
            from . import _lib

            for t in weights.values():
                if type(t).__module__.startswith("torch") and t.is_cuda:
                    _lib.call("owlgpu_weights_declare", t.data_ptr(), 0)
                    self._declared.append(t)

    def release(self) -> None:
        """Forget the declared kernel tensors.  Call it before the weights
        are freed: the library keys its images by device address, and a
        freed address may be reused by another tensor."""
        if self._declared:
            from . import _lib

            for t in self._declared:
                _lib.call("owlgpu_weights_forget", t.data_ptr())
            self._declared = []

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    @staticmethod
    def _relu(a):
        return a.clamp_min(0) if type(a).__module__.startswith("torch") else np.maximum(a, 0)

    def _conv_relu(self, x, w, s):
        from .layers import ACT_RELU

        return self.layers.conv2d_bias_act(x, w, None, [s, s], SAME, ACT_RELU)

    def forward(self, x):
        nn, w, relu = self.nn, self.w, self._relu
        h = self._conv_relu(x, w["stem"], 2)
        h = nn.max_pool2d(h, [2, 2], [2, 2], SAME)
        for si, (cout, stride) in enumerate(STAGES):
            for bi in range(2):
                s = stride if bi == 0 else 1
                pre = f"s{si}b{bi}"
                y = self._conv_relu(h, w[pre + "c1"], s)
                y = nn.conv2d(y, w[pre + "c2"], [1, 1], SAME)
                sc = nn.conv2d(h, w[pre + "proj"], [s, s], SAME) if pre + "proj" in w else h
                h = relu(y + sc)
        side = h.shape[1]
        h = nn.avg_pool2d(h, [side, side], [1, 1], VALID)
        y = nn.conv2d(h, w["head"], [1, 1], SAME)
        return y.reshape(y.shape[0], 10)


# ---- scheduler (host logic, no CUDA) -------------------------------------------


@dataclass
class Stats:
    completed: int = 0
    images: int = 0
    groups: int = 0
    created: int = 0
    evicted: int = 0
    peak_bytes: int = 0
    wall_s: float = 0.0
    latencies: list = field(default_factory=list)

    def summary(self) -> dict:
        lat = np.asarray(self.latencies) * 1e3
        return {"requests": self.completed, "images": self.images, "groups": self.groups,
                "instances_created": self.created, "instances_evicted": self.evicted,
                "wall_s": self.wall_s,
                "req_per_s": self.completed / self.wall_s if self.wall_s else None,
                "images_per_s": self.images / self.wall_s if self.wall_s else None,
                "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
                "p99_ms": float(np.percentile(lat, 99)) if lat.size else None,
                "mean_ms": float(lat.mean()) if lat.size else None,
                "peak_bytes": self.peak_bytes}


class Scheduler:
    """Continuous batching with admission by a device-memory budget.

    The scheduler owns the instances (one captured forward pass of a (side,
    bucket) shape each) and the budget: every instance, busy or idle, counts
    its bytes.  A group reuses an idle instance of its shape; otherwise idle
    instances of other shapes are destroyed, least recently used first,
    until a new one fits; if busy instances hold the memory the group waits.
    Executor interface (CUDA in ``GraphExecutor``, simulated in the tests):
    ``estimate(key)``, ``create(key)`` -> instance with ``nbytes``,
    ``destroy(inst)``, ``launch(inst, requests)``, ``poll(inst)`` -> bool
    (True once finished, with the requests' outputs filled).
    """

    def __init__(self, executor, hbm_budget: int, max_group: int = 128, buckets=BUCKETS,
                 clock: Callable[[], float] = time.perf_counter, idle_sleep: float = 2e-5,
                 sleep: Callable[[float], None] = time.sleep):
        self.ex = executor
        self.budget = hbm_budget
        self.max_group = min(max_group, buckets[-1])
        self.buckets = buckets
        self.clock = clock
        self.idle_sleep = idle_sleep
        self.sleep = sleep
        self.idle: dict = {}        # key -> deque of idle instances
        self.lru: list = []         # idle instances, least recently used first
        self.allocated = 0

    def _acquire(self, key, st: Stats, busy: int):
        q = self.idle.get(key)
        if q:
            inst = q.pop()
            self.lru.remove(inst)
            return inst
        need = self.ex.estimate(key)
        while self.allocated + need > self.budget and self.lru:
            victim = self.lru.pop(0)
            self.idle[victim.key].remove(victim)
            self.allocated -= victim.nbytes
            self.ex.destroy(victim)
            st.evicted += 1
        if self.allocated + need > self.budget and busy:
            return None  # wait for busy instances to finish
        inst = self.ex.create(key)
        inst.key = key
        self.allocated += inst.nbytes
        st.created += 1
        st.peak_bytes = max(st.peak_bytes, self.allocated)
        return inst

    def _release(self, inst) -> None:
        self.idle.setdefault(inst.key, deque()).append(inst)
        self.lru.append(inst)

    def _group_size(self, q: deque) -> int:
        n = 0
        for r in q:
            if n + r.batch > self.max_group:
                break
            n += r.batch
        return n

    def run(self, requests: list, stats: Stats | None = None) -> Stats:
        st = stats or Stats()
        for r in requests:
            if r.batch > self.max_group:
                raise ValueError(f"request {r.rid}: batch {r.batch} > max_group")
        pending = sorted(requests, key=lambda r: r.arrival)
        queues: dict = {}
        inflight: list = []
        nxt = 0
        t0 = self.clock()
        while nxt < len(pending) or any(queues.values()) or inflight:
            now = self.clock() - t0
            while nxt < len(pending) and pending[nxt].arrival <= now:
                r = pending[nxt]
                queues.setdefault(r.side, deque()).append(r)
                nxt += 1
            still = []
            for inst, group in inflight:
                if self.ex.poll(inst):
                    t = self.clock() - t0
                    for r in group:
                        r.done = t
                        st.latencies.append(t - r.arrival)
                        st.completed += 1
                        st.images += r.batch
                    self._release(inst)
                else:
                    still.append((inst, group))
            inflight = still
            # admit groups, the side with the oldest waiting request first
            while True:
                heads = sorted((q[0].arrival, side) for side, q in queues.items() if q)
                admitted = False
                for _, side in heads:
                    q = queues[side]
                    key = (side, bucket_for(self._group_size(q), self.buckets))
                    inst = self._acquire(key, st, len(inflight))
                    if inst is None:
                        continue
                    group, n = [], 0
                    while q and n + q[0].batch <= self.max_group:
                        r = q.popleft()
                        group.append(r)
                        n += r.batch
                    t = self.clock() - t0
                    for r in group:
                        r.admitted = t
                    self.ex.launch(inst, group)
                    inflight.append((inst, group))
                    st.groups += 1
                    admitted = True
                    break
                if not admitted:
                    break
            if not inflight and not any(queues.values()) and nxt < len(pending):
                wait = pending[nxt].arrival - (self.clock() - t0)
                if wait > 0:
                    self.sleep(min(wait, 1e-3))
            elif self.idle_sleep:
                self.sleep(self.idle_sleep)
        st.wall_s = self.clock() - t0
        return st

    def close(self) -> None:
        for inst in list(self.lru):
            self.ex.destroy(inst)
        self.lru.clear()
        self.idle.clear()
        self.allocated = 0


# ---- the CUDA executor --------------------------------------------------------


class _Instance:
    __slots__ = ("key", "graph", "x", "y", "host_y", "stream", "done", "nbytes", "requests")


class GraphExecutor:
    """Captured forward passes: one CUDA graph per instance of a (side,
    bucket) shape, each with its own static input/output buffers, its own
    stream (round-robin over `streams`) and a completion event."""

    def __init__(self, stack: ResidualStack, streams: int = 8, capture: bool = True):
        import torch

        self.torch = torch
        self.stack = stack
        self.capture = capture
        self.streams = [torch.cuda.Stream() for _ in range(streams)]
        self.rr = 0
        self.sizes: dict = {}

    def estimate(self, key) -> int:
        """Bytes of a new instance: measured once one exists, else an upper
        bound of four live copies of the largest activation (stem output)."""
        if key in self.sizes:
            return self.sizes[key]
        side, bucket = key
        return bucket * side * side * 64 * 4 * 4 + (16 << 20)

    def create(self, key) -> _Instance:
        torch = self.torch
        side, bucket = key
        inst = _Instance()
        inst.key = key
        inst.stream = self.streams[self.rr % len(self.streams)]
        self.rr += 1
        torch.cuda.synchronize()
        before = torch.cuda.memory_reserved()
        inst.x = torch.zeros((bucket, side, side, 3), dtype=torch.float32, device="cuda")
        inst.host_y = torch.empty((bucket, 10), dtype=torch.float32, pin_memory=True)
        inst.graph, inst.y = None, None
        if self.capture:
            with torch.cuda.stream(inst.stream):
                self.stack.forward(inst.x)  # first run outside capture
            inst.stream.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=inst.stream):
                inst.y = self.stack.forward(inst.x)
            inst.graph = g
        torch.cuda.synchronize()
        inst.nbytes = max(torch.cuda.memory_reserved() - before, inst.x.numel() * 4)
        self.sizes[key] = max(self.sizes.get(key, 0), inst.nbytes)
        inst.done = torch.cuda.Event()
        inst.requests = None
        return inst

    def destroy(self, inst) -> None:
        inst.graph = None
        inst.x = inst.y = None
        self.torch.cuda.synchronize()
        self.torch.cuda.empty_cache()

    def launch(self, inst, requests) -> None:
        torch = self.torch
        inst.requests = requests
        with torch.cuda.stream(inst.stream):
            o = 0
            for r in requests:
                inst.x[o:o + r.batch].copy_(r.pixels, non_blocking=True)
                o += r.batch
            if o < inst.x.shape[0]:
                inst.x[o:].zero_()
            if inst.graph is not None:
                inst.graph.replay()
            else:
                inst.y = self.stack.forward(inst.x)
            inst.host_y.copy_(inst.y, non_blocking=True)
            inst.done.record(inst.stream)

    def poll(self, inst) -> bool:
        if not inst.done.query():
            return False
        o = 0
        for r in inst.requests:
            r.output = inst.host_y[o:o + r.batch].numpy().copy()
            o += r.batch
        inst.requests = None
        return True


def attach_pixels(requests, seed: int = 1, pool: int = 128, pinned: bool = True):
    """U[0,1] pixels for every request: each side has one pool of `pool`
    images and a request takes `batch` consecutive ones at a random offset
    (so generating inputs costs nothing inside the timed loop)."""
    import torch

    rng = np.random.default_rng(seed)
    pools = {}
    for side in sorted({r.side for r in requests}):
        a = torch.from_numpy(rng.uniform(0, 1, (pool + 64, side, side, 3)).astype(np.float32))
        pools[side] = a.pin_memory() if pinned else a
    for r in requests:
        o = int(rng.integers(0, pool))
        r.pixels = pools[r.side][o:o + r.batch]
    return requests
