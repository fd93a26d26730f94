"""Serving loop host logic on the CPU: the scheduler against a simulated
executor (admission by memory budget, grouping, eviction, continuous
batching), and the residual stack on the oracle (batch independence)."""

import numpy as np
import pytest

from owl_gb300.serving import (Request, ResidualStack, Scheduler, bucket_for, init_stack,
                               poisson_stream, stack_flops, stack_layers)


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-6)


class FakeInst:
    def __init__(self, key, nbytes):
        self.key, self.nbytes = key, nbytes
        self.finish = None
        self.requests = None
        self.alive = True


class FakeExecutor:
    """Runs a group of `n` images of side s in (20 + n * s * s / 1e3) us of
    simulated time; an instance of (side, bucket) holds bucket*side*side
    bytes."""

    def __init__(self, clock):
        self.clock = clock
        self.created, self.destroyed, self.launches = [], [], []
        self.busy_bytes = []

    def estimate(self, key):
        side, bucket = key
        return bucket * side * side

    def create(self, key):
        inst = FakeInst(key, self.estimate(key))
        self.created.append(inst)
        return inst

    def destroy(self, inst):
        assert inst.finish is None or inst.finish <= self.clock()
        inst.alive = False
        self.destroyed.append(inst)

    def launch(self, inst, requests):
        assert inst.alive and sum(r.batch for r in requests) <= inst.key[1]
        side = inst.key[0]
        n = sum(r.batch for r in requests)
        inst.finish = self.clock() + 20e-6 + n * side * side / 1e9
        inst.requests = requests
        self.launches.append((self.clock(), inst.key, [r.rid for r in requests]))

    def poll(self, inst):
        if self.clock() < inst.finish:
            return False
        for r in inst.requests:
            r.output = np.full((r.batch, 10), r.rid, dtype=np.float32)
        return True


def _run(requests, budget, max_group=128):
    clk = FakeClock()
    ex = FakeExecutor(clk)
    sch = Scheduler(ex, budget, max_group=max_group, clock=clk, idle_sleep=5e-6,
                    sleep=clk.sleep)
    st = sch.run(requests)
    return sch, ex, st


def test_bucket_for():
    assert bucket_for(1) == 1 and bucket_for(3) == 4 and bucket_for(17) == 24
    assert bucket_for(128) == 128
    with pytest.raises(ValueError):
        bucket_for(129)


def test_every_request_completes_once_with_its_output():
    reqs = poisson_stream(200, 2000.0, seed=3, max_batch=64)
    _, ex, st = _run(reqs, budget=64 * 224 * 224 * 8)
    assert st.completed == 200 and st.images == sum(r.batch for r in reqs)
    for r in reqs:
        assert r.output.shape == (r.batch, 10) and np.all(r.output == r.rid)
        assert r.arrival <= r.admitted <= r.done
    launched = sorted(rid for _, _, rids in ex.launches for rid in rids)
    assert launched == list(range(200))
    s = st.summary()
    assert s["p50_ms"] <= s["p99_ms"] and s["req_per_s"] > 0


def test_groups_are_same_side_fifo_and_within_max_group():
    reqs = [Request(i, 0.0, 8, 28 if i % 2 else 56) for i in range(40)]
    _, ex, st = _run(reqs, budget=1 << 40, max_group=64)
    assert st.groups < 40  # simultaneous arrivals were grouped
    by_id = {r.rid: r for r in reqs}
    for _, (side, bucket), rids in ex.launches:
        assert all(by_id[i].side == side for i in rids)
        assert sum(by_id[i].batch for i in rids) <= min(bucket, 64)
        assert rids == sorted(rids)  # oldest first within a side


def test_budget_bounds_allocated_memory_and_evicts_idle_instances():
    reqs = poisson_stream(300, 5000.0, seed=4, max_batch=32)
    budget = 96 * 224 * 224 + 32 * 112 * 112  # room for one large and one mid instance
    sch, ex, st = _run(reqs, budget=budget, max_group=96)
    assert st.completed == 300
    assert st.peak_bytes <= budget
    assert st.evicted > 0 and len(ex.destroyed) == st.evicted
    assert sch.allocated <= budget


def test_over_budget_group_runs_alone_rather_than_deadlocking():
    reqs = [Request(0, 0.0, 64, 224), Request(1, 0.0, 4, 14)]
    _, ex, st = _run(reqs, budget=10)  # smaller than any instance
    assert st.completed == 2


def test_continuous_batching_admits_while_others_run():
    # a long 224 group, then small requests that arrive while it runs
    reqs = [Request(0, 0.0, 64, 224)] + [Request(i, 1e-4 * i, 2, 14) for i in range(1, 6)]
    _, ex, st = _run(reqs, budget=1 << 40)
    big_done = reqs[0].done
    assert any(r.admitted < big_done and r.done < big_done for r in reqs[1:])


def test_stack_layout_and_flops():
    layers = stack_layers()
    assert sum(1 for n, *_ in layers if not n.endswith("proj")) == 18
    assert {s[2] for _, s, _ in layers if _ != "head"} >= {3, 64, 128, 256, 512}
    assert abs(stack_flops(224) / 3.434e9 - 1) < 1e-3
    assert stack_flops(28, 4) == 4 * stack_flops(28)


def test_stack_rows_are_independent_of_the_batch(oracle_nn):
    """On the oracle the GEMM blocking depends on the batch, so rows agree
    to float64 rounding rather than bit for bit."""
    w = {k: v.astype(np.float64) for k, v in init_stack(0).items()}
    stack = ResidualStack(w, oracle_nn)
    x = np.random.default_rng(5).uniform(0, 1, (3, 14, 14, 3))
    y = stack.forward(x)
    assert y.shape == (3, 10)
    for i in range(3):
        assert np.allclose(stack.forward(x[i:i + 1].copy())[0], y[i], rtol=0, atol=1e-12)
