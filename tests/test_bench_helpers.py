"""Host logic of bench.py's measurement helpers, on the CPU:

* PinnedRing hands out slab ranges that never overlap a request still in
  flight, waits for the oldest request only when the slab is full, and
  reports each request's latency from its scheduled arrival;
* ClockSampler keeps only the nvidia-smi samples stamped inside the timed
  window (a stand-in nvidia-smi on PATH prints fixed clock lines), reports
  throttle reasons it saw there, and falls back to the nearest samples,
  labelled so, for a window shorter than its interval."""
import importlib.util
import os
import random
import stat
import time

import pytest
import torch

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _HostTorch:
    """torch with pin_memory dropped (no CUDA here)."""
    float32 = torch.float32

    @staticmethod
    def empty(n, dtype, pin_memory):
        return torch.empty(n, dtype=dtype)


class _FakeServer:
    def __init__(self):
        self.waited = []

    def wait(self, ticket, timeout_ms):
        self.waited.append(ticket)
        return 0, {"latency_ms": 2.0}


@pytest.mark.parametrize("slab", [64, 1000, 4096])
def test_pinned_ring_ranges_never_overlap_live_requests(bench, slab):
    rng = random.Random(slab)
    ring = bench.PinnedRing(_HostTorch, slab)
    srv = _FakeServer()
    owner = [None] * slab
    live = {}
    for t in range(3000):
        n = rng.randint(1, slab // 3)
        start, view = ring.take(srv, n)
        assert view.numel() == n and 0 <= start and start + n <= slab
        for tk in [k for k in live if k in srv.waited]:
            a, e = live.pop(tk)
            owner[a:e] = [None] * (e - a)
        assert all(o is None for o in owner[start:start + n]), (t, start, n)
        owner[start:start + n] = [t] * n
        live[t] = (start, start + n)
        ring.add(start, n, t, 0.001)
    ring.drain(srv)
    assert sorted(srv.waited) == list(range(3000))  # every request waited for once
    assert len(ring.lat_ms) == 3000 and all(abs(v - 3.0) < 1e-9 for v in ring.lat_ms)


def test_pinned_ring_waits_only_when_full(bench):
    ring = bench.PinnedRing(_HostTorch, 100)
    srv = _FakeServer()
    for t in range(4):
        s, _ = ring.take(srv, 25)
        ring.add(s, 25, t, 0.0)
    assert srv.waited == []  # 4 x 25 fit exactly
    s, _ = ring.take(srv, 10)
    assert srv.waited == [0] and s == 0  # the oldest range is retired and reused


@pytest.fixture
def fake_smi(tmp_path, monkeypatch):
    def make(line):
        exe = tmp_path / "nvidia-smi"
        exe.write_text("#!/bin/bash\nwhile true; do echo '" + line + "'; sleep 0.02; done\n")
        exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
        monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ["PATH"])
    return make


def test_clock_sampler_window(bench, fake_smi):
    fake_smi("2070, 2070, 900.5, Not Active, Not Active, Not Active, Not Active, Not Active")
    c = bench.ClockSampler(0)
    time.sleep(0.1)
    t0 = time.time()
    time.sleep(0.2)
    out = c.stop(t0, time.time())
    assert out["window"] == "timed region" and out["samples"] >= 4
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["reasons"] == []


def test_clock_sampler_reasons_and_short_window(bench, fake_smi):
    fake_smi("1500, 2070, 1390.0, Active, Not Active, Not Active, Not Active, Active")
    c = bench.ClockSampler(0)
    t0 = time.time()
    out = c.stop(t0, t0 + 0.001)
    assert out["samples"] >= 1 and out["window"].startswith("nearest")
    assert out["reasons"] == ["sw_power_cap"] and out["sm_mhz"] == 1500.0
