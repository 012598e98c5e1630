"""bench.py's workload naming and its in-flight slot assignment, on the CPU: the default line
carries the headline metric verbatim, other sizes name their own size, both arms describe the
same workload, and the timed steps alternate over the slots in order."""
import json
import os
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)


def test_default_metric_is_the_headline_metric():
    import bench

    metric, config = bench.workload_config(bench.parse([]))
    baseline = os.path.join(ROOT, "BASELINE.json")
    if os.path.exists(baseline):
        assert metric == json.load(open(baseline))["metric"]
    assert metric == bench.METRIC
    assert (config["n"], config["dim"], config["queries"], config["M"], config["k"]) == (1_000_000, 1536, 10_000,
                                                                                         64, 10)


def test_other_sizes_name_their_size():
    import bench

    assert "100k×1536" in bench.workload_config(bench.parse(["--n", "100000"]))[0]
    assert "20k×128" in bench.workload_config(bench.parse(["--n", "20000", "--dim", "128"]))[0]
    assert "12345×1536" in bench.workload_config(bench.parse(["--n", "12345"]))[0]
    assert "1M×960" in bench.workload_config(bench.parse(["--workload", "gist960"]))[0]


def test_both_arms_share_the_config():
    import bench

    ours = bench.parse(["--inflight", "3"])
    ref = bench.parse(["--impl", "reference"])
    assert bench.workload_config(ours) == bench.workload_config(ref)
    assert bench.parse([]).inflight == 2


class _FakeStream:
    def __init__(self, log, name):
        self.log, self.name = log, name

    def wait_event(self, ev):
        self.log.append(("wait", self.name))


class _FakeCuda:
    """Just enough of torch.cuda for bench.pipelined_ms: records which stream each step ran on."""

    def __init__(self, log):
        self.log = log
        self.current = "main"
        outer = self

        class Event:
            def __init__(self, enable_timing=False):
                pass

            def record(self, stream=None):
                outer.log.append(("record", outer.current))

            def elapsed_time(self, other):
                return 12.0

        class Ctx:
            def __init__(self, stream):
                self.stream = stream

            def __enter__(self):
                self.prev = outer.current
                outer.current = self.stream.name

            def __exit__(self, *exc):
                outer.current = self.prev

        class Current:
            def wait_stream(self, s):
                outer.log.append(("join", s.name))

        self.Event = Event
        self.stream = Ctx
        self._current = Current()

    def current_stream(self):
        return self._current

    def synchronize(self):
        self.log.append(("sync", None))


def test_pipelined_steps_alternate_over_the_slots():
    import types

    import bench

    log = []
    fake = types.SimpleNamespace(cuda=_FakeCuda(log))
    streams = [_FakeStream(log, f"s{j}") for j in range(3)]
    ran = []
    fns = [(lambda j: (lambda: ran.append((j, fake.cuda.current))))(j) for j in range(3)]
    ms = bench.pipelined_ms(fake, fns, streams, 7)
    assert ran == [(s % 3, f"s{s % 3}") for s in range(7)]  # step s on slot s mod 3, on its stream
    assert ms == 12.0 / 7
    kinds = [k for k, _ in log]
    # both syncs outside the region; every stream waits on the start and is joined before the end
    assert kinds[0] == "sync" and kinds[-1] == "sync"
    start, end = kinds.index("record"), len(kinds) - 1 - kinds[::-1].index("record")
    assert [n for k, n in log[start:end] if k == "wait"] == ["s0", "s1", "s2"]
    assert [n for k, n in log[start:end] if k == "join"] == ["s0", "s1", "s2"]
    assert log[start] == ("record", "main") and log[end] == ("record", "main")
