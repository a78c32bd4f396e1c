"""The request-loop schedule tuner's choice rule (CPU only: the request loop is replaced by a
stand-in that reports fixed spans and latencies per candidate)."""
import pytest

from xtb_gb300 import interface as X
from xtb_gb300 import tuning


class _Res:
    def __init__(self, t_done, latency):
        self.t_submit, self.t_start, self.t_done = 0.0, 0.0, t_done
        self.latency = latency


def _fake_server(table):
    """A Server whose pass of 100 requests, for the candidate it was built with, spans the given
    time and whose two slowest requests take the given latency (its p99)."""
    class Srv:
        def __init__(self, plain_workers, iters_per_step, pool_max_nao, coop_blocks, **kw):
            self.span, self.lat = table[(plain_workers, iters_per_step, pool_max_nao, coop_blocks)]
            self.k = 0

        def submit(self, *a, **kw):
            self.k += 1
            return self.k

        def wait(self, i, check=True):
            return _Res(self.span * i / 100.0, self.lat if i <= 2 else 0.01)

        def close(self):
            pass
    return Srv


@pytest.mark.parametrize("spans,lats,want", [
    # a candidate 2% slower with half the tail latency wins
    ((4.28, 4.36, 5.0), (4.4, 2.2, 1.0), 1),
    # outside the tie band the shortest span wins whatever its latency
    ((4.00, 4.20, 5.0), (4.4, 2.2, 1.0), 0),
    # equal spans: the lower latency
    ((4.0, 4.0, 4.0), (3.0, 2.0, 2.5), 1),
])
def test_span_then_tail_latency(monkeypatch, spans, lats, want):
    cands = ((8, 1, 192, 76), (6, 1, 256, 76), (4, 1, 512, 0))
    table = {c: (s, l) for c, s, l in zip(cands, spans, lats)}
    monkeypatch.setattr(X, "Server", _fake_server(table))
    monkeypatch.setattr(tuning, "_schedules", {})
    reqs = [{"numbers": [1, 1], "positions": [[0.0, 0.0, float(k)], [0.0, 0.0, k + 1.4]], "gradient": False}
            for k in range(100)]
    s = tuning.schedule(reqs, candidates=cands)
    assert (s["plain_workers"], s["iters_per_step"], s["pool_max_nao"], s["coop_blocks"]) == cands[want]
    assert len(s["span_s"]) == len(s["p99_s"]) == 3
    assert tuning.schedule(reqs, candidates=cands) is s                 # kept per stream


def test_finalists_decide_by_median(monkeypatch):
    """A candidate that looks best in its first pass but not in its repeats loses to one that is
    steadily short: the choice goes by the finalists' median span."""
    cands = ((8, 1, 192, 76), (6, 1, 256, -20), (4, 1, 512, 0), (6, 1, 512, 0))
    seq = {cands[0]: [3.60, 4.20, 4.30], cands[1]: [3.80, 3.78, 3.82], cands[2]: [3.90, 4.00, 4.10],
           cands[3]: [5.00]}
    calls = {}

    class Srv:
        def __init__(self, plain_workers, iters_per_step, pool_max_nao, coop_blocks, **kw):
            c = (plain_workers, iters_per_step, pool_max_nao, coop_blocks)
            k = calls.get(c, 0)
            calls[c] = k + 1
            self.span = seq[c][k]
            self.k = 0

        def submit(self, *a, **kw):
            self.k += 1
            return self.k

        def wait(self, i, check=True):
            return _Res(self.span * i / 100.0, 1.0)

        def close(self):
            pass

    monkeypatch.setattr(X, "Server", Srv)
    monkeypatch.setattr(tuning, "_schedules", {})
    reqs = [{"numbers": [1, 1], "positions": [[0.0, 0.0, float(k)], [0.0, 0.0, k + 1.4]], "gradient": False}
            for k in range(100)]
    s = tuning.schedule(reqs, candidates=cands)
    assert (s["plain_workers"], s["iters_per_step"], s["pool_max_nao"], s["coop_blocks"]) == cands[1]
    assert calls == {cands[0]: 3, cands[1]: 3, cands[2]: 3, cands[3]: 1}     # three finalists, two repeats
    assert len(s["span_s"][tuning._label(cands[1])]) == 3
