"""Host side of the serving mode, without a GPU: slot sizing against the
memory budget, the request-stream distributions, and the admission loop
(first in, first out, waiting for free slots, stopping at a time limit)
driven through a stand-in pool with the same interface."""
import math

import numpy as np
import pytest

from ctsm_gb300 import abi, serving


def test_slot_bytes_match_manifest():
    c, p, g = serving.slot_bytes(canopy=True)
    seen, cb, pb, gb = set(), 0, 0, 0
    lv = {"C": 1, "P": 1, "GR": 1, "SS": 37, "ZI": 38, "G": 25, "S": 20, "SN": 12, "PL": 13, "PS": 20}
    for (n, kind, dt, use) in abi.SOILWATER_FIELDS + abi.SOILTEMP_FIELDS + abi.CANOPY_FIELDS:
        if n in seen:
            continue
        seen.add(n)
        b = lv[kind] * (8 if dt == abi.F64 else 4)
        if kind in ("P", "PL", "PS"):
            pb += b
        elif kind == "GR":
            gb += b
        else:
            cb += b
    assert c == cb + 6 * 38 * 8 + 4
    rec = p - (pb + 20 * 8 + 16 + 4)          # rootr, Medlyn pair, filter entry, CanopyFluxes iteration record
    assert rec % 4 == 0 and 0 < rec < 2048
    assert g == gb


def test_capacities_for_150_gb():
    cc, pc, gc = serving.capacities(150e9)
    c, p, g = serving.slot_bytes()
    assert pc == 4 * cc and gc == cc
    assert cc * (c + 4 * p + g) <= 150e9 < (cc + 1) * (c + 4 * p + g)
    assert cc > 5_000_000


def test_stream_distributions():
    arr, ncols, lens, seeds = serving.stream_draws(20000, rate=2.0, seed=5)
    assert arr[0] == 0.0 and np.all(np.diff(arr) >= 0)
    assert abs(np.mean(np.diff(arr)) - 0.5) < 0.02
    assert ncols.min() >= 1 and ncols.max() <= 50000
    lg = np.log(ncols + 0.5)
    assert abs(np.mean(lg) - math.log(50001) / 2) < 0.1          # log-uniform
    assert lens.min() >= 48 and lens.max() <= 17520
    assert abs(lens.mean() - (48 + 17520) / 2) < 150
    assert len(np.unique(seeds)) == 20000


class FakePool:
    """Capacity in columns, one running step per tick, completion visible
    one tick after the last step (like a queued device)."""

    def __init__(self, cap):
        self.cap, self.used, self.run, self.slots, self.done = cap, 0, {}, 0, []
        self.ticks = 0

    def admit(self, q):
        if self.used + q.ncol > self.cap:
            return None
        q.slot = self.slots
        self.slots += 1
        self.used += q.ncol
        self.run[q.slot] = [q, 0]
        return q.slot

    def tick(self):
        self.ticks += 1
        n = 0
        ready = list(self.done)
        self.done = []
        for s, (q, k) in list(self.run.items()):
            if k < q.nsteps:
                self.run[s][1] = k + 1
                n += q.ncol
                if k + 1 == q.nsteps:
                    self.done.append(s)
        self.ready = ready
        return n

    def poll(self):
        r, self.ready = getattr(self, "ready", []), []
        return r

    def evict(self, q):
        q2, k = self.run.pop(q.slot)
        self.used -= q.ncol
        q.steps_done = k
        return k

    def sync(self):
        pass


def _req(i, n, steps, arr):
    return serving.Request(i, i, n, steps, arr, {}, 0, 0, None, {})


def test_serve_fifo_and_waiting():
    reqs = [_req(0, 700, 5, 0), _req(1, 600, 3, 1), _req(2, 200, 2, 1), _req(3, 50, 1, 30)]
    st = serving.serve(FakePool(1000), reqs, tick_clock=True)
    assert st["completed"] == 4 and st["never_admitted"] == 0
    assert reqs[1].t_admit >= reqs[0].t_done and reqs[2].t_admit >= reqs[1].t_admit
    assert st["column_steps"] == sum(q.ncol * q.nsteps for q in reqs)
    assert st["p50_s_per_day"] >= 0


def test_serve_refuses_request_larger_than_pool():
    with pytest.raises(Exception):
        serving.serve(FakePool(100), [_req(0, 101, 2, 0)], tick_clock=True)


def test_serve_time_limit_stops_running():
    reqs = [_req(0, 10, 10 ** 9, 0), _req(1, 10, 3, 0)]
    st = serving.serve(FakePool(100), reqs, time_limit=0.05)
    assert reqs[1].steps_done == 3 and 0 < reqs[0].steps_done < 10 ** 9
    assert st["completed"] == 1 and st["stopped"] == 1


def test_percentile():
    assert serving.percentile([1, 2, 3, 4], 50) == 2.5
    assert math.isnan(serving.percentile([], 99))


def test_command_line_parses(capsys):
    from ctsm_gb300 import serving
    with pytest.raises(SystemExit) as e:
        serving.main(["--help"])
    assert e.value.code == 0 and "--requests" in capsys.readouterr().out
