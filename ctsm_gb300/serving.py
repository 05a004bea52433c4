"""Serving mode: a device-resident pool that run requests join and leave while
others run (continuous batching), with a Poisson request stream and latency
statistics.

A request is a single point or a region: its own columns (with 1-4 patches
each and one gridcell per column), a number of 1800 s model steps and a seed
that draws its state and its perturbed parameters.  `serve` admits arrived
requests in arrival order as soon as the pool has free slot ranges for them
(first in, first out: a request that does not fit holds the ones behind it),
enqueues one tick at a time (every running request advances one step), and
evicts each request as its last step completes: its final state is copied
back into the request's own host buffers, which are page-locked when CUDA is
available.  Columns never interact, so a request's results are the same
whatever else shares the pool.

There is no reference counterpart: CTSM runs one configuration per
executable.  The step each tick runs is the batch engine's full step
(CanopyFluxes, root sink, SoilTemperature, SoilWater)."""
import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import abi, canopy_inputs, full_inputs
from ._lib import load, check, CtsmError

E_FULL = 11
STEPS_PER_DAY = 48          # 1800 s steps


class PoolConfig(C.Structure):
    _fields_ = [("col_capacity", C.c_int32), ("patch_capacity", C.c_int32), ("grid_capacity", C.c_int32),
                ("dtime", C.c_double), ("e_ice", C.c_double), ("snow_thermal_cond_method", C.c_int32),
                ("stomatalcond_method", C.c_int32), ("itmax_canopy_fluxes", C.c_int32), ("with_canopy", C.c_int32),
                ("max_inflight", C.c_int32), ("rootmoist", C.c_int32), ("hydrology", C.c_int32)]


class PoolRequest(C.Structure):
    _fields_ = [("ncol", C.c_int32), ("npatch", C.c_int32), ("ngrid", C.c_int32), ("nsteps", C.c_int32),
                ("sw", C.POINTER(abi.SoilWaterIO)), ("st", C.POINTER(abi.SoilTempIO)), ("cio", C.POINTER(abi.CanopyIO)),
                ("rm", C.POINTER(abi.RootMoistIO)), ("hy", C.POINTER(abi.HydrologyIO)),
                ("rootr", C.POINTER(C.c_double)), ("medlynslope_p", C.POINTER(C.c_double)),
                ("medlynintercept_p", C.POINTER(C.c_double))]


def _bind(L):
    if getattr(L, "_pool_bound", False):
        return
    P = C.POINTER
    L.ctsmg_pool_slot_bytes.argtypes = [C.c_int32, P(C.c_int64), P(C.c_int64), P(C.c_int64)]
    L.ctsmg_pool_slot_bytes_cfg.argtypes = [P(PoolConfig), P(C.c_int64), P(C.c_int64), P(C.c_int64)]
    L.ctsmg_pool_admit_request.argtypes = [C.c_void_p, P(PoolRequest), P(C.c_int32)]
    L.ctsmg_pool_evict_request.argtypes = [C.c_void_p, C.c_int32, P(PoolRequest), P(C.c_int32)]
    L.ctsmg_pool_create.argtypes = [P(C.c_void_p), P(PoolConfig), P(abi.CanopyParams), P(abi.Pftcon)]
    L.ctsmg_pool_admit.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P(abi.SoilWaterIO),
                                   P(abi.SoilTempIO), P(abi.CanopyIO), P(C.c_double), P(C.c_double), P(C.c_double),
                                   P(C.c_int32)]
    L.ctsmg_pool_tick.argtypes = [C.c_void_p, P(C.c_int64)]
    L.ctsmg_pool_poll.argtypes = [C.c_void_p, P(C.c_int32), C.c_int32, P(C.c_int32)]
    L.ctsmg_pool_evict.argtypes = [C.c_void_p, C.c_int32, P(abi.SoilWaterIO), P(abi.SoilTempIO), P(abi.CanopyIO),
                                   P(C.c_int32)]
    L.ctsmg_pool_sync.argtypes = [C.c_void_p]
    L.ctsmg_pool_free.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32), P(C.c_int32)]
    L.ctsmg_pool_destroy.argtypes = [C.c_void_p]
    L._pool_bound = True


def slot_bytes(canopy=True, rootmoist=False, hydrology=False):
    """(column, patch, gridcell) device bytes per slot."""
    L = load()
    _bind(L)
    c, p, g = C.c_int64(), C.c_int64(), C.c_int64()
    cfg = PoolConfig(with_canopy=1 if canopy else 0, rootmoist=1 if rootmoist else 0,
                     hydrology=1 if hydrology else 0)
    check(L.ctsmg_pool_slot_bytes_cfg(C.byref(cfg), C.byref(c), C.byref(p), C.byref(g)))
    return c.value, p.value, g.value


def capacities(budget_bytes, canopy=True, patches_per_column=4, rootmoist=False, hydrology=False):
    """Slot capacities that fit `budget_bytes`: one gridcell and up to
    `patches_per_column` patches per column slot, so patches and gridcells
    never run out before columns do."""
    c, p, g = slot_bytes(canopy, rootmoist, hydrology)
    per_col = c + patches_per_column * p + g
    ncol = int(budget_bytes // per_col)
    if ncol < 1:
        raise ValueError("budget below one column")
    ncol = min(ncol, (2 ** 31 - 1) // patches_per_column)         # int32 slot positions
    return ncol, patches_per_column * ncol, ncol


@dataclass
class Request:
    """One run request.  `state` holds its arrays (dense, 1-based maps); after
    eviction it holds the final state."""
    rid: int
    seed: int
    ncol: int
    nsteps: int
    arrival: float = 0.0
    state: dict = None
    npatch: int = 0
    ngrid: int = 0
    rootr: np.ndarray = None
    factors: dict = None
    slot: int = -1
    t_admit: float = math.nan
    t_done: float = math.nan
    steps_done: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def days(self):
        return self.nsteps / STEPS_PER_DAY

    def column_steps(self):
        return self.ncol * self.nsteps


def _pinned_like(a):
    try:
        import torch
        if torch.cuda.is_available():
            t = torch.empty(a.shape, dtype=getattr(torch, {"f8": "float64", "i4": "int32"}[a.dtype.str[1:]]),
                            pin_memory=True)
            out = t.numpy()
            out[...] = a
            return out, t
    except (ImportError, KeyError, RuntimeError):
        pass
    return np.ascontiguousarray(a), None


def make_request(rid, seed, ncol, nsteps, arrival=0.0, pinned=True, physical=False):
    """A request's state from its seed: the full-step inputs (snow, uneven
    bedrock, 1-4 patches per column) with the eight perturbed parameters
    drawn log-uniformly in [0.5, 1.5] times their defaults, as for ensemble
    members (medlynslope / medlynintercept per patch, om_frac_sf in the soil
    properties; the others are inert on this path).  physical: for a pool
    with the root moisture stress and the hydrology -- the columns without
    snow layers (melted layers are removed only by SnowHydrology, outside the
    path), with the root moisture stress components (transpiration follows
    the soil water) and the hydrology's (drainage takes water out of the
    column and repairs over-dried layers), so that a year-long request stays
    in the physical domain."""
    r = np.random.Generator(np.random.Philox(seed))
    factors = {k: float(np.exp(r.uniform(np.log(0.5), np.log(1.5)))) for k in full_inputs.ENSEMBLE_PARAMS}
    A, npatch, ngrid, rootr = full_inputs.full_state(ncol, om_frac_sf=factors["om_frac_sf"], rng=r)
    if physical:
        full_inputs.snow_free(A)
        full_inputs.add_rootmoist_fields(A, npatch, rootr, rng=r)
        full_inputs.add_hydrology_fields(A, r)
    pft = canopy_inputs.DEFAULT_PFT
    it = A["itype"]
    A["medlynslope_p"] = np.array([row[6] for row in pft])[it] * factors["medlynslope"]
    A["medlynintercept_p"] = np.array([row[7] for row in pft])[it] * factors["medlynintercept"]
    keep = []
    if pinned:
        for k in list(A):
            A[k], t = _pinned_like(A[k])
            if t is not None:
                keep.append(t)
        rootr, t = _pinned_like(rootr)
        if t is not None:
            keep.append(t)
    q = Request(rid, seed, ncol, nsteps, arrival, A, npatch, ngrid, np.ascontiguousarray(rootr), factors)
    q.extra["pinned"] = keep
    return q


def stream_draws(n, rate, seed=0, cols=(1, 50000), steps=(48, 17520)):
    """Arrival times (Poisson process at `rate` per second, first at 0),
    column counts (log-uniform over [cols[0], cols[1]], integer), lengths
    (uniform integers in `steps`) and per-request seeds of n requests."""
    r = np.random.Generator(np.random.Philox(seed))
    gaps = r.exponential(1.0 / rate, n) if rate > 0 else np.zeros(n)
    arr = np.cumsum(gaps) - gaps[0]
    ncols = np.floor(np.exp(r.uniform(np.log(cols[0]), np.log(cols[1] + 1), n))).astype(np.int64)
    ncols = np.clip(ncols, cols[0], cols[1])
    lens = r.integers(steps[0], steps[1] + 1, n)
    seeds = r.integers(1, 2 ** 62, n)
    return arr, ncols, lens, seeds


def request_stream(n, rate, seed=0, cols=(1, 50000), steps=(48, 17520), pinned=True, physical=False):
    """n requests drawn by stream_draws, each with its state."""
    arr, ncols, lens, seeds = stream_draws(n, rate, seed, cols, steps)
    return [make_request(i, int(seeds[i]), int(ncols[i]), int(lens[i]), float(arr[i]), pinned, physical)
            for i in range(n)]


class Pool:
    """Handle on ctsmg_pool: capacities from a device-memory budget or given
    directly."""

    def __init__(self, budget_bytes=None, col_capacity=None, canopy=True, dtime=1800.0, e_ice=6.0,
                 snow_thermal_cond_method=0, stomatalcond_method=1, itmax=40, params=None, pftcon=None,
                 max_inflight=2, patches_per_column=4, rootmoist=False, hydrology=False):
        self.L = load()
        _bind(self.L)
        if col_capacity is None:
            cc, pc, gc = capacities(budget_bytes, canopy, patches_per_column, rootmoist, hydrology)
        else:
            cc, pc, gc = col_capacity, patches_per_column * col_capacity, col_capacity
        self.capacity = (cc, pc, gc)
        self.canopy = canopy
        self.rootmoist = bool(rootmoist and canopy)
        self.hydrology = bool(hydrology)
        cfg = PoolConfig(cc, pc, gc, dtime, e_ice, snow_thermal_cond_method, stomatalcond_method, itmax,
                         1 if canopy else 0, max_inflight, 1 if self.rootmoist else 0, 1 if self.hydrology else 0)
        self._par = params if params is not None else canopy_inputs.make_params()
        self._pft = pftcon if pftcon is not None else canopy_inputs.make_pftcon()
        self.h = C.c_void_p()
        check(self.L.ctsmg_pool_create(C.byref(self.h), C.byref(cfg), C.byref(self._par), C.byref(self._pft)))

    def _ios(self, q):
        A, n, npch, ng = q.state, q.ncol, q.npatch, q.ngrid
        sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, A, n)
        st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, A, n, npch)
        ci = abi.make_io(abi.CanopyIO, abi.CANOPY_FIELDS, A, n, npch, ng, 1) if self.canopy else None
        rm = abi.make_io(abi.RootMoistIO, abi.ROOTMOIST_FIELDS, A, n, npch) if self.rootmoist else None
        hy = abi.make_io(abi.HydrologyIO, abi.HYDROLOGY_FIELDS, A, n) if self.hydrology else None
        return sw, st, ci, rm, hy

    def _request(self, q, ios):
        sw, st, ci, rm, hy = ios
        dp = C.POINTER(C.c_double)
        ptr = lambda io, T: C.pointer(io) if io is not None else C.POINTER(T)()
        return PoolRequest(q.ncol, q.npatch, q.ngrid, q.nsteps, C.pointer(sw), C.pointer(st),
                           ptr(ci, abi.CanopyIO), ptr(rm, abi.RootMoistIO), ptr(hy, abi.HydrologyIO),
                           q.rootr.ctypes.data_as(dp) if self.canopy else dp(),
                           q.state["medlynslope_p"].ctypes.data_as(dp) if "medlynslope_p" in q.state else dp(),
                           q.state["medlynintercept_p"].ctypes.data_as(dp) if "medlynintercept_p" in q.state else dp())

    def admit(self, q):
        """Admits request q; returns its slot, or None when the pool is full."""
        ios = self._ios(q)
        req = self._request(q, ios)
        slot = C.c_int32()
        rc = self.L.ctsmg_pool_admit_request(self.h, C.byref(req), C.byref(slot))
        if rc == E_FULL:
            return None
        check(rc)
        q.slot = slot.value
        return q.slot

    def tick(self):
        n = C.c_int64()
        check(self.L.ctsmg_pool_tick(self.h, C.byref(n)))
        return n.value

    def poll(self, cap=256):
        buf = (C.c_int32 * cap)()
        n = C.c_int32()
        check(self.L.ctsmg_pool_poll(self.h, buf, cap, C.byref(n)))
        return list(buf[:n.value])

    def evict(self, q):
        """Copies q's final state into q.state and frees its slots; returns
        the number of steps it ran."""
        ios = self._ios(q)
        req = self._request(q, ios)
        steps = C.c_int32()
        check(self.L.ctsmg_pool_evict_request(self.h, q.slot, C.byref(req), C.byref(steps)))
        q.steps_done = steps.value
        q.slot = -1
        return steps.value

    def sync(self):
        check(self.L.ctsmg_pool_sync(self.h))

    def largest_free(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        check(self.L.ctsmg_pool_free(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def close(self):
        if self.h:
            self.L.ctsmg_pool_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def percentile(x, q):
    x = np.sort(np.asarray(x, dtype=np.float64))
    if x.size == 0:
        return math.nan
    return float(np.percentile(x, q, method="linear"))


def serve(pool, requests, time_limit=None, tick_clock=False, clock=time.perf_counter):
    """Runs the request stream through the pool.  Arrival times are seconds
    from the start (or tick numbers when tick_clock is set, which makes the
    admission order reproducible; the recorded admission and completion
    times are then tick numbers too).  Requests still running when time_limit
    runs out are stopped and evicted with the steps they ran.  Returns a dict
    of statistics (steady_column_steps_per_s: the rate from the tick at which
    the last request was admitted to the end); each request's record is on
    the request object."""
    queue = sorted(requests, key=lambda q: (q.arrival, q.rid))
    running = {}
    nq = 0
    ticks = 0
    col_steps = 0
    max_running_cols = 0
    t_all, cs_all = None, 0
    t0 = clock()

    def now():
        return float(ticks) if tick_clock else clock() - t0

    def finish(slot):
        q = running.pop(slot)
        pool.evict(q)
        q.t_done = now()
        A = q.state
        if A is not None and "t_soisno" in A:
            bad = ~(np.isfinite(A["t_soisno"]).all(axis=0) & np.isfinite(A["h2osoi_liq"]).all(axis=0))
            if "t_veg" in A:
                bad |= np.bincount(A["patch_column"] - 1, weights=~np.isfinite(A["t_veg"]), minlength=q.ncol) > 0
            q.extra["nonfinite_columns"] = int(bad.sum())

    while nq < len(queue) or running:
        t = now()
        while nq < len(queue) and queue[nq].arrival <= t:
            q = queue[nq]
            if pool.admit(q) is None:
                if not running:
                    raise CtsmError(E_FULL, "request %d does not fit the empty pool" % q.rid)
                break
            q.t_admit = now()
            running[q.slot] = q
            nq += 1
        if not running:
            if tick_clock:
                ticks = int(math.ceil(queue[nq].arrival))
            else:
                time.sleep(max(0.0, min(queue[nq].arrival - now(), 0.05)))
            continue
        if time_limit is not None and clock() - t0 > time_limit:
            break
        n = pool.tick()
        ticks += 1
        col_steps += n
        max_running_cols = max(max_running_cols, n)
        if nq == len(queue) and t_all is None:      # every request admitted: steady part begins
            t_all, cs_all = clock() - t0, col_steps - n
        for slot in pool.poll():
            finish(slot)
    for slot in list(running):          # stopped by the time limit
        finish(slot)
    pool.sync()
    wall = clock() - t0
    done = [q for q in requests if q.steps_done == q.nsteps]
    per_day = [(q.t_done - q.arrival) / q.days for q in done]
    # pace of every request that ran: seconds from arrival to its end (or the
    # time limit) per simulated day it advanced
    pace = [(q.t_done - q.arrival) / (q.steps_done / STEPS_PER_DAY) for q in requests if q.steps_done > 0]
    nonfinite = [q.extra.get("nonfinite_columns", 0) for q in requests if q.steps_done > 0]
    wait = [q.t_admit - q.arrival for q in requests if not math.isnan(q.t_admit)]
    steady = None
    if t_all is not None and wall - t_all > 1.0:
        steady = (col_steps - cs_all) / (wall - t_all)
    return dict(wall_s=wall, ticks=ticks, column_steps=col_steps, column_steps_per_s=col_steps / wall if wall > 0 else 0.0,
                steady_column_steps_per_s=steady, steady_from_s=t_all,
                requests=len(requests), completed=len(done), stopped=len(requests) - len(done) - (len(queue) - nq),
                never_admitted=len(queue) - nq, max_running_columns=max_running_cols,
                p50_s_per_day=percentile(per_day, 50), p99_s_per_day=percentile(per_day, 99),
                p50_pace_s_per_day=percentile(pace, 50), p99_pace_s_per_day=percentile(pace, 99),
                p50_wait_s=percentile(wait, 50), p99_wait_s=percentile(wait, 99),
                nonfinite_requests=int(sum(1 for n in nonfinite if n > 0)), nonfinite_columns=int(sum(nonfinite)))


def main(argv=None):
    """Command line: run a Poisson request stream through a pool and print its
    statistics as one JSON line; --out also writes every request's record
    (arrival, admission, completion, time per simulated day, whether its
    final state is finite, its share of patches at itmax)."""
    import argparse
    import json
    p = argparse.ArgumentParser(prog="python -m ctsm_gb300.serving",
                                description="Poisson request stream through the serving pool")
    p.add_argument("--requests", type=int, default=64)
    p.add_argument("--rate", type=float, default=2.0, help="arrivals per second")
    p.add_argument("--seed", type=int, default=2026)
    p.add_argument("--budget-gb", type=float, default=150.0, help="device memory budget of the pool")
    p.add_argument("--time-limit", type=float, default=None, help="seconds; default: run to completion")
    p.add_argument("--out", default=None, help="JSON file for the statistics and per-request records")
    p.add_argument("--cols-max", type=int, default=50000, help="largest request (columns)")
    p.add_argument("--plain", action="store_true",
                   help="the step without the root moisture stress and the hydrology, on the workload's snowy "
                        "columns")
    a = p.parse_args(argv)
    from . import soil
    soil.init()
    t0 = time.time()
    reqs = request_stream(a.requests, a.rate, seed=a.seed, cols=(1, a.cols_max), physical=not a.plain)
    gen_s = time.time() - t0
    pool = Pool(budget_bytes=a.budget_gb * 1e9, rootmoist=not a.plain, hydrology=not a.plain)
    try:
        st = serve(pool, reqs, time_limit=a.time_limit)
    finally:
        pool.close()
    st["gen_s"] = gen_s
    st["offered_column_steps"] = int(sum(q.column_steps() for q in reqs))
    if a.out:
        recs = []
        for q in reqs:
            A = q.state
            recs.append(dict(rid=q.rid, ncol=q.ncol, nsteps=q.nsteps, days=q.days, arrival=q.arrival,
                             admit=q.t_admit, done=q.t_done, s_per_day=(q.t_done - q.arrival) / q.days,
                             finite=bool(np.isfinite(A["t_soisno"]).all() and np.isfinite(A["t_veg"]).all()),
                             nonfinite_columns=q.extra.get("nonfinite_columns", 0),
                             liq_min=float(A["h2osoi_liq"][abi.NLEVSNO:abi.NLEVSNO + abi.NLEVSOI].min()),
                             itmax_frac=float((A["num_iter"] >= 40).mean())))
        with open(a.out, "w") as f:
            json.dump({"stats": st, "requests": recs}, f)
    print(json.dumps(st), flush=True)


if __name__ == "__main__":
    main()
