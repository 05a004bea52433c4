"""Benchmark: column-timesteps/s of the fused SoilWater + SoilTemperature step.

Workload (N=1): the uneven-column batch -- 524,288 columns of FP64 state,
nbedrock ~ U{3..20}, snl ~ U{0..-12} (snow thickness 0.01-0.5 m, density
50-400 kg/m3, T 230-273.15 K), soil properties and forcing as in the plain
4,096-column case, 1800 s steps.  One bench step = one model step over every
column = one CUDA-graph replay of the fused step kernel.  The resident state
(~3.4 GB) is far larger than L2 (129 MB), so consecutive steps stream from HBM.

Lines reported:
  value  batched resident engine, inputs already in HBM (CUDA events per step)
  e2e    plain drop-in C-ABI calls (ctsmg_soilwater + ctsmg_soiltemperature) on
         pinned host buffers, host<->device copies inside the timed region
  cpu_baseline / --impl reference   the CPU oracle (C++ restatement of the
         reference Fortran, OpenMP over clumps of columns) on the host cores
Extra keys on the same line (rank 0, N = 1):
  canopy    CanopyFluxes + Photosynthesis over 2,097,152 patches (1-4 per
            column): device-resident steps and the plain drop-in call
  ensemble  256 perturbed-parameter members (columns U{512..8192} each) through
            the full soil + canopy step, batched vs one set of plain drop-in
            calls per member
  serving   a Poisson stream of run requests (192 at 8/s; columns log-uniform
            1..50,000, lengths U{48..17,520} steps) through the device pool
            with a 150 GB admission budget, bounded in wall time
Under torchrun each rank advances its own 524,288-column shard (no
collective on the data path; weak scaling); time is the max over ranks.
"""
import argparse
import copy
import ctypes as C
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "column-timesteps/s batched vs plain on 1 GB300 at <=1e-9 rel err; p50/p99 latency"
UNIT = "column-timesteps/s"
WORKLOAD = "uneven-column batch: SoilWater(ZD09)+SoilTemperature, 524288 cols, nbedrock U{3..20}, snl U{0..-12}, dt=1800s"
DT = 1800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=48)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--ncol", type=int, default=524288)
    p.add_argument("--seed", type=int, default=2026)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-gate", action="store_true", help="skip the oracle parity and balance check of the run")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-canopy", action="store_true")
    p.add_argument("--no-ensemble", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--canopy-patches", type=int, default=2097152)
    p.add_argument("--canopy-steps", type=int, default=8)
    p.add_argument("--ens-members", type=int, default=256)
    p.add_argument("--ens-steps", type=int, default=48)
    p.add_argument("--serve-requests", type=int, default=192)
    p.add_argument("--serve-rate", type=float, default=8.0)
    p.add_argument("--serve-seconds", type=float, default=60.0)
    p.add_argument("--serve-budget-gb", type=float, default=150.0)
    p.add_argument("--no-clm5", action="store_true")
    p.add_argument("--clm5-cols", type=int, default=262144)
    p.add_argument("--clm5-steps", type=int, default=8)
    return p.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_seed(seed, rank):
    """Each rank advances its own shard of columns (weak scaling): same size,
    its own draws."""
    return seed + rank


def max_over_ranks(x, ws, device):
    """The slowest rank's time (the job's time); all_reduce on `device` (cuda
    with NCCL, cpu with gloo)."""
    if ws == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(ws, units_per_rank, steps, t_max):
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time."""
    return ws * units_per_rank * steps / t_max


def make_inputs(ncol, seed):
    from ctsm_gb300 import inputs
    return inputs.soil_columns(ncol, seed=seed, snow=True, nbedrock=(3, 20))


# ---------------------------------------------------------------- CPU oracle
def bench_config(A, ncol):
    """The workload's `config` dict: identical on both arms (it describes the
    inputs only; how the GPU arm ran them goes under "tuning")."""
    state_gb = sum(v.nbytes for v in A.values()) / 1e9 * ncol / A["zwt"].shape[0]
    return {"workload": WORKLOAD, "ncol_per_gpu": ncol, "mean_snow_layers": float(-A["snl"].mean()),
            "dtime_s": DT, "l2": "inputs larger than L2 (state %.2f GB vs 129 MB L2)" % state_gb}


class OracleSoilStepper:
    """The CPU oracle (C++ restatement, OpenMP over clumps of columns) stepping
    a private copy of the first `ncol` columns of A through the benched step:
    SoilWater (Zeng-Decker), SoilTemperature, the h2osoi_vol refresh.  With
    noise = (ulps, seed) every libm result of the oracle is perturbed by up to
    `ulps` ulp (a deterministic hash of its arguments); with track_water the
    column water budget error of every step (BalanceCheckMod.F90:592-658 over
    the scoped fluxes) is kept as water_err_max."""

    def __init__(self, A, ncol=None, noise=None, track_water=False):
        from ctsm_gb300 import abi
        from oracle import oracle as orc
        self.L = orc.lib()
        n = A["zwt"].shape[0] if ncol is None else min(ncol, A["zwt"].shape[0])
        self.n = n
        # one patch per column in this workload, so patch arrays slice like column arrays
        self.S = {k: np.array(v[..., :n], order="C", copy=True) for k, v in A.items()}
        self.b = abi.Bounds(1, n, 1, n)
        self.filt = np.arange(1, n + 1, dtype=np.int32)
        self.fp = self.filt.ctypes.data_as(C.POINTER(C.c_int32))
        self.sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS, self.S, n)
        self.st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, self.S, n, n)
        self.noise = noise
        self.water_err_max = np.zeros(n) if track_water else None

    def _water(self):
        from ctsm_gb300.abi import NLEVSNO, NLEVSOI
        S = self.S
        LS = -NLEVSNO + 1
        w = S["h2osfc"] + S["h2osno_no_layers"]
        for j in range(LS, NLEVSOI + 1):
            w = w + np.where(j >= S["snl"] + 1, S["h2osoi_liq"][j - LS] + S["h2osoi_ice"][j - LS], 0.0)
        return w

    def step(self, k=1):
        from ctsm_gb300 import inputs
        from ctsm_gb300.abi import NLEVSNO, NLEVSOI
        if self.noise:
            self.L.oracle_set_libm_noise(int(self.noise[0]), int(self.noise[1]))
        try:
            for _ in range(k):
                w0 = self._water() if self.water_err_max is not None else None
                rc = self.L.oracle_soilwater(C.byref(self.b), self.n, self.fp, C.byref(self.sw), 6.0, DT)
                rc = rc or self.L.oracle_soiltemperature(C.byref(self.b), self.n, self.fp, C.byref(self.st), DT, 0)
                if rc:
                    raise RuntimeError("oracle step failed (rc %d)" % rc)
                if w0 is not None:
                    S = self.S
                    deep = S["zwt"] > S["zi"][NLEVSOI + NLEVSNO]
                    net = (S["qflx_infl"] - S["qflx_rootsoi"].sum(axis=0) - np.where(deep, S["qcharge"], 0.0)) * DT
                    np.maximum(self.water_err_max, np.abs((self._water() - w0) - net), out=self.water_err_max)
                inputs.refresh_h2osoi_vol(self.S)
        finally:
            if self.noise:
                self.L.oracle_set_libm_noise(0, 0)


def host_threads():
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def oracle_rate(A, npatch, target_s=10.0, max_cols=131072):
    """Column-steps/s of the CPU oracle on a bounded sample of the workload
    (the first `max_cols` columns, as many 1800 s steps as fit in ~target_s)."""
    o = OracleSoilStepper(A, max_cols)
    t0 = time.perf_counter()
    o.step()
    t1 = time.perf_counter() - t0
    steps = max(1, min(64, int(target_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    return o.n * steps / dt, o.n, steps, dt, host_threads()


# ---------------------------------------------------------------- correctness gate
# The benched run is checked against the oracle on the same inputs.  State
# variables and well-conditioned outputs are held to 1e-9 relative; the two
# outputs that difference nearly equal terms -- eflx_fgr12 (heat flux between
# levels 1 and 2 from the new temperatures, SoilTemperatureMod.F90:572-595)
# and xmf (latent heat of phase change summed over levels, :1492-1502) -- to
# 1e-9 relative plus the oracle's own spread under 4-ulp libm noise (and, for
# eflx_fgr12, the rounding bound of the two temperatures it differences), the
# test the parity suite applies.  Thresholds of BalanceCheckMod.F90:592-658
# (water) and :1103-1113 (errsoi).
GATE_TOL = 1e-9
GATE_STATE = ("h2osoi_liq", "h2osoi_ice", "t_soisno")
GATE_FLUXES = ("qcharge", "qflx_deficit", "t_grnd", "qflx_snomelt", "t_h2osfc")
GATE_CANCEL = ("eflx_fgr12", "xmf")
GATE_NOISE_ULPS = 4
GATE_NOISE_RUNS = 4


def _rel_err_cols(g, r, band=None):
    """Per-column max relative error |g-r| / (|r| + 1e-12 max|r|) over the
    levels of one field (level-major arrays: columns on the last axis); with a
    band, (|g-r| - band) clipped at 0 over 1e-9 |r| scaled to the same units."""
    g = np.asarray(g, dtype=np.float64)
    r = np.asarray(r, dtype=np.float64)
    scale = float(np.nanmax(np.abs(r))) if r.size else 0.0
    d = np.abs(g - r)
    if band is not None:
        d = np.maximum(d - band, 0.0)
    d = d / (np.abs(r) + 1e-12 * scale + 1e-300)
    d = np.where(np.isnan(g) & np.isnan(r), 0.0, d)
    d = np.where(np.isnan(g) ^ np.isnan(r), np.inf, d)
    return d if d.ndim == 1 else d.max(axis=0)


def compare_states(G, R, fields, tol=GATE_TOL, bands=None):
    """{field: max rel err}, and the per-column bool of any field above tol."""
    errs, worst = {}, None
    for k in fields:
        e = _rel_err_cols(G[k], R[k], None if bands is None else bands.get(k))
        errs[k] = float(e.max()) if e.size else 0.0
        worst = e if worst is None else np.maximum(worst, e)
    return errs, worst > tol


def fgr12_rounding_bound(R, ulps=8):
    """(1-cnfac) tk_1 ulps eps (|T_1| + |T_2|) / (z_2 - z_1): the error of
    eflx_fgr12 that the rounding of the two new temperatures alone allows,
    with tk_1 the interface conductivity of SoilTemperatureMod.F90:822-828."""
    from ctsm_gb300.abi import NLEVSNO
    eps = np.finfo(np.float64).eps
    r1, r2 = 1 + NLEVSNO - 1, 2 + NLEVSNO - 1
    t1, t2 = R["thk"][r1], R["thk"][r2]
    z1, z2, zi = R["z"][r1], R["z"][r2], R["zi"][1 + NLEVSNO]
    tk = t1 * t2 * (z2 - z1) / (t1 * (z2 - zi) + t2 * (zi - z1))
    return 0.5 * np.abs(tk) * ulps * eps * (np.abs(R["t_soisno"][r1]) + np.abs(R["t_soisno"][r2])) / (z2 - z1)


def xmf_rounding_bound(R, ulps=8):
    """ulps eps sum, over the levels that changed phase, of |T_j| / fact_j:
    the error of xmf that the rounding of each such level's temperature alone
    allows (Phasechange, SoilTemperatureMod.F90:1214-1527: xmf sums
    HFUS (wice0 - ice) / dtime with wice0 - ice = hm dtime / HFUS and
    hm = -tinc / fact_j, tinc = TFRZ - T_j)."""
    eps = np.finfo(np.float64).eps
    act = np.asarray(R["imelt"]) > 0
    fact = np.where(act, np.abs(R["fact"]), np.inf)
    return ulps * eps * np.sum(np.where(act, np.abs(R["t_soisno"]) / fact, 0.0), axis=0)


def soil_gate(A0, npatch, G, nsteps, G1, balance, identical, sensitivity_runs=4):
    """Parity of the benched run.
    (1) One step from the GPU's evolved state: the GPU's next step (G1)
        against the oracle's step from the same state (G), every column.
    (2) The trajectory: the GPU state after `nsteps` steps (G) against the
        oracle stepped `nsteps` from the same initial state (A0), every
        column.  Phase change switches on and off at the freezing point on an
        ulp of temperature, so trajectories of an FP64 code part where a level
        sits at the threshold; columns that do are counted, together with the
        columns where the oracle itself parts from its own trajectory when
        every libm result it uses is perturbed by 2 ulp (`sensitivity_runs`
        realisations): the reference's own sensitivity.
    (3) The reference's balance thresholds over every column and every step
        after skip_steps, from a replica batch with the balance check on whose
        final state is bit-identical to the benched one (`identical`), beside
        the oracle's own water budget error over the same steps."""
    from ctsm_gb300 import balance as bal
    state = GATE_STATE + GATE_FLUXES
    # (1)
    o1 = OracleSoilStepper(G)
    o1.step(1)
    bands = {k: np.zeros_like(o1.S[k]) for k in GATE_CANCEL}
    for seed in range(1, GATE_NOISE_RUNS + 1):
        on = OracleSoilStepper(G, noise=(GATE_NOISE_ULPS, seed))
        on.step(1)
        for k in GATE_CANCEL:
            np.maximum(bands[k], np.abs(on.S[k] - o1.S[k]), out=bands[k])
        del on
    bands["eflx_fgr12"] = bands["eflx_fgr12"] + fgr12_rounding_bound(o1.S)
    bands["xmf"] = bands["xmf"] + xmf_rounding_bound(o1.S)
    one, one_bad = compare_states(G1, o1.S, state)
    one_c, one_c_bad = compare_states(G1, o1.S, GATE_CANCEL, bands=bands)
    one.update({k + " (conditioned)": v for k, v in one_c.items()})
    one_bad = one_bad | one_c_bad
    # how much the conditioned outputs lean on their band: the plain relative
    # error and the columns that exceed 1e-9 without it
    band_use = {}
    for k in GATE_CANCEL:
        e_plain, bad_plain = compare_states(G1, o1.S, (k,))
        band_use[k] = {"max_rel_err_without_band": e_plain[k], "columns_above_tol_without_band": int(bad_plain.sum())}
    del o1
    # (2)
    o = OracleSoilStepper(A0, track_water=True)
    t0 = time.perf_counter()
    o.step(nsteps)
    t_oracle = time.perf_counter() - t0
    traj, traj_bad = compare_states(G, o.S, GATE_STATE)
    sens = np.zeros(o.n, dtype=bool)
    for seed in range(1, sensitivity_runs + 1):
        on = OracleSoilStepper(A0, noise=(2, 100 + seed))
        on.step(nsteps)
        sens |= compare_states(on.S, o.S, GATE_STATE)[1]
        del on
    h2o_max, soi_max = balance
    # columns past the reference's stop thresholds: the GPU's, and those of
    # them where the oracle's own water budget is past the stop threshold too
    # (the reference's arithmetic leaves the budget there, the GPU with it)
    stop_gpu = (h2o_max >= bal.ERROR_THRESH) | (soi_max >= bal.ERRSOI_STOP)
    stop_both = stop_gpu & (o.water_err_max >= bal.ERROR_THRESH)
    finite = int(np.count_nonzero(~np.isfinite(G["t_soisno"]).all(axis=0) | ~np.isfinite(G["h2osoi_liq"]).all(axis=0)))
    gate = {"columns": int(o.n), "steps": int(nsteps), "tol": GATE_TOL,
            "one_step_from_evolved_state": {"max_rel_err": one, "columns_above_tol": int(one_bad.sum()),
                                            "conditioned": list(GATE_CANCEL), "band_use": band_use},
            "trajectory": {"max_rel_err": traj, "columns_above_tol": int(traj_bad.sum()),
                           "oracle_self_sensitive_columns": int(sens.sum()),
                           "above_tol_and_sensitive": int((traj_bad & sens).sum()),
                           "sensitivity": "oracle vs itself with every libm result perturbed by up to 2 ulp, "
                                          "%d realisations" % sensitivity_runs},
            "nonfinite_columns": finite,
            "balance": {"errh2o_max_mm": float(np.max(h2o_max)), "errsoi_max_w_m2": float(np.max(soi_max)),
                        "oracle_errh2o_max_mm": float(o.water_err_max.max()),
                        "h2o_warning": bal.H2O_WARNING_THRESH, "h2o_stop": bal.ERROR_THRESH,
                        "errsoi_warning": bal.ERRSOI_WARNING, "errsoi_stop": bal.ERRSOI_STOP,
                        "columns_above_warning": int(np.count_nonzero((h2o_max >= bal.H2O_WARNING_THRESH) |
                                                                      (soi_max >= bal.ERRSOI_WARNING))),
                        "columns_above_stop": int(np.count_nonzero(stop_gpu)),
                        "columns_above_stop_in_oracle_too": int(np.count_nonzero(stop_both)),
                        "replica_bit_identical": bool(identical)}}
    gate["pass"] = bool(not one_bad.any() and finite == 0 and identical and not (stop_gpu & ~stop_both).any()
                        and np.all(np.isfinite(h2o_max)) and np.all(np.isfinite(soi_max)))
    return gate, o.n * nsteps / t_oracle, t_oracle


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


# ---------------------------------------------------------------- clocks
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None
        # raw samples, kept for inspection (CTSMG_CLOCKS_CSV names the file)
        self.path = os.environ.get("CTSMG_CLOCKS_CSV", os.path.join(tempfile.gettempdir(), "clocks_bench.csv"))

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def copied_bytes(reset=False):
    """Host<->device bytes the drop-in entry points copied since the last
    reset, as counted by the library at each copy."""
    import ctypes as C
    from ctsm_gb300 import _lib
    L = _lib.load()
    L.ctsmg_copy_bytes.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int32]
    h2d, d2h = C.c_int64(0), C.c_int64(0)
    _lib.check(L.ctsmg_copy_bytes(C.byref(h2d), C.byref(d2h), 1 if reset else 0))
    return h2d.value, d2h.value


def pipe_trace(enable):
    """Turns the drop-in calls' per-chunk timeline on or off for this thread
    and returns the last recorded call's marks: one (copy-in start, copy-in
    end, kernel start, kernel end, copy-out end, host copy-in enqueued, host
    copy-out enqueued) tuple per chunk, in ms."""
    import ctypes as C
    from ctsm_gb300 import _lib
    L = _lib.load()
    L.ctsmg_pipe_trace.argtypes = [C.c_int32, C.POINTER(C.c_float), C.c_int32, C.POINTER(C.c_int32)]
    buf = (C.c_float * (7 * 64))()
    n = C.c_int32(0)
    _lib.check(L.ctsmg_pipe_trace(1 if enable else 0, buf, 64, C.byref(n)))
    return [tuple(buf[7 * k:7 * k + 7]) for k in range(n.value)]


def pipeline_summary(marks):
    """Busy time of the copy-in stream, the kernels and the copy-out stream of
    one pipelined call, and its span, from its per-chunk marks (ms)."""
    if not marks:
        return {"chunks": 0}

    def union(iv):
        tot, end = 0.0, -1e30
        for a, b in sorted(iv):
            if b > end:
                tot += b - max(a, end)
                end = b
        return tot
    out_iv, prev = [], 0.0
    for m in marks:                       # a chunk's copy-out starts after its kernel and the previous copy-out
        a = max(m[3], prev)
        out_iv.append((a, m[4]))
        prev = m[4]
    return {"chunks": len(marks), "span_ms": round(max(m[4] for m in marks), 3),
            "h2d_busy_ms": round(union([(m[0], m[1]) for m in marks]), 3),
            "kernel_busy_ms": round(union([(m[2], m[3]) for m in marks]), 3),
            "d2h_busy_ms": round(union(out_iv), 3),
            "first_kernel_start_ms": round(marks[0][2], 3), "last_copy_in_end_ms": round(marks[-1][1], 3),
            "marks_ms": [[round(x, 3) for x in m] for m in marks]}


# ---------------------------------------------------------------- arms
def reference_arm(args, ws, rank):
    """The reference's CPU implementation of the path (the oracle port: the
    Fortran cannot be built on either machine) on the same workload and config
    as the GPU arm: every one of the `ncol` columns, W untimed and K timed
    steps, all host threads."""
    if rank != 0:
        return
    A, npatch = make_inputs(args.ncol, rank_seed(args.seed, 0))
    cfg = bench_config(A, args.ncol)
    o = OracleSoilStepper(A)
    o.step(max(0, args.warmup))
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t0
    v = o.n * args.steps / dt
    threads = host_threads()
    sample = "all %d columns of the workload x %d steps (%.1f s) after %d untimed steps" % (
        o.n, args.steps, dt, args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Philox draws; no dataset)", "config": cfg,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "cpu": cpu_model(),
                             "note": "C++ restatement of the reference Fortran (no Fortran compiler on the build "
                                     "image or the GPU box)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)



# ---------------------------------------------------------------- extra workloads
def canopy_leg(args, barrier):
    """CanopyFluxes + Photosynthesis over the canopy workload: resident steps
    (inputs in HBM, CUDA events) and the plain drop-in call on pinned host
    arrays (copies in the timed region)."""
    import torch
    from ctsm_gb300 import abi, canopy, canopy_inputs as ci, roofline
    from ctsm_gb300.engine import SoilBatch
    A, npatch, ncol, ngrid = ci.canopy_patches(args.canopy_patches, seed=args.seed)
    A0 = copy.deepcopy(A)
    b = SoilBatch(A, npatch, canopy=True, ngrid=ngrid, order=2)
    b.run(args.warmup)
    b.sync()
    barrier()
    ms = b.run(args.canopy_steps, timed=True)
    b.sync()
    b.download()
    b.close()
    mean_ms = float(ms.mean())
    passes = float(A["num_iter"].mean())
    flops = roofline.CANOPY_FLOPS_PER_PASS * passes * npatch
    out = {"workload": "CanopyFluxes+Photosynthesis, %d patches, 1-4 per column, itmax 40" % npatch,
           "patches": npatch, "steps": args.canopy_steps, "ms_per_step": mean_ms,
           "patch_steps_per_s": npatch / (mean_ms * 1e-3), "mean_passes": passes,
           "gpu_launches_per_step": 4,
           "fp64": {"achieved": flops / (mean_ms * 1e-3) / 1e12, "unit": "TFLOP/s",
                    "flops_per_pass": roofline.CANOPY_FLOPS_PER_PASS},
           "traffic_bytes_per_patch_step": roofline.CANOPY_TRAFFIC_PER_PATCH_STEP}
    if not args.no_e2e:
        H = {}
        for k, v in A0.items():
            t = torch.empty(v.shape, dtype=torch.float64 if v.dtype == np.float64 else torch.int32).pin_memory()
            h = t.numpy()
            h[...] = v
            H[k] = h
        canopy.set_params()
        bnd = abi.Bounds(1, ncol, 1, npatch)
        filt = np.arange(1, npatch + 1, dtype=np.int32)
        canopy.CanopyFluxes(bnd, npatch, filt, H, DT, ngrid)
        barrier()
        k = 3
        copied_bytes(reset=True)
        t0 = time.perf_counter()
        for _ in range(k):
            canopy.CanopyFluxes(bnd, npatch, filt, H, DT, ngrid)
        barrier()
        te = (time.perf_counter() - t0) / k
        h2d, d2h = copied_bytes()
        out["e2e"] = {"value": npatch / te, "unit": "patch-steps/s", "ms_per_call": 1e3 * te,
                      "h2d_bytes_per_step": h2d // k, "d2h_bytes_per_step": d2h // k,
                      "path": "ctsmg_canopyfluxes (plain drop-in, pinned host arrays)"}
    return out


def member_state(A, member_col, m):
    """Member m of a packed ensemble state as a state of its own (its columns,
    patches and gridcells, index maps rebased)."""
    ncol, npatch = A["zwt"].shape[0], A["wtcol"].shape[0]
    cols = np.nonzero(member_col == m)[0]
    pidx = np.nonzero(np.isin(A["patch_column"] - 1, cols))[0]
    S = {}
    for k, v in A.items():
        if v.shape[-1] == ncol:
            S[k] = np.ascontiguousarray(v[..., cols])
        elif v.shape[-1] == npatch:
            S[k] = np.ascontiguousarray(v[..., pidx])
    S["col_patchi"] = (A["col_patchi"][cols] - pidx[0]).astype(np.int32)
    S["patch_column"] = (A["patch_column"][pidx] - cols[0]).astype(np.int32)
    S["patch_gridcell"] = S["patch_column"].copy()
    return S, len(pidx), len(cols)


def ensemble_leg(args, barrier):
    """The perturbed-parameter ensemble on the CLM5-default step (soil
    resistance, root moisture stress, CanopyFluxes, root sink,
    SoilTemperature, SoilFluxes, the moisture-form SoilWater with the default
    hydrology), six of the eight parameters acting (medlynslope,
    medlynintercept, om_frac_sf, baseflow_scalar, fff, d_max): every member in
    one resident batch (one CUDA graph per step) against the plain form, one
    set of drop-in C-ABI calls per member, timed over every member."""
    from ctsm_gb300 import abi, canopy, full_inputs as fi, soil
    from ctsm_gb300.engine import SoilBatch
    from ctsm_gb300.plain_step import PlainCLM5Step
    A, npatch, ngrid, rootr, member_col, f = fi.ensemble(args.ens_members, seed=args.seed, clm5=True)
    ncol = A["zwt"].shape[0]
    nml = abi.soilwater_movement_nml(1)
    soil.set_soilwater_movement(nml)
    soil.set_soilhydrology_params()
    soil.set_soil_resistance()
    canopy.set_params()
    try:
        b = SoilBatch(copy.deepcopy(A), npatch, canopy=True, ngrid=ngrid, per_patch_medlyn=True, soilfluxes=True,
                      rootmoist=True, soilresis=True, hydrology=True, per_column_hydrology=True)
        block = b.autotune(trial_steps=1)
        b.run(args.warmup)
        b.sync()
        barrier()
        ms = b.run(args.ens_steps, timed=True)
        b.sync()
        b.close()
        batched = ncol * args.ens_steps / (float(ms.sum()) * 1e-3)
        # the plain form: every member, one set of drop-in calls per member and step
        steppers = []
        for m in range(args.ens_members):
            S, npm, ncm = member_state(A, member_col, m)
            steppers.append(PlainCLM5Step(S, npm, ncm, medlyn=(float(f["medlynslope"][m]),
                                                               float(f["medlynintercept"][m])),
                                          d_max=fi.D_MAX * float(f["d_max"][m]),
                                          baseflow_scalar=fi.BASEFLOW_SCALAR * float(f["baseflow_scalar"][m]),
                                          fff=fi.FFF * float(f["fff"][m])))
        for st in steppers[:4]:
            st.step()                                             # warm-up
        kp = 2
        barrier()
        t0 = time.perf_counter()
        for _ in range(kp):
            for st in steppers:
                st.step()
        barrier()
        t_plain = time.perf_counter() - t0
        plain = ncol * kp / t_plain
    finally:
        soil.set_soilwater_movement(abi.soilwater_movement_nml(0, use_bedrock=0))
        soil.set_soilhydrology_params()
        soil.set_soil_resistance()
        canopy.set_params()
    return {"workload": "%d members, columns U{512..8192} each (%d columns, %d patches), CLM5-default step "
                        "(soil resistance, root moisture stress, CanopyFluxes, root sink, SoilTemperature, "
                        "SoilFluxes, moisture-form SoilWater + default hydrology), 8 parameters log-uniform "
                        "x[0.5,1.5], 6 acting (jmaxb1: LUNA, kmax: plant hydraulics, outside the path)"
                        % (args.ens_members, ncol, npatch),
            "columns": ncol, "patches": npatch, "steps": args.ens_steps, "ms_per_step": float(ms.mean()),
            "batched_column_steps_per_s": batched, "block": block,
            "plain_column_steps_per_s": plain,
            "plain_sample": "all %d members x %d steps, one set of %d drop-in C-ABI calls (and 3 parameter setters) per member and step "
                            "(%.2f s)" % (args.ens_members, kp, 14, t_plain),
            "batched_over_plain": batched / plain}


def clm5_leg(args, barrier):
    """The CLM5-default configuration of the whole scoped step in the resident
    engine: soil evaporative resistance and root moisture stress, CanopyFluxes,
    the root sink, SoilTemperature, SoilFluxes, the moisture-form SoilWater
    with the default hydrology around it (saturated excess, infiltration,
    perched / theta-based water tables, lateral flows)."""
    from ctsm_gb300 import abi, full_inputs as fi, soil
    from ctsm_gb300.engine import SoilBatch
    r = np.random.Generator(np.random.Philox(args.seed + 7))
    A, npatch, ngrid, rootr = fi.full_state(args.clm5_cols, seed=args.seed + 7)
    fi.add_soilfluxes_fields(A, npatch, ngrid)
    fi.add_rootmoist_fields(A, npatch, rootr, rng=r)
    fi.add_soilresis_fields(A)
    fi.add_hydrology_fields(A, r)
    nml = abi.soilwater_movement_nml(1)
    soil.set_soilwater_movement(nml)
    soil.set_soilhydrology_params()
    soil.set_soil_resistance()
    try:
        b = SoilBatch(A, npatch, canopy=True, ngrid=ngrid, soilfluxes=True, rootmoist=True, soilresis=True,
                      hydrology=True)
        # two steps first, so the tuner's bucketed order sees sub-step counts
        # of this run rather than the inputs' zeros
        b.run(2)
        tuned = b.tune(trial_steps=2)
        b.run(args.warmup)
        b.sync()
        barrier()
        ms = b.run(args.clm5_steps, timed=True)
        b.sync()
        b.download()
        b.close()
    finally:
        soil.set_soilwater_movement(abi.soilwater_movement_nml(0, use_bedrock=0))
    ncol = A["zwt"].shape[0]
    mean_ms = float(ms.mean())
    return {"workload": "CLM5 default step (soilresis, root moisture stress, CanopyFluxes, root sink, "
                        "SoilTemperature, SoilFluxes, moisture-form SoilWater + default hydrology), %d columns, "
                        "%d patches" % (ncol, npatch),
            "columns": ncol, "patches": npatch, "steps": args.clm5_steps, "ms_per_step": mean_ms,
            "column_steps_per_s": ncol / (mean_ms * 1e-3),
            "mean_substeps": float(A["num_substeps"].mean()), "max_substeps": float(A["num_substeps"].max()),
            "mean_canopy_passes": float(A["num_iter"].mean()), "gpu_launches_per_step": 8,
            "tuning": {"block": tuned["block"], "mf_order": tuned["mf_order"],
                       "ms_per_step": {k: {str(blk): round(v, 3) for blk, v in t.items()}
                                       for k, t in tuned["ms_per_step"].items()}}}


def serving_leg(args):
    """A Poisson stream of run requests through the device pool, bounded in
    wall time: requests still running at the limit are stopped (their steps
    count in the throughput; their pace -- wall seconds per simulated day
    since arrival -- is reported beside the completed requests' latency)."""
    from ctsm_gb300 import serving
    reqs = serving.request_stream(args.serve_requests, args.serve_rate, seed=args.seed, physical=True)
    pool = serving.Pool(budget_bytes=args.serve_budget_gb * 1e9, rootmoist=True, hydrology=True)
    cap = pool.capacity
    st = serving.serve(pool, reqs, time_limit=args.serve_seconds)
    pool.close()
    st.update({"workload": "Poisson arrivals at %.2f/s, %d requests, columns log-uniform 1..50000, "
                           "lengths U{48..17520} steps, snow-free columns, full soil+canopy step with the root "
                           "moisture stress and the aquifer-layer hydrology" % (args.serve_rate, args.serve_requests),
               "budget_gb": args.serve_budget_gb, "capacity_columns": cap[0], "time_limit_s": args.serve_seconds,
               "offered_column_steps": int(sum(q.column_steps() for q in reqs)),
               "latency_note": "headline p50/p99_pace_s_per_day: every request that ran, (completion or time "
                               "limit - arrival) / simulated days it advanced; p50/p99_s_per_day: completed "
                               "requests only, (completion - arrival) / simulated days; nonfinite_*: final "
                               "states with a non-finite temperature or liquid water"})
    return st


def ours_arm(args, ws, rank, local):
    import torch
    from ctsm_gb300 import abi, soil, roofline, _lib
    from ctsm_gb300.engine import SoilBatch

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    soil.init()
    L = _lib.load()
    L.ctsmg_measure_fp64_tflops.argtypes = [C.POINTER(C.c_double)]
    fp64 = C.c_double(0.0)
    L.ctsmg_measure_fp64_tflops(C.byref(fp64))
    L.ctsmg_measure_fp64_lane_cost.argtypes = [C.c_int32, C.POINTER(C.c_float)]
    L.ctsmg_measure_fp64_div_lane_cost.argtypes = [C.c_int32, C.POINTER(C.c_float)]
    lane_cost = {"dfma": {}, "ddiv": {}}
    for lanes in (32, 8, 1):
        t = C.c_float(0.0)
        L.ctsmg_measure_fp64_lane_cost(lanes, C.byref(t))
        lane_cost["dfma"]["ms_%d_lanes" % lanes] = round(float(t.value), 3)
        t = C.c_float(0.0)
        L.ctsmg_measure_fp64_div_lane_cost(lanes, C.byref(t))
        lane_cost["ddiv"]["ms_%d_lanes" % lanes] = round(float(t.value), 3)

    A, npatch = make_inputs(args.ncol, rank_seed(args.seed, rank))
    ncol = args.ncol
    mean_snow = float(-A["snl"].mean())
    cfg = bench_config(A, ncol)

    # ---------------- batched resident engine
    G = copy.deepcopy(A)
    batch = SoilBatch(G, npatch, dtime=DT)
    tuned = batch.tune(trial_steps=2)
    block = tuned["block"]
    batch.run(args.warmup)
    batch.sync()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    clocks = Clocks(local)
    clocks.start()
    barrier()
    t0 = time.perf_counter()
    step_ms = batch.run(args.steps, timed=True)
    batch.sync()
    barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    ev_total_s = float(step_ms.sum()) / 1e3
    t_rank = max_over_ranks(max(ev_total_s, 0.0), ws, "cuda")
    value = job_value(ws, ncol, args.steps, t_rank)
    mean_launch_s = float(step_ms.mean()) / 1e3

    rd, wr = roofline.step_bytes_per_column(mean_snow, 1.0)
    alg_bytes = (rd + wr) * ncol
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        hbm_peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        hbm_peak, peak_src = 6800.0, "fallback"
    achieved = alg_bytes / mean_launch_s / 1e9
    flops_cs = roofline.FLOPS_PER_COLUMN_STEP
    fp64_line = None
    if flops_cs:
        ach_tf = flops_cs * ncol / mean_launch_s / 1e12
        # issue slots of the FP64 pipe: the measured DFMA loop issues
        # peak / 2 FLOP / 32 lanes warp instructions per second
        ach_wi = roofline.FP64_WARP_INST_PER_COLUMN_STEP * ncol / mean_launch_s
        peak_wi = fp64.value * 1e12 / 64.0
        fp64_line = {"achieved": ach_tf, "peak": fp64.value, "unit": "TFLOP/s", "frac": ach_tf / fp64.value,
                     "flops_per_column_step": flops_cs, "peak_source": "measured live (DFMA loop)",
                     "issue": {"achieved_warp_inst_per_s": ach_wi, "peak_warp_inst_per_s": peak_wi,
                               "frac": ach_wi / peak_wi,
                               "warp_inst_per_column_step": roofline.FP64_WARP_INST_PER_COLUMN_STEP}}
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
            "traffic": roofline.TRAFFIC_PER_COLUMN_STEP * ncol if roofline.TRAFFIC_PER_COLUMN_STEP else None,
            "peak_source": peak_src, "algorithmic_bytes_per_column_step": rd + wr,
            "kernel": "soilstep_kernel", "fp64": fp64_line,
            "note": "the step is FP64-pipe bound on GB300; the HBM fraction is reported as required"}

    # ---------------- correctness gate of the benched run (after the timed region)
    gate = None
    cpu = None
    nsteps_run = args.warmup + args.steps
    if not args.no_gate:
        batch.download()                      # G: the state the timed steps left
        G1 = copy.deepcopy(G)
        batch.run(1)
        batch.sync()
        batch.download(G1)                    # one further step from that state
        batch.close()
        del batch
        R = copy.deepcopy(A)
        rb = SoilBatch(R, npatch, dtime=DT, balance=True)
        rb.set_block(block)
        rb.run(nsteps_run)
        rb.sync()
        rb.download()
        h2o_max, soi_max, _, _ = rb.balance()
        rb.close()
        identical = all(np.array_equal(R[k], G[k], equal_nan=True) for k in GATE_STATE + GATE_FLUXES)
        del R
        gate, oracle_cs, t_oracle = soil_gate(A, npatch, G, nsteps_run, G1, (h2o_max, soi_max), identical)
        if rank == 0 and ws == 1 and not args.no_cpu:
            cpu = {"value": oracle_cs, "unit": UNIT, "cores": host_threads(), "kind": "port",
                   "sample": "all %d columns x %d steps (%.1f s): the oracle run of the correctness gate"
                             % (ncol, nsteps_run, t_oracle), "cpu": cpu_model()}
        del G1
    else:
        batch.close()
        del batch

    # ---------------- plain drop-in e2e (host buffers, copies in the timed region)
    e2e = None
    if not args.no_e2e:
        H = {}
        for k, v in A.items():
            t = torch.empty(v.shape, dtype=torch.float64 if v.dtype == np.float64 else torch.int32).pin_memory()
            h = t.numpy()
            h[...] = v
            H[k] = h
        bnd = abi.Bounds(1, ncol, 1, npatch)
        filt = np.arange(1, ncol + 1, dtype=np.int32)
        ke = min(args.steps, 8)
        for _ in range(max(1, min(args.warmup, 2))):
            soil.SoilWater(bnd, ncol, filt, H, DT)
            soil.SoilTemperature(bnd, ncol, filt, H, DT)
        barrier()
        copied_bytes(reset=True)
        t_sw = t_st = 0.0
        t0 = time.perf_counter()
        for _ in range(ke):
            ta = time.perf_counter()
            soil.SoilWater(bnd, ncol, filt, H, DT)       # each call returns with its results on the host
            tb = time.perf_counter()
            soil.SoilTemperature(bnd, ncol, filt, H, DT)
            t_sw += tb - ta
            t_st += time.perf_counter() - tb
        barrier()
        te = max_over_ranks(time.perf_counter() - t0, ws, "cuda")
        h2d, d2h = copied_bytes()
        # one more pair outside the timed region: bytes and the per-chunk
        # timeline of each call
        per_call = {}
        for name, call in (("SoilWater", soil.SoilWater), ("SoilTemperature", soil.SoilTemperature)):
            copied_bytes(reset=True)
            pipe_trace(True)
            call(bnd, ncol, filt, H, DT)
            marks = pipe_trace(False)
            bi, bo = copied_bytes()
            per_call[name] = dict(h2d_bytes=bi, d2h_bytes=bo, **pipeline_summary(marks))
        # the same pairs with the time-constant inputs (soil properties, soil
        # layer geometry) kept on the device between calls, as a host that
        # sets them once at initialisation would opt in to
        Lb = _lib.load()
        Lb.ctsmg_set_time_constant_inputs.argtypes = [C.c_int32]
        _lib.check(Lb.ctsmg_set_time_constant_inputs(1))
        try:
            soil.SoilWater(bnd, ncol, filt, H, DT)
            soil.SoilTemperature(bnd, ncol, filt, H, DT)
            barrier()
            copied_bytes(reset=True)
            t0 = time.perf_counter()
            for _ in range(ke):
                soil.SoilWater(bnd, ncol, filt, H, DT)
                soil.SoilTemperature(bnd, ncol, filt, H, DT)
            barrier()
            tr = max_over_ranks(time.perf_counter() - t0, ws, "cuda")
            h2d_r, d2h_r = copied_bytes()
        finally:
            Lb.ctsmg_set_time_constant_inputs(0)
        e2e = {"value": job_value(ws, ncol, ke, te), "unit": UNIT, "h2d_bytes_per_step": h2d // ke,
               "d2h_bytes_per_step": d2h // ke, "steps": ke, "ms_per_step": 1e3 * te / ke,
               "ms_per_call": {"SoilWater": 1e3 * t_sw / ke, "SoilTemperature": 1e3 * t_st / ke},
               "calls": per_call,
               "time_constant_inputs_resident": {
                   "value": job_value(ws, ncol, ke, tr), "unit": UNIT, "ms_per_step": 1e3 * tr / ke,
                   "h2d_bytes_per_step": h2d_r // ke, "d2h_bytes_per_step": d2h_r // ke,
                   "note": "ctsmg_set_time_constant_inputs(1): soil properties and soil-layer geometry copied "
                           "once, every other input and output copied every call"},
               "path": "ctsmg_soilwater + ctsmg_soiltemperature (plain drop-in, pinned host arrays)"}

    # ---------------- CPU baseline (rank 0 only, N = 1 only) when the gate did not time the oracle
    if cpu is None and rank == 0 and ws == 1 and not args.no_cpu:
        r, n, steps, dt, threads = oracle_rate(A, npatch)
        cpu = {"value": r, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "first %d columns of the workload x %d steps (%.1f s)" % (n, steps, dt),
               "cpu": cpu_model()}

    extra = {}
    if rank == 0 and ws == 1:
        for name, flag, fn in (("canopy", args.no_canopy, lambda: canopy_leg(args, barrier)),
                               ("ensemble", args.no_ensemble, lambda: ensemble_leg(args, barrier)),
                               ("clm5_default", args.no_clm5, lambda: clm5_leg(args, barrier)),
                               ("serving", args.no_serving, lambda: serving_leg(args))):
            if not flag:
                try:
                    extra[name] = fn()
                except Exception as exc:          # a failed leg is reported, not hidden
                    extra[name] = {"error": "%s: %s" % (type(exc).__name__, exc)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * t_rank / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded Philox draws; no dataset)", "config": cfg,
                "tuning": {"block": block, "column_order": tuned["order"], "graph": "one CUDA graph per step",
                           "autotune_ms_per_step": tuned["ms_per_step"], "mean_snow_layers": mean_snow},
                "parity": gate,
                "gpu_launches": int(args.steps), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clk, "wall_s_timed": wall, "fp64_peak_tflops": fp64.value,
                "fp64_lane_cost": lane_cost}
        line.update(extra)
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, ws, rank)
        return
    ours_arm(args, ws, rank, local)


if __name__ == "__main__":
    main()
