"""Python handle on the batched resident mode of libctsm_gpu.so."""
import ctypes as C

import numpy as np

from . import abi
from ._lib import load, check


def _bind(L):
    if getattr(L, "_batch_bound", False):
        return
    P = C.POINTER
    L.ctsmg_batch_create.argtypes = [P(C.c_void_p), P(abi.SoilWaterIO), P(abi.SoilTempIO), C.c_int32, C.c_int32,
                                     C.c_double, C.c_double, C.c_int32]
    L.ctsmg_batch_run.argtypes = [C.c_void_p, C.c_int32, P(C.c_float)]
    L.ctsmg_batch_sync.argtypes = [C.c_void_p]
    L.ctsmg_batch_download.argtypes = [C.c_void_p, P(abi.SoilWaterIO), P(abi.SoilTempIO)]
    L.ctsmg_batch_autotune.argtypes = [C.c_void_p, C.c_int32, P(C.c_int32)]
    L.ctsmg_batch_set_block.argtypes = [C.c_void_p, C.c_int32]
    L.ctsmg_batch_state_bytes.argtypes = [C.c_void_p]
    L.ctsmg_batch_state_bytes.restype = C.c_int64
    L.ctsmg_batch_destroy.argtypes = [C.c_void_p]
    L.ctsmg_batch_create2.argtypes = [P(C.c_void_p), P(BatchConfig), P(abi.SoilWaterIO), P(abi.SoilTempIO),
                                      P(abi.CanopyIO), P(C.c_double), P(C.c_double), P(C.c_double),
                                      P(abi.CanopyParams), P(abi.Pftcon)]
    L.ctsmg_batch_download2.argtypes = [C.c_void_p, P(abi.SoilWaterIO), P(abi.SoilTempIO), P(abi.CanopyIO)]
    L.ctsmg_batch_create3.argtypes = [P(C.c_void_p), P(BatchConfig), P(abi.SoilWaterIO), P(abi.SoilTempIO),
                                      P(abi.CanopyIO), P(abi.SoilFluxesIO), P(C.c_double), P(C.c_double),
                                      P(C.c_double), P(abi.CanopyParams), P(abi.Pftcon)]
    L.ctsmg_batch_download3.argtypes = [C.c_void_p, P(abi.SoilWaterIO), P(abi.SoilTempIO), P(abi.CanopyIO),
                                        P(abi.SoilFluxesIO)]
    L.ctsmg_batch_balance.argtypes = [C.c_void_p] + [P(C.c_double)] * 4
    L.ctsmg_batch_open.argtypes = [P(C.c_void_p), P(BatchConfig), P(BatchInputs)]
    L.ctsmg_batch_fetch.argtypes = [C.c_void_p, P(BatchInputs)]
    L._batch_bound = True


def _ref(x):
    return None if x is None else C.byref(x)


class BatchConfig(C.Structure):
    _fields_ = [("ncol", C.c_int32), ("npatch", C.c_int32), ("ngrid", C.c_int32), ("dtime", C.c_double),
                ("e_ice", C.c_double), ("snow_thermal_cond_method", C.c_int32), ("stomatalcond_method", C.c_int32),
                ("itmax_canopy_fluxes", C.c_int32), ("order", C.c_int32), ("with_canopy", C.c_int32),
                ("bucket", C.c_int32), ("balance", C.c_int32), ("skip_steps", C.c_int32), ("soilfluxes", C.c_int32),
                ("soilresis", C.c_int32), ("rootmoist", C.c_int32), ("hydrology", C.c_int32)]


class BatchInputs(C.Structure):
    _fields_ = [("sw", C.POINTER(abi.SoilWaterIO)), ("st", C.POINTER(abi.SoilTempIO)),
                ("cio", C.POINTER(abi.CanopyIO)), ("sf", C.POINTER(abi.SoilFluxesIO)),
                ("rm", C.POINTER(abi.RootMoistIO)), ("rootr", C.POINTER(C.c_double)),
                ("medlynslope_p", C.POINTER(C.c_double)), ("medlynintercept_p", C.POINTER(C.c_double)),
                ("cpar", C.POINTER(abi.CanopyParams)), ("pft", C.POINTER(abi.Pftcon)),
                ("sr", C.POINTER(abi.SoilResisIO)), ("hy", C.POINTER(abi.HydrologyIO)),
                ("baseflow_scalar_c", C.POINTER(C.c_double)), ("fff_c", C.POINTER(C.c_double)),
                ("d_max_c", C.POINTER(C.c_double))]


def _pt(x):
    return None if x is None else C.pointer(x)


class SoilBatch:
    """Resident batch of columns advanced by model steps: SoilWater +
    SoilTemperature (order 0), or, with canopy=True, CanopyFluxes + root sink +
    SoilTemperature + SoilWater in the driver's order (order 1), or
    CanopyFluxes alone (order 2; `state` then needs only the canopy
    components)."""

    def __init__(self, state, npatch, dtime=1800.0, e_ice=6.0, snow_thermal_cond_method=0, canopy=False,
                 ngrid=None, rootr=None, order=None, bucket=True, stomatalcond_method=1, itmax=40,
                 params=None, pftcon=None, per_patch_medlyn=False, balance=False, skip_steps=None,
                 soilfluxes=False, rootmoist=False, soilresis=False, hydrology=False, per_column_hydrology=False):
        from . import canopy_inputs
        self.L = load()
        _bind(self.L)
        self.state = state
        self.canopy_only = order == 2
        self.ncol = state["forc_pbot" if self.canopy_only else "zwt"].shape[0]
        self.npatch = npatch
        self.canopy = canopy
        self.ngrid = ngrid if ngrid is not None else self.ncol
        if self.canopy_only:
            self._sw = self._st = None
        else:
            self._sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS +
                                   [x for x in abi.SOILWATER_EXTRA if x[0] in state], state, self.ncol)
            self._st = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, state, self.ncol, npatch)
        from .balance import skip_steps as _skip
        self.balance_on = balance
        cfg = BatchConfig(self.ncol, npatch, self.ngrid, dtime, e_ice, snow_thermal_cond_method, stomatalcond_method,
                          itmax, (1 if canopy else 0) if order is None else order, 1 if canopy else 0,
                          1 if bucket else 0, 1 if balance else 0,
                          _skip(dtime) if skip_steps is None else skip_steps, 1 if soilfluxes else 0,
                          1 if soilresis else 0, 1 if rootmoist else 0, 1 if hydrology else 0)
        self.soilresis = soilresis
        self.hydrology = hydrology
        self.soilfluxes = soilfluxes
        self.rootmoist = rootmoist
        self.h = C.c_void_p()
        if canopy:
            self._ci = abi.make_io(abi.CanopyIO, abi.CANOPY_FIELDS, state, self.ncol, npatch, self.ngrid, 1)
            dp = C.POINTER(C.c_double)
            ms = state["medlynslope_p"].ctypes.data_as(dp) if per_patch_medlyn else None
            mi = state["medlynintercept_p"].ctypes.data_as(dp) if per_patch_medlyn else None
            self._par = params if params is not None else canopy_inputs.make_params()
            self._pft = pftcon if pftcon is not None else canopy_inputs.make_pftcon()
            self._rootr = None if rootr is None else np.ascontiguousarray(rootr, dtype=np.float64)
            self._sf = abi.make_io(abi.SoilFluxesIO, abi.SOILFLUXES_FIELDS, state, self.ncol, npatch) \
                if soilfluxes else None
            self._rm = abi.make_io(abi.RootMoistIO, abi.ROOTMOIST_FIELDS, state, self.ncol, npatch) \
                if rootmoist else None
            self._sr = abi.make_io(abi.SoilResisIO, abi.SOILRESIS_FIELDS, state, self.ncol) if soilresis else None
            self._open(cfg, dp, ms, mi, C.pointer(self._ci), C.pointer(self._par), C.pointer(self._pft),
                       per_column_hydrology)
        elif hydrology:
            self._sf = self._rm = self._sr = self._rootr = None
            self._open(cfg, C.POINTER(C.c_double), None, None, None, None, None, per_column_hydrology)
        else:
            check(self.L.ctsmg_batch_create2(C.byref(self.h), C.byref(cfg), C.byref(self._sw), C.byref(self._st),
                                             None, None, None, None, None, None))

    def _open(self, cfg, dp, ms, mi, ci, par, pft, per_column_hydrology):
        st = self.state
        self._hy = abi.make_io(abi.HydrologyIO, abi.HYDROLOGY_FIELDS, st, self.ncol) if self.hydrology else None
        pc = self.hydrology and per_column_hydrology
        self._in = BatchInputs(_pt(self._sw), _pt(self._st), ci, _pt(self._sf), _pt(self._rm),
                               None if self._rootr is None else self._rootr.ctypes.data_as(dp), ms, mi, par, pft,
                               _pt(self._sr), _pt(self._hy),
                               st["baseflow_scalar_c"].ctypes.data_as(dp) if pc else None,
                               st["fff_c"].ctypes.data_as(dp) if pc else None,
                               st["d_max_c"].ctypes.data_as(dp) if (self.soilresis and "d_max_c" in st) else None)
        check(self.L.ctsmg_batch_open(C.byref(self.h), C.byref(cfg), C.byref(self._in)))

    def run(self, nsteps, timed=False):
        if timed:
            ms = (C.c_float * nsteps)()
            check(self.L.ctsmg_batch_run(self.h, nsteps, ms))
            return np.array(ms[:], dtype=np.float64)
        check(self.L.ctsmg_batch_run(self.h, nsteps, None))
        return None

    def sync(self):
        check(self.L.ctsmg_batch_sync(self.h))

    def download(self, state=None):
        st = state if state is not None else self.state
        if self.canopy_only:
            sw = tt = None
        else:
            sw = abi.make_io(abi.SoilWaterIO, abi.SOILWATER_FIELDS +
                             [x for x in abi.SOILWATER_EXTRA if x[0] in st], st, self.ncol)
            tt = abi.make_io(abi.SoilTempIO, abi.SOILTEMP_FIELDS, st, self.ncol, self.npatch)
        if self.hydrology and not self.canopy:
            hy = abi.make_io(abi.HydrologyIO, abi.HYDROLOGY_FIELDS, st, self.ncol)
            check(self.L.ctsmg_batch_fetch(self.h, C.byref(BatchInputs(_pt(sw), _pt(tt), None, None, None, None, None,
                                                                       None, None, None, None, _pt(hy)))))
        elif self.canopy:
            ci = abi.make_io(abi.CanopyIO, abi.CANOPY_FIELDS, st, self.ncol, self.npatch, self.ngrid, 1)
            sf = abi.make_io(abi.SoilFluxesIO, abi.SOILFLUXES_FIELDS, st, self.ncol, self.npatch) \
                if self.soilfluxes else None
            rm = abi.make_io(abi.RootMoistIO, abi.ROOTMOIST_FIELDS, st, self.ncol, self.npatch) \
                if self.rootmoist else None
            sr = abi.make_io(abi.SoilResisIO, abi.SOILRESIS_FIELDS, st, self.ncol) if self.soilresis else None
            hy = abi.make_io(abi.HydrologyIO, abi.HYDROLOGY_FIELDS, st, self.ncol) if self.hydrology else None
            check(self.L.ctsmg_batch_fetch(self.h, C.byref(BatchInputs(_pt(sw), _pt(tt), C.pointer(ci), _pt(sf),
                                                                       _pt(rm), None, None, None, None, None,
                                                                       _pt(sr), _pt(hy)))))
        else:
            check(self.L.ctsmg_batch_download(self.h, C.byref(sw), C.byref(tt)))
        return st

    def balance(self):
        """(errh2o_max, errsoi_max, errh2o_last, errsoi_last) per column."""
        out = [np.zeros(self.ncol) for _ in range(4)]
        dp = C.POINTER(C.c_double)
        check(self.L.ctsmg_batch_balance(self.h, *[o.ctypes.data_as(dp) for o in out]))
        return tuple(out)

    def autotune(self, trial_steps=2):
        b = C.c_int32()
        check(self.L.ctsmg_batch_autotune(self.h, trial_steps, C.byref(b)))
        return b.value

    def tune(self, trial_steps=2):
        """ctsmg_batch_autotune2: the fastest (column order, moisture-form
        work order, threads per block) on the batch's own data.  Returns
        {"block", "order", "mf_order", "ms_per_step": {candidate name:
        {block: ms}}}; mf_order is "sub-steps,bedrock", "positions" or None
        (no moisture form), and a candidate name is the column order's, with
        the work order after a slash for a moisture-form batch."""
        L = self.L
        L.ctsmg_batch_autotune2.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                            C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(C.c_int32)]
        L.ctsmg_batch_order_name.restype = C.c_char_p
        b, o, m, n = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        ms = (C.c_float * 24)()
        check(L.ctsmg_batch_autotune2(self.h, trial_steps, C.byref(b), C.byref(o), C.byref(m), ms, C.byref(n)))
        mf_names = ("sub-steps,bedrock", "positions")
        nmf = 2 if m.value >= 0 else 1
        norders = n.value // (3 * nmf)
        table = {}
        for i in range(norders):
            oname = L.ctsmg_batch_order_name(i if norders > 1 else o.value).decode()
            for j in range(nmf):
                name = oname + ("/" + mf_names[j] if nmf == 2 else "")
                table[name] = {blk: float(ms[(i * nmf + j) * 3 + k]) for k, blk in enumerate((64, 128, 256))}
        return {"block": b.value, "order": L.ctsmg_batch_order_name(o.value).decode(),
                "mf_order": (mf_names[0] if m.value == 1 else mf_names[1]) if m.value >= 0 else None,
                "ms_per_step": table}

    def set_block(self, block):
        check(self.L.ctsmg_batch_set_block(self.h, block))

    def set_mf_order(self, sorted_):
        """ctsmg_batch_set_mf_order: True buckets the moisture-form columns by
        the previous step's sub-step count and bedrock depth, False takes
        them in position order."""
        check(self.L.ctsmg_batch_set_mf_order(self.h, 1 if sorted_ else 0))

    def save(self, path):
        """ctsmg_batch_save: write the resident state to a checkpoint file."""
        self.L.ctsmg_batch_save.argtypes = [C.c_void_p, C.c_char_p]
        check(self.L.ctsmg_batch_save(self.h, str(path).encode()))

    def load(self, path):
        """ctsmg_batch_load: restore the resident state from a checkpoint file."""
        self.L.ctsmg_batch_load.argtypes = [C.c_void_p, C.c_char_p]
        check(self.L.ctsmg_batch_load(self.h, str(path).encode()))

    def save_restart(self, path):
        """The resident state's restart variables, in the reference's restart
        layout, to a NetCDF-3 file at `path` (ctsm_gb300/restart.py); returns
        the variable names written."""
        import os
        import tempfile
        from . import restart
        with tempfile.TemporaryDirectory() as d:
            ck = os.path.join(d, "state.ckpt")
            self.save(ck)
            return restart.checkpoint_to_restart(restart.read_checkpoint(ck), path)

    def load_restart(self, path):
        """Replace the resident components that the restart file at `path`
        holds variables for (and h2osoi_vol, formed from them); the others
        keep their resident values.  Returns the variable names read."""
        import os
        import tempfile
        from . import restart
        with tempfile.TemporaryDirectory() as d:
            ck = os.path.join(d, "state.ckpt")
            self.save(ck)
            merged, read = restart.restart_into_checkpoint(path, restart.read_checkpoint(ck))
            restart.write_checkpoint(ck, merged)
            self.load(ck)
        return read

    def state_bytes(self):
        return int(self.L.ctsmg_batch_state_bytes(self.h))

    def close(self):
        if self.h:
            self.L.ctsmg_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
