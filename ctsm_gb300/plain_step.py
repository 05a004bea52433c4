"""The plain form of a model step: what a CTSM host does with the drop-in
calls alone -- CanopyFluxes, the root water sink, SoilTemperature, SoilWater
and the between-step h2osoi_vol refresh, each call copying its arrays from
and back to host memory (src/main/clm_driver.F90:766, 900, 950; the sink of
src/biogeophys/SoilWaterPlantSinkMod.F90:332-420 and the refresh of
src/biogeophys/HydrologyNoDrainageMod.F90:580,590 run on the host, as they
do in the reference).  It is the baseline the batched engine is compared
with: one member or region per set of calls, no state kept on the device."""
import numpy as np

from . import abi, canopy, canopy_inputs, inputs, soil

DT = 1800.0


def root_sink(A, rootr):
    """qflx_rootsoi (levels 1..nlevsoi, columns) from the patches' transpiration
    and root fractions, summed over each column's patches in patch order."""
    ncol = A["zwt"].shape[0]
    npch = A["wtcol"].shape[0]
    pcol = np.repeat(np.arange(ncol), A["col_npatches"])
    tw = A["qflx_tran_veg"] * A["wtcol"]
    rc = np.zeros((abi.NLEVSOI, ncol))
    for j in range(abi.NLEVSOI):
        rc[j] = np.bincount(pcol, weights=rootr[j, :npch] * A["qflx_tran_veg"] * A["wtcol"], minlength=ncol)
    temp = np.bincount(pcol, weights=tw, minlength=ncol)
    rc = np.where(temp != 0.0, rc / np.where(temp != 0.0, temp, 1.0), rc)
    A["qflx_rootsoi"][...] = rc * temp


def full_step(A, npatch, ngrid, rootr, displa0, z0mv0, medlyn=None, params=None):
    """One plain full step in place on A.  medlyn = (slope, intercept) factors
    of an ensemble member, applied through the pftcon rows (the drop-in reads
    the parameters from pftcon)."""
    ncol = A["zwt"].shape[0]
    if medlyn is not None:
        rows = [list(r) for r in canopy_inputs.DEFAULT_PFT]
        for r in rows:
            r[6] *= medlyn[0]
            r[7] *= medlyn[1]
        canopy.set_params(params, canopy_inputs.make_pftcon(rows))
    A["displa"][:] = displa0
    A["z0mv"][:] = z0mv0
    A["cgrnds"][:] = 0.0
    A["cgrndl"][:] = 0.0
    b = abi.Bounds(1, ncol, 1, npatch)
    canopy.CanopyFluxes(b, npatch, np.arange(1, npatch + 1, dtype=np.int32), A, DT, ngrid)
    root_sink(A, rootr)
    filt = np.arange(1, ncol + 1, dtype=np.int32)
    soil.SoilTemperature(b, ncol, filt, A, DT)
    soil.SoilWater(b, ncol, filt, A, DT)
    inputs.refresh_h2osoi_vol(A)
