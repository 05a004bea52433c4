"""Restart files in the reference's layout for the state of the path.

The batched engine checkpoints its resident state in a self-describing binary
(`ctsmg_batch_save` / `ctsmg_batch_load`: magic, batch sizes, one record per
component in the caller's column order and the C-ABI's level layout).  This
module reads and writes that format on the host and converts it to and from a
NetCDF-3 file (scipy.io.netcdf_file; NetCDF-4 / PIO are absent here) whose
variables carry the names, types, dimensions and on-file dimension order of
the reference's restart variables for the prognostic state of SoilWater,
SoilTemperature and CanopyFluxes:

    T_SOISNO, T_VEG, TH2OSFC, T_GRND       src/biogeophys/TemperatureType.F90:951-981
    H2OSFC, H2OSNO_NO_LAYERS, H2OSOI_LIQ,
    H2OSOI_ICE, SNOCAN, LIQCAN, WA         src/biogeophys/WaterStateType.F90:629-696
    INT_SNOW                               src/biogeophys/WaterStateBulkType.F90:223
    FH2OSFC, SNOW_DEPTH, SNOMELT_ACCUM,
    frac_sno_eff                           src/biogeophys/WaterDiagnosticBulkType.F90:830-858
    FROST_TABLE, ZWT, ZWT_PERCH            src/biogeophys/SoilHydrologyType.F90:307-320
    SNLSNO                                 src/main/subgridRestMod.F90:537

Dimensions follow src/main/restFileMod.F90:551-562 ('column', 'pft',
'levtot' = nlevsno + nlevgrnd here).  A variable declared with
switchdim=.true. (the level arrays) is stored with each column's levels
contiguous, i.e. (column, levtot) in C order (src/main/ncdio_pio.F90.in:
1278-1282, 2712-2719), where the C-ABI keeps levels outermost; the
conversion transposes.  Only the components a batch holds are written; a
restart read back into a checkpoint replaces those components and leaves the
others as the template checkpoint has them.
"""
import struct

import numpy as np

from . import abi

MAGIC = b"CTSMGCK1"
# level kinds in the order of the C enum (ctsm_gb300/csrc/capi_internal.h)
KINDS = ("C", "P", "SS", "ZI", "G", "S", "SN", "PL", "GR", "PS", "PG")
_NLEV = {"C": 1, "P": 1, "GR": 1, "SS": abi.NLEVSNO + abi.NLEVGRND, "ZI": abi.NLEVSNO + abi.NLEVGRND + 1,
         "G": abi.NLEVGRND, "PG": abi.NLEVGRND, "S": abi.NLEVSOI, "PS": abi.NLEVSOI, "SN": abi.NLEVSNO,
         "PL": abi.NLEVSNO + 1}
_PATCH_KINDS = ("P", "PL", "PS", "PG")

# restart variable -> (component, NetCDF type code, dimensions in C order on file)
RESTART_VARS = {
    "T_SOISNO": ("t_soisno", "d", ("column", "levtot")),
    "T_VEG": ("t_veg", "d", ("pft",)),
    "TH2OSFC": ("t_h2osfc", "d", ("column",)),
    "T_GRND": ("t_grnd", "d", ("column",)),
    "H2OSFC": ("h2osfc", "d", ("column",)),
    "H2OSNO_NO_LAYERS": ("h2osno_no_layers", "d", ("column",)),
    "H2OSOI_LIQ": ("h2osoi_liq", "d", ("column", "levtot")),
    "H2OSOI_ICE": ("h2osoi_ice", "d", ("column", "levtot")),
    "SNOCAN": ("snocan", "d", ("pft",)),
    "LIQCAN": ("liqcan", "d", ("pft",)),
    "WA": ("wa", "d", ("column",)),
    "INT_SNOW": ("int_snow", "d", ("column",)),
    "FH2OSFC": ("frac_h2osfc", "d", ("column",)),
    "SNOW_DEPTH": ("snow_depth", "d", ("column",)),
    "SNOMELT_ACCUM": ("snomelt_accum", "d", ("column",)),
    "frac_sno_eff": ("frac_sno_eff", "d", ("column",)),
    "FROST_TABLE": ("frost_table", "d", ("column",)),
    "ZWT": ("zwt", "d", ("column",)),
    "ZWT_PERCH": ("zwt_perched", "d", ("column",)),
    "SNLSNO": ("snl", "i", ("column",)),
}
_LEVEL_DIMS = {"levtot": "SS"}


class Checkpoint:
    """The content of a checkpoint file: batch sizes and, per component, its
    level kind and an array (levels outermost for level kinds, caller's
    column / patch order)."""

    def __init__(self, ncol, npatch, ngrid, fields=None):
        self.ncol, self.npatch, self.ngrid = int(ncol), int(npatch), int(ngrid)
        self.fields = dict(fields or {})          # name -> (kind, array)

    def shape(self, kind):
        n = self.npatch if kind in _PATCH_KINDS else self.ngrid if kind == "GR" else self.ncol
        return (n,) if _NLEV[kind] == 1 else (_NLEV[kind], n)


def read_checkpoint(path):
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != MAGIC:
        raise ValueError("%s is not a checkpoint file" % path)
    ncol, npatch, ngrid, nrec = struct.unpack_from("<4i", data, 8)
    ck = Checkpoint(ncol, npatch, ngrid)
    off = 24
    for _ in range(nrec):
        (nl,) = struct.unpack_from("<H", data, off)
        off += 2
        name = data[off:off + nl].decode()
        off += nl
        kind_i, esize, nbytes = struct.unpack_from("<iiq", data, off)
        off += 16
        kind = KINDS[kind_i]
        dt = {8: np.float64, 4: np.int32}[esize]
        arr = np.frombuffer(data, dtype=dt, count=nbytes // esize, offset=off).reshape(ck.shape(kind)).copy()
        off += nbytes
        ck.fields[name] = (kind, arr)
    if off != len(data):
        raise ValueError("%s: %d trailing bytes" % (path, len(data) - off))
    return ck


def write_checkpoint(path, ck):
    with open(path, "wb") as f:
        f.write(MAGIC + struct.pack("<4i", ck.ncol, ck.npatch, ck.ngrid, len(ck.fields)))
        for name, (kind, arr) in ck.fields.items():
            a = np.ascontiguousarray(arr)
            if a.shape != ck.shape(kind) or a.dtype not in (np.float64, np.int32):
                raise ValueError("component %s: shape %s / type %s do not fit kind %s" % (name, a.shape, a.dtype, kind))
            nb = name.encode()
            f.write(struct.pack("<H", len(nb)) + nb + struct.pack("<iiq", KINDS.index(kind), a.itemsize, a.nbytes))
            f.write(a.tobytes())


def _netcdf():
    from scipy.io import netcdf_file
    return netcdf_file


def checkpoint_to_restart(ck, path):
    """Write the restart variables of the components `ck` holds to a NetCDF-3
    file at `path`; returns the names written."""
    dims = {"column": ck.ncol, "pft": ck.npatch, "levtot": _NLEV["SS"]}
    written = []
    f = _netcdf()(str(path), "w", version=2)
    try:
        f.title = "CTSM restart variables of the column biogeophysics path"
        for d, n in dims.items():
            f.createDimension(d, n)
        for var, (comp, code, vdims) in RESTART_VARS.items():
            if comp not in ck.fields:
                continue
            kind, arr = ck.fields[comp]
            if len(vdims) == 2 and kind != _LEVEL_DIMS[vdims[1]]:
                raise ValueError("component %s has level kind %s, %s wants %s" % (comp, kind, var, vdims[1]))
            v = f.createVariable(var, code, vdims)
            v[:] = np.ascontiguousarray(arr.T) if arr.ndim == 2 else arr
            written.append(var)
    finally:
        f.close()
    return written


def restart_into_checkpoint(path, ck):
    """A copy of checkpoint `ck` with every component that the restart file
    at `path` holds a variable for replaced by the file's values; returns
    (checkpoint, names read)."""
    out = Checkpoint(ck.ncol, ck.npatch, ck.ngrid, ck.fields)
    read = []
    f = _netcdf()(str(path), "r", mmap=False)
    try:
        if f.dimensions["column"] != ck.ncol or f.dimensions["pft"] != ck.npatch:
            raise ValueError("restart sizes (column %s, pft %s) differ from the checkpoint's (%d, %d)" %
                             (f.dimensions["column"], f.dimensions["pft"], ck.ncol, ck.npatch))
        for var, (comp, code, vdims) in RESTART_VARS.items():
            if var not in f.variables or comp not in ck.fields:
                continue
            v = f.variables[var]
            if tuple(v.dimensions) != vdims:
                raise ValueError("%s has dimensions %s, expected %s" % (var, v.dimensions, vdims))
            kind, old = ck.fields[comp]
            a = np.array(v[:], dtype=old.dtype)
            out.fields[comp] = (kind, np.ascontiguousarray(a.T) if a.ndim == 2 else a)
            read.append(var)
    finally:
        f.close()
    # h2osoi_vol is not a restart variable: the driver forms it from the water
    # contents between steps (HydrologyNoDrainageMod.F90:580,590)
    F = out.fields
    if read and all(k in F for k in ("h2osoi_vol", "h2osoi_liq", "h2osoi_ice", "dz")):
        vol = F["h2osoi_vol"][1].copy()
        liq, ice, dz = F["h2osoi_liq"][1], F["h2osoi_ice"][1], F["dz"][1]
        for j in range(1, abi.NLEVSOI + 1):
            row = j + abi.NLEVSNO - 1
            vol[j - 1] = liq[row] / (dz[row] * 1.000e3) + ice[row] / (dz[row] * 0.917e3)
        F["h2osoi_vol"] = (F["h2osoi_vol"][0], vol)
    return out, read
