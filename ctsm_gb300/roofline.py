"""Algorithmic bytes per column-step of the fused soil step, from the ABI
manifest (ctsm_gb300/abi.py): every component the step reads is counted once,
every component it writes once, on the levels the column actually uses
(snow arrays on its |snl| active layers only)."""
from . import abi

NLEVSNO, NLEVSOI, NLEVGRND = abi.NLEVSNO, abi.NLEVSOI, abi.NLEVGRND

# Per column-step of soilstep_kernel on the uneven-column workload, from an
# ncu capture of one launch over 65,536 columns of the same workload (state
# 420 MB, larger than L2): FP64 FLOPs (DADD + DMUL + 2 x DFMA executed, libm
# included), FP64-pipe warp instructions (every FP64 instruction one issue
# slot of the pipe, whatever its lanes) and DRAM bytes read + written.  The
# full 524,288-column launch is scaled from it by columns.
FLOPS_PER_COLUMN_STEP = (150967449 + 161048536 + 2 * 403756673) / 65536.0
FP64_WARP_INST_PER_COLUMN_STEP = 28241444 / 65536.0
TRAFFIC_PER_COLUMN_STEP = (575314944 + 351197952) / 65536.0

# FP64 floating-point operations per CanopyFluxes pass of one patch
# (canopy_iterate_kernel: DADD + DMUL + 2 x DFMA executed over 262,144 patches
# of the canopy workload, 5.508 passes per patch on average), and DRAM bytes
# per patch-step of that kernel from a capture of one launch over 262,144
# patches of the same workload (3.5 GB of traffic, larger than L2), scaled to
# the full launch by patches.
CANOPY_FLOPS_PER_PASS = (489099825 + 889105990 + 2 * 2293152799) / (262144 * 5.507728576660156)
CANOPY_TRAFFIC_PER_PATCH_STEP = (2404084224 + 1122854912) / 262144.0


def _active_levels(kind, nsnow):
    return {"C": 1, "P": 1, "SS": nsnow + NLEVGRND, "ZI": nsnow + NLEVGRND + 1, "G": NLEVGRND,
            "S": NLEVSOI, "SN": nsnow, "PL": nsnow + 1}[kind]


def step_bytes_per_column(mean_snow_layers, patches_per_column=1.0):
    """(bytes read, bytes written) per column for one SoilWater + SoilTemperature
    step with the between-step h2osoi_vol refresh."""
    fields = {}
    for (n, k, t, u) in abi.SOILWATER_FIELDS + abi.SOILTEMP_FIELDS:
        r, w = fields.get(n, (False, False, k, t))[:2]
        fields[n] = (r or u in ("in", "inout"), w or u in ("out", "inout"), k, t)
    fields["h2osoi_vol"] = (True, True, "G", "f8")  # refreshed at the end of the step
    rd = wr = 0.0
    for n, (r, w, k, t) in fields.items():
        size = 8 if t == "f8" else 4
        lev = _active_levels(k, mean_snow_layers)
        if k == "G" and n == "h2osoi_vol":
            lev = NLEVSOI
        mult = patches_per_column if k in ("P", "PL") else 1.0
        if r:
            rd += lev * size * mult
        if w:
            wr += lev * size * mult
    return rd, wr
