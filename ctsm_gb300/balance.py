"""Balance-check constants of BalanceCheckMod (src/biogeophys/BalanceCheckMod.F90)."""

SKIP_SIZE = 3600.0          # :56  seconds of start-up during which the check is skipped
ERROR_THRESH = 1.e-5        # :65  water error stop threshold (mm)
H2O_WARNING_THRESH = 1.e-9  # :506 water error warning threshold (mm)
ERRSOI_WARNING = 1.e-5      # :1105 soil energy error warning threshold (W/m2)
ERRSOI_STOP = 1.e-4         # :1111 soil energy error stop threshold (W/m2)


def _nint(x):
    """Fortran nint: round half away from zero."""
    import math
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def skip_steps(dtime):
    """max(2, nint(skip_size / dtime)) + 1  (BalanceCheckMod.F90:91)."""
    return max(2, _nint(SKIP_SIZE / dtime)) + 1
