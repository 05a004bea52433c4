// Host build of the device root finder (ctsm_gb300/csrc/rootfind.cuh) for the
// CPU test that compares its evaluation trace with the oracle's hybrid/brent.
#include <cstdint>
#include "rootfind.cuh"
#include "rootfind_testfns.h"

extern "C" int rf_trace(int k, const double* prm, double x0, double* xs, int cap, int* not_bracketed) {
    ctsmg::RootFind rf;
    rf.start(x0);
    int n = 0;
    for (;;) {
        if (n < cap) xs[n] = rf.x;
        ++n;
        if (!rf.next(rf_testfn(k, prm, rf.x))) break;
    }
    *not_bracketed = rf.not_bracketed ? 1 : 0;
    return n;
}
