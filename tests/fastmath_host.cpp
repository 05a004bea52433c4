// Host build of the column kernels' table-driven log / log10 / exp / pow
// (ctsm_gb300/csrc/fastmath.cuh) for the tests: the same arithmetic as the
// device code, one explicitly rounded operation at a time.  Built with
// -ffp-contract=off by tests/fastmath_host.py.
#include "fastmath.cuh"

extern "C" void fm_eval(int n, const double* x, const double* y, double* out) {
    for (int i = 0; i < n; ++i) {
        out[i] = ctsmg::fm::log(x[i]);
        out[n + i] = ctsmg::fm::log10(x[i]);
        out[2 * n + i] = ctsmg::fm::exp(y[i]);
        out[3 * n + i] = ctsmg::fm::pow(x[i], y[i]);
    }
}
