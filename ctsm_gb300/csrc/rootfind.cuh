// rootfind.cuh -- the Ci root finder of Photosynthesis: the secant iteration
// of hybrid (src/biogeophys/PhotosynthesisMod.F90:2251-2368) with its Brent
// fallback (:2371-2485), written as a resumable state machine with a single
// evaluation point.  The caller evaluates f at rf.x, passes the value to
// rf.next(f) and repeats while next() returns true:
//
//     rf.start(x0);
//     do { f = ci_func(rf.x, ...); } while (rf.next(f));
//
// The points evaluated, their order and the last evaluation (whose side
// effects -- ac, aj, ap, ag, an, gs_mol -- are what Photosynthesis keeps) are
// those of the reference's nested hybrid -> brent calls.  With one call site
// the evaluation is compiled once, and the lanes of a warp that are at
// different places of the iteration (first points, secant steps, Brent steps,
// the final re-evaluation at the minimum) evaluate together.
#pragma once
#include <cmath>

#ifndef __CUDACC__
#define CTSMG_HD
#else
#define CTSMG_HD __host__ __device__
#endif

namespace ctsmg {

struct RootFind {
    double x;                                   // next point to evaluate
    double x0, x1, f0, f1, minx, minf, tol;     // hybrid
    double a, b, c, fa, fb, fc, d, e;           // brent
    int mode, iter, biter;
    bool not_bracketed;                         // brent's endrun condition (:2412-2415)

    enum { M_X0, M_X1, M_SECANT, M_BRENT, M_MIN };

    CTSMG_HD void start(double xs) {
        x = xs;
        x0 = xs;
        mode = M_X0;
        not_bracketed = false;
    }

    // Next secant point (:2321-2331); false when |dx| < tol (converged).
    CTSMG_HD bool secant() {
        const double dx = -f1 * (x1 - x0) / (f1 - f0);
        const double xn = x1 + dx;
        tol = std::fabs(xn) * 1.e-2;
        if (std::fabs(dx) < tol) return false;
        x0 = x1;
        f0 = f1;
        x1 = xn;
        x = xn;
        mode = M_SECANT;
        return true;
    }

    // One Brent iteration up to its evaluation (:2420-2472); false when it
    // has converged.
    CTSMG_HD bool brent_step() {
        const double eps = 1.e-2;
        if ((fb > 0.0 && fc > 0.0) || (fb < 0.0 && fc < 0.0)) { c = a; fc = fa; d = b - a; e = d; }
        if (std::fabs(fc) < std::fabs(fb)) { a = b; b = c; c = a; fa = fb; fb = fc; fc = fa; }
        const double tol1 = 2.0 * eps * std::fabs(b) + 0.5 * tol;
        const double xm = 0.5 * (c - b);
        if (std::fabs(xm) <= tol1 || fb == 0.) return false;
        if (std::fabs(e) >= tol1 && std::fabs(fa) > std::fabs(fb)) {
            const double s = fb / fa;
            double p, q;
            if (a == c) {
                p = 2.0 * xm * s;
                q = 1.0 - s;
            } else {
                q = fa / fc;
                const double r = fb / fc;
                p = s * (2.0 * xm * q * (q - r) - (b - a) * (r - 1.0));
                q = (q - 1.0) * (r - 1.0) * (s - 1.0);
            }
            if (p > 0.0) q = -q;
            p = std::fabs(p);
            if (2.0 * p < std::fmin(3.0 * xm * q - std::fabs(tol1 * q), std::fabs(e * q))) { e = d; d = p / q; }
            else { d = xm; e = d; }
        } else {
            d = xm;
            e = d;
        }
        a = b;
        fa = fb;
        if (std::fabs(d) > tol1) b = b + d;
        else b = b + std::copysign(std::fabs(tol1), xm);
        x = b;
        mode = M_BRENT;
        return true;
    }

    // Consume f(x); true when another evaluation (at x) is needed.
    CTSMG_HD bool next(double f) {
        switch (mode) {
        case M_X0:                                        // :2297-2304
            f0 = f;
            if (f0 == 0.0) return false;
            minx = x0;
            minf = f0;
            x1 = x0 * 0.99;
            x = x1;
            mode = M_X1;
            return true;
        case M_X1:                                        // :2306-2316
            f1 = f;
            if (f1 == 0.0) return false;
            if (f1 < minf) { minx = x1; minf = f1; }
            iter = 1;
            return secant();
        case M_SECANT:                                    // :2333-2354
            f1 = f;
            if (f1 < minf) { minx = x1; minf = f1; }
            if (std::fabs(f1) <= 1.e-4) return false;
            if (f1 * f0 < 0.0) {                          // brent(x0, x1, f0, f1, tol): :2408-2418
                a = x0; b = x1; fa = f0; fb = f1;
                if ((fa > 0.0 && fb > 0.0) || (fa < 0.0 && fb < 0.0)) { not_bracketed = true; return false; }
                c = b; fc = fb; d = 0.0; e = 0.0;
                biter = 0;
                return brent_step();
            }
            if (iter > 40) { x = minx; mode = M_MIN; return true; }   // :2355-2364
            ++iter;
            return secant();
        case M_BRENT:                                     // :2474-2479 (itmax = 20)
            fb = f;
            if (fb == 0.0) return false;
            if (++biter == 20) return false;
            return brent_step();
        default:                                          // f(minx) evaluated
            return false;
        }
    }
};

} // namespace ctsmg
