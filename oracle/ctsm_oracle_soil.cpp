// ctsm_oracle_soil.cpp -- CPU oracle (test infrastructure only) for the soil path.
//
// A plain C++ restatement of the reference Fortran routines, used only by the
// tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  It is
// never linked into the product library.  Each function follows the reference
// routine named in its comment statement by statement, keeping the reference's
// evaluation order (Fortran left-to-right, no FMA contraction: built with
// -ffp-contract=off) and the reference's single-precision literals, which are
// reproduced as (double)(float)x.
//
// Parity is unpinned at the level of SoilWater / SoilTemperature outputs: the
// reference ships no test for these routines and cannot be compiled here (no
// Fortran compiler).  LAPACK dgbsv / dgtsv are restated from the published
// reference-LAPACK algorithm (dgbtf2 + dgbtrs, netlib LAPACK 3.x) and checked
// against scipy.linalg.lapack in the CPU tests.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include "ctsm_gpu.h"
#include "ctsm_oracle.h"
#include "oracle_libm.h"

namespace oracle_libm {
int g_noise_ulps = 0;
uint64_t g_noise_seed = 0;
}

namespace {

// physical constants: tools/mksurfdata_esmf/src/shr_const_mod.F90:14-56 and
// src/main/clm_varcon.F90:48-121
const double TFRZ = 273.15;
const double GRAV = 9.80616;
const double SB = 5.67e-8;
const double DENH2O = 1.000e3;
const double DENICE = 0.917e3;
const double CPLIQ = 4.188e3;
const double CPICE = 2.11727e3;
const double HFUS = 3.337e5;
const double TKAIR = 0.023;
const double TKICE = 2.290;
const double TKWAT = 0.57;
const double CAPR = 0.34;
const double CNFAC = 0.5;
const double THK_BEDROCK = 3.0;
const double CSOL_BEDROCK = 2.0e6;
const double THIN_SFCLAYER = 1.0e-6;   // SoilTemperatureMod.F90:47

const int NLEVSNO = CTSMG_NLEVSNO;
const int NLEVSOI = CTSMG_NLEVSOI;
const int NLEVGRND = CTSMG_NLEVGRND;

inline double sp(float x) { return (double)x; }   // Fortran default-real literal

// gfortran expands x**4 and x**3 into square-and-multiply chains
inline double ipow4(double x) { double x2 = x * x; return x2 * x2; }
inline double ipow3(double x) { double x2 = x * x; return x2 * x; }

// Column-array view: element (c, j) of a field with lower bound lb
struct F {
    const double* b; int ld; int lb;
    double operator()(int c, int j) const { return b[c + (j - lb) * (size_t)ld]; }
};
struct FW {
    double* b; int ld; int lb;
    double& operator()(int c, int j) const { return b[c + (j - lb) * (size_t)ld]; }
};
struct IW {
    int32_t* b; int ld; int lb;
    int32_t& operator()(int c, int j) const { return b[c + (j - lb) * (size_t)ld]; }
};

thread_local int g_err = 0, g_err_idx = 0, g_err_lev = 0;

using oracle_libm::o_pow;
using oracle_libm::o_log10;
void set_err(int code, int idx, int lev) {
    if (g_err == 0) { g_err = code; g_err_idx = idx; g_err_lev = lev; }
}

} // namespace

// Optional libm noise for conditioning studies: when ulps > 0 every pow /
// log10 / exp / log / atan result is scaled by (1 + k eps) with k in
// [-ulps, ulps] drawn from a hash of the call's arguments and the seed
// (deterministic and thread-safe).  Off (0) for every parity run.
extern "C" void oracle_set_libm_noise(int ulps, unsigned long long seed) {
    oracle_libm::g_noise_ulps = ulps;
    oracle_libm::g_noise_seed = seed;
}

// ============================================================ Tridiagonal
// src/biogeophys/TridiagonalMod.F90:23-91 (Thomas algorithm, no pivoting),
// for one column with levels lbj..ubj (arrays indexed 0..n-1 here), jtop = lbj.
extern "C" void oracle_tridiagonal(int n, const double* a, const double* b,
                                   const double* c, const double* r, double* u) {
    std::vector<double> gam(n);
    double bet = b[0];
    for (int j = 0; j < n; ++j) {
        if (j == 0) {
            u[j] = r[j] / bet;
        } else {
            gam[j] = c[j - 1] / bet;
            bet = b[j] - a[j] * gam[j];
            u[j] = (r[j] - a[j] * u[j - 1]) / bet;
        }
    }
    for (int j = n - 2; j >= 0; --j) u[j] = u[j] - gam[j + 1] * u[j + 1];
}

// ============================================================ dgbsv
// Reference-LAPACK dgbsv = dgbtf2 (unblocked band LU with partial pivoting;
// dgbtrf takes this path because ilaenv gives NB=1 for KU<=64) followed by
// dgbtrs ('N') with one right-hand side.  ab is LAPACK band storage,
// ldab = 2*kl+ku+1, column-major: AB(i,j) = ab[(i-1) + (j-1)*ldab].
// Returns info (0, or the 1-based index of a zero pivot).
extern "C" int oracle_dgbsv(int n, int kl, int ku, double* ab, int ldab,
                            int* ipiv, double* bvec) {
    auto AB = [&](int i, int j) -> double& { return ab[(i - 1) + (size_t)(j - 1) * ldab]; };
    const int kv = ku + kl;
    int info = 0;
    // dgbtf2: zero the fill-in elements in columns ku+2 .. min(kv,n)
    for (int j = ku + 2; j <= std::min(kv, n); ++j)
        for (int i = kv - j + 2; i <= kl; ++i) AB(i, j) = 0.0;
    int ju = 1;
    for (int j = 1; j <= n; ++j) {
        if (j + kv <= n)
            for (int i = 1; i <= kl; ++i) AB(i, j + kv) = 0.0;
        int km = std::min(kl, n - j);
        // idamax over km+1 entries starting at AB(kv+1, j)
        int jp = 1;
        double dmax = std::fabs(AB(kv + 1, j));
        for (int i = 2; i <= km + 1; ++i) {
            double v = std::fabs(AB(kv + i, j));
            if (v > dmax) { jp = i; dmax = v; }
        }
        ipiv[j - 1] = jp + j - 1;
        if (AB(kv + jp, j) != 0.0) {
            ju = std::max(ju, std::min(j + ku + jp - 1, n));
            if (jp != 1) {
                // dswap(ju-j+1, AB(kv+jp,j), ldab-1, AB(kv+1,j), ldab-1)
                for (int k = 0; k <= ju - j; ++k) {
                    double& x = AB(kv + jp - k, j + k);
                    double& y = AB(kv + 1 - k, j + k);
                    double t = x; x = y; y = t;
                }
            }
            if (km > 0) {
                double rp = 1.0 / AB(kv + 1, j);          // dscal(km, one/piv, ...)
                for (int i = 1; i <= km; ++i) AB(kv + 1 + i, j) = AB(kv + 1 + i, j) * rp;
                if (ju > j) {
                    // dger(km, ju-j, -one, x=AB(kv+2,j), y=AB(kv,j+1) stride ldab-1,
                    //      A=AB(kv+1,j+1) lda=ldab-1)
                    for (int k = 1; k <= ju - j; ++k) {
                        double yk = AB(kv + 1 - k, j + k);
                        if (yk != 0.0) {
                            double temp = -1.0 * yk;
                            for (int i = 1; i <= km; ++i)
                                AB(kv + 1 + i - k, j + k) = AB(kv + 1 + i - k, j + k) + AB(kv + 1 + i, j) * temp;
                        }
                    }
                }
            }
        } else if (info == 0) {
            info = j;
        }
    }
    if (info != 0) return info;
    // dgbtrs, no transpose: apply P and L
    const int kd = ku + kl + 1;
    if (kl > 0) {
        for (int j = 1; j <= n - 1; ++j) {
            int lm = std::min(kl, n - j);
            int l = ipiv[j - 1];
            if (l != j) { double t = bvec[l - 1]; bvec[l - 1] = bvec[j - 1]; bvec[j - 1] = t; }
            double y = bvec[j - 1];
            if (y != 0.0) {
                double temp = -1.0 * y;
                for (int i = 1; i <= lm; ++i) bvec[j - 1 + i] = bvec[j - 1 + i] + AB(kd + i, j) * temp;
            }
        }
    }
    // dtbsv('Upper','No transpose','Non-unit', n, kl+ku, ab, ldab, b, 1)
    const int k = kl + ku, kplus1 = k + 1;
    for (int j = n; j >= 1; --j) {
        if (bvec[j - 1] != 0.0) {
            int l = kplus1 - j;
            bvec[j - 1] = bvec[j - 1] / AB(kplus1, j);
            double temp = bvec[j - 1];
            for (int i = j - 1; i >= std::max(1, j - k); --i)
                bvec[i - 1] = bvec[i - 1] - temp * AB(l + i, j);
        }
    }
    return 0;
}

// ============================================================ SoilWater (ZD09)
// src/biogeophys/SoilWaterMovementMod.F90:414-972, one column at a time (the
// reference's column-inner loops carry no dependence between columns).
static void zd09_column(int c, const ctsmg_soilwater_io* io, double e_ice, double dtime) {
    const int ld = io->ldc;
    F z{io->z, ld, -NLEVSNO + 1}, zi{io->zi, ld, -NLEVSNO}, dz{io->dz, ld, -NLEVSNO + 1};
    F watsat{io->watsat, ld, 1}, hksat{io->hksat, ld, 1}, bsw{io->bsw, ld, 1}, sucsat{io->sucsat, ld, 1};
    F h2osoi_ice{io->h2osoi_ice, ld, -NLEVSNO + 1}, h2osoi_vol{io->h2osoi_vol, ld, 1};
    F t_soisno{io->t_soisno, ld, -NLEVSNO + 1}, qflx_rootsoi{io->qflx_rootsoi, ld, 1};
    FW h2osoi_liq{io->h2osoi_liq, ld, -NLEVSNO + 1};
    FW icefrac{io->icefrac, ld, 1}, smp_l{io->smp_l, ld, 1}, hk_l{io->hk_l, ld, 1};
    FW qin_col{io->qin, ld, 1}, qout_col{io->qout, ld, 1};
    const double zwt = io->zwt[c], smpmin = io->smpmin[c], qflx_infl = io->qflx_infl[c];

    const int N1 = NLEVSOI + 2;  // 1-based arrays up to nlevsoi+1
    double zmm[N1], dzmm[N1], zimm[N1], vol_ice[N1], vwc_liq[N1], vol_eq[N1], zq[N1];
    double hk[N1], dhkdw[N1], smp[N1], dsmpdw[N1], imped[N1];
    double amx[N1], bmx[N1], cmx[N1], rmx[N1], qin[N1], qout[N1];
    double dqidw0[N1], dqidw1[N1], dqodw1[N1], dqodw2[N1], dwat2[N1];
    double icef[N1];

    for (int j = 1; j <= NLEVSOI; ++j) {
        zmm[j] = z(c, j) * 1.e3;
        dzmm[j] = dz(c, j) * 1.e3;
        zimm[j] = zi(c, j) * 1.e3;
        vol_ice[j] = std::min(watsat(c, j), h2osoi_ice(c, j) / (dz(c, j) * DENICE));
        icef[j] = std::min(1.0, vol_ice[j] / watsat(c, j));
        icefrac(c, j) = icef[j];
        vwc_liq[j] = std::max(h2osoi_liq(c, j), 1.0e-6) / (dz(c, j) * DENH2O);
    }
    zimm[0] = 0.0;
    const double zwtmm = zwt * 1.e3;

    // jwt: layer right above the water table (:638-647)
    int jwt = NLEVSOI;
    for (int j = 1; j <= NLEVSOI; ++j) {
        if (zwt <= zi(c, j)) { jwt = j - 1; break; }
    }
    // vwc at water-table depth (:649-665)
    double vwc_zwt = watsat(c, NLEVSOI);
    if (t_soisno(c, jwt + 1) < TFRZ) {
        vwc_zwt = vwc_liq[NLEVSOI];
        for (int j = NLEVSOI; j <= NLEVGRND; ++j) {
            if (zwt <= zi(c, j)) {
                double smp1 = HFUS * (TFRZ - t_soisno(c, j)) / (GRAV * t_soisno(c, j)) * 1000.0;
                smp1 = std::max(sucsat(c, NLEVSOI), smp1);
                vwc_zwt = watsat(c, NLEVSOI) * o_pow(smp1 / sucsat(c, NLEVSOI), -1.0 / bsw(c, NLEVSOI));
                vwc_zwt = std::min(vwc_zwt, sp(0.5f) * (watsat(c, NLEVSOI) + h2osoi_vol(c, NLEVSOI)));
                break;
            }
        }
    }
    // equilibrium water content (:670-712)
    for (int j = 1; j <= NLEVSOI; ++j) {
        const double ss = sucsat(c, j), ws = watsat(c, j), bb = bsw(c, j);
        if (zwtmm <= zimm[j - 1]) {
            vol_eq[j] = ws;
        } else if ((zwtmm < zimm[j]) && (zwtmm > zimm[j - 1])) {
            double tempi = 1.0;
            double temp0 = o_pow(((ss + zwtmm - zimm[j - 1]) / ss), 1.0 - 1.0 / bb);
            double voleq1 = -ss * ws / (1.0 - 1.0 / bb) / (zwtmm - zimm[j - 1]) * (tempi - temp0);
            vol_eq[j] = (voleq1 * (zwtmm - zimm[j - 1]) + ws * (zimm[j] - zwtmm)) / (zimm[j] - zimm[j - 1]);
            vol_eq[j] = std::min(ws, vol_eq[j]);
            vol_eq[j] = std::max(vol_eq[j], 0.0);
        } else {
            double tempi = o_pow(((ss + zwtmm - zimm[j]) / ss), 1.0 - 1.0 / bb);
            double temp0 = o_pow(((ss + zwtmm - zimm[j - 1]) / ss), 1.0 - 1.0 / bb);
            vol_eq[j] = -ss * ws / (1.0 - 1.0 / bb) / (zimm[j] - zimm[j - 1]) * (tempi - temp0);
            vol_eq[j] = std::max(vol_eq[j], 0.0);
            vol_eq[j] = std::min(ws, vol_eq[j]);
        }
        zq[j] = -ss * o_pow(std::max(vol_eq[j] / ws, 0.01), -bb);
        zq[j] = std::max(smpmin, zq[j]);
    }
    // aquifer-layer zq (:715-728)
    {
        const int j = NLEVSOI;
        if (jwt == NLEVSOI) {
            const double ss = sucsat(c, j), ws = watsat(c, j), bb = bsw(c, j);
            double tempi = 1.0;
            double temp0 = o_pow(((ss + zwtmm - zimm[j]) / ss), 1.0 - 1.0 / bb);
            vol_eq[j + 1] = -ss * ws / (1.0 - 1.0 / bb) / (zwtmm - zimm[j]) * (tempi - temp0);
            vol_eq[j + 1] = std::max(vol_eq[j + 1], 0.0);
            vol_eq[j + 1] = std::min(ws, vol_eq[j + 1]);
            zq[j + 1] = -ss * o_pow(std::max(vol_eq[j + 1] / ws, 0.01), -bb);
            zq[j + 1] = std::max(smpmin, zq[j + 1]);
        }
    }
    // conductivity, matric potential and derivatives (:730-784)
    const double sdamp = 0.0;
    for (int j = 1; j <= NLEVSOI; ++j) {
        const int jp = std::min(NLEVSOI, j + 1);
        double s1 = 0.5 * (vwc_liq[j] + vwc_liq[jp]) / (0.5 * (watsat(c, j) + watsat(c, jp)));
        s1 = std::min(1.0, s1);
        double s2 = hksat(c, j) * o_pow(s1, 2.0 * bsw(c, j) + 2.0);
        imped[j] = o_pow(10.0, -e_ice * (0.5 * (icef[j] + icef[jp])));
        hk[j] = imped[j] * s1 * s2;
        dhkdw[j] = imped[j] * (2.0 * bsw(c, j) + 3.0) * s2 * (1.0 / (watsat(c, j) + watsat(c, jp)));
        double s_node = std::max(vwc_liq[j] / watsat(c, j), 0.01);
        s_node = std::min(1.0, s_node);
        smp[j] = -sucsat(c, j) * o_pow(s_node, -bsw(c, j));
        smp[j] = std::max(smpmin, smp[j]);
        dsmpdw[j] = -bsw(c, j) * smp[j] / vwc_liq[j];
        smp_l(c, j) = smp[j];
        hk_l(c, j) = hk[j];
    }
    // aquifer layer geometry (:787-796)
    zmm[NLEVSOI + 1] = sp(0.5f) * (1.e3 * zwt + zmm[NLEVSOI]);
    if (jwt < NLEVSOI) dzmm[NLEVSOI + 1] = dzmm[NLEVSOI];
    else dzmm[NLEVSOI + 1] = (1.e3 * zwt - zmm[NLEVSOI]);

    // top node (:801-818)
    {
        const int j = 1;
        qin[j] = qflx_infl;
        double den = (zmm[j + 1] - zmm[j]);
        double dzq = (zq[j + 1] - zq[j]);
        double num = (smp[j + 1] - smp[j]) - dzq;
        qout[j] = -hk[j] * num / den;
        dqodw1[j] = -(-hk[j] * dsmpdw[j] + num * dhkdw[j]) / den;
        dqodw2[j] = -(hk[j] * dsmpdw[j + 1] + num * dhkdw[j]) / den;
        rmx[j] = qin[j] - qout[j] - qflx_rootsoi(c, j);
        amx[j] = 0.0;
        bmx[j] = dzmm[j] * (sdamp + 1.0 / dtime) + dqodw1[j];
        cmx[j] = dqodw2[j];
        qin_col(c, j) = qin[j];
        qout_col(c, j) = qout[j];
    }
    // interior nodes (:822-846)
    for (int j = 2; j <= NLEVSOI - 1; ++j) {
        double den = (zmm[j] - zmm[j - 1]);
        double dzq = (zq[j] - zq[j - 1]);
        double num = (smp[j] - smp[j - 1]) - dzq;
        qin[j] = -hk[j - 1] * num / den;
        dqidw0[j] = -(-hk[j - 1] * dsmpdw[j - 1] + num * dhkdw[j - 1]) / den;
        dqidw1[j] = -(hk[j - 1] * dsmpdw[j] + num * dhkdw[j - 1]) / den;
        den = (zmm[j + 1] - zmm[j]);
        dzq = (zq[j + 1] - zq[j]);
        num = (smp[j + 1] - smp[j]) - dzq;
        qout[j] = -hk[j] * num / den;
        dqodw1[j] = -(-hk[j] * dsmpdw[j] + num * dhkdw[j]) / den;
        dqodw2[j] = -(hk[j] * dsmpdw[j + 1] + num * dhkdw[j]) / den;
        rmx[j] = qin[j] - qout[j] - qflx_rootsoi(c, j);
        amx[j] = -dqidw0[j];
        bmx[j] = dzmm[j] / dtime - dqidw1[j] + dqodw1[j];
        cmx[j] = dqodw2[j];
        qin_col(c, j) = qin[j];
        qout_col(c, j) = qout[j];
    }
    // bottom node (:850-894)
    {
        const int j = NLEVSOI;
        if (j > jwt) {
            double den = (zmm[j] - zmm[j - 1]);
            double dzq = (zq[j] - zq[j - 1]);
            double num = (smp[j] - smp[j - 1]) - dzq;
            qin[j] = -hk[j - 1] * num / den;
            dqidw0[j] = -(-hk[j - 1] * dsmpdw[j - 1] + num * dhkdw[j - 1]) / den;
            dqidw1[j] = -(hk[j - 1] * dsmpdw[j] + num * dhkdw[j - 1]) / den;
            qout[j] = 0.0;
            dqodw1[j] = 0.0;
            rmx[j] = qin[j] - qout[j] - qflx_rootsoi(c, j);
            amx[j] = -dqidw0[j];
            bmx[j] = dzmm[j] / dtime - dqidw1[j] + dqodw1[j];
            cmx[j] = 0.0;
            qin_col(c, j) = qin[j];
            qout_col(c, j) = qout[j];
            rmx[j + 1] = 0.0;
            amx[j + 1] = 0.0;
            bmx[j + 1] = dzmm[j + 1] / dtime;
            cmx[j + 1] = 0.0;
        } else {
            double s_node = std::max(sp(0.5f) * ((vwc_zwt + vwc_liq[j]) / watsat(c, j)), 0.01);
            s_node = std::min(1.0, s_node);
            double smp1 = -sucsat(c, j) * o_pow(s_node, -bsw(c, j));
            smp1 = std::max(smpmin, smp1);
            double dsmpdw1 = -bsw(c, j) * smp1 / (s_node * watsat(c, j));
            double den = (zmm[j] - zmm[j - 1]);
            double dzq = (zq[j] - zq[j - 1]);
            double num = (smp[j] - smp[j - 1]) - dzq;
            qin[j] = -hk[j - 1] * num / den;
            dqidw0[j] = -(-hk[j - 1] * dsmpdw[j - 1] + num * dhkdw[j - 1]) / den;
            dqidw1[j] = -(hk[j - 1] * dsmpdw[j] + num * dhkdw[j - 1]) / den;
            den = (zmm[j + 1] - zmm[j]);
            dzq = (zq[j + 1] - zq[j]);
            num = (smp1 - smp[j]) - dzq;
            qout[j] = -hk[j] * num / den;
            dqodw1[j] = -(-hk[j] * dsmpdw[j] + num * dhkdw[j]) / den;
            dqodw2[j] = -(hk[j] * dsmpdw1 + num * dhkdw[j]) / den;
            rmx[j] = qin[j] - qout[j] - qflx_rootsoi(c, j);
            amx[j] = -dqidw0[j];
            bmx[j] = dzmm[j] / dtime - dqidw1[j] + dqodw1[j];
            cmx[j] = dqodw2[j];
            qin[j + 1] = qout[j];
            dqidw0[j + 1] = -(-hk[j] * dsmpdw[j] + num * dhkdw[j]) / den;
            dqidw1[j + 1] = -(hk[j] * dsmpdw1 + num * dhkdw[j]) / den;
            qout[j + 1] = 0.0;
            dqodw1[j + 1] = 0.0;
            rmx[j + 1] = qin[j + 1] - qout[j + 1];
            amx[j + 1] = -dqidw0[j + 1];
            bmx[j + 1] = dzmm[j + 1] / dtime - dqidw1[j + 1] + dqodw1[j + 1];
            cmx[j + 1] = 0.0;
            qin_col(c, j) = qin[j];
            qout_col(c, j) = qout[j];
        }
    }
    // solve (:898-906), Tridiagonal with jtop = 1 over 1..nlevsoi+1
    oracle_tridiagonal(NLEVSOI + 1, amx + 1, bmx + 1, cmx + 1, rmx + 1, dwat2 + 1);

    // renew liquid water, recharge (:912-955)
    for (int j = 1; j <= NLEVSOI; ++j) h2osoi_liq(c, j) = h2osoi_liq(c, j) + dwat2[j] * dzmm[j];
    double qcharge;
    if (jwt < NLEVSOI) {
        const double wh_zwt = 0.0;
        double s_node = std::max(h2osoi_vol(c, jwt + 1) / watsat(c, jwt + 1), 0.01);
        double s1 = std::min(1.0, s_node);
        double ka = imped[jwt + 1] * hksat(c, jwt + 1) * o_pow(s1, 2.0 * bsw(c, jwt + 1) + 3.0);
        double smp1 = std::max(smpmin, smp[std::max(1, jwt)]);
        double wh = smp1 - zq[std::max(1, jwt)];
        if (jwt == 0) {
            qcharge = -ka * (wh_zwt - wh) / ((zwt + sp(1.e-3f)) * 1000.0);
        } else {
            qcharge = -ka * (wh_zwt - wh) / ((zwt - z(c, jwt)) * 1000.0 * sp(2.0f));
        }
        qcharge = std::max(-10.0 / dtime, qcharge);
        qcharge = std::min(10.0 / dtime, qcharge);
    } else {
        qcharge = dwat2[NLEVSOI + 1] * dzmm[NLEVSOI + 1] / dtime;
    }
    io->qcharge[c] = qcharge;
    // water deficit (:958-968)
    double deficit = 0.0;
    for (int j = 1; j <= NLEVSOI; ++j)
        if (h2osoi_liq(c, j) < 0.0) deficit = deficit - h2osoi_liq(c, j);
    io->qflx_deficit[c] = deficit;
}

extern "C" int oracle_soilwater(const ctsmg_bounds* bounds, int num_hydrologyc,
                                const int32_t* filter_hydrologyc,
                                const ctsmg_soilwater_io* io, double e_ice, double dtime) {
    g_err = 0;
#pragma omp parallel for schedule(static)
    for (int fc = 0; fc < num_hydrologyc; ++fc)
        zd09_column(filter_hydrologyc[fc] - bounds->begc, io, e_ice, dtime);
    return 0;
}

// ============================================================ SoilTemperature
// src/biogeophys/SoilTemperatureMod.F90:92-508 with SoilThermProp (:602-901),
// ComputeGroundHeatFluxAndDeriv (:1543-1796), ComputeHeatDiffFluxAndFactor
// (:1799-1910), SetRHSVec* (:1913-2353), SetMatrix* (:2356-2926),
// BandDiagonal (BandDiagonalMod.F90:29-221), PhaseChangeH2osfc (:904-1130)
// and Phasechange (:1133-1540); natural-vegetation columns.
static int soiltemp_column(int c, const ctsmg_bounds* bounds, const ctsmg_soiltemp_io* io,
                           double dtime, int snow_method) {
    const int ld = io->ldc, ldp = io->ldp;
    const int LS = -NLEVSNO + 1;
    F z{io->z, ld, LS}, zi{io->zi, ld, -NLEVSNO}, dz{io->dz, ld, LS};
    F watsat{io->watsat, ld, 1}, bsw{io->bsw, ld, 1}, sucsat{io->sucsat, ld, 1};
    F tkmg{io->tkmg, ld, 1}, tkdry{io->tkdry, ld, 1}, csol{io->csol, ld, 1};
    FW t_soisno{io->t_soisno, ld, LS}, h2osoi_liq{io->h2osoi_liq, ld, LS}, h2osoi_ice{io->h2osoi_ice, ld, LS};
    FW thk{io->thk, ld, LS}, fact{io->fact, ld, LS}, bw{io->bw, ld, LS};
    FW eflx_fgr{io->eflx_fgr, ld, 1};
    FW qflx_snomelt_lyr{io->qflx_snomelt_lyr, ld, LS}, qflx_snofrz_lyr{io->qflx_snofrz_lyr, ld, LS};
    IW imelt{io->imelt, ld, LS};
    F sabg_lyr{io->sabg_lyr, ldp, LS};

    const int snl = io->snl[c];
    const int nbedrock = io->nbedrock[c];
    const double frac_sno = io->frac_sno_eff[c];
    const double frac_h2osfc = io->frac_h2osfc[c];
    const double emg = io->emg[c];

    // index helpers for level arrays -nlevsno+1..nlevgrnd
    const int NL = NLEVSNO + NLEVGRND + 2;
    auto L = [](int j) { return j + NLEVSNO; };     // j in -nlevsno..nlevgrnd+1 -> 0..
    double tk[NL], cv[NL], fn[NL], fn1[NL];
    for (int i = 0; i < NL; ++i) { tk[i] = cv[i] = fn[i] = fn1[i] = NAN; }

    // ---------------- SoilThermProp
    for (int j = LS; j <= NLEVGRND; ++j) {
        if (j >= 1) {
            double satw = (h2osoi_liq(c, j) / DENH2O + h2osoi_ice(c, j) / DENICE + 0.0 / DENICE) / (dz(c, j) * watsat(c, j));
            satw = std::min(1.0, satw);
            double t;
            if (satw > .1e-6) {
                double dke;
                if (t_soisno(c, j) >= TFRZ) dke = std::max(0.0, o_log10(satw) + 1.0);
                else dke = satw;
                double fl = (h2osoi_liq(c, j) / (DENH2O * dz(c, j))) /
                            (h2osoi_liq(c, j) / (DENH2O * dz(c, j)) + h2osoi_ice(c, j) / (DENICE * dz(c, j)) + 0.0 / (DENICE * dz(c, j)));
                double dksat = tkmg(c, j) * o_pow(TKWAT, fl * watsat(c, j)) * o_pow(TKICE, (1.0 - fl) * watsat(c, j));
                t = dke * dksat + (1.0 - dke) * tkdry(c, j);
            } else {
                t = tkdry(c, j);
            }
            if (j > nbedrock) t = THK_BEDROCK;
            thk(c, j) = t;
        }
        if (snl + 1 < 1 && (j >= snl + 1) && (j <= 0)) {
            bw(c, j) = (h2osoi_ice(c, j) + h2osoi_liq(c, j)) / (frac_sno * dz(c, j));
            double b = bw(c, j);
            if (snow_method == 0) {
                thk(c, j) = TKAIR + (7.75e-5 * b + 1.105e-6 * b * b) * (TKICE - TKAIR);
            } else {
                if (b <= 156) thk(c, j) = sp(0.023f) + sp(0.234f) * (b / 1000);
                else thk(c, j) = sp(0.138f) - sp(1.01f) * (b / 1000) + (sp(3.233f) * ((b / 1000) * (b / 1000)));
            }
        }
    }
    for (int j = LS; j <= NLEVGRND; ++j) {
        if (j >= snl + 1 && j <= NLEVGRND - 1) {
            tk[L(j)] = thk(c, j) * thk(c, j + 1) * (z(c, j + 1) - z(c, j)) /
                       (thk(c, j) * (z(c, j + 1) - zi(c, j)) + thk(c, j + 1) * (zi(c, j) - z(c, j)));
        } else if (j == NLEVGRND) {
            tk[L(j)] = 0.0;
        }
    }
    double tk_h2osfc;
    {
        double zh2osfc = sp(1.0e-3f) * (sp(0.5f) * io->h2osfc[c]);
        tk_h2osfc = TKWAT * thk(c, 1) * (z(c, 1) + zh2osfc) / (TKWAT * z(c, 1) + thk(c, 1) * zh2osfc);
    }
    for (int j = 1; j <= NLEVGRND; ++j) {
        cv[L(j)] = csol(c, j) * (1.0 - watsat(c, j)) * dz(c, j) + (h2osoi_ice(c, j) * CPICE + h2osoi_liq(c, j) * CPLIQ) + 0.0 * CPICE;
        if (j > nbedrock) cv[L(j)] = CSOL_BEDROCK * dz(c, j);
    }
    if (io->h2osno_no_layers[c] > 0.0) cv[L(1)] = cv[L(1)] + CPICE * io->h2osno_no_layers[c];
    for (int j = LS; j <= 0; ++j) {
        if (snl + 1 < 1 && j >= snl + 1) {
            if (frac_sno > 0.0)
                cv[L(j)] = std::max(THIN_SFCLAYER, (CPLIQ * h2osoi_liq(c, j) + CPICE * h2osoi_ice(c, j)) / frac_sno);
            else
                cv[L(j)] = THIN_SFCLAYER;
        }
    }

    // ---------------- ComputeGroundHeatFluxAndDeriv
    const double t_grnd = io->t_grnd[c];
    const double lwrad_emit = emg * SB * ipow4(t_grnd);
    const double dlwrad_emit = 4.0 * emg * SB * ipow3(t_grnd);
    const double lwrad_emit_snow = emg * SB * ipow4(t_soisno(c, snl + 1));
    const double lwrad_emit_soil = emg * SB * ipow4(t_soisno(c, 1));
    const double lwrad_emit_h2osfc = emg * SB * ipow4(io->t_h2osfc[c]);
    double hs_soil = 0.0, hs_h2osfc = 0.0, hs = 0.0, dhsdT = 0.0;
    const int p0 = io->col_patchi[c] - bounds->begp, np = io->col_npatches[c];
    const double forc_lwrad = io->forc_lwrad[c], htvp = io->htvp[c];
    for (int p = p0; p < p0 + np; ++p) {
        const double fv = (double)io->frac_veg_nosno[p];
        double gnet = io->sabg[p] + io->dlrad[p] + (1.0 - fv) * emg * forc_lwrad - lwrad_emit -
                      (io->eflx_sh_grnd[p] + io->qflx_evap_soi[p] * htvp);
        io->eflx_gnet[p] = gnet;
        io->sabg_chk[p] = frac_sno * io->sabg_snow[p] + (1.0 - frac_sno) * io->sabg_soil[p];
        double gsoil = io->sabg_soil[p] + io->dlrad[p] + (1.0 - fv) * emg * forc_lwrad - lwrad_emit_soil -
                       (io->eflx_sh_soil[p] + io->qflx_ev_soil[p] * htvp);
        double gh2o = io->sabg_soil[p] + io->dlrad[p] + (1.0 - fv) * emg * forc_lwrad - lwrad_emit_h2osfc -
                      (io->eflx_sh_h2osfc[p] + io->qflx_ev_h2osfc[p] * htvp);
        double dg = -io->cgrnd[p] - dlwrad_emit;
        io->dgnetdT[p] = dg;
        const double w = io->wtcol[p];
        hs = hs + gnet * w;
        dhsdT = dhsdT + dg * w;
        hs_soil = hs_soil + gsoil * w;
        hs_h2osfc = hs_h2osfc + gh2o * w;
    }
    (void)hs;
    double sabg_lyr_col[NLEVSNO + 2];
    for (int j = LS; j <= 1; ++j) sabg_lyr_col[j + NLEVSNO] = 0.0;
    double hs_top = 0.0, hs_top_snow = 0.0;
    const int lyr_top = snl + 1;
    for (int p = p0; p < p0 + np; ++p) {
        const double fv = (double)io->frac_veg_nosno[p];
        const double w = io->wtcol[p];
        double gtop = sabg_lyr(p, lyr_top) + io->dlrad[p] + (1.0 - fv) * emg * forc_lwrad - lwrad_emit -
                      (io->eflx_sh_grnd[p] + io->qflx_evap_soi[p] * htvp);
        hs_top = hs_top + gtop * w;
        double gsnow = sabg_lyr(p, lyr_top) + io->dlrad[p] + (1.0 - fv) * emg * forc_lwrad - lwrad_emit_snow -
                       (io->eflx_sh_snow[p] + io->qflx_ev_snow[p] * htvp);
        hs_top_snow = hs_top_snow + gsnow * w;
        for (int j = lyr_top; j <= 1; ++j)
            sabg_lyr_col[j + NLEVSNO] = sabg_lyr_col[j + NLEVSNO] + sabg_lyr(p, j) * w;
    }
    (void)hs_top;
    auto SLC = [&](int j) { return sabg_lyr_col[j + NLEVSNO]; };

    // ---------------- ComputeHeatDiffFluxAndFactor
    for (int j = LS; j <= NLEVGRND; ++j) {
        if (j >= snl + 1) {
            if (j == snl + 1) {
                fact(c, j) = dtime / cv[L(j)] * dz(c, j) / (0.5 * (z(c, j) - zi(c, j - 1) + CAPR * (z(c, j + 1) - zi(c, j - 1))));
                fn[L(j)] = tk[L(j)] * (t_soisno(c, j + 1) - t_soisno(c, j)) / (z(c, j + 1) - z(c, j));
            } else if (j <= NLEVGRND - 1) {
                fact(c, j) = dtime / cv[L(j)];
                fn[L(j)] = tk[L(j)] * (t_soisno(c, j + 1) - t_soisno(c, j)) / (z(c, j + 1) - z(c, j));
            } else {
                fact(c, j) = dtime / cv[L(j)];
                fn[L(j)] = io->eflx_bot[c];
            }
        }
    }
    // surface water thermal properties (:348-357)
    double c_h2osfc, dz_h2osfc;
    if ((io->h2osfc[c] > THIN_SFCLAYER) && (frac_h2osfc > THIN_SFCLAYER)) {
        c_h2osfc = std::max(THIN_SFCLAYER, CPLIQ * io->h2osfc[c] / frac_h2osfc);
        dz_h2osfc = std::max(THIN_SFCLAYER, sp(1.0e-3f) * io->h2osfc[c] / frac_h2osfc);
    } else {
        c_h2osfc = THIN_SFCLAYER;
        dz_h2osfc = THIN_SFCLAYER;
    }
    io->c_h2osfc[c] = c_h2osfc;

    // ---------------- SetRHSVec: rows -nlevsno..nlevgrnd -> index r + NLEVSNO
    const int NR = NLEVSNO + NLEVGRND + 1;
    double rvec[NR];
    auto R = [&](int r) -> double& { return rvec[r + NLEVSNO]; };
    for (int i = 0; i < NR; ++i) rvec[i] = NAN;
    const double t_h2osfc0 = io->t_h2osfc[c];
    for (int j = LS; j <= 0; ++j) {          // SetRHSVec_Snow
        if (j == snl + 1) {
            R(j - 1) = t_soisno(c, j) + fact(c, j) * (hs_top_snow - dhsdT * t_soisno(c, j) + CNFAC * fn[L(j)]);
        } else if (j > snl + 1) {
            R(j - 1) = t_soisno(c, j) + CNFAC * fact(c, j) * (fn[L(j)] - fn[L(j - 1)]);
            R(j - 1) = R(j - 1) + fact(c, j) * SLC(j);
        }
    }
    double fn_h2osfc;
    {                                         // SetRHSVec_StandingSurfaceWater
        double dzm = (sp(0.5f) * dz_h2osfc + z(c, 1));
        fn_h2osfc = tk_h2osfc * (t_soisno(c, 1) - t_h2osfc0) / dzm;
        R(0) = t_h2osfc0 + (dtime / c_h2osfc) * (hs_h2osfc - dhsdT * t_h2osfc0 + CNFAC * fn_h2osfc);
    }
    for (int j = 1; j <= NLEVGRND; ++j) {    // SetRHSVec_Soil
        if (j == snl + 1) {
            R(j) = t_soisno(c, j) + fact(c, j) * (hs_top_snow - dhsdT * t_soisno(c, j) + CNFAC * fn[L(j)]);
        } else if (j == 1) {
            R(j) = t_soisno(c, j) + fact(c, j) *
                   ((1.0 - frac_sno) * (hs_soil - dhsdT * t_soisno(c, j)) + CNFAC * (fn[L(j)] - frac_sno * fn[L(j - 1)]));
            R(j) = R(j) + frac_sno * fact(c, j) * SLC(j);
        } else if (j <= NLEVGRND - 1) {
            R(j) = t_soisno(c, j) + CNFAC * fact(c, j) * (fn[L(j)] - fn[L(j - 1)]);
        } else {
            R(j) = t_soisno(c, j) - CNFAC * fact(c, j) * fn[L(j - 1)] + fact(c, j) * fn[L(j)];
        }
    }
    if (frac_h2osfc != 0.0)
        R(1) = R(1) - frac_h2osfc * fact(c, 1) * ((hs_soil - dhsdT * t_soisno(c, 1)) + CNFAC * fn_h2osfc);

    // ---------------- SetMatrix: bmat[band 1..5][row]
    double bm[6][NR];
    for (int k = 0; k < 6; ++k) for (int i = 0; i < NR; ++i) bm[k][i] = 0.0;
    auto B = [&](int k, int r) -> double& { return bm[k][r + NLEVSNO]; };
    for (int j = LS; j <= 0; ++j) {          // SetMatrix_Snow
        if (j >= snl + 1) {
            double dzp = z(c, j + 1) - z(c, j);
            if (j == snl + 1) {
                B(4, j - 1) = 0.0;
                B(3, j - 1) = 1.0 + (1.0 - CNFAC) * fact(c, j) * tk[L(j)] / dzp - fact(c, j) * dhsdT;
            } else {
                double dzm = (z(c, j) - z(c, j - 1));
                B(4, j - 1) = -(1.0 - CNFAC) * fact(c, j) * tk[L(j - 1)] / dzm;
                B(3, j - 1) = 1.0 + (1.0 - CNFAC) * fact(c, j) * (tk[L(j)] / dzp + tk[L(j - 1)] / dzm);
            }
            if (j != 0) B(2, j - 1) = -(1.0 - CNFAC) * fact(c, j) * tk[L(j)] / dzp;
            else B(1, j - 1) = -(1.0 - CNFAC) * fact(c, j) * tk[L(j)] / dzp;   // snow -> soil (band 1 of row -1)
        }
    }
    // the assembly copies band 4 of the top snow row only for rows >= -nlevsno+1
    // and band 2 of row -1 is never copied (AssembleMatrixFromSubmatrices, :2459-2480);
    // both entries are zero by construction above, so no masking is needed here.
    for (int j = 1; j <= NLEVGRND; ++j) {    // SetMatrix_Soil
        if (j == snl + 1) {
            double dzp = z(c, j + 1) - z(c, j);
            if (j != 1) B(4, j) = 0.0; else B(5, j) = 0.0;
            B(3, j) = 1.0 + (1.0 - CNFAC) * fact(c, j) * tk[L(j)] / dzp - fact(c, j) * dhsdT;
            B(2, j) = -(1.0 - CNFAC) * fact(c, j) * tk[L(j)] / dzp;
        } else if (j == 1) {
            double dzm = (z(c, j) - z(c, j - 1));
            double dzp = (z(c, j + 1) - z(c, j));
            B(2, j) = -(1.0 - CNFAC) * fact(c, j) * tk[L(j)] / dzp;
            B(3, j) = 1.0 + (1.0 - CNFAC) * fact(c, j) * (tk[L(j)] / dzp + frac_sno * tk[L(j - 1)] / dzm) -
                      (1.0 - frac_sno) * fact(c, j) * dhsdT;
            B(5, j) = -frac_sno * (1.0 - CNFAC) * fact(c, j) * tk[L(j - 1)] / dzm;
        } else if (j <= NLEVGRND - 1) {
            double dzm = (z(c, j) - z(c, j - 1));
            double dzp = (z(c, j + 1) - z(c, j));
            B(2, j) = -(1.0 - CNFAC) * fact(c, j) * tk[L(j)] / dzp;
            B(3, j) = 1.0 + (1.0 - CNFAC) * fact(c, j) * (tk[L(j)] / dzp + tk[L(j - 1)] / dzm);
            B(4, j) = -(1.0 - CNFAC) * fact(c, j) * tk[L(j - 1)] / dzm;
        } else {
            double dzm = (z(c, j) - z(c, j - 1));
            B(2, j) = 0.0;
            B(3, j) = 1.0 + (1.0 - CNFAC) * fact(c, j) * tk[L(j - 1)] / dzm;
            B(4, j) = -(1.0 - CNFAC) * fact(c, j) * tk[L(j - 1)] / dzm;
        }
    }
    {
        double dzm = (sp(0.5f) * dz_h2osfc + z(c, 1));
        if (frac_h2osfc != 0.0)
            B(3, 1) = B(3, 1) + frac_h2osfc * ((1.0 - CNFAC) * fact(c, 1) * tk_h2osfc / dzm + fact(c, 1) * dhsdT);
        // SetMatrix_StandingSurfaceWater
        B(3, 0) = 1.0 + (1.0 - CNFAC) * (dtime / c_h2osfc) * tk_h2osfc / dzm - (dtime / c_h2osfc) * dhsdT;
        B(2, 0) = -(1.0 - CNFAC) * (dtime / c_h2osfc) * tk_h2osfc / dzm;
        if (frac_h2osfc != 0.0)
            B(4, 1) = -frac_h2osfc * (1.0 - CNFAC) * fact(c, 1) * tk_h2osfc / dzm;
    }
    // AssembleMatrixFromSubmatrices: band 2 of row 25 and band 4 of row 1 from
    // soil are not copied; band 4 of row 1 is the ssw coupling set just above.
    B(2, NLEVGRND) = 0.0;

    // ---------------- BandDiagonal (BandDiagonalMod.F90:167-219)
    const int jtop = snl, jbot = NLEVGRND;
    const int n = jbot - jtop + 1;
    const int kl = 2, ku = 2, m = 2 * kl + ku + 1;
    std::vector<double> ab((size_t)m * n, 0.0), res(n);
    std::vector<int> ipiv(n);
    auto AB = [&](int i, int jj) -> double& { return ab[(i - 1) + (size_t)(jj - 1) * m]; };
    for (int jj = 3; jj <= n; ++jj) AB(kl + ku - 1, jj) = B(1, jtop + jj - 3);
    for (int jj = 2; jj <= n; ++jj) AB(kl + ku + 0, jj) = B(2, jtop + jj - 2);
    for (int jj = 1; jj <= n; ++jj) AB(kl + ku + 1, jj) = B(3, jtop + jj - 1);
    for (int jj = 1; jj <= n - 1; ++jj) AB(kl + ku + 2, jj) = B(4, jtop + jj);
    for (int jj = 1; jj <= n - 2; ++jj) AB(kl + ku + 3, jj) = B(5, jtop + jj + 1);
    for (int jj = 1; jj <= n; ++jj) res[jj - 1] = R(jtop + jj - 1);
    int info = oracle_dgbsv(n, kl, ku, ab.data(), m, ipiv.data(), res.data());
    if (info != 0) return info;
    auto TV = [&](int r) { return res[r - jtop]; };

    // unpack (:422-434)
    for (int j = snl + 1; j <= 0; ++j) t_soisno(c, j) = TV(j - 1);
    for (int j = 1; j <= NLEVGRND; ++j) t_soisno(c, j) = TV(j);
    double t_h2osfc;
    if (frac_h2osfc == 0.0) t_h2osfc = t_soisno(c, 1);
    else t_h2osfc = TV(0);
    io->t_h2osfc[c] = t_h2osfc;

    // fn1 (:438-483)
    for (int j = LS; j <= NLEVGRND; ++j) {
        if (j >= snl + 1) {
            if (j <= NLEVGRND - 1) fn1[L(j)] = tk[L(j)] * (t_soisno(c, j + 1) - t_soisno(c, j)) / (z(c, j + 1) - z(c, j));
            else fn1[L(j)] = 0.0;
        }
    }

    // ---------------- PhaseChangeH2osfc (:904-1130)
    io->xmf_h2osfc[c] = 0.0;
    io->qflx_h2osfc_to_ice[c] = 0.0;
    io->eflx_h2osfc_to_snow[c] = 0.0;
    {
        double h2osno_total = io->h2osno_no_layers[c];
        for (int j = snl + 1; j <= 0; ++j) h2osno_total = h2osno_total + h2osoi_ice(c, j) + h2osoi_liq(c, j);
        if (frac_h2osfc > 0.0 && t_h2osfc <= TFRZ) {
            double tinc = TFRZ - t_h2osfc;
            t_h2osfc = TFRZ;
            double hm = frac_h2osfc * (dhsdT * tinc - tinc * c_h2osfc / dtime);
            double xm = hm * dtime / HFUS;
            double temp1 = io->h2osfc[c] + xm;
            double z_avg = frac_sno * io->snow_depth[c];
            double rho_avg;
            if (z_avg > 0.0) rho_avg = std::min(800.0, h2osno_total / z_avg);
            else rho_avg = 200.0;
            if (temp1 >= 0.0) {
                io->int_snow[c] = io->int_snow[c] - xm;
                if (snl == 0) io->h2osno_no_layers[c] = io->h2osno_no_layers[c] - xm;
                else h2osoi_ice(c, 0) = h2osoi_ice(c, 0) - xm;
                h2osno_total = h2osno_total - xm;
                io->h2osfc[c] = io->h2osfc[c] + xm;
                io->xmf_h2osfc[c] = hm;
                io->qflx_h2osfc_to_ice[c] = -xm / dtime;
                if (frac_sno > 0 && snl < 0) io->snow_depth[c] = h2osno_total / (rho_avg * frac_sno);
                else io->snow_depth[c] = h2osno_total / DENICE;
                if (snl == 0) {
                    t_soisno(c, 0) = t_h2osfc;
                    io->eflx_h2osfc_to_snow[c] = 0.;
                } else {
                    double c1, c2;
                    if (snl == -1) c1 = frac_sno * (dtime / fact(c, 0) - dhsdT * dtime);
                    else c1 = frac_sno / fact(c, 0) * dtime;
                    if (frac_h2osfc != 0.0) c2 = (-CPLIQ * xm - frac_h2osfc * dhsdT * dtime);
                    else c2 = 0.0;
                    t_soisno(c, 0) = (c1 * t_soisno(c, 0) + c2 * t_h2osfc) / (c1 + c2);
                    io->eflx_h2osfc_to_snow[c] = (t_h2osfc - t_soisno(c, 0)) * c2 / dtime;
                }
            } else {
                rho_avg = (h2osno_total * rho_avg + io->h2osfc[c] * DENICE) / (h2osno_total + io->h2osfc[c]);
                io->int_snow[c] = io->int_snow[c] + io->h2osfc[c];
                if (snl == 0) io->h2osno_no_layers[c] = io->h2osno_no_layers[c] + io->h2osfc[c];
                else h2osoi_ice(c, 0) = h2osoi_ice(c, 0) + io->h2osfc[c];
                h2osno_total = h2osno_total + io->h2osfc[c];
                io->qflx_h2osfc_to_ice[c] = io->h2osfc[c] / dtime;
                t_h2osfc = t_h2osfc - temp1 * HFUS / (dtime * dhsdT - c_h2osfc);
                io->xmf_h2osfc[c] = (hm - frac_h2osfc * temp1 * HFUS / dtime);
                if (snl == 0) {
                    t_soisno(c, 0) = t_h2osfc;
                } else if (snl == -1) {
                    double c1 = frac_sno * (dtime / fact(c, 0) - dhsdT * dtime);
                    double c2 = (frac_h2osfc != 0.0) ? frac_h2osfc * (c_h2osfc - dtime * dhsdT) : 0.0;
                    t_soisno(c, 0) = (c1 * t_soisno(c, 0) + c2 * t_h2osfc) / (c1 + c2);
                    t_h2osfc = t_soisno(c, 0);
                } else {
                    double c1 = frac_sno / fact(c, 0) * dtime;
                    double c2 = (frac_h2osfc != 0.0) ? frac_h2osfc * (c_h2osfc - dtime * dhsdT) : 0.0;
                    t_soisno(c, 0) = (c1 * t_soisno(c, 0) + c2 * t_h2osfc) / (c1 + c2);
                    t_h2osfc = t_soisno(c, 0);
                }
                io->h2osfc[c] = 0.0;
                if (frac_sno > 0 && snl < 0) io->snow_depth[c] = h2osno_total / (rho_avg * frac_sno);
                else io->snow_depth[c] = h2osno_total / DENICE;
            }
            io->t_h2osfc[c] = t_h2osfc;
        }
    }

    // ---------------- Phasechange (:1133-1540)
    double xmf = 0.0, qflx_snomelt = 0.0, qflx_snofrz = 0.0, qflx_snow_drain = 0.0;
    double hm[NL], xm[NL], wice0[NL], wliq0[NL], wmass0[NL], tinc[NL], supercool[NL];
    for (int j = LS; j <= NLEVGRND; ++j) {
        if (j >= snl + 1) {
            imelt(c, j) = 0;
            hm[L(j)] = 0.0;
            xm[L(j)] = 0.0;
            wice0[L(j)] = h2osoi_ice(c, j);
            wliq0[L(j)] = h2osoi_liq(c, j);
            wmass0[L(j)] = h2osoi_ice(c, j) + h2osoi_liq(c, j) + 0.0;
        }
        if (j <= 0) {
            qflx_snomelt_lyr(c, j) = 0.0;
            qflx_snofrz_lyr(c, j) = 0.0;
        }
    }
    for (int j = LS; j <= 0; ++j) {
        if (j >= snl + 1) {
            if (h2osoi_ice(c, j) > 0.0 && t_soisno(c, j) > TFRZ) {
                imelt(c, j) = 1;
                tinc[L(j)] = TFRZ - t_soisno(c, j);
                t_soisno(c, j) = TFRZ;
            }
            if (h2osoi_liq(c, j) > 0.0 && t_soisno(c, j) < TFRZ) {
                imelt(c, j) = 2;
                tinc[L(j)] = TFRZ - t_soisno(c, j);
                t_soisno(c, j) = TFRZ;
            }
        }
    }
    const double h2osno_nl = io->h2osno_no_layers[c];
    for (int j = 1; j <= NLEVGRND; ++j) {
        supercool[L(j)] = 0.0;
        if (h2osoi_ice(c, j) > 0. && t_soisno(c, j) > TFRZ) {
            imelt(c, j) = 1;
            tinc[L(j)] = TFRZ - t_soisno(c, j);
            t_soisno(c, j) = TFRZ;
        }
        supercool[L(j)] = 0.0;
        if (t_soisno(c, j) < TFRZ) {
            double smp = HFUS * (TFRZ - t_soisno(c, j)) / (GRAV * t_soisno(c, j)) * 1000.0;
            supercool[L(j)] = watsat(c, j) * o_pow(smp / sucsat(c, j), -1.0 / bsw(c, j));
            supercool[L(j)] = supercool[L(j)] * dz(c, j) * 1000.0;
        }
        if (h2osoi_liq(c, j) > supercool[L(j)] && t_soisno(c, j) < TFRZ) {
            imelt(c, j) = 2;
            tinc[L(j)] = TFRZ - t_soisno(c, j);
            t_soisno(c, j) = TFRZ;
        }
        if (h2osno_nl > 0.0 && j == 1) {
            if (t_soisno(c, j) > TFRZ) {
                imelt(c, j) = 1;
                tinc[L(j)] = TFRZ - t_soisno(c, j);
                t_soisno(c, j) = TFRZ;
            }
        }
    }
    for (int j = LS; j <= NLEVGRND; ++j) {
        if (j < snl + 1) continue;
        const int lj = L(j);
        if (imelt(c, j) > 0) {
            if (j == snl + 1) {
                if (j > 0) hm[lj] = dhsdT * tinc[lj] - tinc[lj] / fact(c, j);
                else hm[lj] = frac_sno * (dhsdT * tinc[lj] - tinc[lj] / fact(c, j));
                if (j == 1 && frac_h2osfc != 0.0) hm[lj] = hm[lj] - frac_h2osfc * (dhsdT * tinc[lj]);
            } else if (j == 1) {
                hm[lj] = (1.0 - frac_sno - frac_h2osfc) * dhsdT * tinc[lj] - tinc[lj] / fact(c, j);
            } else {
                if (j < 1) hm[lj] = -frac_sno * (tinc[lj] / fact(c, j));
                else hm[lj] = -tinc[lj] / fact(c, j);
            }
        }
        if (imelt(c, j) == 1 && hm[lj] < 0.0) { hm[lj] = 0.0; imelt(c, j) = 0; }
        if (imelt(c, j) == 2 && hm[lj] > 0.0) { hm[lj] = 0.0; imelt(c, j) = 0; }
        if (imelt(c, j) > 0 && std::fabs(hm[lj]) > 0.0) {
            xm[lj] = hm[lj] * dtime / HFUS;
            if (j == 1) {
                if (io->h2osno_no_layers[c] > 0.0 && xm[lj] > 0.0) {
                    double temp1 = io->h2osno_no_layers[c];
                    io->h2osno_no_layers[c] = std::max(0.0, temp1 - xm[lj]);
                    double propor = io->h2osno_no_layers[c] / temp1;
                    io->snow_depth[c] = propor * io->snow_depth[c];
                    double heatr = hm[lj] - HFUS * (temp1 - io->h2osno_no_layers[c]) / dtime;
                    if (heatr > 0.0) { xm[lj] = heatr * dtime / HFUS; hm[lj] = heatr; }
                    else { xm[lj] = 0.0; hm[lj] = 0.0; }
                    qflx_snomelt = std::max(0.0, (temp1 - io->h2osno_no_layers[c])) / dtime;
                    xmf = HFUS * qflx_snomelt;
                    qflx_snow_drain = qflx_snomelt;
                }
            }
            double heatr = 0.0;
            if (xm[lj] > 0.0) {
                h2osoi_ice(c, j) = std::max(0.0, wice0[lj] - xm[lj]);
                if (j >= 1) {
                    heatr = hm[lj] - HFUS * (0.0 - 0.0 + wice0[lj] - h2osoi_ice(c, j)) / dtime;
                } else {
                    heatr = hm[lj] - HFUS * (wice0[lj] - h2osoi_ice(c, j)) / dtime;
                }
            } else if (xm[lj] < 0.0) {
                if (j <= 0) {
                    h2osoi_ice(c, j) = std::min(wmass0[lj], wice0[lj] - xm[lj]);
                } else {
                    if (wmass0[lj] - 0.0 < supercool[lj]) h2osoi_ice(c, j) = 0.0;
                    else h2osoi_ice(c, j) = std::min(wmass0[lj] - 0.0 - supercool[lj], wice0[lj] - xm[lj]);
                }
                heatr = hm[lj] - HFUS * (wice0[lj] - h2osoi_ice(c, j)) / dtime;
            }
            h2osoi_liq(c, j) = std::max(0.0, wmass0[lj] - h2osoi_ice(c, j) - 0.0);
            if (std::fabs(heatr) > 0.0) {
                if (j == snl + 1) {
                    if (j == 1) {
                        t_soisno(c, j) = t_soisno(c, j) + fact(c, j) * heatr / (1.0 - (1.0 - frac_h2osfc) * fact(c, j) * dhsdT);
                    } else {
                        t_soisno(c, j) = t_soisno(c, j) + (fact(c, j) / frac_sno) * heatr / (1.0 - fact(c, j) * dhsdT);
                    }
                } else if (j == 1) {
                    t_soisno(c, j) = t_soisno(c, j) + fact(c, j) * heatr /
                                     (1.0 - (1.0 - frac_sno - frac_h2osfc) * fact(c, j) * dhsdT);
                } else {
                    if (j > 0) t_soisno(c, j) = t_soisno(c, j) + fact(c, j) * heatr;
                    else if (frac_sno > 0.0) t_soisno(c, j) = t_soisno(c, j) + (fact(c, j) / frac_sno) * heatr;
                }
                if (j <= 0) {
                    if (h2osoi_liq(c, j) * h2osoi_ice(c, j) > 0.0) t_soisno(c, j) = TFRZ;
                }
            }
            if (j >= 1) {
                xmf = xmf + HFUS * (wice0[lj] - h2osoi_ice(c, j)) / dtime + HFUS * (0.0 - 0.0) / dtime;
            } else {
                xmf = xmf + HFUS * (wice0[lj] - h2osoi_ice(c, j)) / dtime;
            }
            if (imelt(c, j) == 1 && j < 1) {
                qflx_snomelt_lyr(c, j) = std::max(0.0, (wice0[lj] - h2osoi_ice(c, j))) / dtime;
                qflx_snomelt = qflx_snomelt + qflx_snomelt_lyr(c, j);
                io->snomelt_accum[c] = io->snomelt_accum[c] + qflx_snomelt_lyr(c, j) * dtime * 1.e-3;
            }
            if (imelt(c, j) == 2 && j < 1) {
                qflx_snofrz_lyr(c, j) = std::max(0.0, (h2osoi_ice(c, j) - wice0[lj])) / dtime;
                qflx_snofrz = qflx_snofrz + qflx_snofrz_lyr(c, j);
            }
        }
    }
    io->xmf[c] = xmf;
    io->qflx_snomelt[c] = qflx_snomelt;
    io->qflx_snofrz[c] = qflx_snofrz;
    io->qflx_snow_drain[c] = qflx_snow_drain;
    io->eflx_snomelt[c] = qflx_snomelt * HFUS;
    (void)wliq0;

    // ---------------- t_grnd (:457-477)
    double tg;
    if (snl < 0) {
        if (frac_h2osfc != 0.0)
            tg = frac_sno * t_soisno(c, snl + 1) + (1.0 - frac_sno - frac_h2osfc) * t_soisno(c, 1) + frac_h2osfc * io->t_h2osfc[c];
        else
            tg = frac_sno * t_soisno(c, snl + 1) + (1.0 - frac_sno) * t_soisno(c, 1);
    } else {
        if (frac_h2osfc != 0.0) tg = (1.0 - frac_h2osfc) * t_soisno(c, 1) + frac_h2osfc * io->t_h2osfc[c];
        else tg = t_soisno(c, 1);
    }
    io->t_grnd[c] = tg;

    // ---------------- eflx_fgr12, eflx_fgr (:479-504)
    io->eflx_fgr12[c] = -CNFAC * fn[L(1)] - (1.0 - CNFAC) * fn1[L(1)];
    for (int j = 1; j <= NLEVGRND; ++j) {
        if (j < NLEVGRND) eflx_fgr(c, j) = -CNFAC * fn[L(j)] - (1.0 - CNFAC) * fn1[L(j)];
        else eflx_fgr(c, j) = 0.0;
    }
    return 0;
}

extern "C" int oracle_soiltemperature(const ctsmg_bounds* bounds, int num_nolakec,
                                      const int32_t* filter_nolakec,
                                      const ctsmg_soiltemp_io* io, double dtime, int snow_method) {
    int first_bad = 0, bad_c = 0;
#pragma omp parallel for schedule(static)
    for (int fc = 0; fc < num_nolakec; ++fc) {
        int c = filter_nolakec[fc] - bounds->begc;
        int info = soiltemp_column(c, bounds, io, dtime, snow_method);
        if (info != 0) {
#pragma omp critical
            { if (first_bad == 0 || fc < bad_c) { first_bad = info; bad_c = fc; } }
        }
    }
    if (first_bad) { set_err(CTSMG_E_SINGULAR, filter_nolakec[bad_c], first_bad); return CTSMG_E_SINGULAR; }
    return 0;
}

extern "C" int oracle_last_error(int* idx, int* lev) {
    if (idx) *idx = g_err_idx;
    if (lev) *lev = g_err_lev;
    return g_err;
}

// Compute_EffecRootFrac_And_VertTranSink_Default
// (src/biogeophys/SoilWaterPlantSinkMod.F90:332-420) for dense arrays
// (columns 1..ncol, patches col_patchi..col_patchi+npatches-1, 1-based).
extern "C" void oracle_rootsink(int ncol, int ldp, const int32_t* col_patchi, const int32_t* col_npatches,
                                const double* wtcol, const double* qflx_tran_veg, const double* rootr,
                                double* qflx_rootsoi) {
    for (int c = 0; c < ncol; ++c) {
        const int p0 = col_patchi[c] - 1, np = col_npatches[c];
        double rc[NLEVSOI + 1];
        for (int j = 1; j <= NLEVSOI; ++j) rc[j] = 0.0;
        for (int j = 1; j <= NLEVSOI; ++j)
            for (int p = p0; p < p0 + np; ++p) rc[j] = rc[j] + rootr[p + (size_t)(j - 1) * ldp] * qflx_tran_veg[p] * wtcol[p];
        double temp = 0.0;
        for (int p = p0; p < p0 + np; ++p) temp = temp + qflx_tran_veg[p] * wtcol[p];
        const double tran_col = temp;
        for (int j = 1; j <= NLEVSOI; ++j) {
            if (temp != 0.0) rc[j] = rc[j] / temp;
            qflx_rootsoi[c + (size_t)(j - 1) * ncol] = rc[j] * tran_col;
        }
    }
}

// Compute_EffecRootFrac_And_VertTranSink_Default
// (src/biogeophys/SoilWaterPlantSinkMod.F90:332-420) over a column filter with
// the drop-in's io struct: rootr_col zeroed (:376-381), accumulated level by
// level over the column's patches (:383-393), temp summed (:394-401), then
// the quotient and qflx_rootsoi = rootr_col * qflx_tran_veg_col (:403-412);
// a NULL qflx_tran_veg_col stands for the wtcol-weighted patch sum.
extern "C" int oracle_root_sink(const ctsmg_bounds* b, int nf, const int32_t* filt, const ctsmg_rootsink_io* io) {
    const int ldc = io->ldc, ldp = io->ldp;
    std::vector<double> temp(b->endc - b->begc + 1, 0.0);
    for (int j = 1; j <= NLEVSOI; ++j)
        for (int fc = 0; fc < nf; ++fc) io->rootr_col[(filt[fc] - b->begc) + (size_t)(j - 1) * ldc] = 0.0;
    for (int j = 1; j <= NLEVSOI; ++j)
        for (int fc = 0; fc < nf; ++fc) {
            const int c = filt[fc] - b->begc;
            const int p0 = io->col_patchi[c] - b->begp, np = io->col_npatches[c];
            double& r = io->rootr_col[c + (size_t)(j - 1) * ldc];
            for (int p = p0; p < p0 + np; ++p) r = r + io->rootr[p + (size_t)(j - 1) * ldp] * io->qflx_tran_veg[p] * io->wtcol[p];
        }
    for (int fc = 0; fc < nf; ++fc) {
        const int c = filt[fc] - b->begc;
        const int p0 = io->col_patchi[c] - b->begp, np = io->col_npatches[c];
        for (int p = p0; p < p0 + np; ++p) temp[c] = temp[c] + io->qflx_tran_veg[p] * io->wtcol[p];
    }
    for (int j = 1; j <= NLEVSOI; ++j)
        for (int fc = 0; fc < nf; ++fc) {
            const int c = filt[fc] - b->begc;
            double& r = io->rootr_col[c + (size_t)(j - 1) * ldc];
            if (temp[c] != 0.0) r = r / temp[c];
            const double tcol = io->qflx_tran_veg_col ? io->qflx_tran_veg_col[c] : temp[c];
            io->qflx_rootsoi[c + (size_t)(j - 1) * ldc] = r * tcol;
        }
    return 0;
}
