// baregrnd_kernels.cu -- BareGroundFluxes (src/biogeophys/BareGroundFluxesMod.F90:73-545)
// in FP64 on sm_103a: one thread per patch of filter_noexposedvegp.  Three
// Monin-Obukhov iterations with the general FrictionVelocity
// (FrictionVelocityMod.F90:754-1117: separate roughness lengths for momentum,
// heat and moisture, which ZengWang2007 makes differ over bare ground), then
// the ground fluxes, their temperature derivatives and the 2 m diagnostics.
#include <cuda_runtime.h>
#include <cstdint>
#include "ctsm_device.cuh"
#include "qsat.cuh"
#include "baregrnd_kernels.cuh"

namespace ctsmg {
namespace bare {

constexpr double PI = 3.14159265358979323846;
constexpr double VKC = 0.4;
constexpr double CPAIR = 1.00464e3;
constexpr double RGAS = 6.02214e26 * 1.38065e-23;
constexpr double NU_PARAM = 1.5e-5;
constexpr double ZII = 1000.0;    // convective boundary height (m), FrictionVelocity cold start
constexpr double BETA = 1.0;      // coefficient of the convective velocity

// FrictionVelocityMod.F90:1120-1155
__device__ __forceinline__ double stab1(double zeta) {
    const double chik2 = sqrt(1.0 - 16.0 * zeta);
    const double chik = sqrt(chik2);
    return 2.0 * log((1.0 + chik) * 0.5) + log((1.0 + chik2) * 0.5) - 2.0 * atan(chik) + PI * 0.5;
}
__device__ __forceinline__ double stab2(double zeta) { return 2.0 * log((1.0 + sqrt(1.0 - 16.0 * zeta)) * 0.5); }

struct FV { double ustar, temp1, temp2, temp12m, temp22m, u10_clm, va, vds, u10; };

// FrictionVelocityMod.F90:754-1117 for one patch
__device__ void friction_velocity(double displa, double z0m, double z0h, double z0q, double obu, int iter, double ur,
                                  double um, double hgt_u, double hgt_t, double hgt_q, double& fm, FV& o) {
    const double zetam = 1.574, zetat = 0.465;
    const double zldis = hgt_u - displa;
    const double zeta = zldis / obu;
    double ustar;
    if (zeta < -zetam)
        ustar = VKC * um / (log(-zetam * obu / z0m) - stab1(-zetam) + stab1(z0m / obu) +
                            1.14 * (pow(-zeta, 0.333) - pow(zetam, 0.333)));
    else if (zeta < 0.0)
        ustar = VKC * um / (log(zldis / z0m) - stab1(zeta) + stab1(z0m / obu));
    else if (zeta <= 1.0)
        ustar = VKC * um / (log(zldis / z0m) + 5.0 * zeta - 5.0 * z0m / obu);
    else
        ustar = VKC * um / (log(obu / z0m) + 5.0 - 5.0 * z0m / obu + (5.0 * log(zeta) + zeta - 1.0));
    o.ustar = ustar;
    o.vds = (zeta < 0.0) ? 2.e-3 * ustar * (1.0 + pow(300.0 / (-obu), 0.666)) : 2.e-3 * ustar;
    if (zldis - z0m <= 10.0) {
        o.u10_clm = um;
    } else {
        const double z10 = 10.0 + z0m;
        if (zeta < -zetam)
            o.u10_clm = um - (ustar / VKC * (log(-zetam * obu / z10) - stab1(-zetam) + stab1(z10 / obu) +
                                              1.14 * (pow(-zeta, 0.333) - pow(zetam, 0.333))));
        else if (zeta < 0.0)
            o.u10_clm = um - (ustar / VKC * (log(zldis / z10) - stab1(zeta) + stab1(z10 / obu)));
        else if (zeta <= 1.0)
            o.u10_clm = um - (ustar / VKC * (log(zldis / z10) + 5.0 * zeta - 5.0 * z10 / obu));
        else
            o.u10_clm = um - (ustar / VKC * (log(obu / z10) + 5.0 - 5.0 * z10 / obu + (5.0 * log(zeta) + zeta - 1.0)));
    }
    o.va = um;
    auto tprof = [&](double zl, double z0) {
        const double zt = zl / obu;
        if (zt < -zetat)
            return VKC / (log(-zetat * obu / z0) - stab2(-zetat) + stab2(z0 / obu) +
                          0.8 * (pow(zetat, -0.333) - pow(-zt, -0.333)));
        else if (zt < 0.0)
            return VKC / (log(zl / z0) - stab2(zt) + stab2(z0 / obu));
        else if (zt <= 1.0)
            return VKC / (log(zl / z0) + 5.0 * zt - 5.0 * z0 / obu);
        return VKC / (log(obu / z0) + 5.0 - 5.0 * z0 / obu + (5.0 * log(zt) + zt - 1.0));
    };
    o.temp1 = tprof(hgt_t - displa, z0h);
    o.temp2 = (hgt_q == hgt_t && z0q == z0h) ? o.temp1 : tprof(hgt_q - displa, z0q);
    o.temp12m = tprof(2.0 + z0h, z0h);
    o.temp22m = (z0q == z0h) ? o.temp12m : tprof(2.0 + z0q, z0q);
    double fmnew;
    const double zc = fmin(zeta, 1.0);
    if (zc < 0.0) {
        const double tmp1 = pow(1.0 - 16.0 * zc, 0.25);
        const double tmp2 = log((1.0 + tmp1 * tmp1) / 2.0);
        const double tmp3 = log((1.0 + tmp1) / 2.0);
        fmnew = 2.0 * tmp3 + tmp2 - 2.0 * atan(tmp1) + 1.5707963;
    } else {
        fmnew = -5.0 * zc;
    }
    fm = (iter == 1) ? fmnew : 0.5 * (fm + fmnew);
    double zeta10 = fmin(10.0 / obu, 1.0);
    if (zeta == 0.0) zeta10 = 0.0;
    double fm10;
    if (zeta10 < 0.0) {
        const double tmp1 = pow(1.0 - 16.0 * zeta10, 0.25);
        const double tmp2 = log((1.0 + tmp1 * tmp1) / 2.0);
        const double tmp3 = log((1.0 + tmp1) / 2.0);
        fm10 = 2.0 * tmp3 + tmp2 - 2.0 * atan(tmp1) + 1.5707963;
    } else {
        fm10 = -5.0 * zeta10;
    }
    const double tmp4 = log(fmax(1.0, hgt_u / 10.0));
    o.u10 = ur - ustar / VKC * (tmp4 - fm + fm10);
}

// BareGroundFluxesMod.F90:558-578
__device__ __forceinline__ double dewpoint(double e, double t) {
    double d;
    if (t < TFRZ) d = 273.86 * log(e / 611.21) / (22.587 - log(e / 611.21));
    else d = 243.04 * log(e / 610.94) / (17.625 - log(e / 610.94));
    return d + TFRZ;
}

__global__ void __launch_bounds__(128)
baregrnd_kernel(ctsmg_baregrnd_io io, int begc, int begp, int nfp, const int32_t* __restrict__ filt, BareArgs A,
                int* __restrict__ last) {
    const int fp = blockIdx.x * blockDim.x + threadIdx.x;
    if (fp >= nfp) return;
    const int p = filt[fp] - begp;
    const int c = io.patch_column[p] - begc;
    const int g = io.patch_gridcell[p] - io.begg;
    const int ldp = io.ldp;
    const double forc_t = io.forc_t[c], forc_pbot = io.forc_pbot[c], forc_q = io.forc_q[c], forc_th = io.forc_th[c];
    const double forc_rho = io.forc_rho[c], thv = io.thv[c], t_grnd = io.t_grnd[c], thm = io.thm[p];
    // (:194-207)
    io.btran[p] = 0.0;
    io.t_veg[p] = forc_t;
    const double cf_bare = forc_pbot / (RGAS * 0.001 * thm) * 1.e06;
    io.rssun[p] = 1.0 / 1.e15 * cf_bare;
    io.rssha[p] = 1.0 / 1.e15 * cf_bare;
#pragma unroll 1
    for (int j = 1; j <= NLEVGRND; ++j) {
        io.rootr[p + (size_t)(j - 1) * ldp] = 0.0;
        io.rresis[p + (size_t)(j - 1) * ldp] = 0.0;
    }
    // (:209-243)
    const double displa = 0.0;
    io.displa[p] = 0.0; io.z0mv[p] = 0.0; io.z0hv[p] = 0.0; io.z0qv[p] = 0.0;
    io.dlrad[p] = 0.0; io.ulrad[p] = 0.0; io.dhsdt_canopy[p] = 0.0; io.eflx_sh_stem[p] = 0.0;
    const double fu = io.forc_u[g], fvv = io.forc_v[g];
    const double ur = fmax(A.wind_min, sqrt(fu * fu + fvv * fvv));
    const double dth = thm - t_grnd;
    const double dqh = forc_q - io.qg[c];
    const double dthv = dth * (1.0 + 0.61 * forc_q) + 0.61 * forc_th * dqh;
    const double zldis = io.forc_hgt_u_patch[p];
    const double z0mg = io.z0mg[c];
    double z0hg = io.z0hg[c], z0qg = io.z0qg[c];
    // MoninObukIni (FrictionVelocityMod.F90:1158-1209)
    double um, obu;
    {
        const double wc = 0.5;
        um = (dthv >= 0.0) ? fmax(ur, 0.1) : sqrt(ur * ur + wc * wc);
        const double rib = GRAV * zldis * dthv / (thv * um * um);
        double zeta;
        if (rib >= 0.0) {
            zeta = rib * log(zldis / z0mg) / (1.0 - 5.0 * fmin(rib, 0.19));
            zeta = fmin(A.zetamaxstable, fmax(zeta, 0.01));
        } else {
            zeta = rib * log(zldis / z0mg);
            zeta = fmax(-100.0, fmin(zeta, -0.01));
        }
        obu = zldis / zeta;
    }
    double hgt_u = io.forc_hgt_u_patch[p], hgt_t = io.forc_hgt_t_patch[p], hgt_q = io.forc_hgt_q_patch[p];
    double fm = 0.0, zeta = 0.0;
    FV o{};
    int num_iter = 0;
    // stability iteration (:245-295)
#pragma unroll 1
    for (int iter = 1; iter <= 3; ++iter) {
        friction_velocity(displa, z0mg, z0hg, z0qg, obu, iter, ur, um, hgt_u, hgt_t, hgt_q, fm, o);
        const double ustar = o.ustar;
        const double tstar = o.temp1 * dth;
        const double qstar = o.temp2 * dqh;
        z0hg = z0mg / exp(A.a_coef * pow(ustar * z0mg / NU_PARAM, A.a_exp));
        z0qg = z0hg;
        hgt_u = io.forc_hgt_u[g] + z0mg + displa;
        hgt_t = io.forc_hgt_t[g] + z0hg + displa;
        hgt_q = io.forc_hgt_q[g] + z0qg + displa;
        const double thvstar = tstar * (1.0 + 0.61 * forc_q) + 0.61 * forc_th * qstar;
        zeta = zldis * VKC * GRAV * thvstar / (ustar * ustar * thv);
        if (zeta >= 0.0) {
            zeta = fmin(A.zetamaxstable, fmax(zeta, 0.01));
            um = fmax(ur, 0.1);
        } else {
            zeta = fmax(-100.0, fmin(zeta, -0.01));
            const double wc = BETA * pow(-GRAV * ustar * thvstar * ZII / thv, 0.333);
            um = sqrt(ur * ur + wc * wc);
        }
        obu = zldis / zeta;
        num_iter = iter;
    }
    io.forc_hgt_u_patch[p] = hgt_u; io.forc_hgt_t_patch[p] = hgt_t; io.forc_hgt_q_patch[p] = hgt_q;
    io.z0mg_patch[p] = z0mg; io.z0hg_patch[p] = z0hg; io.z0qg_patch[p] = z0qg;
    io.zeta[p] = zeta; io.obu[p] = obu; io.num_iter[p] = num_iter; io.fm[p] = fm;
    io.u10_clm[p] = o.u10_clm; io.u10[p] = o.u10; io.va[p] = o.va; io.vds[p] = o.vds; io.fv[p] = o.ustar;
    // fluxes (:297-385)
    const double ustar = o.ustar;
    const double ram = 1.0 / (ustar * ustar / um);
    const double rah = 1.0 / (o.temp1 * ustar);
    const double raw = 1.0 / (o.temp2 * ustar);
    const double raih = forc_rho * CPAIR / rah;
    double forc_qs, forc_esat;
    qsat(forc_t, forc_pbot, forc_qs, forc_esat, nullptr);
    const double forc_e = fmax((forc_q * forc_pbot) / (forc_q + 0.622), 0.01 * forc_esat);
    const double forc_dewpoint = dewpoint(forc_e, t_grnd);
    double raiw = 0.0;
    if (dqh > 0.0) {
        raiw = (t_grnd > forc_dewpoint) ? 0.0 : forc_rho / raw;
    } else if (A.soil_resis_method == 0) {
        raiw = (t_grnd > forc_dewpoint) ? 0.0 : io.soilbeta[c] * forc_rho / raw;
    } else {
        raiw = forc_rho / (raw + io.soilresis[c]);
    }
    io.ram1[p] = ram;
    io.cgrnds[p] = raih;
    io.cgrndl[p] = raiw * io.dqgdT[c];
    io.cgrnd[p] = raih + io.htvp[c] * (raiw * io.dqgdT[c]);
    io.taux[p] = -forc_rho * io.forc_u[g] / ram;
    io.tauy[p] = -forc_rho * io.forc_v[g] / ram;
    const double sh = -raih * dth;
    io.eflx_sh_grnd[p] = sh;
    io.eflx_sh_tot[p] = sh;
    const int snl = io.snl[c], ld = io.ldc;
    io.eflx_sh_snow[p] = -raih * (thm - io.t_soisno[c + (size_t)(snl + 1 - LS) * ld]);
    io.eflx_sh_soil[p] = -raih * (thm - io.t_soisno[c + (size_t)(1 - LS) * ld]);
    io.eflx_sh_h2osfc[p] = -raih * (thm - io.t_h2osfc[c]);
    io.qflx_tran_veg[p] = 0.0;
    io.qflx_evap_veg[p] = 0.0;
    const double ev = -raiw * dqh;
    io.qflx_evap_soi[p] = ev;
    io.qflx_evap_tot[p] = ev;
    io.qflx_ev_snow[p] = -raiw * (forc_q - io.qg_snow[c]);
    io.qflx_ev_soil[p] = -raiw * (forc_q - io.qg_soil[c]);
    io.qflx_ev_h2osfc[p] = -raiw * (forc_q - io.qg_h2osfc[c]);
    const double t2 = thm + o.temp1 * dth * (1.0 / o.temp12m - 1.0 / o.temp1);
    const double q2 = forc_q + o.temp2 * dqh * (1.0 / o.temp22m - 1.0 / o.temp2);
    io.t_ref2m[p] = t2;
    io.q_ref2m[p] = q2;
    double qsat2, e2;
    qsat(t2, forc_pbot, qsat2, e2, nullptr);
    io.rh_ref2m[p] = fmin(100.0, q2 / qsat2 * 100.0);
    io.kbm1[p] = log(z0mg / z0hg);
    atomicMax(&last[c], fp);          // the column takes the values of its last patch in the filter
}

// z0hg_col / z0qg_col = the values of the column's last patch in filter
// order (:381-382), written after every patch has read the old ones.
__global__ void __launch_bounds__(128)
baregrnd_col_kernel(ctsmg_baregrnd_io io, int begc, int begp, int nfp, const int32_t* __restrict__ filt,
                    const int* __restrict__ last) {
    const int fp = blockIdx.x * blockDim.x + threadIdx.x;
    if (fp >= nfp) return;
    const int p = filt[fp] - begp;
    const int c = io.patch_column[p] - begc;
    if (last[c] != fp) return;
    io.z0hg[c] = io.z0hg_patch[p];
    io.z0qg[c] = io.z0qg_patch[p];
}

} // namespace bare

cudaError_t launch_baregrnd(const ctsmg_baregrnd_io& io, int begc, int begp, int nfp, const int32_t* d_filt,
                            const BareArgs& a, int* d_last, int ncol, cudaStream_t s) {
    if (nfp <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(d_last, 0xff, (size_t)ncol * sizeof(int), s);
    if (e != cudaSuccess) return e;
    bare::baregrnd_kernel<<<(nfp + 127) / 128, 128, 0, s>>>(io, begc, begp, nfp, d_filt, a, d_last);
    bare::baregrnd_col_kernel<<<(nfp + 127) / 128, 128, 0, s>>>(io, begc, begp, nfp, d_filt, d_last);
    return cudaGetLastError();
}

} // namespace ctsmg
