/* ctsm_oracle.h -- CPU oracle entry points (test infrastructure only; never
 * linked into the product library).  Each restates a reference routine; see
 * the comments in the .cpp files for the file:line each one follows. */
#ifndef CTSM_ORACLE_H
#define CTSM_ORACLE_H
#include <stdint.h>
#include "ctsm_gpu.h"
#ifdef __cplusplus
extern "C" {
#endif
void oracle_tridiagonal(int n, const double* a, const double* b, const double* c,
                        const double* r, double* u);
int  oracle_dgbsv(int n, int kl, int ku, double* ab, int ldab, int* ipiv, double* b);
int  oracle_soilwater(const ctsmg_bounds* bounds, int num_hydrologyc,
                      const int32_t* filter_hydrologyc, const ctsmg_soilwater_io* io,
                      double e_ice, double dtime);
int  oracle_soiltemperature(const ctsmg_bounds* bounds, int num_nolakec,
                            const int32_t* filter_nolakec, const ctsmg_soiltemp_io* io,
                            double dtime, int snow_method);
int  oracle_last_error(int* idx, int* lev);
void oracle_rootsink(int ncol, int ldp, const int32_t* col_patchi, const int32_t* col_npatches,
                     const double* wtcol, const double* qflx_tran_veg, const double* rootr, double* qflx_rootsoi);
void oracle_set_libm_noise(int ulps, unsigned long long seed);
void oracle_set_canopy_params(const ctsmg_canopy_params* p, const ctsmg_pftcon* pft, int method, int itmax);
void oracle_set_patch_medlyn(const double* slope, const double* intercept);
int  oracle_quadratic(double a, double b, double c, double* r1, double* r2);
void oracle_qsat(double T, double p, double* qs, double* es, double* qsdT);
int  oracle_hydrology(const ctsmg_bounds* b, int n, const int32_t* filt, const ctsmg_hydrology_io* io, int which,
                      const ctsmg_soilhydrology_params* P, double dtime);
int  oracle_baregroundfluxes(const ctsmg_bounds* b, int nump, const int32_t* filtp, const ctsmg_baregrnd_io* io,
                             int soil_resis_method);
int  oracle_soilevap_resis(const ctsmg_bounds* b, int num_nolakec, const int32_t* filter_nolakec,
                           const ctsmg_soilresis_io* io, const ctsmg_soil_resistance_params* par);
int  oracle_dgtsv(int n, double* dl, double* d, double* du, double* b);
int  oracle_soilwater_mf(const ctsmg_bounds* bounds, int num_hydrologyc, const int32_t* filter_hydrologyc,
                         const ctsmg_soilwater_io* io, double e_ice, double dtime,
                         const ctsmg_soilwater_movement_nml* nml, int* err_col);
void oracle_set_soil_water_fractions(const ctsmg_bounds* bounds, int num_hydrologyc, const int32_t* filter_hydrologyc,
                                     const ctsmg_soilwater_io* io);
void oracle_flexcn_fix(const ctsmg_bounds* bounds, int num_hydrologyc, const int32_t* filter_hydrologyc,
                       const ctsmg_soilwater_io* io);
int  oracle_root_moist_stress(const ctsmg_bounds* b, int nump, const int32_t* filtp, const ctsmg_rootmoist_io* io);
int  oracle_soilfluxes(const ctsmg_bounds* b, int num_nolakec, const int32_t* filter_nolakec, int num_nolakep,
                       const int32_t* filter_nolakep, const ctsmg_soilfluxes_io* io, double dtime);
int  oracle_canopyfluxes(const ctsmg_bounds* b, int num_exposedvegp, const int32_t* filter_exposedvegp,
                         const ctsmg_canopy_io* io, double dtime, int* err_index);
#ifdef __cplusplus
}
#endif
#endif
