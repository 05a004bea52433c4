/*
 * ctsm_gpu.h -- C-ABI of the GB300 (sm_103a) column biogeophysics library.
 *
 * This is the boundary a CTSM host binds through ISO_C_BINDING in place of the
 * column-parallel calls of the land driver:
 *
 *   SoilWater        src/biogeophys/SoilWaterMovementMod.F90:240-243
 *                    (called from src/biogeophys/HydrologyNoDrainageMod.F90:346)
 *   SoilTemperature  src/biogeophys/SoilTemperatureMod.F90:92-95
 *                    (called from src/main/clm_driver.F90:900)
 *   CanopyFluxes     src/biogeophys/CanopyFluxesMod.F90:191-198
 *                    (called from src/main/clm_driver.F90:766)
 *   SoilFluxes       src/biogeophys/SoilFluxesMod.F90:36-41
 *                    (called from src/main/clm_driver.F90:921)
 *
 * Array convention (identical to the Fortran storage of the derived types):
 *   every 2-D column field is declared (begc:endc, lb:ub) in Fortran, so
 *   element (c, j) lives at  base[(c - begc) + (j - lb) * ldc].
 *   The Fortran side passes  c_loc(inst%field(begc, lb))  and  ldc = endc-begc+1.
 *   Patch fields use (p - begp) + (j - lb) * ldp the same way.
 *   Lower bounds used below (nlevsno = 12, nlevsoi = 20, nlevgrnd = 25):
 *     [SS] (c, -nlevsno+1 : nlevgrnd)   snow + soil levels (t_soisno, dz, ...)
 *     [ZI] (c, -nlevsno   : nlevgrnd)   interfaces (col%zi)
 *     [G ] (c, 1 : nlevgrnd)            soil + bedrock levels (watsat, ...)
 *     [S ] (c, 1 : nlevsoi)             hydrologically active levels
 *     [SN] (c, -nlevsno+1 : 0)          snow levels only
 *     [PL] (p, -nlevsno+1 : 1)          patch snow levels + top soil (sabg_lyr)
 *     [PG] (p, 1 : nlevgrnd)            patch soil + bedrock levels (rootfr, rootr)
 *   Filters are the reference's 1-based global indices (filter_hydrologyc(fc)
 *   holds c with begc <= c <= endc).
 *
 * Error behaviour: the reference calls endrun (abort).  Every entry point here
 * returns 0 on success or a CTSMG_E* code; ctsmg_last_error() returns the
 * message and ctsmg_last_error_index() the (column or patch, level) context, so
 * the Fortran wrapper can call endrun(subgrid_index=..., subgrid_level=...)
 * exactly where the reference would.
 *
 * All entry points are host-pointer, copy-in / copy-out calls that may be made
 * concurrently from several host threads (one per clump, as the
 * !$OMP PARALLEL DO of src/main/clm_driver.F90:525 does): each calling thread
 * gets its own CUDA stream and device workspace.
 */
#ifndef CTSM_GPU_H
#define CTSM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- sizes */
#define CTSMG_NLEVSNO   12
#define CTSMG_NLEVSOI   20
#define CTSMG_NLEVGRND  25
#define CTSMG_NLEV_SS   (CTSMG_NLEVSNO + CTSMG_NLEVGRND)      /* 37 */
#define CTSMG_NLEV_ZI   (CTSMG_NLEVSNO + CTSMG_NLEVGRND + 1)  /* 38 */

/* ---------------------------------------------------------------- status */
#define CTSMG_OK               0
#define CTSMG_E_ARG            1   /* bad argument / size (host check)            */
#define CTSMG_E_CUDA           2   /* CUDA runtime error                          */
#define CTSMG_E_NOT_INIT       3   /* ctsmg_init not called                       */
#define CTSMG_E_SINGULAR       4   /* band solve: dgbsv info /= 0
                                      (src/biogeophys/BandDiagonalMod.F90:200-213) */
#define CTSMG_E_DISCRIMINANT   5   /* quadratic: negative discriminant
                                      (src/utils/quadraticMod.F90:50-58)          */
#define CTSMG_E_NOT_BRACKETED  6   /* brent: root not bracketed
                                      (src/biogeophys/PhotosynthesisMod.F90:2412-2415) */
#define CTSMG_E_FORCING_HEIGHT 7   /* forcing height below canopy
                                      (src/biogeophys/CanopyFluxesMod.F90:997-1002) */
#define CTSMG_E_BALANCE        8   /* water / energy balance above stop threshold
                                      (src/biogeophys/BalanceCheckMod.F90:626,1111) */
#define CTSMG_E_TIMEOUT        9   /* a bounded device wait ran out                */
#define CTSMG_E_UNSUPPORTED   10   /* option not built (e.g. urban columns)        */

/* ---------------------------------------------------------------- bounds */
/* src/main/decompMod.F90:58-70 (bounds_type: begg/endg, begl/endl, begc/endc, begp/endp) */
typedef struct {
    int32_t begc, endc;
    int32_t begp, endp;
} ctsmg_bounds;

/* ---------------------------------------------------------------- options */
/* Namelist values the reference keeps as module state:
 *   soilwater_movement_method, lower_boundary_condition
 *     (src/biogeophys/SoilWaterMovementMod.F90:67-78, defaults
 *      bld/namelist_files/namelist_defaults_ctsm.xml:471-477)
 *   snow_thermal_cond_method (src/main/clm_varctl.F90; default Jordan1991,
 *      Sturm1997 for clm6_0: namelist_defaults_ctsm.xml:555-556)
 *   itmax_canopy_fluxes (src/biogeophys/CanopyFluxesMod.F90:83)             */
typedef struct {
    int32_t soilwater_movement_method;   /* 0 = Zeng-Decker 2009, 1 = moisture form */
    int32_t snow_thermal_cond_method;    /* 0 = Jordan1991, 1 = Sturm1997           */
    int32_t itmax_canopy_fluxes;         /* 40                                      */
    int32_t stomatalcond_method;         /* 0 = Ball-Berry 1987, 1 = Medlyn 2011    */
    int32_t nlevsno, nlevsoi, nlevgrnd;  /* must equal the CTSMG_NLEV* constants    */
} ctsmg_options;

/* Scalar parameters read from the parameter file by readParams:
 *   e_ice  src/biogeophys/SoilWaterMovementMod.F90:89-106                       */
typedef struct {
    double e_ice;
} ctsmg_soilwater_params;

/* ---------------------------------------------------------------- SoilWater */
/* Components of the derived types that soilwater_zengdecker2009 reads and
 * writes (src/biogeophys/SoilWaterMovementMod.F90:537-566).                  */
typedef struct {
    int32_t ldc;                 /* leading dimension of every column array       */
    /* col (ColumnType) */
    const double* z;             /* [SS] layer depth (m)                          */
    const double* zi;            /* [ZI] interface depth (m)                      */
    const double* dz;            /* [SS] layer thickness (m)                      */
    /* soilhydrology_inst */
    const double* zwt;           /* (c)  water table depth (m)                    */
    double*       qcharge;       /* (c)  out: aquifer recharge (mm/s)             */
    double*       icefrac;       /* [G]  out: ice fraction, levels 1..nlevsoi     */
    double*       qin;           /* [S]  out: flux into layer (mm/s)              */
    double*       qout;          /* [S]  out: flux out of layer (mm/s)            */
    /* soilstate_inst */
    const double* smpmin;        /* (c)  minimum soil potential (mm)              */
    const double* watsat;        /* [G]  porosity                                 */
    const double* hksat;         /* [G]  saturated conductivity (mm/s)            */
    const double* bsw;           /* [G]  Clapp-Hornberger b                       */
    const double* sucsat;        /* [G]  saturated suction (mm)                   */
    double*       smp_l;         /* [G]  out: matric potential (mm)               */
    double*       hk_l;          /* [G]  out: conductivity (mm/s)                 */
    /* waterstatebulk_inst */
    const double* h2osoi_ice;    /* [SS] ice (kg/m2)                              */
    double*       h2osoi_liq;    /* [SS] inout: liquid (kg/m2)                    */
    const double* h2osoi_vol;    /* [G]  volumetric water (previous step)         */
    /* waterfluxbulk_inst */
    double*       qflx_deficit;  /* (c)  out: deficit to keep liquid >= 0 (mm/s)  */
    const double* qflx_infl;     /* (c)  infiltration (mm/s)                      */
    const double* qflx_rootsoi;  /* [S]  root water sink (mm/s)                   */
    /* temperature_inst */
    const double* t_soisno;      /* [SS] soil temperature (K)                     */
    /* Read or written only by the moisture form (soilwater_movement_method = 1,
     * SoilWaterMovementMod.F90:1172-1186) or by the use_flexibleCN
     * negative-liquid fix (:331-368); NULL otherwise.  With the moisture form
     * icefrac is an INPUT (set by SetSoilWaterFractions,
     * SoilHydrologyMod.F90:200-245, before SoilWater) and h2osoi_vol,
     * qflx_deficit and t_soisno are not used.                                */
    const int32_t* nbedrock;     /* (c)  index of the bottom soil layer (nlayers) */
    const double* eff_porosity;  /* [G]  porosity - ice volume (over-saturation)  */
    double*       num_substeps;  /* (c)  out: adaptive sub-steps taken (trials)   */
    double*       wa;            /* (c)  inout: aquifer water, flexibleCN fix (mm)*/
} ctsmg_soilwater_io;

/* Namelist soilwater_movement_inparm (init_soilwater_movement,
 * src/biogeophys/SoilWaterMovementMod.F90:108-216) and use_flexibleCN
 * (clm_varctl).  Boundary conditions: 0 bc_head, 1 bc_flux, 2 bc_zero_flux,
 * 3 bc_waterTable, 4 bc_aquifer (:47-51).  flux_calculation = 42 is the
 * reference's `expensive` error estimate (:1321-1336), any other value the
 * inexpensive one.  The same consistency checks as the reference apply
 * (ZD09 needs bc_aquifer; use_bedrock needs bc_zero_flux), and the forms the
 * reference cannot complete are refused: bc_head at either boundary (the
 * boundary water contents are never set, and the lower one ends in endrun),
 * bc_aquifer with the moisture form (:1764-1861 has no case for it).       */
typedef struct {
    int32_t soilwater_movement_method;   /* 0 ZD09, 1 moisture form              */
    int32_t upper_boundary_condition;    /* 1                                     */
    int32_t lower_boundary_condition;    /* 4 with ZD09, 2 with the moisture form */
    int32_t flux_calculation;            /* 1 inexpensive, 42 expensive           */
    int32_t use_flexibleCN;              /* 0 / 1                                 */
    int32_t use_bedrock;                 /* 1 (namelist_defaults_ctsm.xml:259)   */
    double  dtmin;                       /* 60 s                                  */
    double  verySmall;                   /* 1e-8 s                                */
    double  xTolerUpper;                 /* 1e-1: halve the sub-step above        */
    double  xTolerLower;                 /* 1e-2: double the sub-step below       */
} ctsmg_soilwater_movement_nml;

/* ---------------------------------------------------------------- SoilTemperature */
/* Components read and written by SoilTemperature and the routines it calls
 * (SoilThermProp, ComputeGroundHeatFluxAndDeriv, ComputeHeatDiffFluxAndFactor,
 *  SetRHSVec*, SetMatrix*, BandDiagonal, PhaseChangeH2osfc, Phasechange):
 *  src/biogeophys/SoilTemperatureMod.F90:184-256, 661-688, 960-981, 1191-1219,
 *  1603-1653.  Natural-vegetation (soil/crop) columns only; urban, lake,
 *  glacier, wetland and excess-ice branches are not built.                    */
typedef struct {
    int32_t ldc, ldp;
    /* col (ColumnType) and patch (PatchType) */
    const int32_t* snl;          /* (c)  number of snow layers (<= 0)             */
    const int32_t* nbedrock;     /* (c)  index of deepest soil layer              */
    const double*  z;            /* [SS] */
    const double*  zi;           /* [ZI] */
    const double*  dz;           /* [SS] */
    const int32_t* col_patchi;   /* (c)  first patch of column (global index)     */
    const int32_t* col_npatches; /* (c)  patches in column                        */
    const double*  wtcol;        /* (p)  patch weight on column                   */
    const int32_t* frac_veg_nosno; /* (p) 0/1                                     */
    /* atm2lnd / solarabs (patch) */
    const double* forc_lwrad;    /* (c)  downward longwave (W/m2)                 */
    const double* sabg;          /* (p) */
    const double* sabg_soil;     /* (p) */
    const double* sabg_snow;     /* (p) */
    const double* sabg_lyr;      /* [PL] */
    double*       sabg_chk;      /* (p)  out */
    /* energyflux_inst (patch inputs, patch/col outputs) */
    const double* htvp;          /* (c) */
    const double* cgrnd;         /* (p) */
    const double* dlrad;         /* (p) */
    const double* eflx_sh_grnd;  /* (p) */
    const double* eflx_sh_snow;  /* (p) */
    const double* eflx_sh_soil;  /* (p) */
    const double* eflx_sh_h2osfc;/* (p) */
    const double* qflx_evap_soi; /* (p) */
    const double* qflx_ev_snow;  /* (p) */
    const double* qflx_ev_soil;  /* (p) */
    const double* qflx_ev_h2osfc;/* (p) */
    const double* eflx_bot;      /* (c) */
    double*       eflx_gnet;     /* (p)  out */
    double*       dgnetdT;       /* (p)  out */
    double*       eflx_fgr12;    /* (c)  out */
    double*       eflx_fgr;      /* [G]  out */
    double*       eflx_snomelt;  /* (c)  out */
    double*       eflx_h2osfc_to_snow; /* (c) out */
    /* temperature_inst */
    const double* emg;           /* (c) */
    double*       t_soisno;      /* [SS] inout */
    double*       t_h2osfc;      /* (c)  inout */
    double*       t_grnd;        /* (c)  inout (input: previous ground T)         */
    double*       fact;          /* [SS] out */
    double*       c_h2osfc;      /* (c)  out */
    double*       xmf;           /* (c)  out */
    double*       xmf_h2osfc;    /* (c)  out */
    int32_t*      imelt;         /* [SS] out */
    /* soilstate_inst */
    const double* watsat;        /* [G] */
    const double* bsw;           /* [G] */
    const double* sucsat;        /* [G] */
    const double* tkmg;          /* [G] */
    const double* tkdry;         /* [G] */
    const double* csol;          /* [G] */
    double*       thk;           /* [SS] out */
    /* waterstatebulk / waterdiagnosticbulk / waterfluxbulk */
    double*       h2osoi_liq;    /* [SS] inout */
    double*       h2osoi_ice;    /* [SS] inout */
    double*       h2osfc;        /* (c)  inout */
    double*       h2osno_no_layers; /* (c) inout */
    double*       int_snow;      /* (c)  inout */
    double*       snow_depth;    /* (c)  inout */
    double*       snomelt_accum; /* (c)  inout */
    const double* frac_sno_eff;  /* (c) */
    const double* frac_h2osfc;   /* (c) */
    double*       bw;            /* [SN] out */
    double*       qflx_snomelt;  /* (c)  out */
    double*       qflx_snofrz;   /* (c)  out */
    double*       qflx_snow_drain; /* (c) out */
    double*       qflx_snomelt_lyr; /* [SN] out */
    double*       qflx_snofrz_lyr;  /* [SN] out */
    double*       qflx_h2osfc_to_ice; /* (c) out */
} ctsmg_soiltemp_io;

/* ---------------------------------------------------------------- CanopyFluxes */
/* Scalar parameters of CanopyFluxes (readParams, src/biogeophys/CanopyFluxesMod.F90:159-188),
 * FrictionVelocity (zetamaxstable, FrictionVelocityMod.F90:136,511) and
 * Photosynthesis (params_type, src/biogeophys/PhotosynthesisMod.F90:92-140;
 * module constants :85-89).  Values of the parameter file are not shipped
 * with the reference; ctsm_gb300/canopy_inputs.py records the ones used.   */
typedef struct {
    /* CanopyFluxes */
    double lai_dl, z_dl, a_coef, a_exp, csoilc, cv, wind_min, zetamaxstable;
    /* Photosynthesis */
    double kc25_coef, ko25_coef, cp25_yr2000, kcha, koha, cpha;
    double vcmaxha, jmaxha, tpuha, lmrha, vcmaxhd, jmaxhd, tpuhd, lmrhd, lmrse;
    double vcmaxse_sf, jmaxse_sf, tpuse_sf, jmax25top_sf;
    double fnr, act25, theta_psii, theta_ip, tpu25ratio, kp25ratio, fnps, leaf_mr_vcm;
    int32_t light_inhibit;                 /* 1 = respiration x 0.67 in light (:1828-1830) */
} ctsmg_canopy_params;

/* pftcon arrays used on the path, indexed by patch%itype (0 .. npft-1)
 * (src/main/pftconMod.F90): c3psn, slatop, leafcn, flnr, fnitr, dleaf,
 * medlynslope, medlynintercept, mbbopt, Photosynthesis' theta_cj, and the
 * soil water potentials at full stomatal opening / closure smpso, smpsc (mm)
 * of the root moisture stress.                                            */
#define CTSMG_MAX_PFT 80
typedef struct {
    int32_t npft;
    double c3psn[CTSMG_MAX_PFT], slatop[CTSMG_MAX_PFT], leafcn[CTSMG_MAX_PFT];
    double flnr[CTSMG_MAX_PFT], fnitr[CTSMG_MAX_PFT], dleaf[CTSMG_MAX_PFT];
    double medlynslope[CTSMG_MAX_PFT], medlynintercept[CTSMG_MAX_PFT], theta_cj[CTSMG_MAX_PFT];
    double mbbopt[CTSMG_MAX_PFT];
    double smpso[CTSMG_MAX_PFT], smpsc[CTSMG_MAX_PFT];
} ctsmg_pftcon;

/* Components CanopyFluxes reads and writes on the natural-vegetation,
 * satellite-phenology path (associate block src/biogeophys/CanopyFluxesMod.F90:420-640):
 * ZengWang2007 roughness, no biomass heat storage, no FATES / LUNA / hydraulic
 * stress / ozone, soil resistance by sl14 (soilresis given).  Patch arrays
 * (p) use ldp, column arrays (c) ldc, gridcell arrays (g) ldg; patch_column
 * and patch_gridcell hold the reference's global indices (patch%column,
 * patch%gridcell).  btran comes from calc_root_moist_stress, the sun/shade
 * PAR, lai and vcmaxcint from SurfaceRadiation / SurfaceAlbedo.           */
typedef struct {
    int32_t ldp, ldc, ldg, begg;
    /* patch (PatchType) */
    const int32_t* itype; const int32_t* patch_column; const int32_t* patch_gridcell;
    /* gridcell forcing (atm2lnd_inst) */
    const double *forc_u, *forc_v, *forc_hgt_u, *forc_hgt_t, *forc_hgt_q, *forc_pco2, *forc_po2, *dayl, *max_dayl;
    /* column inputs */
    const int32_t* snl;
    const double *forc_pbot, *forc_th, *forc_q, *forc_rho, *forc_lwrad, *thv, *t_grnd, *qg, *qg_snow, *qg_soil,
        *qg_h2osfc, *dqgdT, *emg, *htvp, *z0mg, *snow_depth, *frac_sno_eff, *frac_h2osfc, *soilresis, *t_h2osfc;
    const double* t_soisno;                /* [SS] */
    /* patch inputs */
    const int32_t* frac_veg_nosno;
    const double *elai, *esai, *htop, *emv, *fwet, *fdry, *laisun, *laisha, *btran, *sabv, *thm, *t_a10,
        *parsun_z, *parsha_z, *vcmaxcintsun, *vcmaxcintsha;
    /* patch in/out */
    double *displa, *z0mv, *t_veg, *liqcan, *snocan, *cgrnds, *cgrndl;
    /* patch outputs */
    double *z0hv, *z0qv, *forc_hgt_u_patch, *forc_hgt_t_patch, *forc_hgt_q_patch, *taf, *qaf, *ustar, *um, *obu,
        *zeta, *ram1, *rah1, *raw1, *rah2, *raw2, *rb1, *uaf, *vpd, *rhaf;
    double *eflx_sh_veg, *qflx_evap_veg, *qflx_tran_veg, *eflx_sh_grnd, *eflx_sh_snow, *eflx_sh_soil,
        *eflx_sh_h2osfc, *qflx_evap_soi, *qflx_ev_snow, *qflx_ev_soil, *qflx_ev_h2osfc;
    double *t_ref2m, *q_ref2m, *rh_ref2m, *vpd_ref2m, *dlrad, *ulrad, *t_skin, *cgrnd, *taux, *tauy, *err_canopy;
    double *rssun, *rssha, *psnsun, *psnsha, *lmrsun, *lmrsha, *cisun, *cisha, *gs_mol_sun, *gs_mol_sha,
        *rh_leaf, *vpd_can, *u10_clm, *u10, *fv, *vds, *fm;
    int32_t* num_iter;
} ctsmg_canopy_io;

/* ---------------------------------------------------------------- lifecycle */
/* Replaces the namelist reads init_soilwater_movement
 * (src/biogeophys/SoilWaterMovementMod.F90:110-216), CanopyFluxesReadNML
 * (src/biogeophys/CanopyFluxesMod.F90:92-157) and Photosynthesis ReadNML
 * (src/biogeophys/PhotosynthesisMod.F90:939-1015).  Selects device 0.       */
int32_t ctsmg_init(const ctsmg_options* opt);

/* Replaces init_soilwater_movement (SoilWaterMovementMod.F90:108-216).
 * ctsmg_init sets the reference's defaults for its soilwater_movement_method;
 * this call replaces all of them.                                          */
int32_t ctsmg_set_soilwater_movement(const ctsmg_soilwater_movement_nml* nml);

/* Replaces readParams of SoilWaterMovementMod (src/biogeophys/SoilWaterMovementMod.F90:89-106). */
int32_t ctsmg_set_soilwater_params(const ctsmg_soilwater_params* p);

/* Replaces readParams of CanopyFluxesMod / PhotosynthesisMod and the pftcon
 * reads (src/biogeophys/CanopyFluxesMod.F90:159-188, PhotosynthesisMod.F90:809-912). */
int32_t ctsmg_set_canopy_params(const ctsmg_canopy_params* p, const ctsmg_pftcon* pft);

/* Frees every device buffer and stream. */
int32_t ctsmg_finalize(void);

/* Message and (index, level) context of the last error on the calling thread. */
const char* ctsmg_last_error(void);
int32_t ctsmg_last_error_index(int32_t* index, int32_t* level);

/* ---------------------------------------------------------------- drop-in calls */
/* SoilWater, Zeng-Decker 2009 form:
 *   src/biogeophys/SoilWaterMovementMod.F90:240-243 (dispatch :297-329) and
 *   soilwater_zengdecker2009 :414-972.  num_urbanc/filter_urbanc are unused by
 *   that form and omitted. */
int32_t ctsmg_soilwater(const ctsmg_bounds* bounds,
                        int32_t num_hydrologyc, const int32_t* filter_hydrologyc,
                        const ctsmg_soilwater_io* io, double dtime);

/* SoilTemperature: src/biogeophys/SoilTemperatureMod.F90:92-508 (urban
 * filters omitted: urban columns are not built). */
int32_t ctsmg_soiltemperature(const ctsmg_bounds* bounds,
                              int32_t num_nolakec, const int32_t* filter_nolakec,
                              const ctsmg_soiltemp_io* io, double dtime);

/* CanopyFluxes: src/biogeophys/CanopyFluxesMod.F90:191-1768 with
 * FrictionVelocity / MoninObukIni (FrictionVelocityMod.F90:754-1209), QSat
 * (QSatMod.F90:61-127) and Photosynthesis sun + shade with hybrid / brent /
 * ci_func / quadratic (PhotosynthesisMod.F90:1243-2701, quadraticMod.F90:17-74),
 * over the exposed-vegetation patch filter (1-based patch indices).       */
int32_t ctsmg_canopyfluxes(const ctsmg_bounds* bounds, int32_t num_exposedvegp,
                           const int32_t* filter_exposedvegp, const ctsmg_canopy_io* io, double dtime);

/* ---------------------------------------------------------------- root moisture stress */
/* The first part of CanopyFluxes' setup (src/biogeophys/CanopyFluxesMod.F90:
 * 709, 833-895): effective porosity and volumetric liquid water of the soil
 * levels (SoilMoistStressMod.F90:70-114, 171-217) and the default root
 * moisture stress (calc_root_moist_stress_clm45default, :312-435, with the
 * Clapp-Hornberger suction): btran and the effective root fractions rootr
 * that the root water sink uses.  [PG] = (p, 1:nlevgrnd).  The reference runs
 * it inside CanopyFluxes; here it is its own call, made right before
 * ctsmg_canopyfluxes, which takes btran as an input.                      */
typedef struct {
    int32_t ldc, ldp;
    const double*  h2osoi_liq;       /* [SS]                                    */
    const double*  h2osoi_ice;       /* [SS]                                    */
    const double*  dz;               /* [SS]                                    */
    const double*  t_soisno;         /* [SS]                                    */
    const double*  watsat;           /* [G]                                     */
    const double*  sucsat;           /* [G]                                     */
    const double*  bsw;              /* [G]                                     */
    double*        eff_porosity;     /* [G]  out                                */
    double*        h2osoi_liqvol;    /* [G]  out                                */
    const int32_t* patch_column;     /* (p)  1-based (begc)                     */
    const int32_t* itype;            /* (p)                                     */
    const double*  rootfr;           /* [PG] root fraction                      */
    double*        btran;            /* (p)  out: transpiration wetness factor  */
    double*        rootr;            /* [PG] out: effective root fraction       */
    double*        rresis;           /* [PG] inout: root soil water stress      */
} ctsmg_rootmoist_io;

/* calc_root_moist_stress for the exposed-vegetation patch filter (pftcon
 * smpso / smpsc from ctsmg_set_canopy_params).                             */
int32_t ctsmg_root_moist_stress(const ctsmg_bounds* bounds, int32_t num_exposedvegp,
                                const int32_t* filter_exposedvegp, const ctsmg_rootmoist_io* io);

/* SetSoilWaterFractions (src/biogeophys/SoilHydrologyMod.F90:236-249, called
 * at src/biogeophys/HydrologyNoDrainageMod.F90:302 before SoilWater), without
 * excess ice: eff_porosity and icefrac on levels 1..nlevsoi from dz,
 * h2osoi_ice and watsat of the SoilWater io struct.                      */
int32_t ctsmg_set_soil_water_fractions(const ctsmg_bounds* bounds, int32_t num_hydrologyc,
                                       const int32_t* filter_hydrologyc, const ctsmg_soilwater_io* io);

/* ---------------------------------------------------------------- root water sink */
/* Components of Compute_EffecRootFrac_And_VertTranSink_Default
 * (src/biogeophys/SoilWaterPlantSinkMod.F90:332-420), the transpiration sink
 * SoilWater's Zeng-Decker and moisture forms take (called from
 * src/biogeophys/SoilWaterPlantSinkMod.F90:55-120 before SoilWater).  Every
 * patch of a filtered column is active (patch%active).                    */
typedef struct {
    int32_t ldc, ldp;
    const int32_t* col_patchi;        /* (c)  first patch of the column (global)     */
    const int32_t* col_npatches;      /* (c)                                        */
    const double*  wtcol;             /* (p)  patch weight on the column             */
    const double*  qflx_tran_veg;     /* (p)  patch transpiration (mm/s)             */
    const double*  qflx_tran_veg_col; /* (c)  column transpiration (mm/s); NULL = the
                                         wtcol-weighted sum of the patches'          */
    const double*  rootr;             /* [PG] patch effective root fraction (levels
                                         1..nlevsoi read)                           */
    double*        rootr_col;         /* [G]  out: column effective root fraction,
                                         levels 1..nlevsoi                          */
    double*        qflx_rootsoi;      /* [S]  out: soil water sink (mm/s)            */
} ctsmg_rootsink_io;

int32_t ctsmg_root_sink(const ctsmg_bounds* bounds, int32_t num_filterc, const int32_t* filterc,
                        const ctsmg_rootsink_io* io);

/* ------------------------------------------------------- hydrology neighbours of SoilWater */
/* The water-table and drainage routines of the default (no aquifer layer)
 * hydrology around SoilWater, for natural soil columns outside hillslopes
 * (src/biogeophys/HydrologyNoDrainageMod.F90:302-372,
 *  src/biogeophys/HydrologyDrainageMod.F90:132-146):
 *   SaturatedExcessRunoff, TOPMODEL fsat (SaturatedExcessRunoffMod.F90:200-360)
 *   PerchedWaterTable      (SoilHydrologyMod.F90:1525-1641)
 *   ThetaBasedWaterTable   (SoilHydrologyMod.F90:1933-2025)
 *   PerchedLateralFlow     (SoilHydrologyMod.F90:1645-1929)
 *   SubsurfaceLateralFlow  (SoilHydrologyMod.F90:2029-2565)
 * The parameter-file values are aq_sp_yield_min, n_baseflow, baseflow_scalar,
 * perched_baseflow_scalar, e_ice (SoilHydrologyMod.F90:61-67, 174-199) and
 * fff (SaturatedExcessRunoffMod.F90:56, 194).  The hillslope branches, the
 * urban columns and the volumetric discharge diagnostics are not built.   */
typedef struct {
    double aq_sp_yield_min, n_baseflow, baseflow_scalar, perched_baseflow_scalar, e_ice, fff;
    /* surface water (SurfaceWaterMod.F90:42-43, 68-70) and soilhydrology_inst%h2osfcflag (1) */
    double pc, mu;
    int32_t h2osfcflag;
} ctsmg_soilhydrology_params;

typedef struct {
    int32_t ldc;
    const int32_t* nbedrock;          /* (c)                                        */
    const double* z;                  /* [SS]                                       */
    const double* zi;                 /* [ZI]                                       */
    const double* dz;                 /* [SS]                                       */
    const double* t_soisno;           /* [SS]                                       */
    double* h2osoi_liq;               /* [SS] inout                                 */
    double* h2osoi_ice;               /* [SS] inout                                 */
    double* h2osoi_vol;               /* [G]  inout (the water tables refresh it)   */
    double* h2osfc;                   /* (c)  inout (mm)                            */
    double* zwt;                      /* (c)  inout: water table depth (m)          */
    double* zwt_perched;              /* (c)  inout: perched water table depth (m)  */
    double* frost_table;              /* (c)  inout: frost table depth (m)          */
    double* icefrac;                  /* [G]  out                                   */
    const double* watsat;             /* [G]                                        */
    const double* hksat;              /* [G]  (mm/s)                                */
    const double* bsw;                /* [G]                                        */
    const double* sucsat;             /* [G]  (mm)                                  */
    const double* eff_porosity;       /* [G]                                        */
    const double* topo_slope;         /* (c)  (degrees)                             */
    const double* wtfact;             /* (c)  maximum saturated fraction            */
    const double* qflx_rain_plus_snomelt; /* (c) (mm/s)                             */
    const double* qflx_snwcp_liq;     /* (c)  (mm/s)                                */
    double* fsat;                     /* (c)  out: saturated fraction               */
    double* fcov;                     /* (c)  out                                   */
    double* qflx_sat_excess_surf;     /* (c)  out (mm/s)                            */
    double* qflx_drain_perched;       /* (c)  out (mm/s)                            */
    double* qflx_latflow_out;         /* (c)  out (mm/s)                            */
    double* qflx_latflow_in;          /* (c)  out (mm/s)                            */
    double* qflx_rsub_sat;            /* (c)  out (mm/s)                            */
    double* qflx_drain;               /* (c)  out (mm/s)                            */
    double* qflx_qrgwl;               /* (c)  out (mm/s)                            */
    double* qflx_ice_runoff_xs;       /* (c)  out (mm/s)                            */
    /* the infiltration chain before SoilWater (SetQflxInputs,
     * InfiltrationExcessRunoff with the hksat qinmax, RouteInfiltrationExcess,
     * UpdateH2osfc, Infiltration)                                          */
    const int32_t* snl;               /* (c)                                        */
    const double* frac_sno_eff;       /* (c)                                        */
    const double* frac_h2osfc;        /* (c)                                        */
    const double* frac_h2osfc_nosnow; /* (c)                                        */
    const double* h2osfc_thresh;      /* (c)  (mm)                                  */
    const double* qflx_snow_h2osfc;   /* (c)  (mm/s)                                */
    const double* qflx_floodc;        /* (c)  (mm/s)                                */
    /* the column averages (qflx_*_col), distinct from the patch fluxes of
     * SoilTemperature / SoilFluxes with the same base name                  */
    const double* qflx_ev_soil_col;   /* (c)  (mm/s)                                */
    const double* qflx_liqevap_from_top_layer_col; /* (c) (mm/s)                    */
    const double* qflx_ev_h2osfc_col; /* (c)  (mm/s)                                */
    double* qflx_top_soil;            /* (c)  out                                   */
    double* qflx_in_soil;             /* (c)  out                                   */
    double* qflx_top_soil_to_h2osfc;  /* (c)  out                                   */
    double* qinmax;                   /* (c)  out                                   */
    double* qflx_infl_excess;         /* (c)  out                                   */
    double* qflx_in_soil_limited;     /* (c)  out                                   */
    double* qflx_in_h2osfc;           /* (c)  out                                   */
    double* qflx_infl_excess_surf;    /* (c)  out                                   */
    double* qflx_h2osfc_surf;         /* (c)  out                                   */
    double* qflx_h2osfc_drain;        /* (c)  out                                   */
    double* qflx_infl;                /* (c)  out: infiltration, SoilWater's input  */
    /* the aquifer-layer path (WaterTable, Drainage; SoilWater's ZD09 form)  */
    double* wa;                       /* (c)  inout: aquifer water (mm)             */
    const double* qcharge;            /* (c)  aquifer recharge from SoilWater (mm/s)*/
    const double* hkdepth;            /* (c)  decay factor depth (m)                */
} ctsmg_hydrology_io;

/* readParams of SoilHydrologyMod and SaturatedExcessRunoffMod. */
int32_t ctsmg_set_soilhydrology_params(const ctsmg_soilhydrology_params* p);
/* One entry per reference routine, over filter_hydrologyc (1-based). */
/* SetQflxInputs (SoilHydrologyMod.F90:298-366), InfiltrationExcessRunoff
 * (InfiltrationExcessRunoffMod.F90:196-304), RouteInfiltrationExcess
 * (SoilHydrologyMod.F90:369-423), UpdateH2osfc (SurfaceWaterMod.F90:345-556)
 * and Infiltration (SoilHydrologyMod.F90:426-457), in this order, after
 * SaturatedExcessRunoff.                                                  */
int32_t ctsmg_infiltration_chain(const ctsmg_bounds* bounds, int32_t num_hydrologyc,
                                 const int32_t* filter_hydrologyc, const ctsmg_hydrology_io* io, double dtime);
/* The aquifer-layer path that follows the Zeng-Decker SoilWater
 * (use_aquifer_layer, HydrologyNoDrainageMod.F90:356-359,
 * HydrologyDrainageMod.F90:132-137): WaterTable (SoilHydrologyMod.F90:607-861)
 * and Drainage (:864-1410, the non-VIC branch).                          */
int32_t ctsmg_water_table(const ctsmg_bounds* bounds, int32_t num_hydrologyc, const int32_t* filter_hydrologyc,
                          const ctsmg_hydrology_io* io, double dtime);
int32_t ctsmg_drainage(const ctsmg_bounds* bounds, int32_t num_hydrologyc, const int32_t* filter_hydrologyc,
                       const ctsmg_hydrology_io* io, double dtime);
int32_t ctsmg_saturated_excess_runoff(const ctsmg_bounds* bounds, int32_t num_hydrologyc,
                                      const int32_t* filter_hydrologyc, const ctsmg_hydrology_io* io);
int32_t ctsmg_perched_water_table(const ctsmg_bounds* bounds, int32_t num_hydrologyc,
                                  const int32_t* filter_hydrologyc, const ctsmg_hydrology_io* io);
int32_t ctsmg_theta_based_water_table(const ctsmg_bounds* bounds, int32_t num_hydrologyc,
                                      const int32_t* filter_hydrologyc, const ctsmg_hydrology_io* io);
int32_t ctsmg_perched_lateral_flow(const ctsmg_bounds* bounds, int32_t num_hydrologyc,
                                   const int32_t* filter_hydrologyc, const ctsmg_hydrology_io* io, double dtime);
int32_t ctsmg_subsurface_lateral_flow(const ctsmg_bounds* bounds, int32_t num_hydrologyc,
                                      const int32_t* filter_hydrologyc, const ctsmg_hydrology_io* io, double dtime);

/* ------------------------------------------------------------ BareGroundFluxes */
/* Components BareGroundFluxes reads and writes for the patches without
 * exposed vegetation (src/biogeophys/BareGroundFluxesMod.F90:73-545;
 * called at clm_driver.F90:718): three Monin-Obukhov iterations with
 * FrictionVelocity, ZengWang2007 roughness, the ground evaporation
 * resistance of the soil resistance method in force (sl_14: soilresis,
 * leepielke_1992: soilbeta), the 2 m diagnostics.  The human-stress
 * indices, lch4 and the landunit-level reference-temperature copies are not
 * built.  a_coef, a_exp, wind_min and zetamaxstable are taken from
 * ctsmg_set_canopy_params (the reference reads the same parameter names).  */
typedef struct {
    int32_t ldp, ldc, ldg, begg;
    const int32_t* patch_column; const int32_t* patch_gridcell;
    /* gridcell forcing */
    const double *forc_u, *forc_v, *forc_hgt_u, *forc_hgt_t, *forc_hgt_q;
    /* column */
    const int32_t* snl;
    const double *forc_t, *forc_pbot, *forc_q, *forc_th, *forc_rho, *thv, *t_grnd, *qg, *qg_snow, *qg_soil,
                 *qg_h2osfc, *dqgdT, *htvp, *z0mg, *soilresis, *soilbeta, *t_h2osfc;
    const double* t_soisno;                        /* [SS]                              */
    double *z0hg, *z0qg;                           /* (c) inout: the last step's roughness in, this step's out */
    /* patch */
    const double* thm;
    double *forc_hgt_u_patch;                      /* (p) inout: the last step's height in */
    double *forc_hgt_t_patch, *forc_hgt_q_patch;   /* (p) inout                         */
    double *btran, *t_veg, *rssun, *rssha, *displa, *z0mv, *z0hv, *z0qv, *dlrad, *ulrad, *dhsdt_canopy,
           *eflx_sh_stem, *z0mg_patch, *z0hg_patch, *z0qg_patch, *zeta, *obu, *ram1, *cgrnds, *cgrndl, *cgrnd,
           *taux, *tauy, *eflx_sh_grnd, *eflx_sh_tot, *eflx_sh_snow, *eflx_sh_soil, *eflx_sh_h2osfc,
           *qflx_tran_veg, *qflx_evap_veg, *qflx_evap_soi, *qflx_evap_tot, *qflx_ev_snow, *qflx_ev_soil,
           *qflx_ev_h2osfc, *t_ref2m, *q_ref2m, *rh_ref2m, *kbm1, *u10_clm, *u10, *va, *vds, *fv, *fm;
    int32_t* num_iter;
    double *rootr, *rresis;                        /* [PG] out: zero                    */
} ctsmg_baregrnd_io;

/* Replaces BareGroundFluxes over filter_noexposedvegp (1-based patches). */
int32_t ctsmg_baregroundfluxes(const ctsmg_bounds* bounds, int32_t num_noexposedvegp,
                               const int32_t* filter_noexposedvegp, const ctsmg_baregrnd_io* io);

/* ------------------------------------------------------- soil evaporative resistance */
/* calc_soilevap_resis (src/biogeophys/SurfaceResistanceMod.F90:190-227),
 * called from BiogeophysPreFluxCalcs before CanopyFluxes
 * (BiogeophysPreFluxCalcsMod.F90:113), for natural-vegetation soil columns
 * (the wetland, glacier and urban branches are not built).
 * soil_resis_method 1 = sl_14 (dry surface layer: dsl, soilresis; the CLM5
 * default, namelist_defaults_ctsm.xml:270), 0 = leepielke_1992 (soilbeta).
 * d_max (mm) and frac_sat_soil_dsl_init come from the parameter file
 * (readParams, :101-111).                                                   */
typedef struct {
    int32_t soil_resis_method;
    double  d_max;
    double  frac_sat_soil_dsl_init;
} ctsmg_soil_resistance_params;

typedef struct {
    int32_t ldc;
    const double* dz;             /* [SS] layer thickness (m)                    */
    const double* t_soisno;       /* [SS] (K)                                    */
    const double* h2osoi_liq;     /* [SS] (kg/m2)                                */
    const double* h2osoi_ice;     /* [SS] (kg/m2)                                */
    const double* watsat;         /* [G]                                         */
    const double* bsw;            /* [G]                                         */
    const double* sucsat;         /* [G]  (mm)                                   */
    const double* watfc;          /* [G]  field capacity (leepielke_1992 only)   */
    const double* frac_sno;       /* (c)  (leepielke_1992 only)                  */
    const double* frac_h2osfc;    /* (c)  (leepielke_1992 only)                  */
    double*       dsl;            /* (c)  out: dry surface layer thickness (mm)  */
    double*       soilresis;      /* (c)  out: soil evaporative resistance (s/m) */
    double*       soilbeta;       /* (c)  out: evaporation factor (leepielke)    */
} ctsmg_soilresis_io;

/* Replaces soil_resistance_readNL (:60-96) and readParams (:101-111). */
int32_t ctsmg_set_soil_resistance(const ctsmg_soil_resistance_params* p);
/* Replaces calc_soilevap_resis over the column filter; the components the
 * method does not use may be NULL.                                          */
int32_t ctsmg_soilevap_resis(const ctsmg_bounds* bounds, int32_t num_nolakec, const int32_t* filter_nolakec,
                             const ctsmg_soilresis_io* io);

/* ---------------------------------------------------------------- SoilFluxes */
/* Components SoilFluxes reads and writes for natural-vegetation columns and
 * patches (src/biogeophys/SoilFluxesMod.F90:36-518; the urban branches and the
 * _r/_u copies are not built).  tssbef and t_h2osfc_bef are the temperatures
 * saved before SoilTemperature (temperature_inst%t_ssbef_col,
 * t_h2osfc_bef_col); patch_column is 1-based (begc); eflx_sh_stem is zero
 * (no biomass heat storage).                                                */
typedef struct {
    int32_t ldc, ldp;
    /* columns */
    const int32_t* snl;
    const int32_t* col_patchi;       /* (c) first patch (1-based, begp)         */
    const int32_t* col_npatches;
    const double*  frac_sno_eff;
    const double*  frac_h2osfc;
    const double*  t_grnd;
    const double*  t_h2osfc;
    const double*  t_h2osfc_bef;
    const double*  c_h2osfc;
    const double*  emg;
    const double*  forc_lwrad;
    const double*  htvp;
    const double*  xmf;
    const double*  xmf_h2osfc;
    const double*  eflx_h2osfc_to_snow;
    const double*  t_soisno;         /* [SS] after SoilTemperature              */
    const double*  tssbef;           /* [SS] before SoilTemperature             */
    const double*  fact;             /* [SS] from SoilTemperature               */
    const double*  h2osoi_liq;       /* [SS]                                    */
    const double*  h2osoi_ice;       /* [SS]                                    */
    double*        errsoi_col;       /* out: soil energy error (W/m2), p2c      */
    /* patches */
    const int32_t* patch_column;
    const int32_t* frac_veg_nosno;
    const double*  wtcol;
    const double*  cgrnds;
    const double*  cgrndl;
    const double*  sabg_soil;
    const double*  sabg_snow;
    const double*  dlrad;
    const double*  ulrad;
    const double*  eflx_sh_veg;
    const double*  qflx_evap_veg;
    const double*  qflx_tran_veg;
    double*        eflx_sh_grnd;     /* inout: updated for the T increment     */
    double*        qflx_evap_soi;    /* inout                                   */
    double*        qflx_ev_snow;     /* inout                                   */
    double*        qflx_ev_soil;     /* inout                                   */
    double*        qflx_ev_h2osfc;   /* inout                                   */
    double*        qflx_liqevap_from_top_layer;
    double*        qflx_solidevap_from_top_layer;
    double*        qflx_soliddew_to_top_layer;
    double*        qflx_liqdew_to_top_layer;
    double*        eflx_soil_grnd;
    double*        eflx_sh_tot;
    double*        qflx_evap_tot;
    double*        eflx_lh_tot;
    double*        qflx_evap_can;
    double*        eflx_lh_vege;
    double*        eflx_lh_vegt;
    double*        eflx_lh_grnd;
    double*        eflx_lwrad_out;
    double*        eflx_lwrad_net;
    double*        errsoi_patch;
    double*        t_skin;           /* inout: written where frac_veg_nosno = 0 */
} ctsmg_soilfluxes_io;

/* SoilFluxes (src/biogeophys/SoilFluxesMod.F90:36-518): the ground sensible
 * and latent fluxes for the temperature increment of the step, top-layer
 * evaporation / dew and its limits, eflx_soil_grnd, the total, latent and
 * longwave fluxes and the soil energy error errsoi (patch, and column by
 * p2c over filter_nolakec).  Called after SoilTemperature
 * (src/main/clm_driver.F90:921).                                         */
int32_t ctsmg_soilfluxes(const ctsmg_bounds* bounds, int32_t num_nolakec, const int32_t* filter_nolakec,
                         int32_t num_nolakep, const int32_t* filter_nolakep, const ctsmg_soilfluxes_io* io,
                         double dtime);

/* Allocation-free SoilTemperature.  No counterpart in the reference: it is an
 * extra entry point for callers that cannot allocate device memory -- a host
 * whose device memory belongs to another runtime (an OpenACC or OpenMP-offload
 * Fortran build that keeps the derived types resident and budgets device
 * memory itself) or one that must not call cudaMalloc on this path.  Every
 * pointer in io_dev and filter_nolakec_dev is DEVICE memory owned by the
 * caller (filter NULL = begc..begc+num_nolakec-1); the call allocates nothing:
 * the band-solve scratch is a fixed array inside the library, sized for at
 * most 16384 columns per call (larger filters return CTSMG_E_ARG).  The first
 * call on a device after ctsmg_init looks up that array's address (make it
 * before any stream capture); ctsmg_finalize forgets the addresses, so after a
 * device reset the caller runs ctsmg_finalize and ctsmg_init again.  Without
 * ctsmg_init the call returns CTSMG_E_NOT_INIT.  A filter entry outside
 * begc..endc, or a column whose snl, nbedrock or patch range is out of bounds,
 * is skipped and returns CTSMG_E_ARG with its filter position as the index;
 * the other columns are computed.  All calls share the one array, so calls
 * that overlap on the GPU (other streams, other host threads) race: serialise
 * them.  stream is a cudaStream_t (NULL = default stream); the call waits for
 * it to finish. */
int32_t ctsmg_soiltemperature_noalloc(const ctsmg_bounds* bounds, int32_t num_nolakec,
                                      const int32_t* filter_nolakec_dev, const ctsmg_soiltemp_io* io_dev,
                                      double dtime, void* stream);

/* ---------------------------------------------------------------- batched resident mode */
/* Many columns kept resident in HBM across model steps.  The reference has no
 * counterpart object: it is the clump loop of src/main/clm_driver.F90:525-1346
 * restricted to the three scoped calls, with state kept on the device.  Each
 * step is SoilWater (ZD09), then SoilTemperature, then the between-step
 * refresh h2osoi_vol = liq/(dz denh2o) + ice/(dz denice) on levels 1..nlevsoi
 * that the driver makes in src/biogeophys/HydrologyNoDrainageMod.F90:580,590.
 * Host arrays are dense (begc = begp = 1, ldc = ncol, ldp = npatch); columns
 * are reordered on the device by (snl, nbedrock) so that warps see uniform
 * level counts, and restored to the caller's order by ctsmg_batch_download. */
typedef struct ctsmg_batch_s* ctsmg_batch;

/* Full configuration of a batch.  with_canopy = 1 adds CanopyFluxes over all
 * npatch patches before the soil step and the root water sink that couples
 * transpiration into SoilWater (Compute_EffecRootFrac_And_VertTranSink_Default,
 * src/biogeophys/SoilWaterPlantSinkMod.F90:332-420); order = 1 is the driver's
 * order CanopyFluxes, SoilTemperature, SoilWater (src/main/clm_driver.F90:766,900,950),
 * order = 0 is SoilWater then SoilTemperature, order = 2 runs CanopyFluxes
 * alone (the soil state is then read but not advanced).  bucket = 1 reorders the
 * columns by (snl, nbedrock) on the device.                               */
typedef struct {
    int32_t ncol, npatch, ngrid;
    double dtime, e_ice;
    int32_t snow_thermal_cond_method, stomatalcond_method, itmax_canopy_fluxes;
    int32_t order, with_canopy, bucket;
    /* balance = 1 evaluates every step's column water error (mm) and soil
     * energy error errsoi (W/m2) as BalanceCheck does
     * (src/biogeophys/BalanceCheckMod.F90:592-658, 1103-1113; errsoi from
     * src/biogeophys/SoilFluxesMod.F90:399-445) and keeps their maxima over
     * the steps after the first skip_steps (BalanceCheckMod.F90:91).       */
    int32_t balance, skip_steps;
    /* soilfluxes = 1 (with_canopy, order 1) runs SoilFluxes between
     * SoilTemperature and SoilWater as the driver does (clm_driver.F90:921);
     * sf (ctsmg_batch_create3) then carries its components.               */
    int32_t soilfluxes;
    /* soilresis = 1 (with_canopy) computes dsl and soilresis (sl_14, the
     * parameters of ctsmg_set_soil_resistance) from the resident soil state
     * at the start of every step, as BiogeophysPreFluxCalcs does before
     * CanopyFluxes (BiogeophysPreFluxCalcsMod.F90:113); the inputs' sr
     * carries the components.                                              */
    int32_t soilresis;
    /* rootmoist = 1 (with_canopy) computes btran and rootr from the resident
     * soil state at the start of every step, as CanopyFluxes does before its
     * iteration (src/biogeophys/CanopyFluxesMod.F90:833-895); the root sink
     * then uses that rootr.  The inputs' rm carries the components.       */
    int32_t rootmoist;
    /* hydrology = 1 (with the moisture form) runs the default hydrology's
     * water tables and lateral flows around SoilWater in every step:
     * SaturatedExcessRunoff before it, PerchedWaterTable,
     * ThetaBasedWaterTable, PerchedLateralFlow and SubsurfaceLateralFlow after
     * it (HydrologyNoDrainageMod.F90:308-368, HydrologyDrainageMod.F90:139-143),
     * with the parameters of ctsmg_set_soilhydrology_params, or per column
     * baseflow_scalar / fff from the inputs (ensemble members).          */
    int32_t hydrology;
} ctsmg_batch_config;

/* Everything a batch can hold, in one struct (NULL = not used).           */
typedef struct {
    const ctsmg_soilwater_io* sw;
    const ctsmg_soiltemp_io* st;
    const ctsmg_canopy_io* cio;
    const ctsmg_soilfluxes_io* sf;
    const ctsmg_rootmoist_io* rm;
    const double* rootr;                 /* (p, 1:nlevsoi), ldp = npatch; unused with rootmoist */
    const double* medlynslope_p;
    const double* medlynintercept_p;
    const ctsmg_canopy_params* cpar;
    const ctsmg_pftcon* pft;
    const ctsmg_soilresis_io* sr;
    const ctsmg_hydrology_io* hy;
    const double* baseflow_scalar_c;     /* (c) or NULL */
    const double* fff_c;                 /* (c) or NULL */
    const double* d_max_c;               /* (c) or NULL: per-column d_max of the sl_14
                                            soil resistance (ensemble members)     */
} ctsmg_batch_inputs;

/* Create a batch from `in` (the arrays are copied); ctsmg_batch_create*
 * are shorthands for it.  ctsmg_batch_fetch copies the state the steps
 * write back into every table `in` names, in the caller's column order.   */
int32_t ctsmg_batch_open(ctsmg_batch* out, const ctsmg_batch_config* cfg, const ctsmg_batch_inputs* in);
int32_t ctsmg_batch_fetch(ctsmg_batch b, const ctsmg_batch_inputs* in);

/* cio/rootr/medlyn*_p may be NULL when with_canopy = 0.  rootr is (p, 1:nlevsoi)
 * with ldp = npatch; medlynslope_p / medlynintercept_p (p) override the pftcon
 * values per patch (perturbed-parameter ensemble members) or are NULL.     */
int32_t ctsmg_batch_create2(ctsmg_batch* out, const ctsmg_batch_config* cfg, const ctsmg_soilwater_io* sw,
                            const ctsmg_soiltemp_io* st, const ctsmg_canopy_io* cio, const double* rootr,
                            const double* medlynslope_p, const double* medlynintercept_p,
                            const ctsmg_canopy_params* cpar, const ctsmg_pftcon* pft);
/* As ctsmg_batch_create2, plus the SoilFluxes components when cfg->soilfluxes
 * (sf->tssbef / t_h2osfc_bef are filled by the step itself).               */
int32_t ctsmg_batch_create3(ctsmg_batch* out, const ctsmg_batch_config* cfg, const ctsmg_soilwater_io* sw,
                            const ctsmg_soiltemp_io* st, const ctsmg_canopy_io* cio, const ctsmg_soilfluxes_io* sf,
                            const double* rootr, const double* medlynslope_p, const double* medlynintercept_p,
                            const ctsmg_canopy_params* cpar, const ctsmg_pftcon* pft);
/* As ctsmg_batch_download2, plus the SoilFluxes components (sf may be NULL). */
int32_t ctsmg_batch_download3(ctsmg_batch b, const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st,
                              const ctsmg_canopy_io* cio, const ctsmg_soilfluxes_io* sf);
int32_t ctsmg_batch_create(ctsmg_batch* out, const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st,
                           int32_t ncol, int32_t npatch, double dtime, double e_ice,
                           int32_t snow_thermal_cond_method);
/* Enqueue nsteps steps (one CUDA graph replay each).  If step_ms is not NULL
 * each step is timed with CUDA events on the batch's stream (synchronising). */
int32_t ctsmg_batch_run(ctsmg_batch b, int32_t nsteps, float* step_ms);
/* Wait for the batch's stream; returns CTSMG_E_SINGULAR with the column if a
 * band solve failed in any step since creation. */
int32_t ctsmg_batch_sync(ctsmg_batch b);
/* Copy the resident state back into the caller's host arrays (caller order). */
int32_t ctsmg_batch_download(ctsmg_batch b, const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st);
/* Same, and the canopy components as well when the batch runs CanopyFluxes. */
int32_t ctsmg_batch_download2(ctsmg_batch b, const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st,
                              const ctsmg_canopy_io* cio);
/* Per-column balance results in the caller's column order (any pointer may be
 * NULL): maxima of |errh2o| and |errsoi| over the checked steps, and the last
 * step's signed errors. */
int32_t ctsmg_batch_balance(ctsmg_batch b, double* errh2o_max, double* errsoi_max, double* errh2o_last,
                            double* errsoi_last);
/* Time trial_steps steps for each candidate threads-per-block (64, 128, 256)
 * on the batch's own data, keep the fastest, restore the state. */
int32_t ctsmg_batch_autotune(ctsmg_batch b, int32_t trial_steps, int32_t* block_out);
/* Autotuner over (column order, moisture-form work order, threads per
 * block).  The batch holds its columns in one of four orders -- sorted by
 * (snl, nbedrock, zwt), by (snl, zwt, nbedrock), by (nbedrock, snl, zwt), or
 * the caller's order -- which decides how uniform the level loops and
 * branches of a warp's 32 lanes are.  With the moisture form, its persistent
 * sub-step kernel takes the columns either bucketed by the sub-step count of
 * the previous step and the bedrock depth (rebuilt on the device every step)
 * or in position order.  Every candidate is timed at 64, 128 and 256 threads
 * per block over trial_steps steps of the batch's own data, the fastest is
 * kept (the resident columns are moved into its order on the device) and the
 * state restored.  Column orders are tuned for batches without CanopyFluxes
 * (with it, the column order in force is kept).  ms_out (NULL or 24 floats)
 * receives the milliseconds per step of every candidate, indexed
 * (order * n_mf + mf) * 3 + block, n_mf = 2 with the moisture form (mf 0 the
 * bucketed work order) else 1; order_out the chosen column order (0..3,
 * ctsmg_batch_order_name names it), mf_sort_out 1 / 0 for the chosen work
 * order (-1 without the moisture form), ncand_out the candidates timed.
 * No reference counterpart: the reference runs its clump loop in one fixed
 * order (src/main/clm_driver.F90:525).                                    */
int32_t ctsmg_batch_autotune2(ctsmg_batch b, int32_t trial_steps, int32_t* block_out, int32_t* order_out,
                              int32_t* mf_sort_out, float* ms_out, int32_t* ncand_out);
const char* ctsmg_batch_order_name(int32_t order);
/* The moisture-form work order of a batch with the moisture form: 1 buckets
 * the columns by the previous step's sub-step count and bedrock depth and
 * runs the sub-step kernel on a copy of its components moved into that order
 * (and the written ones moved back), 0 takes them in position order (the
 * default).  Results do not depend on it. */
int32_t ctsmg_batch_set_mf_order(ctsmg_batch b, int32_t sorted);
int32_t ctsmg_batch_set_block(ctsmg_batch b, int32_t block);
int64_t ctsmg_batch_state_bytes(ctsmg_batch b);
/* Checkpoint / restart of a batch's resident state (the restart role of
 * src/main/restFileMod.F90; NetCDF/PIO are absent here, so the file is a
 * self-describing binary: the magic "CTSMGCK1", the batch sizes, then one
 * record per component -- name, kind, element size, byte count and the
 * array in the caller's column order and the reference's level layout).
 * ctsmg_batch_load restores a file into a batch created with the same sizes
 * and components; every component the batch holds must be in the file.    */
int32_t ctsmg_batch_save(ctsmg_batch b, const char* path);
int32_t ctsmg_batch_load(ctsmg_batch b, const char* path);
int32_t ctsmg_batch_destroy(ctsmg_batch b);

/* ---------------------------------------------------------------- serving pool */
/* A device-resident pool of column, patch and gridcell slots that independent
 * run requests (a single point or a region: their own columns, patches,
 * gridcells and step count) are admitted into while others are running.  No
 * reference counterpart: CTSM runs one configuration per executable.  Each
 * tick advances every admitted, unfinished request by one model step -- the
 * same step as a batch with with_canopy (CanopyFluxes, root sink,
 * SoilTemperature, SoilWater, h2osoi_vol refresh) or, with_canopy = 0,
 * SoilWater then SoilTemperature -- through one CUDA graph whose kernels run
 * over filters of the active slots (1-based positions; each request's
 * columns are stored sorted by (snl, nbedrock, water-table depth) and are
 * returned in the caller's order).  Columns never interact, so a request's results do not depend
 * on what else is in the pool.  Calls on one pool must come from one host
 * thread at a time. */
typedef struct ctsmg_pool_s* ctsmg_pool;

typedef struct {
    int32_t col_capacity, patch_capacity, grid_capacity;   /* slots of each kind  */
    double dtime, e_ice;
    int32_t snow_thermal_cond_method, stomatalcond_method, itmax_canopy_fluxes;
    int32_t with_canopy;
    int32_t max_inflight;     /* ticks queued ahead of the device (>= 1)      */
    int32_t rootmoist;        /* 1: each tick starts with the root moisture
                                 stress (btran, rootr from the soil state;
                                 needs with_canopy)                        */
    int32_t hydrology;        /* 1: the aquifer-layer hydrology around the
                                 Zeng-Decker SoilWater (saturated excess,
                                 infiltration, water table, drainage) with
                                 the parameters of ctsmg_set_soilhydrology_params
                                 at creation                               */
} ctsmg_pool_config;

/* One request's host arrays for ctsmg_pool_admit_request /
 * ctsmg_pool_evict_request (dense: begc = begp = begg = 1, ldc = ncol, ldp =
 * npatch, ldg = ngrid).  cio with with_canopy; rm with rootmoist; hy with
 * hydrology; rootr (p, 1:nlevsoi) with with_canopy and no rootmoist;
 * medlynslope_p / medlynintercept_p (p) may be NULL (pftcon values). */
typedef struct {
    int32_t ncol, npatch, ngrid, nsteps;
    const ctsmg_soilwater_io* sw;
    const ctsmg_soiltemp_io* st;
    const ctsmg_canopy_io* cio;
    const ctsmg_rootmoist_io* rm;
    const ctsmg_hydrology_io* hy;
    const double* rootr;
    const double* medlynslope_p;
    const double* medlynintercept_p;
} ctsmg_pool_request;

#define CTSMG_E_FULL          11   /* pool: no free range large enough (nothing changed) */

/* Device bytes one slot of each kind takes in a pool (resident fields, band
 * scratch, filters, root fractions, per-patch Medlyn parameters), for sizing
 * the capacities from a memory budget.                                      */
int32_t ctsmg_pool_slot_bytes(int32_t with_canopy, int64_t* col_bytes, int64_t* patch_bytes, int64_t* grid_bytes);
/* The same for the configuration cfg (its with_canopy, rootmoist and
 * hydrology; the capacities are ignored). */
int32_t ctsmg_pool_slot_bytes_cfg(const ctsmg_pool_config* cfg, int64_t* col_bytes, int64_t* patch_bytes,
                                  int64_t* grid_bytes);
/* cpar / pft may be NULL when with_canopy = 0. */
int32_t ctsmg_pool_create(ctsmg_pool* out, const ctsmg_pool_config* cfg, const ctsmg_canopy_params* cpar,
                          const ctsmg_pftcon* pft);
/* Admit one request: its host arrays are dense (begc = begp = begg = 1, ldc =
 * ncol, ldp = npatch, ldg = ngrid, 1-based col_patchi / patch_column /
 * patch_gridcell within the request), copied to free slot ranges before the
 * call returns.  rootr is (p, 1:nlevsoi) with ldp = npatch; medlynslope_p /
 * medlynintercept_p (p) may be NULL (pftcon values).  Returns CTSMG_E_FULL,
 * changing nothing, when a range of the needed size is not free.  nsteps >= 1
 * model steps run from the next tick on; *slot_out identifies the request. */
int32_t ctsmg_pool_admit(ctsmg_pool p, int32_t ncol, int32_t npatch, int32_t ngrid, int32_t nsteps,
                         const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st, const ctsmg_canopy_io* cio,
                         const double* rootr, const double* medlynslope_p, const double* medlynintercept_p,
                         int32_t* slot_out);
/* ctsmg_pool_admit with every component a configuration can use. */
int32_t ctsmg_pool_admit_request(ctsmg_pool p, const ctsmg_pool_request* req, int32_t* slot_out);
/* Enqueue one step of every running request (returns at once unless
 * max_inflight ticks are already queued).  *ncol_stepped (may be NULL) is
 * the number of columns the tick advances. */
int32_t ctsmg_pool_tick(ctsmg_pool p, int64_t* ncol_stepped);
/* Requests whose last step has completed on the device (up to cap slots). */
int32_t ctsmg_pool_poll(ctsmg_pool p, int32_t* slots, int32_t cap, int32_t* n);
/* Copy a request's state to the host arrays (dense, as for admit; the index
 * components are not written back) and free its slots.  A request that has
 * not finished is stopped after the steps already enqueued.  *steps_done
 * (may be NULL) is the number of steps it ran. */
int32_t ctsmg_pool_evict(ctsmg_pool p, int32_t slot, const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st,
                         const ctsmg_canopy_io* cio, int32_t* steps_done);
/* ctsmg_pool_evict that also returns the root moisture stress and
 * hydrology components (req->rm / req->hy may be NULL; the sizes in req are
 * not used). */
int32_t ctsmg_pool_evict_request(ctsmg_pool p, int32_t slot, const ctsmg_pool_request* req, int32_t* steps_done);
/* Wait for the device; reports a band-solve or CanopyFluxes failure as its
 * status with the request slot in ctsmg_last_error_index and the column (or
 * patch) within the request in the level slot. */
int32_t ctsmg_pool_sync(ctsmg_pool p);
/* Free slots of each kind (largest free range in *_largest; any may be NULL). */
int32_t ctsmg_pool_free(ctsmg_pool p, int32_t* cols_largest, int32_t* patches_largest, int32_t* grids_largest);
int32_t ctsmg_pool_destroy(ctsmg_pool p);

/* ---------------------------------------------------------------- measurement */
/* Host<->device bytes copied by the drop-in entry points of this process
 * (host arrays in, written components back, filters and status reads) since
 * the last reset; reset != 0 zeroes the counters after reading them.  No
 * reference counterpart. */
int32_t ctsmg_copy_bytes(int64_t* h2d, int64_t* d2h, int32_t reset);
/* How the pipelined drop-in calls (ctsmg_soilwater, ctsmg_soiltemperature
 * over an ascending filter of at least 32,768 columns) copy their inputs in:
 * mode 0 (the default) with one gather kernel per chunk that reads the
 * caller's arrays through their device-mapped addresses when every array the
 * call copies in is page-locked (cudaHostAlloc / cudaHostRegister) and
 * element-aligned, else with the copy engines; mode 1 with the copy engines
 * always.  Results do not depend on it.  No reference counterpart. */
int32_t ctsmg_set_copy_mode(int32_t mode);
/* Time-constant inputs of the pipelined drop-in calls.  With resident = 1,
 * ctsmg_soilwater (Zeng-Decker form: levels 1..nlevsoi of z, dz and zi,
 * smpmin, watsat, hksat, bsw, sucsat) and ctsmg_soiltemperature (watsat, bsw,
 * sucsat, tkmg, tkdry, csol) keep their device copy of each such host array
 * between calls -- keyed by the array's address, leading dimension, size
 * and the rows the call reads -- and copy it in again only for columns not
 * yet covered.  These are the
 * components CTSM sets at initialisation (SoilStateInitTimeConstMod) and the
 * soil-layer geometry; a caller that changes one on the host calls
 * ctsmg_invalidate_time_constant_inputs() before its next call.  Default 0:
 * every input is copied in on every call.  No reference counterpart. */
int32_t ctsmg_set_time_constant_inputs(int32_t resident);
int32_t ctsmg_invalidate_time_constant_inputs(void);
/* Per-chunk timeline of the calling thread's pipelined drop-in calls
 * (ctsmg_soilwater, ctsmg_soiltemperature over an ascending filter of at
 * least 32,768 columns).  enable = 1 / 0 turns the recording on / off for
 * later calls, -1 leaves it.  With ms_out (7 floats per chunk, at most
 * max_chunks chunks) the last recorded call's marks are read first, in ms
 * from its first copy-in: on the GPU copy-in start, copy-in end, kernel
 * start, kernel end, copy-out end; on the host clock the moments the calling
 * thread finished enqueuing the chunk's copy-in and its copy-out;
 * *nchunks_out = its chunks.  No reference counterpart. */
int32_t ctsmg_pipe_trace(int32_t enable, float* ms_out, int32_t max_chunks, int32_t* nchunks_out);
/* FP64 FMA throughput of the current GPU in TFLOP/s (a DFMA loop over every
 * SM); the denominator of the FP64 roofline fraction.  No reference counterpart. */
int32_t ctsmg_measure_fp64_tflops(double* tflops);
/* Milliseconds of the same DFMA loop (512 x 128 FMAs per thread, 8 blocks of
 * 256 threads per SM) when only the first active_lanes (1..32) lanes of each
 * warp run it: equal times for 1 and 32 lanes mean an FP64 warp instruction
 * costs its issue slot whatever its active lanes.  No reference counterpart. */
int32_t ctsmg_measure_fp64_lane_cost(int32_t active_lanes, float* ms_out);
/* The same for a loop of FP64 divisions (256 x 8 per thread): whether a
 * division's cost follows its active lanes.  No reference counterpart. */
int32_t ctsmg_measure_fp64_div_lane_cost(int32_t active_lanes, float* ms_out);
#ifdef __cplusplus
}
#endif
#endif /* CTSM_GPU_H */
