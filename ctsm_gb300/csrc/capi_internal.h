// capi_internal.h -- field tables and helpers shared by the C-ABI sources.
#pragma once
#include <cstddef>
#include <cstdint>
#include "ctsm_gpu.h"

namespace ctsmg {
enum Kind { K_C, K_P, K_SS, K_ZI, K_G, K_S, K_SN, K_PL, K_GR, K_PS, K_PG };
enum Use { U_IN, U_OUT, U_INOUT };
// A component of an io struct.  The drop-in calls copy rows [lev0, lev0 +
// nlev) of its storage (nlev = 0: every row), and skip the copy-in when
// no_in is set (an output the call writes over that whole range).
struct FieldDesc {
    size_t offset; int kind; int esize; int use; const char* name;
    int lev0 = 0, nlev = 0, no_in = 0;
    // rows copied in when they differ from the rows copied out (in_nlev > 0):
    // an output the call writes on some rows only needs the others copied in
    int in_lev0 = 0, in_nlev = 0;
};

extern const FieldDesc SOILWATER_TABLE[];
extern const int SOILWATER_NFIELDS;
extern const FieldDesc SOILWATER_MF_TABLE[];
extern const int SOILWATER_MF_NFIELDS;
extern const FieldDesc SOILWATER_FLEXCN_TABLE[];
extern const int SOILWATER_FLEXCN_NFIELDS;
extern const FieldDesc SOILRESIS_SL14_TABLE[];
extern const int SOILRESIS_SL14_NFIELDS;
extern const FieldDesc HYD_SAT_TABLE[], HYD_PWT_TABLE[], HYD_TWT_TABLE[], HYD_PLF_TABLE[], HYD_SLF_TABLE[],
    HYD_INF_TABLE[], HYD_WT_TABLE[], HYD_DR_TABLE[];
extern const int HYD_SAT_TABLE_N, HYD_PWT_TABLE_N, HYD_TWT_TABLE_N, HYD_PLF_TABLE_N, HYD_SLF_TABLE_N, HYD_INF_TABLE_N,
    HYD_WT_TABLE_N, HYD_DR_TABLE_N;
extern const FieldDesc SOILTEMP_TABLE[];
extern const int SOILTEMP_NFIELDS;
extern const FieldDesc CANOPY_TABLE[];
extern const int CANOPY_NFIELDS;
extern const FieldDesc ROOTMOIST_TABLE[];
extern const int ROOTMOIST_NFIELDS;
extern const FieldDesc SOILFLUXES_TABLE[];
extern const int SOILFLUXES_NFIELDS;

int kind_levels(int kind);
size_t field_bytes(const FieldDesc& f, int ldc, int ldp, int ldg = 0);
int set_error(int code, const char* what, int index, int level);
int check_filter(const ctsmg_bounds* b, int nf, const int32_t* filt);
int current_snow_method();
// false when ctsmg_init has not been called (or ctsmg_finalize came after it);
// otherwise the snow thermal conductivity method in force goes to *method
bool snow_method_if_init(int* method);
// drops the per-device addresses the allocation-free SoilTemperature looked up
// (ctsmg_finalize; the next call after ctsmg_init looks them up again)
void noalloc_forget_devices();
// the soilwater_movement_inparm namelist in force (ctsmg_init / ctsmg_set_soilwater_movement)
ctsmg_soilwater_movement_nml current_soilwater_nml();
ctsmg_soil_resistance_params current_soil_resistance();
ctsmg_soilhydrology_params current_soilhydrology_params();
} // namespace ctsmg
