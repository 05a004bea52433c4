// engine.cu -- batched resident mode: many columns (and their patches) kept in
// HBM across model steps, columns bucketed by level count, each step replayed
// as one CUDA graph: [CanopyFluxes -> root sink ->] SoilWater / SoilTemperature
// -> h2osoi_vol refresh.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>
#include "ctsm_gpu.h"
#include "ctsm_device.cuh"
#include "soil_kernels.cuh"
#include "canopy_kernels.cuh"
#include "balance_kernels.cuh"
#include "rootmoist_kernels.cuh"
#include "moisture_form_kernels.cuh"
#include "surface_resistance.cuh"
#include "capi_internal.h"

namespace ctsmg {

struct UField {              // one resident component (shared by every io struct naming it)
    std::string name;
    int kind, esize, use;
    void* dptr = nullptr;
    size_t bytes = 0;
};

struct Batch {
    ctsmg_batch_config cfg{};
    int block = 128;
    std::vector<UField> fields;
    std::map<std::string, int> index;
    ctsmg_soilwater_io dsw{};
    ctsmg_soiltemp_io dst{};
    ctsmg_soilfluxes_io dsf{};
    ctsmg_rootmoist_io drm{};
    ctsmg_soilwater_movement_nml swm{};   // the namelist when the batch was created
    ctsmg_soilresis_io dsr{};
    SoilResisArgs sra{};
    HydroStepArgs hya{};
    double* hyd_params = nullptr;         // per-column baseflow_scalar / fff (positions order)
    double* dmax_c = nullptr;             // per-column d_max of the soil resistance (positions order)
    MoistureFormArgs mfa{};
    CanopyArgs cargs{};
    double* rootr = nullptr;
    double* mslope = nullptr;
    double* mint = nullptr;
    int* counter = nullptr;
    int* mf_work = nullptr;        // work counter and work order of the persistent moisture-form kernel
    void* mf_compact = nullptr;    // the moisture form's components moved into the work order
    bool mf_sort = false;          // its columns bucketed by previous sub-steps and bedrock depth
    double* cws = nullptr;         // CanopyFluxes iteration records
    int32_t* d_perm = nullptr;     // sorted position -> original column index (0-based)
    std::vector<int32_t> h_perm;   // host copy of d_perm
    // the keys the column orders sort by, in the caller's column order
    std::vector<int32_t> key_snl, key_nbedrock;
    std::vector<double> key_zwt;
    int order_key = 0;             // the column order in force (COLUMN_ORDERS)
    double* ws = nullptr;
    DevError* err = nullptr;
    void* snapshot = nullptr;
    size_t state_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    BalanceState bal{};
    void* bal_mem = nullptr;
};

static int cuda_err(cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return set_error(CTSMG_E_CUDA, m.c_str(), 0, 0);
}
#define CK(call, where) do { cudaError_t _e = (call); if (_e != cudaSuccess) return cuda_err(_e, where); } while (0)

static void* io_ptr(const void* io, const FieldDesc& f) {
    return *reinterpret_cast<void* const*>(reinterpret_cast<const char*>(io) + f.offset);
}
static void set_io_ptr(void* io, const FieldDesc& f, void* p) {
    *reinterpret_cast<void**>(reinterpret_cast<char*>(io) + f.offset) = p;
}

static cudaError_t enqueue_step(Batch* b) {
    cudaError_t e = cudaSuccess;
    const int ncol = b->cfg.ncol;
    if (b->cfg.balance || b->cfg.soilfluxes) {
        e = launch_prestep(b->dst, ncol, b->bal, b->stream);
        if (e != cudaSuccess) return e;
    }
    if (b->cfg.soilresis) {
        e = launch_soilevap_resis(b->dsr, 1, ncol, nullptr, b->sra, b->stream);
        if (e != cudaSuccess) return e;
    }
    if (b->cfg.rootmoist) {
        e = launch_rootmoist(b->drm, b->cargs.pft, 1, 1, b->cfg.npatch, nullptr, b->stream);
        if (e != cudaSuccess) return e;
    }
    if (b->cfg.with_canopy) {
        e = launch_canopy(b->cargs, b->cfg.npatch, nullptr, b->cfg.dtime, b->counter, b->err, b->cws, b->stream);
        if (e != cudaSuccess || b->cfg.order == 2) return e;
        e = launch_rootsink(b->dst.col_patchi, b->dst.col_npatches, b->dst.wtcol, b->cargs.io.qflx_tran_veg,
                            b->cfg.rootmoist ? b->drm.rootr : b->rootr, b->cfg.npatch, (double*)b->dsw.qflx_rootsoi, ncol, b->stream);
        if (e != cudaSuccess) return e;
    }
    // the moisture form runs in its own kernel: before the heat solve in
    // order 0 (SoilWater first), after it (and SoilFluxes) otherwise
    const int ord = b->cfg.soilfluxes ? 2 : b->cfg.order;
    const bool mf = b->swm.soilwater_movement_method == 1;
    // with the hydrology, the Zeng-Decker form also leaves the fused kernel
    const HydroStepArgs* hy = b->cfg.hydrology ? &b->hya : nullptr;
    const bool own = mf || hy;
    auto water_step = [&](int refresh) {
        if (mf)
            return launch_mf_step(b->dsw, ncol, b->mfa, b->swm.use_flexibleCN, refresh, b->err, nullptr, b->stream,
                                  b->mf_work, hy, b->mf_sort, b->mf_compact);
        return launch_zd09_step(b->dsw, ncol, b->cfg.e_ice, b->cfg.dtime, b->swm.use_flexibleCN, refresh, nullptr,
                                b->stream, hy);
    };
    if (own && ord == 0) {
        e = water_step(0);
        if (e != cudaSuccess) return e;
    }
    SoilStepFlags fl;
    fl.water = own ? 0 : 1;
    fl.flexcn = b->swm.use_flexibleCN;
    fl.refresh = (own && ord >= 1) ? 0 : 1;
    e = launch_soilstep(b->dsw, b->dst, ncol, b->cfg.e_ice, b->cfg.dtime, b->cfg.snow_thermal_cond_method, b->ws,
                        ncol, b->err, b->stream, b->block, ord, nullptr, b->cfg.soilfluxes ? &b->dsf : nullptr, fl);
    if (e == cudaSuccess && own && ord >= 1) e = water_step(1);
    if (e != cudaSuccess || !b->cfg.balance) return e;
    return launch_balance(b->dsw, b->dst, ncol, b->cfg.dtime, b->bal, b->stream);
}

static int build_graph(Batch* b) {
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    cudaError_t le = enqueue_step(b);
    cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (le != cudaSuccess) return cuda_err(le, "step capture");
    if (ce != cudaSuccess) return cuda_err(ce, "cudaStreamEndCapture");
    cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return cuda_err(ie, "cudaGraphInstantiate");
    return 0;
}

static void batch_free(Batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (auto& f : b->fields) if (f.dptr) cudaFree(f.dptr);
    for (void* p : {(void*)b->d_perm, (void*)b->ws, (void*)b->err, b->snapshot, (void*)b->rootr, (void*)b->mslope,
                    (void*)b->mint, (void*)b->counter, (void*)b->cws, b->bal_mem, (void*)b->hyd_params, (void*)b->dmax_c,
                    (void*)b->mf_work, b->mf_compact})
        if (p) cudaFree(p);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// A device io struct starts as the caller's leading dimensions with every
// component pointer NULL; the tables of the step then fill in the device
// copies of exactly the components the step's kernels use.
template <class T>
static void dev_io(T& d, const T* h, size_t header_bytes) {
    std::memset(&d, 0, sizeof d);
    std::memcpy(&d, h, header_bytes);
}

static bool is_column_kind(int k) { return !(k == K_P || k == K_PL || k == K_PS || k == K_PG || k == K_GR); }

} // namespace ctsmg

using namespace ctsmg;

struct ctsmg_batch_s { Batch* b; };

namespace ctsmg {
// Column orders the batch can hold its columns in (position -> caller's
// column): sorted by snow layers, bedrock depth and water-table depth in the
// three priorities below, or the caller's own order.  A warp's lanes hold 32
// consecutive positions, so the order decides how uniform their level loops
// and branches are.
constexpr int N_COLUMN_ORDERS = 4;
static const char* const COLUMN_ORDER_NAMES[N_COLUMN_ORDERS] = {
    "snl,nbedrock,zwt", "snl,zwt,nbedrock", "nbedrock,snl,zwt", "caller"};

static std::vector<int32_t> column_order(int key, const std::vector<int32_t>& snl, const std::vector<int32_t>& nb,
                                         const std::vector<double>& zwt) {
    const int n = (int)snl.size();
    std::vector<int32_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    auto by = [&](auto first, auto second, auto third) {
        std::stable_sort(perm.begin(), perm.end(), [&](int a, int c) {
            if (first(a) != first(c)) return first(a) < first(c);
            if (second(a) != second(c)) return second(a) < second(c);
            return third(a) < third(c);
        });
    };
    auto S = [&](int i) { return (double)snl[i]; };
    auto N = [&](int i) { return (double)nb[i]; };
    auto Z = [&](int i) { return zwt[i]; };
    if (key == 0) by(S, N, Z);
    else if (key == 1) by(S, Z, N);
    else if (key == 2) by(N, S, Z);
    return perm;
}
} // namespace ctsmg



extern "C" int32_t ctsmg_batch_open(ctsmg_batch* out, const ctsmg_batch_config* cfg, const ctsmg_batch_inputs* in) {
    if (!in) return set_error(CTSMG_E_ARG, "null inputs", 0, 0);
    const ctsmg_soilwater_io* sw = in->sw;
    const ctsmg_soiltemp_io* st = in->st;
    const ctsmg_canopy_io* cio = in->cio;
    const ctsmg_soilfluxes_io* sf = in->sf;
    const ctsmg_rootmoist_io* rm = in->rm;
    const double* rootr = in->rootr;
    const double* medlynslope_p = in->medlynslope_p;
    const double* medlynintercept_p = in->medlynintercept_p;
    const ctsmg_canopy_params* cpar = in->cpar;
    const ctsmg_pftcon* pft = in->pft;
    const ctsmg_soilresis_io* sr = in->sr;
    const ctsmg_hydrology_io* hy = in->hy;
    const bool canopy_only = cfg && cfg->order == 2;
    if (!out || !cfg || (!canopy_only && (!sw || !st))) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    const int ncol = cfg->ncol, npatch = cfg->npatch;
    if (ncol <= 0 || npatch < 0) return set_error(CTSMG_E_ARG, "ncol must be positive", 0, 0);
    if (!canopy_only && (sw->ldc != ncol || st->ldc != ncol || st->ldp != npatch))
        return set_error(CTSMG_E_ARG, "batch arrays must be dense: ldc = ncol, ldp = npatch", 0, 0);
    if (!(cfg->dtime > 0.0)) return set_error(CTSMG_E_ARG, "dtime must be positive", 0, 0);
    if (cfg->order < 0 || cfg->order > 2 || (cfg->order == 2 && (!cfg->with_canopy || cfg->balance)))
        return set_error(CTSMG_E_ARG, "order must be 0, 1, or 2 (CanopyFluxes only: with_canopy, no balance)", 0, 0);
    if (cfg->soilfluxes && (!cfg->with_canopy || cfg->order != 1 || !sf))
        return set_error(CTSMG_E_ARG, "soilfluxes needs with_canopy, order 1 and the SoilFluxes components", 0, 0);
    if (cfg->soilfluxes && (sf->ldc != ncol || sf->ldp != npatch))
        return set_error(CTSMG_E_ARG, "SoilFluxes arrays must be dense: ldc = ncol, ldp = npatch", 0, 0);
    const ctsmg_soil_resistance_params sres = current_soil_resistance();
    if (cfg->soilresis && (!cfg->with_canopy || !sr || sres.soil_resis_method != 1))
        return set_error(CTSMG_E_ARG, "soilresis needs with_canopy, the sl_14 method and its components", 0, 0);
    if (cfg->soilresis && sr->ldc != ncol)
        return set_error(CTSMG_E_ARG, "soil resistance arrays must be dense: ldc = ncol", 0, 0);
    if (cfg->rootmoist && (!cfg->with_canopy || !rm))
        return set_error(CTSMG_E_ARG, "rootmoist needs with_canopy and the root moisture stress components", 0, 0);
    if (cfg->rootmoist && (rm->ldc != ncol || rm->ldp != npatch))
        return set_error(CTSMG_E_ARG, "root moisture stress arrays must be dense: ldc = ncol, ldp = npatch", 0, 0);
    if (cfg->with_canopy) {
        if (!cio || (!rootr && !canopy_only && !cfg->rootmoist) || !cpar || !pft)
            return set_error(CTSMG_E_ARG, "with_canopy needs cio, rootr, params", 0, 0);
        if (cio->ldc != ncol || cio->ldp != npatch || cio->ldg != cfg->ngrid || cio->begg != 1)
            return set_error(CTSMG_E_ARG, "canopy arrays must be dense (ldg = ngrid, begg = 1)", 0, 0);
        for (int p = 0; p < npatch; ++p) {
            const int cc = cio->patch_column[p], gg = cio->patch_gridcell[p], it = cio->itype[p];
            if (cc < 1 || cc > ncol || gg < 1 || gg > cfg->ngrid || it < 0 || it >= pft->npft)
                return set_error(CTSMG_E_ARG, "patch column / gridcell / itype out of range", p + 1, 0);
        }
    }
    for (int c = 0; c < (canopy_only ? 0 : ncol); ++c) {
        const int s = st->snl[c], pi = st->col_patchi[c], np = st->col_npatches[c];
        if (s > 0 || s < -NLEVSNO) return set_error(CTSMG_E_ARG, "snl outside -nlevsno..0", c + 1, 0);
        if (np < 0 || pi < 1 || pi + np - 1 > npatch)
            return set_error(CTSMG_E_ARG, "column patches outside 1..npatch", c + 1, 0);
    }
    const ctsmg_soilwater_movement_nml swm = current_soilwater_nml();
    if (!canopy_only && swm.soilwater_movement_method == 1) {
        if (!sw->nbedrock || !sw->eff_porosity || !sw->num_substeps || (swm.use_flexibleCN && !sw->wa))
            return set_error(CTSMG_E_ARG, "the moisture form needs nbedrock, eff_porosity, num_substeps (and wa with "
                             "use_flexibleCN)", 0, 0);
        for (int c = 0; c < ncol; ++c) {
            const int nb = st->nbedrock[c];
            if (nb < 2 || nb > NLEVSOI) return set_error(CTSMG_E_ARG, "nbedrock outside 2..nlevsoi", c + 1, 0);
            if (swm.lower_boundary_condition == 3 && nb != NLEVSOI)
                return set_error(CTSMG_E_ARG, "bc_waterTable needs nbedrock = nlevsoi", c + 1, 0);
        }
    }
    if (!canopy_only && swm.use_flexibleCN && !sw->wa) return set_error(CTSMG_E_ARG, "use_flexibleCN needs wa", 0, 0);
    if (cfg->hydrology && (canopy_only || !hy || hy->ldc != ncol))
        return set_error(CTSMG_E_ARG, "hydrology needs the soil step and dense hydrology arrays", 0, 0);
    if (cfg->hydrology && cfg->balance)
        return set_error(CTSMG_E_UNSUPPORTED, "the balance check does not count the lateral and surface fluxes of the "
                         "hydrology routines", 0, 0);
    if (cfg->balance && swm.use_flexibleCN)
        return set_error(CTSMG_E_UNSUPPORTED, "the balance check does not count the aquifer water the flexibleCN fix "
                         "moves", 0, 0);
    Batch* b = new Batch();
    b->cfg = *cfg;
    b->swm = swm;
    b->mfa = MoistureFormArgs{cfg->e_ice, cfg->dtime, swm.dtmin, swm.verySmall, swm.xTolerUpper, swm.xTolerLower,
                              swm.lower_boundary_condition, swm.flux_calculation == 42 ? 1 : 0,
                              moisture_form_max_trials(cfg->dtime, swm.dtmin)};
    auto fail = [&](int rc) { batch_free(b); return rc; };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(cuda_err(e, "stream"));
    if ((e = cudaEventCreate(&b->ev0)) != cudaSuccess) return fail(cuda_err(e, "event"));
    if ((e = cudaEventCreate(&b->ev1)) != cudaSuccess) return fail(cuda_err(e, "event"));

    // bucket columns: more snow layers first, then shallower bedrock, then a
    // shallower water table (the water-table position selects the branches
    // of the equilibrium profile and recharge in SoilWater); only the order
    // in which threads take columns changes
    std::vector<int32_t> perm(ncol), inv(ncol);
    std::iota(perm.begin(), perm.end(), 0);
    if (!canopy_only) {
        b->key_snl.assign(st->snl, st->snl + ncol);
        b->key_nbedrock.assign(st->nbedrock, st->nbedrock + ncol);
        b->key_zwt.assign(sw->zwt, sw->zwt + ncol);
        b->order_key = cfg->bucket ? 0 : 3;
        perm = column_order(b->order_key, b->key_snl, b->key_nbedrock, b->key_zwt);
    }
    b->h_perm = perm;
    for (int i = 0; i < ncol; ++i) inv[perm[i]] = i;
    if ((e = cudaMalloc(&b->d_perm, (size_t)ncol * 4)) != cudaSuccess) return fail(cuda_err(e, "perm"));
    if ((e = cudaMemcpy(b->d_perm, perm.data(), (size_t)ncol * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(cuda_err(e, "perm H2D"));
    std::vector<int32_t> pcol_new;
    if (cfg->with_canopy) {
        pcol_new.resize(npatch);
        for (int p = 0; p < npatch; ++p) pcol_new[p] = inv[cio->patch_column[p] - 1] + 1;
    }

    auto add = [&](const FieldDesc* tab, int nf, const void* hio, void* dio) -> int {
        for (int i = 0; i < nf; ++i) {
            const FieldDesc& f = tab[i];
            auto it = b->index.find(f.name);
            if (it == b->index.end()) {
                UField u;
                u.name = f.name; u.kind = f.kind; u.esize = f.esize; u.use = f.use;
                u.bytes = field_bytes(f, ncol, npatch, cfg->ngrid);
                cudaError_t ee = cudaMalloc(&u.dptr, u.bytes);
                if (ee != cudaSuccess) return cuda_err(ee, "cudaMalloc(field)");
                const void* hp = io_ptr(hio, f);
                if (!hp) return set_error(CTSMG_E_ARG, (std::string("null component ") + f.name).c_str(), 0, 0);
                if (std::string(f.name) == "patch_column") hp = pcol_new.data();
                if (!is_column_kind(f.kind)) {
                    ee = cudaMemcpy(u.dptr, hp, u.bytes, cudaMemcpyHostToDevice);
                } else {
                    void* tmp = nullptr;
                    ee = cudaMalloc(&tmp, u.bytes);
                    if (ee == cudaSuccess) ee = cudaMemcpy(tmp, hp, u.bytes, cudaMemcpyHostToDevice);
                    if (ee == cudaSuccess) ee = launch_permute(u.dptr, tmp, b->d_perm, ncol, kind_levels(f.kind), f.esize, 0, b->stream);
                    if (ee == cudaSuccess) ee = cudaStreamSynchronize(b->stream);
                    if (tmp) cudaFree(tmp);
                }
                if (ee != cudaSuccess) return cuda_err(ee, "upload");
                b->index[f.name] = (int)b->fields.size();
                b->fields.push_back(u);
                it = b->index.find(f.name);
            } else if (b->fields[it->second].kind != f.kind || b->fields[it->second].esize != f.esize) {
                return set_error(CTSMG_E_ARG, (std::string("component ") + f.name +
                                               " is given with two layouts by the tables of the step").c_str(), 0, 0);
            } else if (b->fields[it->second].use == U_IN && f.use != U_IN) {
                b->fields[it->second].use = f.use;      // written by some call of the step
            }
            set_io_ptr(dio, f, b->fields[it->second].dptr);
        }
        return 0;
    };
    int rc;
    if (!canopy_only) {
        dev_io(b->dsw, sw, sizeof(int32_t));
        dev_io(b->dst, st, 2 * sizeof(int32_t));
        if ((rc = add(SOILWATER_TABLE, SOILWATER_NFIELDS, sw, &b->dsw))) return fail(rc);
        if ((rc = add(SOILTEMP_TABLE, SOILTEMP_NFIELDS, st, &b->dst))) return fail(rc);
        if (swm.soilwater_movement_method == 1) {
            if ((rc = add(SOILWATER_MF_TABLE, SOILWATER_MF_NFIELDS, sw, &b->dsw))) return fail(rc);
            b->fields[b->index["eff_porosity"]].use = U_OUT;     // SetSoilWaterFractions runs in the step
        }
        if (swm.use_flexibleCN && (rc = add(SOILWATER_FLEXCN_TABLE, SOILWATER_FLEXCN_NFIELDS, sw, &b->dsw)))
            return fail(rc);
        if (cfg->hydrology) {
            dev_io(b->hya.io, hy, sizeof(int32_t));
            const bool aq = swm.soilwater_movement_method == 0;     // aquifer-layer path
            const FieldDesc* tabs[6] = {HYD_SAT_TABLE, HYD_INF_TABLE, aq ? HYD_WT_TABLE : HYD_PWT_TABLE,
                                        aq ? HYD_DR_TABLE : HYD_TWT_TABLE, HYD_PLF_TABLE, HYD_SLF_TABLE};
            const int ns[6] = {HYD_SAT_TABLE_N, HYD_INF_TABLE_N, aq ? HYD_WT_TABLE_N : HYD_PWT_TABLE_N,
                               aq ? HYD_DR_TABLE_N : HYD_TWT_TABLE_N, HYD_PLF_TABLE_N, HYD_SLF_TABLE_N};
            for (int k = 0; k < (aq ? 4 : 6); ++k)
                if ((rc = add(tabs[k], ns[k], hy, &b->hya.io))) return fail(rc);
            if (aq) {       // SetSoilWaterFractions runs in the step and writes eff_porosity
                static const FieldDesc EFFPOR[] = {
                    {offsetof(ctsmg_soilwater_io, eff_porosity), K_G, 8, U_OUT, "eff_porosity"}};
                if ((rc = add(EFFPOR, 1, sw, &b->dsw))) return fail(rc);
            }
            b->hya.par = current_soilhydrology_params();
            const double* hc[2] = {in->baseflow_scalar_c, in->fff_c};
            if (hc[0] || hc[1]) {
                const size_t cb = (size_t)ncol * 8;
                if ((e = cudaMalloc(&b->hyd_params, 3 * cb)) != cudaSuccess) return fail(cuda_err(e, "hydrology params"));
                double* tmp = b->hyd_params + 2 * (size_t)ncol;
                for (int k = 0; k < 2; ++k) {
                    if (!hc[k]) continue;
                    double* dst = b->hyd_params + k * (size_t)ncol;
                    if ((e = cudaMemcpy(tmp, hc[k], cb, cudaMemcpyHostToDevice)) != cudaSuccess)
                        return fail(cuda_err(e, "hydrology params"));
                    if ((e = launch_permute(dst, tmp, b->d_perm, ncol, 1, 8, 0, b->stream)) != cudaSuccess ||
                        (e = cudaStreamSynchronize(b->stream)) != cudaSuccess)
                        return fail(cuda_err(e, "hydrology params"));
                    if (k == 0) b->hya.baseflow_scalar_c = dst;
                    else b->hya.fff_c = dst;
                }
            }
        }
    }
    if (cfg->with_canopy) {
        dev_io(b->cargs.io, cio, 4 * sizeof(int32_t));
        if ((rc = add(CANOPY_TABLE, CANOPY_NFIELDS, cio, &b->cargs.io))) return fail(rc);
        b->cargs.par = *cpar;
        b->cargs.pft = *pft;
        b->cargs.method = cfg->stomatalcond_method;
        b->cargs.itmax = cfg->itmax_canopy_fluxes;
        b->cargs.begc = 1;
        b->cargs.begp = 1;
        b->cargs.engine = 1;
        const size_t pb = (size_t)npatch * 8;
        if (cfg->soilresis) {
            dev_io(b->dsr, sr, sizeof(int32_t));
            if ((rc = add(SOILRESIS_SL14_TABLE, SOILRESIS_SL14_NFIELDS, sr, &b->dsr))) return fail(rc);
            b->sra = SoilResisArgs{1, sres.d_max, sres.frac_sat_soil_dsl_init};
            if (in->d_max_c) {      // per-column d_max, in the batch's position order
                const size_t cb = (size_t)ncol * 8;
                if ((e = cudaMalloc(&b->dmax_c, 2 * cb)) != cudaSuccess) return fail(cuda_err(e, "d_max"));
                if ((e = cudaMemcpy(b->dmax_c + ncol, in->d_max_c, cb, cudaMemcpyHostToDevice)) != cudaSuccess ||
                    (e = launch_permute(b->dmax_c, b->dmax_c + ncol, b->d_perm, ncol, 1, 8, 0, b->stream)) != cudaSuccess ||
                    (e = cudaStreamSynchronize(b->stream)) != cudaSuccess)
                    return fail(cuda_err(e, "d_max"));
                b->sra.d_max_c = b->dmax_c;
            }
        }
        if (cfg->rootmoist) {
            dev_io(b->drm, rm, 2 * sizeof(int32_t));
            if ((rc = add(ROOTMOIST_TABLE, ROOTMOIST_NFIELDS, rm, &b->drm))) return fail(rc);
        } else if (!canopy_only) {
            if ((e = cudaMalloc(&b->rootr, pb * NLEVSOI)) != cudaSuccess) return fail(cuda_err(e, "rootr"));
            if ((e = cudaMemcpy(b->rootr, rootr, pb * NLEVSOI, cudaMemcpyHostToDevice)) != cudaSuccess)
                return fail(cuda_err(e, "rootr"));
        }
        if (medlynslope_p) {
            if ((e = cudaMalloc(&b->mslope, pb)) != cudaSuccess) return fail(cuda_err(e, "mslope"));
            if ((e = cudaMemcpy(b->mslope, medlynslope_p, pb, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(cuda_err(e, "mslope"));
        }
        if (medlynintercept_p) {
            if ((e = cudaMalloc(&b->mint, pb)) != cudaSuccess) return fail(cuda_err(e, "mint"));
            if ((e = cudaMemcpy(b->mint, medlynintercept_p, pb, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(cuda_err(e, "mint"));
        }
        b->cargs.medlynslope_p = b->mslope;
        b->cargs.medlynintercept_p = b->mint;
        if (cfg->soilfluxes) {
            dev_io(b->dsf, sf, 2 * sizeof(int32_t));
            if ((rc = add(SOILFLUXES_TABLE, SOILFLUXES_NFIELDS, sf, &b->dsf))) return fail(rc);
        }
        if ((e = cudaMalloc(&b->counter, 256)) != cudaSuccess) return fail(cuda_err(e, "counter"));
        if ((e = cudaMalloc(&b->cws, canopy_ws_bytes(npatch))) != cudaSuccess) return fail(cuda_err(e, "canopy ws"));
    }
    if (cfg->balance || cfg->soilfluxes) {
        const size_t ssb = (size_t)ncol * (NLEVSNO + NLEVGRND) * 8, cb = (size_t)ncol * 8;
        if ((e = cudaMalloc(&b->bal_mem, ssb + 6 * cb + 256)) != cudaSuccess) return fail(cuda_err(e, "balance"));
        if ((e = cudaMemset(b->bal_mem, 0, ssb + 6 * cb + 256)) != cudaSuccess) return fail(cuda_err(e, "balance"));
        char* m = (char*)b->bal_mem;
        b->bal.tssbef = (double*)m; m += ssb;
        b->bal.th2osfc_bef = (double*)m; m += cb;
        b->bal.w_bef = (double*)m; m += cb;
        b->bal.errh2o = (double*)m; m += cb;
        b->bal.errsoi = (double*)m; m += cb;
        b->bal.errh2o_max = (double*)m; m += cb;
        b->bal.errsoi_max = (double*)m; m += cb;
        b->bal.step = (int*)m;
        b->bal.skip_steps = cfg->skip_steps;
        b->bal.mf_lbc = swm.soilwater_movement_method == 1 ? swm.lower_boundary_condition : 0;
        if (cfg->soilfluxes) {                  // the prestep saves straight into SoilFluxes' inputs
            b->bal.tssbef = const_cast<double*>(b->dsf.tssbef);
            b->bal.th2osfc_bef = const_cast<double*>(b->dsf.t_h2osfc_bef);
        }
    }
    if (swm.soilwater_movement_method == 1 && ((e = cudaMalloc(&b->mf_work, mf_work_bytes(ncol))) != cudaSuccess ||
                                                (e = cudaMalloc(&b->mf_compact, mf_compact_bytes(ncol))) != cudaSuccess))
        return fail(cuda_err(e, "moisture-form work order"));
    for (auto& f : b->fields) b->state_bytes += f.bytes;
    if ((e = cudaMalloc(&b->ws, (size_t)SOILTEMP_WS_DOUBLES_PER_COL * ncol * 8)) != cudaSuccess) return fail(cuda_err(e, "ws"));
    if ((e = cudaMalloc(&b->err, sizeof(DevError))) != cudaSuccess) return fail(cuda_err(e, "err"));
    if ((e = cudaMemset(b->err, 0xff, sizeof(DevError))) != cudaSuccess) return fail(cuda_err(e, "err"));
    if ((rc = build_graph(b))) return fail(rc);
    *out = new ctsmg_batch_s{b};
    return 0;
}

extern "C" int32_t ctsmg_batch_create3(ctsmg_batch* out, const ctsmg_batch_config* cfg, const ctsmg_soilwater_io* sw,
                                       const ctsmg_soiltemp_io* st, const ctsmg_canopy_io* cio,
                                       const ctsmg_soilfluxes_io* sf, const double* rootr,
                                       const double* medlynslope_p, const double* medlynintercept_p,
                                       const ctsmg_canopy_params* cpar, const ctsmg_pftcon* pft) {
    if (cfg && cfg->rootmoist) return set_error(CTSMG_E_ARG, "rootmoist needs ctsmg_batch_open", 0, 0);
    if (cfg && cfg->soilresis) return set_error(CTSMG_E_ARG, "soilresis needs ctsmg_batch_open", 0, 0);
    if (cfg && cfg->hydrology) return set_error(CTSMG_E_ARG, "hydrology needs ctsmg_batch_open", 0, 0);
    const ctsmg_batch_inputs in = {sw, st, cio, sf, nullptr, rootr, medlynslope_p, medlynintercept_p, cpar, pft,
                                   nullptr, nullptr, nullptr, nullptr};
    return ctsmg_batch_open(out, cfg, &in);
}

extern "C" int32_t ctsmg_batch_create2(ctsmg_batch* out, const ctsmg_batch_config* cfg, const ctsmg_soilwater_io* sw,
                                       const ctsmg_soiltemp_io* st, const ctsmg_canopy_io* cio, const double* rootr,
                                       const double* medlynslope_p, const double* medlynintercept_p,
                                       const ctsmg_canopy_params* cpar, const ctsmg_pftcon* pft) {
    if (cfg && cfg->soilfluxes) return set_error(CTSMG_E_ARG, "soilfluxes needs ctsmg_batch_create3", 0, 0);
    return ctsmg_batch_create3(out, cfg, sw, st, cio, nullptr, rootr, medlynslope_p, medlynintercept_p, cpar, pft);
}

extern "C" int32_t ctsmg_batch_create(ctsmg_batch* out, const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st,
                                      int32_t ncol, int32_t npatch, double dtime, double e_ice,
                                      int32_t snow_thermal_cond_method) {
    ctsmg_batch_config cfg{};
    cfg.ncol = ncol; cfg.npatch = npatch; cfg.ngrid = 0;
    cfg.dtime = dtime; cfg.e_ice = e_ice;
    cfg.snow_thermal_cond_method = snow_thermal_cond_method;
    cfg.stomatalcond_method = 1; cfg.itmax_canopy_fluxes = 40;
    cfg.order = 0; cfg.with_canopy = 0; cfg.bucket = 1;
    cfg.balance = 0; cfg.skip_steps = 0; cfg.soilfluxes = 0; cfg.soilresis = 0; cfg.rootmoist = 0;
    cfg.hydrology = 0;
    return ctsmg_batch_create2(out, &cfg, sw, st, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
}

extern "C" int32_t ctsmg_batch_run(ctsmg_batch bh, int32_t nsteps, float* step_ms) {
    if (!bh || nsteps < 0) return set_error(CTSMG_E_ARG, "bad batch or nsteps", 0, 0);
    Batch* b = bh->b;
    for (int s = 0; s < nsteps; ++s) {
        if (step_ms) CK(cudaEventRecord(b->ev0, b->stream), "event");
        CK(cudaGraphLaunch(b->graph, b->stream), "cudaGraphLaunch");
        if (step_ms) {
            CK(cudaEventRecord(b->ev1, b->stream), "event");
            CK(cudaEventSynchronize(b->ev1), "event sync");
            CK(cudaEventElapsedTime(&step_ms[s], b->ev0, b->ev1), "elapsed");
        }
    }
    return 0;
}

extern "C" int32_t ctsmg_batch_sync(ctsmg_batch bh) {
    if (!bh) return set_error(CTSMG_E_ARG, "null batch", 0, 0);
    Batch* b = bh->b;
    CK(cudaStreamSynchronize(b->stream), "batch sync");
    DevError h;
    CK(cudaMemcpy(&h, b->err, sizeof h, cudaMemcpyDeviceToHost), "err D2H");
    if (h.key != ~0ull) {
        const int code = (int)(h.key & 0xff);
        int idx = (int)(h.key >> 32);
        if (code == CTSMG_E_SINGULAR && idx >= 1 && idx <= b->cfg.ncol) {
            int32_t orig = 0;
            cudaMemcpy(&orig, b->d_perm + idx - 1, 4, cudaMemcpyDeviceToHost);
            idx = orig + 1;
        }
        return set_error(code, code == CTSMG_E_SINGULAR ? "BandDiagonal ERROR: dgbsv returned error code"
                                                        : "CanopyFluxes error", idx,
                         (int)((h.key >> 8) & 0xffffff) - 1024);
    }
    return 0;
}

static int download_table(Batch* b, const FieldDesc* tab, int nf, const void* hio) {
    for (int i = 0; i < nf; ++i) {
        const FieldDesc& f = tab[i];
        void* hp = io_ptr(hio, f);
        auto it = b->index.find(f.name);
        if (it == b->index.end() || !hp) continue;
        const UField& u = b->fields[it->second];
        if (u.use == U_IN && u.name != "h2osoi_vol" && u.name != "qflx_rootsoi") continue;
        if (!is_column_kind(u.kind)) {
            CK(cudaMemcpy(hp, u.dptr, u.bytes, cudaMemcpyDeviceToHost), "D2H");
        } else {
            void* tmp = nullptr;
            CK(cudaMalloc(&tmp, u.bytes), "tmp");
            cudaError_t e = launch_permute(tmp, u.dptr, b->d_perm, b->cfg.ncol, kind_levels(u.kind), u.esize, 1, b->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
            if (e == cudaSuccess) e = cudaMemcpy(hp, tmp, u.bytes, cudaMemcpyDeviceToHost);
            cudaFree(tmp);
            if (e != cudaSuccess) return cuda_err(e, "download");
        }
    }
    return 0;
}

extern "C" int32_t ctsmg_batch_fetch(ctsmg_batch bh, const ctsmg_batch_inputs* in) {
    if (!bh || !in) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    int rc = ctsmg_batch_download3(bh, in->sw, in->st, in->cio, in->sf);
    if (rc) return rc;
    if (in->rm && bh->b->cfg.rootmoist && (rc = download_table(bh->b, ROOTMOIST_TABLE, ROOTMOIST_NFIELDS, in->rm)))
        return rc;
    if (in->sr && bh->b->cfg.soilresis &&
        (rc = download_table(bh->b, SOILRESIS_SL14_TABLE, SOILRESIS_SL14_NFIELDS, in->sr)))
        return rc;
    if (in->hy && bh->b->cfg.hydrology) {
        const bool aq = bh->b->swm.soilwater_movement_method == 0;
        const FieldDesc* tabs[6] = {HYD_SAT_TABLE, HYD_INF_TABLE, aq ? HYD_WT_TABLE : HYD_PWT_TABLE,
                                    aq ? HYD_DR_TABLE : HYD_TWT_TABLE, HYD_PLF_TABLE, HYD_SLF_TABLE};
        const int ns[6] = {HYD_SAT_TABLE_N, HYD_INF_TABLE_N, aq ? HYD_WT_TABLE_N : HYD_PWT_TABLE_N,
                           aq ? HYD_DR_TABLE_N : HYD_TWT_TABLE_N, HYD_PLF_TABLE_N, HYD_SLF_TABLE_N};
        for (int k = 0; k < (aq ? 4 : 6); ++k)
            if ((rc = download_table(bh->b, tabs[k], ns[k], in->hy))) return rc;
    }
    return 0;
}

extern "C" int32_t ctsmg_batch_download3(ctsmg_batch bh, const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st,
                                         const ctsmg_canopy_io* cio, const ctsmg_soilfluxes_io* sf) {
    int rc = ctsmg_batch_download2(bh, sw, st, cio);
    if (rc || !sf || !bh->b->cfg.soilfluxes) return rc;
    return download_table(bh->b, SOILFLUXES_TABLE, SOILFLUXES_NFIELDS, sf);
}

extern "C" int32_t ctsmg_batch_download2(ctsmg_batch bh, const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st,
                                         const ctsmg_canopy_io* cio) {
    if (!bh) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    Batch* b = bh->b;
    if (b->cfg.order != 2 && (!sw || !st)) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    CK(cudaStreamSynchronize(b->stream), "sync");
    int rc;
    if (sw && (rc = download_table(b, SOILWATER_TABLE, SOILWATER_NFIELDS, sw))) return rc;
    if (sw && b->swm.soilwater_movement_method == 1 &&
        (rc = download_table(b, SOILWATER_MF_TABLE, SOILWATER_MF_NFIELDS, sw))) return rc;
    if (sw && b->swm.use_flexibleCN &&
        (rc = download_table(b, SOILWATER_FLEXCN_TABLE, SOILWATER_FLEXCN_NFIELDS, sw))) return rc;
    if (st && (rc = download_table(b, SOILTEMP_TABLE, SOILTEMP_NFIELDS, st))) return rc;
    if (cio && b->cfg.with_canopy && (rc = download_table(b, CANOPY_TABLE, CANOPY_NFIELDS, cio))) return rc;
    return 0;
}

extern "C" int32_t ctsmg_batch_download(ctsmg_batch bh, const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st) {
    return ctsmg_batch_download2(bh, sw, st, nullptr);
}

extern "C" int32_t ctsmg_batch_balance(ctsmg_batch bh, double* errh2o_max, double* errsoi_max, double* errh2o_last,
                                       double* errsoi_last) {
    if (!bh) return set_error(CTSMG_E_ARG, "null batch", 0, 0);
    Batch* b = bh->b;
    if (!b->cfg.balance) return set_error(CTSMG_E_ARG, "batch was created without balance = 1", 0, 0);
    CK(cudaStreamSynchronize(b->stream), "sync");
    const int ncol = b->cfg.ncol;
    double* outs[4] = {errh2o_max, errsoi_max, errh2o_last, errsoi_last};
    double* srcs[4] = {b->bal.errh2o_max, b->bal.errsoi_max, b->bal.errh2o, b->bal.errsoi};
    for (int k = 0; k < 4; ++k) {
        if (!outs[k]) continue;
        double* tmp = nullptr;
        CK(cudaMalloc(&tmp, (size_t)ncol * 8), "tmp");
        cudaError_t e = launch_permute(tmp, srcs[k], b->d_perm, ncol, 1, 8, 1, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e == cudaSuccess) e = cudaMemcpy(outs[k], tmp, (size_t)ncol * 8, cudaMemcpyDeviceToHost);
        cudaFree(tmp);
        if (e != cudaSuccess) return cuda_err(e, "balance download");
    }
    return 0;
}

// Times `trial_steps` graph replays per candidate threads-per-block on the
// batch's own data and keeps the fastest; the state is restored afterwards.
extern "C" int32_t ctsmg_batch_autotune(ctsmg_batch bh, int32_t trial_steps, int32_t* block_out) {
    if (!bh) return set_error(CTSMG_E_ARG, "null batch", 0, 0);
    Batch* b = bh->b;
    if (trial_steps < 1) trial_steps = 1;
    if (!b->snapshot) CK(cudaMalloc(&b->snapshot, b->state_bytes), "snapshot");
    size_t off = 0;
    for (auto& f : b->fields) {
        CK(cudaMemcpyAsync((char*)b->snapshot + off, f.dptr, f.bytes, cudaMemcpyDeviceToDevice, b->stream), "snap");
        off += f.bytes;
    }
    const int cands[3] = {64, 128, 256};
    int best = b->block;
    float best_ms = 1e30f;
    for (int k = 0; k < 3; ++k) {
        b->block = cands[k];
        int rc = build_graph(b);
        if (rc) return rc;
        CK(cudaGraphLaunch(b->graph, b->stream), "warm");
        CK(cudaEventRecord(b->ev0, b->stream), "ev");
        for (int s = 0; s < trial_steps; ++s) CK(cudaGraphLaunch(b->graph, b->stream), "trial");
        CK(cudaEventRecord(b->ev1, b->stream), "ev");
        CK(cudaEventSynchronize(b->ev1), "ev sync");
        float ms;
        CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1), "elapsed");
        if (ms < best_ms) { best_ms = ms; best = cands[k]; }
    }
    off = 0;
    for (auto& f : b->fields) {
        CK(cudaMemcpyAsync(f.dptr, (char*)b->snapshot + off, f.bytes, cudaMemcpyDeviceToDevice, b->stream), "restore");
        off += f.bytes;
    }
    CK(cudaMemsetAsync(b->err, 0xff, sizeof(DevError), b->stream), "err reset");
    if (b->cfg.balance) {
        const int ncol = b->cfg.ncol;
        const size_t ssb = (size_t)ncol * (NLEVSNO + NLEVGRND) * 8, cb = (size_t)ncol * 8;
        CK(cudaMemsetAsync(b->bal_mem, 0, ssb + 6 * cb + 256, b->stream), "balance reset");
    }
    CK(cudaStreamSynchronize(b->stream), "sync");
    cudaFree(b->snapshot);
    b->snapshot = nullptr;
    b->block = best;
    int rc = build_graph(b);
    if (rc) return rc;
    if (block_out) *block_out = best;
    return 0;
}

// Moves every resident column component (and the per-column parameter
// buffers) to the column order `key`: a gather on the device from the order
// in force.  Only for batches without patches of their own in the step
// (no CanopyFluxes): patch arrays are indexed through col_patchi, which moves
// with its column.
static int reorder_columns(Batch* b, int key) {
    if (key == b->order_key) return 0;
    const int ncol = b->cfg.ncol;
    const std::vector<int32_t> np = column_order(key, b->key_snl, b->key_nbedrock, b->key_zwt);
    std::vector<int32_t> inv(ncol), g(ncol);
    for (int i = 0; i < ncol; ++i) inv[b->h_perm[i]] = i;
    for (int i = 0; i < ncol; ++i) g[i] = inv[np[i]];        // new position i <- current position g[i]
    size_t maxb = 8 * (size_t)ncol;
    for (auto& f : b->fields) maxb = std::max(maxb, f.bytes);
    int32_t* dg = nullptr;
    void* tmp = nullptr;
    cudaError_t e = cudaMalloc(&dg, (size_t)ncol * 4);
    if (e == cudaSuccess) e = cudaMalloc(&tmp, maxb);
    if (e == cudaSuccess) e = cudaMemcpy(dg, g.data(), (size_t)ncol * 4, cudaMemcpyHostToDevice);
    auto move = [&](void* p, int nlev, int esize, size_t bytes) {
        if (e == cudaSuccess) e = launch_permute(tmp, p, dg, ncol, nlev, esize, 0, b->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(p, tmp, bytes, cudaMemcpyDeviceToDevice, b->stream);
    };
    for (auto& f : b->fields)
        if (is_column_kind(f.kind)) move(f.dptr, kind_levels(f.kind), f.esize, f.bytes);
    if (b->hyd_params) {
        if (b->hya.baseflow_scalar_c) move(b->hyd_params, 1, 8, (size_t)ncol * 8);
        if (b->hya.fff_c) move(b->hyd_params + ncol, 1, 8, (size_t)ncol * 8);
    }
    if (b->dmax_c) move(b->dmax_c, 1, 8, (size_t)ncol * 8);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_perm, np.data(), (size_t)ncol * 4, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (dg) cudaFree(dg);
    if (tmp) cudaFree(tmp);
    if (e != cudaSuccess) return cuda_err(e, "column reorder");
    b->h_perm = np;
    b->order_key = key;
    return 0;
}

// Times trial_steps steps for every (column order, moisture-form work order,
// threads per block) candidate on the batch's own data and keeps the fastest;
// the state is restored (in the chosen column order) afterwards.  Column
// orders are tuned for batches without CanopyFluxes; the moisture-form work
// order (bucketed or filter order) for batches with the moisture form.
extern "C" int32_t ctsmg_batch_autotune2(ctsmg_batch bh, int32_t trial_steps, int32_t* block_out,
                                         int32_t* order_out, int32_t* mf_sort_out, float* ms_out,
                                         int32_t* ncand_out) {
    if (!bh) return set_error(CTSMG_E_ARG, "null batch", 0, 0);
    Batch* b = bh->b;
    if (trial_steps < 1) trial_steps = 1;
    const bool orders = !b->cfg.with_canopy && !b->key_snl.empty();
    const int norders = orders ? N_COLUMN_ORDERS : 1;
    const bool mf = b->mf_work != nullptr;
    const int nmf = mf ? 2 : 1;
    const int cands[3] = {64, 128, 256};
    const int key0 = b->order_key;
    const bool sort0 = b->mf_sort;
    if (!b->snapshot) CK(cudaMalloc(&b->snapshot, b->state_bytes), "snapshot");
    auto copy_state = [&](bool save) -> int {
        size_t off = 0;
        for (auto& f : b->fields) {
            void* snap = (char*)b->snapshot + off;
            CK(cudaMemcpyAsync(save ? snap : f.dptr, save ? f.dptr : snap, f.bytes, cudaMemcpyDeviceToDevice,
                               b->stream), "snapshot");
            off += f.bytes;
        }
        return 0;
    };
    int rc = 0;
    int best_block = b->block, best_key = key0;
    bool best_sort = sort0;
    float best_ms = 1e30f;
    for (int o = 0; o < norders; ++o) {
        const int key = orders ? o : key0;
        // the snapshot is taken in the candidate's column order, restored
        // after each timing, and the columns go back to the order in force
        if ((rc = reorder_columns(b, key)) || (rc = copy_state(true))) return rc;
        for (int m = 0; m < nmf; ++m) {
            b->mf_sort = mf ? (m == 0) : sort0;
            for (int k = 0; k < 3; ++k) {
                b->block = cands[k];
                if ((rc = build_graph(b))) return rc;
                CK(cudaGraphLaunch(b->graph, b->stream), "warm");
                CK(cudaEventRecord(b->ev0, b->stream), "ev");
                for (int st = 0; st < trial_steps; ++st) CK(cudaGraphLaunch(b->graph, b->stream), "trial");
                CK(cudaEventRecord(b->ev1, b->stream), "ev");
                CK(cudaEventSynchronize(b->ev1), "ev sync");
                float ms;
                CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1), "elapsed");
                ms /= trial_steps;
                if (ms_out) ms_out[(o * nmf + m) * 3 + k] = ms;
                if (ms < best_ms) { best_ms = ms; best_block = cands[k]; best_key = key; best_sort = b->mf_sort; }
            }
            if ((rc = copy_state(false))) return rc;
        }
        if ((rc = reorder_columns(b, key0))) return rc;
    }
    CK(cudaMemsetAsync(b->err, 0xff, sizeof(DevError), b->stream), "err reset");
    if (b->cfg.balance) {
        const int ncol = b->cfg.ncol;
        const size_t ssb = (size_t)ncol * (NLEVSNO + NLEVGRND) * 8, cb = (size_t)ncol * 8;
        CK(cudaMemsetAsync(b->bal_mem, 0, ssb + 6 * cb + 256, b->stream), "balance reset");
    }
    CK(cudaStreamSynchronize(b->stream), "sync");
    cudaFree(b->snapshot);
    b->snapshot = nullptr;
    if ((rc = reorder_columns(b, best_key))) return rc;
    b->block = best_block;
    b->mf_sort = best_sort;
    if ((rc = build_graph(b))) return rc;
    if (block_out) *block_out = best_block;
    if (order_out) *order_out = best_key;
    if (mf_sort_out) *mf_sort_out = mf ? (best_sort ? 1 : 0) : -1;
    if (ncand_out) *ncand_out = norders * nmf * 3;
    return 0;
}

extern "C" const char* ctsmg_batch_order_name(int32_t key) {
    return (key >= 0 && key < N_COLUMN_ORDERS) ? COLUMN_ORDER_NAMES[key] : "";
}

extern "C" int32_t ctsmg_batch_set_mf_order(ctsmg_batch bh, int32_t sorted) {
    if (!bh || (sorted != 0 && sorted != 1)) return set_error(CTSMG_E_ARG, "sorted must be 0 or 1", 0, 0);
    if (!bh->b->mf_work) return set_error(CTSMG_E_ARG, "the batch has no moisture form", 0, 0);
    bh->b->mf_sort = sorted == 1;
    return build_graph(bh->b);
}

extern "C" int32_t ctsmg_batch_set_block(ctsmg_batch bh, int32_t block) {
    if (!bh || (block != 64 && block != 128 && block != 256))
        return set_error(CTSMG_E_ARG, "block must be 64, 128 or 256", 0, 0);
    bh->b->block = block;
    return build_graph(bh->b);
}

// Host copy of one component in the caller's column order.
static int field_to_host(Batch* b, const UField& u, std::vector<char>& out) {
    out.resize(u.bytes);
    cudaError_t e;
    if (!is_column_kind(u.kind)) {
        e = cudaMemcpy(out.data(), u.dptr, u.bytes, cudaMemcpyDeviceToHost);
    } else {
        void* tmp = nullptr;
        e = cudaMalloc(&tmp, u.bytes);
        if (e == cudaSuccess) e = launch_permute(tmp, u.dptr, b->d_perm, b->cfg.ncol, kind_levels(u.kind), u.esize, 1, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (e == cudaSuccess) e = cudaMemcpy(out.data(), tmp, u.bytes, cudaMemcpyDeviceToHost);
        if (tmp) cudaFree(tmp);
    }
    return e == cudaSuccess ? 0 : cuda_err(e, "checkpoint D2H");
}

static int field_from_host(Batch* b, const UField& u, const std::vector<char>& in) {
    cudaError_t e;
    if (!is_column_kind(u.kind)) {
        e = cudaMemcpy(u.dptr, in.data(), u.bytes, cudaMemcpyHostToDevice);
    } else {
        void* tmp = nullptr;
        e = cudaMalloc(&tmp, u.bytes);
        if (e == cudaSuccess) e = cudaMemcpy(tmp, in.data(), u.bytes, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = launch_permute(u.dptr, tmp, b->d_perm, b->cfg.ncol, kind_levels(u.kind), u.esize, 0, b->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        if (tmp) cudaFree(tmp);
    }
    return e == cudaSuccess ? 0 : cuda_err(e, "restart H2D");
}

static const char CK_MAGIC[8] = {'C', 'T', 'S', 'M', 'G', 'C', 'K', '1'};

extern "C" int32_t ctsmg_batch_save(ctsmg_batch bh, const char* path) {
    if (!bh || !path) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    Batch* b = bh->b;
    CK(cudaStreamSynchronize(b->stream), "sync");
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_error(CTSMG_E_ARG, "cannot open the checkpoint file for writing", 0, 0);
    int rc = 0;
    const int32_t head[4] = {b->cfg.ncol, b->cfg.npatch, b->cfg.ngrid, (int32_t)b->fields.size()};
    bool ok = std::fwrite(CK_MAGIC, 1, 8, f) == 8 && std::fwrite(head, 4, 4, f) == 4;
    std::vector<char> buf;
    for (size_t i = 0; ok && i < b->fields.size(); ++i) {
        const UField& u = b->fields[i];
        if ((rc = field_to_host(b, u, buf))) break;
        const uint16_t nl = (uint16_t)u.name.size();
        const int32_t ke[2] = {u.kind, u.esize};
        const int64_t nb = (int64_t)u.bytes;
        ok = std::fwrite(&nl, 2, 1, f) == 1 && std::fwrite(u.name.data(), 1, nl, f) == nl &&
             std::fwrite(ke, 4, 2, f) == 2 && std::fwrite(&nb, 8, 1, f) == 1 &&
             std::fwrite(buf.data(), 1, u.bytes, f) == u.bytes;
    }
    if (std::fclose(f) != 0) ok = false;
    if (rc) return rc;
    return ok ? 0 : set_error(CTSMG_E_ARG, "writing the checkpoint file failed", 0, 0);
}

extern "C" int32_t ctsmg_batch_load(ctsmg_batch bh, const char* path) {
    if (!bh || !path) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    Batch* b = bh->b;
    CK(cudaStreamSynchronize(b->stream), "sync");
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_error(CTSMG_E_ARG, "cannot open the checkpoint file", 0, 0);
    auto bad = [&](const char* m) { std::fclose(f); return set_error(CTSMG_E_ARG, m, 0, 0); };
    char magic[8];
    int32_t head[4];
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, CK_MAGIC, 8) != 0) return bad("not a checkpoint file");
    if (std::fread(head, 4, 4, f) != 4) return bad("truncated checkpoint header");
    if (head[0] != b->cfg.ncol || head[1] != b->cfg.npatch || head[2] != b->cfg.ngrid)
        return bad("checkpoint sizes differ from the batch's (ncol, npatch, ngrid)");
    std::vector<char> seen(b->fields.size(), 0), buf;
    for (int32_t r = 0; r < head[3]; ++r) {
        uint16_t nl;
        int32_t ke[2];
        int64_t nb;
        if (std::fread(&nl, 2, 1, f) != 1) return bad("truncated checkpoint record");
        std::string name(nl, '\0');
        if (std::fread(&name[0], 1, nl, f) != nl || std::fread(ke, 4, 2, f) != 2 || std::fread(&nb, 8, 1, f) != 1)
            return bad("truncated checkpoint record");
        auto it = b->index.find(name);
        if (it == b->index.end()) {               // a component this batch does not hold
            if (std::fseek(f, (long)nb, SEEK_CUR) != 0) return bad("truncated checkpoint record");
            continue;
        }
        const UField& u = b->fields[it->second];
        if (ke[0] != u.kind || ke[1] != u.esize || (size_t)nb != u.bytes)
            return bad("checkpoint component has another layout than the batch's");
        buf.resize(u.bytes);
        if (std::fread(buf.data(), 1, u.bytes, f) != u.bytes) return bad("truncated checkpoint data");
        int rc = field_from_host(b, u, buf);
        if (rc) { std::fclose(f); return rc; }
        seen[it->second] = 1;
    }
    std::fclose(f);
    for (size_t i = 0; i < seen.size(); ++i)
        if (!seen[i]) return set_error(CTSMG_E_ARG, (std::string("checkpoint lacks component ") + b->fields[i].name).c_str(), 0, 0);
    return 0;
}

extern "C" int64_t ctsmg_batch_state_bytes(ctsmg_batch bh) { return bh ? (int64_t)bh->b->state_bytes : 0; }

extern "C" int32_t ctsmg_batch_destroy(ctsmg_batch bh) {
    if (!bh) return 0;
    batch_free(bh->b);
    delete bh;
    return 0;
}
