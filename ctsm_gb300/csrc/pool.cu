// pool.cu -- serving mode: a device-resident pool of column, patch and
// gridcell slots.  Run requests are admitted into free slot ranges while
// other requests are running, every tick advances all running requests by
// one model step through one CUDA graph over filters of the active slots,
// and finished requests are copied out and their ranges freed.
//
// The step is the batch engine's (optionally the root moisture stress, then
// CanopyFluxes, root sink, SoilTemperature, SoilWater -- optionally inside the
// aquifer-layer hydrology -- and the h2osoi_vol refresh in the order of
// src/main/clm_driver.F90:709, 766, 900, 950; or SoilWater then
// SoilTemperature without the canopy), run over
// the filter of active positions the way the reference runs each clump over
// filter_nolakec / filter_exposedvegp.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#include "ctsm_gpu.h"
#include "ctsm_device.cuh"
#include "soil_kernels.cuh"
#include "canopy_kernels.cuh"
#include "rootmoist_kernels.cuh"
#include "moisture_form_kernels.cuh"
#include "capi_internal.h"

namespace ctsmg {

// First-fit allocator of contiguous ranges in [0, cap) with coalescing.
struct RangeAlloc {
    int cap = 0;
    std::map<int, int> free_;                    // start -> length
    void init(int n) { cap = n; free_.clear(); if (n > 0) free_[0] = n; }
    bool take(int n, int* start) {
        if (n == 0) { *start = 0; return true; }
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *start = it->first;
                const int rest = it->second - n, s = it->first + n;
                free_.erase(it);
                if (rest > 0) free_[s] = rest;
                return true;
            }
        }
        return false;
    }
    void give(int start, int n) {
        if (n == 0) return;
        auto it = free_.emplace(start, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
        }
    }
    int largest() const { int m = 0; for (auto& kv : free_) m = std::max(m, kv.second); return m; }
};

struct PField {
    std::string name;
    int kind, esize, use;
    void* dptr = nullptr;
};

enum ReqState { R_FREE, R_RUNNING, R_DONE };

struct Request {
    int state = R_FREE;
    int c0 = 0, nc = 0, p0 = 0, np = 0, g0 = 0, ng = 0;
    int nsteps = 0, enq = 0;
    cudaEvent_t done = nullptr;               // recorded after its last enqueued step
    std::vector<int32_t> perm;                // pool position c0 + i holds the request's column perm[i]
};

struct Pool {
    ctsmg_pool_config cfg{};
    std::vector<PField> fields;
    std::map<std::string, int> index;
    ctsmg_soilwater_io dsw{};
    ctsmg_soiltemp_io dst{};
    ctsmg_rootmoist_io drm{};
    HydroStepArgs hya{};
    CanopyArgs cargs{};
    double* rootr = nullptr;
    double* mslope = nullptr;
    double* mint = nullptr;
    int* counter = nullptr;
    double* cws = nullptr;                    // CanopyFluxes iteration records
    double* ws = nullptr;
    DevError* err = nullptr;
    int32_t* d_cfilt = nullptr;
    int32_t* d_pfilt = nullptr;
    int32_t* h_cfilt = nullptr;               // pinned staging of the filters
    int32_t* h_pfilt = nullptr;
    cudaEvent_t filt_ev = nullptr;            // last filter upload
    int ncol_act = 0, npat_act = 0;
    bool dirty = true;
    RangeAlloc cols, pats, grids;
    std::vector<Request> req;
    cudaStream_t stream = nullptr, copy = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::vector<cudaEvent_t> ring;
    size_t ring_next = 0, ring_used = 0;
    int block = 128;
};

static int pcuda(cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return set_error(CTSMG_E_CUDA, m.c_str(), 0, 0);
}
#define PK(call, where) do { cudaError_t _e = (call); if (_e != cudaSuccess) return pcuda(_e, where); } while (0)

static void* fptr(const void* io, const FieldDesc& f) {
    return *reinterpret_cast<void* const*>(reinterpret_cast<const char*>(io) + f.offset);
}
static void set_fptr(void* io, const FieldDesc& f, void* p) {
    *reinterpret_cast<void**>(reinterpret_cast<char*>(io) + f.offset) = p;
}
static bool patch_kind(int k) { return k == K_P || k == K_PL || k == K_PS || k == K_PG; }

// Capacity (leading dimension) and first position of a field's kind.
static int kind_cap(const Pool* P, int k) {
    return patch_kind(k) ? P->cfg.patch_capacity : (k == K_GR ? P->cfg.grid_capacity : P->cfg.col_capacity);
}
static int kind_start(const Request& r, int k) { return patch_kind(k) ? r.p0 : (k == K_GR ? r.g0 : r.c0); }
static int kind_count(const Request& r, int k) { return patch_kind(k) ? r.np : (k == K_GR ? r.ng : r.nc); }

// The aquifer-layer hydrology around the Zeng-Decker form (the batch
// engine's tables): saturated excess, infiltration, water table, drainage;
// eff_porosity, which SetSoilWaterFractions writes in the step, is the
// pool's own (neither copied in nor out).
static const FieldDesc* const HYD_TABS[4] = {HYD_SAT_TABLE, HYD_INF_TABLE, HYD_WT_TABLE, HYD_DR_TABLE};
static const int* const HYD_NS[4] = {&HYD_SAT_TABLE_N, &HYD_INF_TABLE_N, &HYD_WT_TABLE_N, &HYD_DR_TABLE_N};
static const FieldDesc POOL_EFFPOR[] = {{offsetof(ctsmg_soilwater_io, eff_porosity), K_G, 8, U_OUT, "eff_porosity"}};

static void for_tables(const ctsmg_pool_config& c, void (*fn)(const FieldDesc&, void*), void* ctx) {
    for (int i = 0; i < SOILWATER_NFIELDS; ++i) fn(SOILWATER_TABLE[i], ctx);
    for (int i = 0; i < SOILTEMP_NFIELDS; ++i) fn(SOILTEMP_TABLE[i], ctx);
    if (c.with_canopy)
        for (int i = 0; i < CANOPY_NFIELDS; ++i) fn(CANOPY_TABLE[i], ctx);
    if (c.with_canopy && c.rootmoist)
        for (int i = 0; i < ROOTMOIST_NFIELDS; ++i) fn(ROOTMOIST_TABLE[i], ctx);
    if (c.hydrology) {
        for (int t = 0; t < 4; ++t)
            for (int i = 0; i < *HYD_NS[t]; ++i) fn(HYD_TABS[t][i], ctx);
        fn(POOL_EFFPOR[0], ctx);
    }
}

struct SlotBytes { int64_t c = 0, p = 0, g = 0; std::map<std::string, int> seen; };

static void add_slot_bytes(const FieldDesc& f, void* ctx) {
    SlotBytes* s = (SlotBytes*)ctx;
    if (s->seen.count(f.name)) return;
    s->seen[f.name] = 1;
    const int64_t b = (int64_t)kind_levels(f.kind) * f.esize;
    if (patch_kind(f.kind)) s->p += b;
    else if (f.kind == K_GR) s->g += b;
    else s->c += b;
}

static void slot_bytes(const ctsmg_pool_config& cfg, int64_t* cb, int64_t* pb, int64_t* gb) {
    SlotBytes s;
    const int with_canopy = cfg.with_canopy;
    for_tables(cfg, add_slot_bytes, &s);
    s.c += (int64_t)SOILTEMP_WS_DOUBLES_PER_COL * 8 + 4;            // band scratch, filter entry
    if (with_canopy)       // rootr, Medlyn slope/intercept, filter, iteration record
        s.p += (int64_t)NLEVSOI * 8 + 2 * 8 + 4 + (int64_t)canopy_ws_bytes_per_patch();
    else s.p += 4;
    *cb = s.c; *pb = s.p; *gb = s.g;
}

static cudaError_t enqueue_tick(Pool* P) {
    cudaError_t e = cudaSuccess;
    const int nc = P->ncol_act;
    if (P->cfg.with_canopy) {
        if (P->cfg.rootmoist) {
            e = launch_rootmoist(P->drm, P->cargs.pft, 1, 1, P->npat_act, P->d_pfilt, P->stream);
            if (e != cudaSuccess) return e;
        }
        e = launch_canopy(P->cargs, P->npat_act, P->d_pfilt, P->cfg.dtime, P->counter, P->err, P->cws, P->stream);
        if (e != cudaSuccess) return e;
        e = launch_rootsink(P->dst.col_patchi, P->dst.col_npatches, P->dst.wtcol, P->cargs.io.qflx_tran_veg,
                            P->cfg.rootmoist ? P->drm.rootr : P->rootr,
                            P->cfg.patch_capacity, (double*)P->dsw.qflx_rootsoi, nc, P->stream, P->cfg.col_capacity,
                            P->d_cfilt);
        if (e != cudaSuccess) return e;
    }
    const int ord = P->cfg.with_canopy ? 1 : 0;
    if (!P->cfg.hydrology)
        return launch_soilstep(P->dsw, P->dst, nc, P->cfg.e_ice, P->cfg.dtime, P->cfg.snow_thermal_cond_method, P->ws,
                               P->cfg.col_capacity, P->err, P->stream, P->block, ord, P->d_cfilt);
    // SoilWater with the hydrology in its own kernel, before the heat solve
    // without the canopy (order 0) and after it with (order 1)
    if (ord == 0) {
        e = launch_zd09_step(P->dsw, nc, P->cfg.e_ice, P->cfg.dtime, 0, 0, P->d_cfilt, P->stream, &P->hya);
        if (e != cudaSuccess) return e;
    }
    SoilStepFlags fl;
    fl.water = 0;
    fl.flexcn = 0;
    fl.refresh = ord == 0 ? 1 : 0;
    e = launch_soilstep(P->dsw, P->dst, nc, P->cfg.e_ice, P->cfg.dtime, P->cfg.snow_thermal_cond_method, P->ws,
                        P->cfg.col_capacity, P->err, P->stream, P->block, ord, P->d_cfilt, nullptr, fl);
    if (e != cudaSuccess || ord == 0) return e;
    return launch_zd09_step(P->dsw, nc, P->cfg.e_ice, P->cfg.dtime, 0, 1, P->d_cfilt, P->stream, &P->hya);
}

// Filters of the running requests in pool-position order (each request's
// columns sit in its range sorted by (snl, nbedrock, water-table depth), so
// consecutive threads read consecutive columns of the same bucket), uploaded
// in stream order, and the tick graph.
static int rebuild(Pool* P) {
    PK(cudaEventSynchronize(P->filt_ev), "filter staging");
    std::vector<const Request*> run;
    for (auto& r : P->req) if (r.state == R_RUNNING) run.push_back(&r);
    std::sort(run.begin(), run.end(), [](const Request* a, const Request* b) { return a->c0 < b->c0; });
    int nc = 0, np = 0;
    for (const Request* r : run) {
        for (int c = r->c0; c < r->c0 + r->nc; ++c) P->h_cfilt[nc++] = c + 1;
        for (int p = r->p0; p < r->p0 + r->np; ++p) P->h_pfilt[np++] = p + 1;
    }
    P->ncol_act = nc;
    P->npat_act = np;
    if (nc > 0) PK(cudaMemcpyAsync(P->d_cfilt, P->h_cfilt, (size_t)nc * 4, cudaMemcpyHostToDevice, P->stream), "filter");
    if (np > 0) PK(cudaMemcpyAsync(P->d_pfilt, P->h_pfilt, (size_t)np * 4, cudaMemcpyHostToDevice, P->stream), "filter");
    PK(cudaEventRecord(P->filt_ev, P->stream), "filter event");
    if (P->graph) { cudaGraphExecDestroy(P->graph); P->graph = nullptr; }
    if (nc > 0) {
        cudaGraph_t g;
        PK(cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal), "capture");
        cudaError_t le = enqueue_tick(P);
        cudaError_t ce = cudaStreamEndCapture(P->stream, &g);
        if (le != cudaSuccess) return pcuda(le, "tick capture");
        if (ce != cudaSuccess) return pcuda(ce, "cudaStreamEndCapture");
        cudaError_t ie = cudaGraphInstantiate(&P->graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) return pcuda(ie, "cudaGraphInstantiate");
    }
    P->dirty = false;
    return 0;
}

static void pool_free(Pool* P) {
    if (!P) return;
    if (P->stream) cudaStreamSynchronize(P->stream);
    if (P->copy) cudaStreamSynchronize(P->copy);
    if (P->graph) cudaGraphExecDestroy(P->graph);
    for (auto& f : P->fields) if (f.dptr) cudaFree(f.dptr);
    for (void* p : {(void*)P->rootr, (void*)P->mslope, (void*)P->mint, (void*)P->counter, (void*)P->cws, (void*)P->ws, (void*)P->err,
                    (void*)P->d_cfilt, (void*)P->d_pfilt})
        if (p) cudaFree(p);
    if (P->h_cfilt) cudaFreeHost(P->h_cfilt);
    if (P->h_pfilt) cudaFreeHost(P->h_pfilt);
    for (auto& r : P->req) if (r.done) cudaEventDestroy(r.done);
    for (auto ev : P->ring) if (ev) cudaEventDestroy(ev);
    if (P->filt_ev) cudaEventDestroy(P->filt_ev);
    if (P->stream) cudaStreamDestroy(P->stream);
    if (P->copy) cudaStreamDestroy(P->copy);
    delete P;
}

// Strided copy of one field between a request's dense host array and its
// range in the pool (level-major, capacity as leading dimension).
static cudaError_t copy_field(const Pool* P, const PField& f, const Request& r, void* host, bool to_device) {
    const int n = kind_count(r, f.kind);
    if (n == 0) return cudaSuccess;
    const size_t w = (size_t)n * f.esize, pitch = (size_t)kind_cap(P, f.kind) * f.esize;
    char* dev = (char*)f.dptr + (size_t)kind_start(r, f.kind) * f.esize;
    const int h = kind_levels(f.kind);
    if (to_device) return cudaMemcpy2DAsync(dev, pitch, host, w, w, h, cudaMemcpyHostToDevice, P->copy);
    return cudaMemcpy2DAsync(host, w, dev, pitch, w, h, cudaMemcpyDeviceToHost, P->copy);
}

} // namespace ctsmg

using namespace ctsmg;

struct ctsmg_pool_s { Pool* P; };

extern "C" int32_t ctsmg_pool_slot_bytes_cfg(const ctsmg_pool_config* cfg, int64_t* col_bytes, int64_t* patch_bytes,
                                             int64_t* grid_bytes) {
    if (!cfg) return set_error(CTSMG_E_ARG, "null configuration", 0, 0);
    int64_t c, p, g;
    slot_bytes(*cfg, &c, &p, &g);
    if (col_bytes) *col_bytes = c;
    if (patch_bytes) *patch_bytes = p;
    if (grid_bytes) *grid_bytes = g;
    return 0;
}

extern "C" int32_t ctsmg_pool_slot_bytes(int32_t with_canopy, int64_t* col_bytes, int64_t* patch_bytes,
                                         int64_t* grid_bytes) {
    int64_t c, p, g;
    ctsmg_pool_config cfg{};
    cfg.with_canopy = with_canopy;
    slot_bytes(cfg, &c, &p, &g);
    if (col_bytes) *col_bytes = c;
    if (patch_bytes) *patch_bytes = p;
    if (grid_bytes) *grid_bytes = g;
    return 0;
}

extern "C" int32_t ctsmg_pool_create(ctsmg_pool* out, const ctsmg_pool_config* cfg, const ctsmg_canopy_params* cpar,
                                     const ctsmg_pftcon* pft) {
    if (!out || !cfg) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    if (cfg->col_capacity <= 0 || cfg->patch_capacity <= 0 || cfg->grid_capacity < 0)
        return set_error(CTSMG_E_ARG, "pool column and patch capacities must be positive", 0, 0);
    if (!(cfg->dtime > 0.0)) return set_error(CTSMG_E_ARG, "dtime must be positive", 0, 0);
    if (cfg->with_canopy && (!cpar || !pft || cfg->patch_capacity <= 0 || cfg->grid_capacity <= 0))
        return set_error(CTSMG_E_ARG, "with_canopy needs params, pftcon, patch and gridcell capacity", 0, 0);
    if (cfg->rootmoist && !cfg->with_canopy)
        return set_error(CTSMG_E_ARG, "rootmoist needs with_canopy", 0, 0);
    const ctsmg_soilwater_movement_nml swm = current_soilwater_nml();
    if (swm.soilwater_movement_method != 0 || swm.use_flexibleCN)
        return set_error(CTSMG_E_UNSUPPORTED, "the serving pool steps the Zeng-Decker form without the flexibleCN fix",
                         0, 0);
    Pool* P = new Pool();
    P->cfg = *cfg;
    if (P->cfg.max_inflight < 1) P->cfg.max_inflight = 1;
    auto fail = [&](int rc) { pool_free(P); return rc; };
    cudaError_t e;
    const int CC = cfg->col_capacity, PC = cfg->patch_capacity, GC = cfg->grid_capacity;
    if ((e = cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(pcuda(e, "stream"));
    if ((e = cudaStreamCreateWithFlags(&P->copy, cudaStreamNonBlocking)) != cudaSuccess) return fail(pcuda(e, "stream"));
    if ((e = cudaEventCreateWithFlags(&P->filt_ev, cudaEventDisableTiming)) != cudaSuccess) return fail(pcuda(e, "event"));
    P->ring.assign(P->cfg.max_inflight, nullptr);
    for (auto& ev : P->ring)
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return fail(pcuda(e, "event"));

    auto add = [&](const FieldDesc* tab, int nf, void* dio) -> int {
        for (int i = 0; i < nf; ++i) {
            const FieldDesc& f = tab[i];
            auto it = P->index.find(f.name);
            if (it == P->index.end()) {
                PField u;
                u.name = f.name; u.kind = f.kind; u.esize = f.esize; u.use = f.use;
                const size_t bytes = field_bytes(f, CC, PC, GC);
                cudaError_t ee = cudaMalloc(&u.dptr, bytes);
                if (ee != cudaSuccess) return pcuda(ee, "cudaMalloc(pool field)");
                ee = cudaMemset(u.dptr, 0, bytes);
                if (ee != cudaSuccess) { cudaFree(u.dptr); return pcuda(ee, "cudaMemset(pool field)"); }
                P->index[f.name] = (int)P->fields.size();
                P->fields.push_back(u);
                it = P->index.find(f.name);
            } else if (P->fields[it->second].use == U_IN && f.use != U_IN) {
                P->fields[it->second].use = f.use;
            }
            set_fptr(dio, f, P->fields[it->second].dptr);
        }
        return 0;
    };
    int rc;
    P->dsw.ldc = CC;
    P->dst.ldc = CC;
    P->dst.ldp = PC;
    if ((rc = add(SOILWATER_TABLE, SOILWATER_NFIELDS, &P->dsw))) return fail(rc);
    if ((rc = add(SOILTEMP_TABLE, SOILTEMP_NFIELDS, &P->dst))) return fail(rc);
    if (cfg->with_canopy) {
        P->cargs.io.ldp = PC; P->cargs.io.ldc = CC; P->cargs.io.ldg = GC; P->cargs.io.begg = 1;
        if ((rc = add(CANOPY_TABLE, CANOPY_NFIELDS, &P->cargs.io))) return fail(rc);
        P->cargs.par = *cpar;
        P->cargs.pft = *pft;
        P->cargs.method = cfg->stomatalcond_method;
        P->cargs.itmax = cfg->itmax_canopy_fluxes;
        P->cargs.begc = 1;
        P->cargs.begp = 1;
        P->cargs.engine = 1;
        const size_t pb = (size_t)PC * 8;
        if ((e = cudaMalloc(&P->rootr, pb * NLEVSOI)) != cudaSuccess) return fail(pcuda(e, "rootr"));
        if ((e = cudaMalloc(&P->mslope, pb)) != cudaSuccess) return fail(pcuda(e, "mslope"));
        if ((e = cudaMalloc(&P->mint, pb)) != cudaSuccess) return fail(pcuda(e, "mint"));
        P->cargs.medlynslope_p = P->mslope;
        P->cargs.medlynintercept_p = P->mint;
        if ((e = cudaMalloc(&P->counter, 256)) != cudaSuccess) return fail(pcuda(e, "counter"));
        if ((e = cudaMalloc(&P->cws, canopy_ws_bytes(PC))) != cudaSuccess) return fail(pcuda(e, "canopy ws"));
        if (cfg->rootmoist) {
            P->drm.ldc = CC;
            P->drm.ldp = PC;
            if ((rc = add(ROOTMOIST_TABLE, ROOTMOIST_NFIELDS, &P->drm))) return fail(rc);
        }
    }
    if (cfg->hydrology) {
        P->hya.io.ldc = CC;
        for (int t = 0; t < 4; ++t)
            if ((rc = add(HYD_TABS[t], *HYD_NS[t], &P->hya.io))) return fail(rc);
        if ((rc = add(POOL_EFFPOR, 1, &P->dsw))) return fail(rc);
        P->hya.par = current_soilhydrology_params();
        P->hya.baseflow_scalar_c = nullptr;
        P->hya.fff_c = nullptr;
    }
    if ((e = cudaMalloc(&P->ws, (size_t)SOILTEMP_WS_DOUBLES_PER_COL * CC * 8)) != cudaSuccess) return fail(pcuda(e, "ws"));
    if ((e = cudaMalloc(&P->err, sizeof(DevError))) != cudaSuccess) return fail(pcuda(e, "err"));
    if ((e = cudaMemset(P->err, 0xff, sizeof(DevError))) != cudaSuccess) return fail(pcuda(e, "err"));
    if ((e = cudaMalloc(&P->d_cfilt, (size_t)CC * 4)) != cudaSuccess) return fail(pcuda(e, "filter"));
    if ((e = cudaHostAlloc(&P->h_cfilt, (size_t)CC * 4, cudaHostAllocDefault)) != cudaSuccess) return fail(pcuda(e, "filter"));
    if ((e = cudaMalloc(&P->d_pfilt, (size_t)PC * 4)) != cudaSuccess) return fail(pcuda(e, "filter"));
    if ((e = cudaHostAlloc(&P->h_pfilt, (size_t)PC * 4, cudaHostAllocDefault)) != cudaSuccess) return fail(pcuda(e, "filter"));
    if ((e = cudaEventRecord(P->filt_ev, P->stream)) != cudaSuccess) return fail(pcuda(e, "event"));
    P->cols.init(CC);
    P->pats.init(PC);
    P->grids.init(GC);
    *out = new ctsmg_pool_s{P};
    return 0;
}

extern "C" int32_t ctsmg_pool_admit(ctsmg_pool ph, int32_t ncol, int32_t npatch, int32_t ngrid, int32_t nsteps,
                                    const ctsmg_soilwater_io* sw, const ctsmg_soiltemp_io* st,
                                    const ctsmg_canopy_io* cio, const double* rootr, const double* medlynslope_p,
                                    const double* medlynintercept_p, int32_t* slot_out) {
    ctsmg_pool_request R{ncol, npatch, ngrid, nsteps, sw, st, cio, nullptr, nullptr, rootr, medlynslope_p,
                         medlynintercept_p};
    return ctsmg_pool_admit_request(ph, &R, slot_out);
}

extern "C" int32_t ctsmg_pool_admit_request(ctsmg_pool ph, const ctsmg_pool_request* req, int32_t* slot_out) {
    if (!ph || !req || !slot_out) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    const int32_t ncol = req->ncol, npatch = req->npatch, ngrid = req->ngrid, nsteps = req->nsteps;
    const ctsmg_soilwater_io* sw = req->sw;
    const ctsmg_soiltemp_io* st = req->st;
    const ctsmg_canopy_io* cio = req->cio;
    const ctsmg_rootmoist_io* rm = req->rm;
    const ctsmg_hydrology_io* hyio = req->hy;
    const double* rootr = req->rootr;
    const double* medlynslope_p = req->medlynslope_p;
    const double* medlynintercept_p = req->medlynintercept_p;
    if (!sw || !st) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    Pool* P = ph->P;
    const bool can = P->cfg.with_canopy != 0;
    const bool rms = can && P->cfg.rootmoist != 0;
    const bool hyd = P->cfg.hydrology != 0;
    if (hyd && (!hyio || hyio->ldc != ncol))
        return set_error(CTSMG_E_ARG, "a hydrology pool needs the request's hydrology components (dense)", 0, 0);
    if (ncol <= 0 || npatch < 0 || ngrid < 0 || nsteps < 1) return set_error(CTSMG_E_ARG, "bad request sizes", 0, 0);
    if (sw->ldc != ncol || st->ldc != ncol || st->ldp != npatch)
        return set_error(CTSMG_E_ARG, "request arrays must be dense: ldc = ncol, ldp = npatch", 0, 0);
    if (can && (!cio || (!rootr && !rms) || cio->ldc != ncol || cio->ldp != npatch || cio->ldg != ngrid ||
                cio->begg != 1))
        return set_error(CTSMG_E_ARG, "canopy request needs cio (ldg = ngrid, begg = 1) and rootr", 0, 0);
    if (rms && (!rm || rm->ldc != ncol || rm->ldp != npatch))
        return set_error(CTSMG_E_ARG, "a rootmoist pool needs the request's root moisture stress components (dense)",
                         0, 0);
    for (int c = 0; c < ncol; ++c) {
        const int s = st->snl[c], pi = st->col_patchi[c], np = st->col_npatches[c], nb = st->nbedrock[c];
        if (s > 0 || s < -NLEVSNO) return set_error(CTSMG_E_ARG, "snl outside -nlevsno..0", c + 1, 0);
        if (nb < 1 || nb > NLEVGRND) return set_error(CTSMG_E_ARG, "nbedrock outside 1..nlevgrnd", c + 1, 0);
        if (np < 0 || pi < 1 || pi + np - 1 > npatch)
            return set_error(CTSMG_E_ARG, "column patches outside 1..npatch", c + 1, 0);
    }
    if (can)
        for (int p = 0; p < npatch; ++p) {
            const int cc = cio->patch_column[p], gg = cio->patch_gridcell[p], it = cio->itype[p];
            if (cc < 1 || cc > ncol || gg < 1 || gg > ngrid || it < 0 || it >= P->cargs.pft.npft)
                return set_error(CTSMG_E_ARG, "patch column / gridcell / itype out of range", p + 1, 0);
        }
    Request r;
    if (!P->cols.take(ncol, &r.c0)) return set_error(CTSMG_E_FULL, "pool: no free column range", ncol, 0);
    if (!P->pats.take(npatch, &r.p0)) {
        P->cols.give(r.c0, ncol);
        return set_error(CTSMG_E_FULL, "pool: no free patch range", npatch, 0);
    }
    if (!P->grids.take(ngrid, &r.g0)) {
        P->cols.give(r.c0, ncol);
        P->pats.give(r.p0, npatch);
        return set_error(CTSMG_E_FULL, "pool: no free gridcell range", ngrid, 0);
    }
    r.nc = ncol; r.np = npatch; r.ng = ngrid; r.nsteps = nsteps; r.enq = 0;
    auto release = [&]() { P->cols.give(r.c0, r.nc); P->pats.give(r.p0, r.np); P->grids.give(r.g0, r.ng); };
    // the request's columns in bucket order: more snow layers, shallower
    // bedrock, shallower water table (the batch engine's order)
    r.perm.resize(ncol);
    std::vector<int32_t> inv(ncol);
    for (int i = 0; i < ncol; ++i) r.perm[i] = i;
    std::stable_sort(r.perm.begin(), r.perm.end(), [&](int a, int b) {
        if (st->snl[a] != st->snl[b]) return st->snl[a] < st->snl[b];
        if (st->nbedrock[a] != st->nbedrock[b]) return st->nbedrock[a] < st->nbedrock[b];
        return sw->zwt[a] < sw->zwt[b];
    });
    bool identity = true;
    for (int i = 0; i < ncol; ++i) { inv[r.perm[i]] = i; identity = identity && r.perm[i] == i; }
    if (identity) r.perm.clear();
    // index components rebased to the pool positions
    std::vector<int32_t> patchi(ncol), pcol, pgrid;
    for (int i = 0; i < ncol; ++i) patchi[i] = st->col_patchi[identity ? i : r.perm[i]] + r.p0;
    if (can) {
        pcol.resize(npatch);
        pgrid.assign(cio->patch_gridcell, cio->patch_gridcell + npatch);
        for (int p = 0; p < npatch; ++p) pcol[p] = inv[cio->patch_column[p] - 1] + 1 + r.c0;
        for (auto& v : pgrid) v += r.g0;
    }
    std::vector<double> ms, mi;
    std::vector<char> gathered;
    auto upload = [&](const FieldDesc* tab, int nf, const void* hio) -> cudaError_t {
        for (int i = 0; i < nf; ++i) {
            const FieldDesc& f = tab[i];
            const PField& u = P->fields[P->index[f.name]];
            const void* hp = fptr(hio, f);
            if (!hp) return cudaErrorInvalidValue;
            if (u.name == "col_patchi") hp = patchi.data();
            else if (u.name == "patch_column") hp = pcol.data();
            else if (u.name == "patch_gridcell") hp = pgrid.data();
            else if (!identity && !patch_kind(u.kind) && u.kind != K_GR) {
                const int lev = kind_levels(u.kind), es = u.esize;
                gathered.resize((size_t)lev * ncol * es);
                const char* src = static_cast<const char*>(hp);
                for (int l = 0; l < lev; ++l)
                    for (int c = 0; c < ncol; ++c)
                        std::memcpy(&gathered[((size_t)l * ncol + c) * es], src + ((size_t)l * ncol + r.perm[c]) * es, es);
                hp = gathered.data();
            }
            cudaError_t ee = copy_field(P, u, r, const_cast<void*>(hp), true);
            if (ee == cudaSuccess && hp == gathered.data()) ee = cudaStreamSynchronize(P->copy);   // buffer reused
            if (ee != cudaSuccess) return ee;
        }
        return cudaSuccess;
    };
    cudaError_t e = upload(SOILWATER_TABLE, SOILWATER_NFIELDS, sw);
    if (e == cudaSuccess) e = upload(SOILTEMP_TABLE, SOILTEMP_NFIELDS, st);
    if (e == cudaSuccess && can) e = upload(CANOPY_TABLE, CANOPY_NFIELDS, cio);
    if (e == cudaSuccess && rms) e = upload(ROOTMOIST_TABLE, ROOTMOIST_NFIELDS, rm);
    for (int t = 0; t < 4 && hyd && e == cudaSuccess; ++t) e = upload(HYD_TABS[t], *HYD_NS[t], hyio);
    if (e == cudaSuccess && can && npatch > 0) {
        if (rootr)
            e = cudaMemcpy2DAsync(P->rootr + r.p0, (size_t)P->cfg.patch_capacity * 8, rootr, (size_t)npatch * 8,
                                  (size_t)npatch * 8, NLEVSOI, cudaMemcpyHostToDevice, P->copy);
        ms.resize(npatch); mi.resize(npatch);
        for (int p = 0; p < npatch; ++p) {
            ms[p] = medlynslope_p ? medlynslope_p[p] : P->cargs.pft.medlynslope[cio->itype[p]];
            mi[p] = medlynintercept_p ? medlynintercept_p[p] : P->cargs.pft.medlynintercept[cio->itype[p]];
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(P->mslope + r.p0, ms.data(), (size_t)npatch * 8, cudaMemcpyHostToDevice, P->copy);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(P->mint + r.p0, mi.data(), (size_t)npatch * 8, cudaMemcpyHostToDevice, P->copy);
    }
    cudaError_t se = cudaStreamSynchronize(P->copy);
    if (e == cudaSuccess) e = se;
    if (e != cudaSuccess) { release(); return e == cudaErrorInvalidValue ? set_error(CTSMG_E_ARG, "null component", 0, 0)
                                                                          : pcuda(e, "admit copy"); }
    int slot = -1;
    for (size_t i = 0; i < P->req.size(); ++i) if (P->req[i].state == R_FREE) { slot = (int)i; break; }
    if (slot < 0) { slot = (int)P->req.size(); P->req.emplace_back(); }
    Request& dst = P->req[slot];
    cudaEvent_t ev = dst.done;
    if (!ev && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) { release(); return pcuda(e, "event"); }
    dst = r;
    dst.done = ev;
    dst.state = R_RUNNING;
    P->dirty = true;
    *slot_out = slot;
    return 0;
}

extern "C" int32_t ctsmg_pool_tick(ctsmg_pool ph, int64_t* ncol_stepped) {
    if (!ph) return set_error(CTSMG_E_ARG, "null pool", 0, 0);
    Pool* P = ph->P;
    if (ncol_stepped) *ncol_stepped = 0;
    int rc;
    if (P->dirty && (rc = rebuild(P))) return rc;
    if (P->ncol_act == 0) return 0;
    if (P->ring_used == P->ring.size()) {           // bound the ticks queued ahead of the device
        PK(cudaEventSynchronize(P->ring[P->ring_next]), "tick throttle");
        --P->ring_used;
    }
    PK(cudaGraphLaunch(P->graph, P->stream), "cudaGraphLaunch");
    PK(cudaEventRecord(P->ring[P->ring_next], P->stream), "tick event");
    P->ring_next = (P->ring_next + 1) % P->ring.size();
    ++P->ring_used;
    for (auto& r : P->req) {
        if (r.state != R_RUNNING) continue;
        if (++r.enq == r.nsteps) {
            PK(cudaEventRecord(r.done, P->stream), "done event");
            r.state = R_DONE;
            P->dirty = true;
        }
    }
    if (ncol_stepped) *ncol_stepped = P->ncol_act;
    return 0;
}

extern "C" int32_t ctsmg_pool_poll(ctsmg_pool ph, int32_t* slots, int32_t cap, int32_t* n) {
    if (!ph || !n || (cap > 0 && !slots)) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    Pool* P = ph->P;
    int k = 0;
    for (size_t i = 0; i < P->req.size() && k < cap; ++i) {
        if (P->req[i].state != R_DONE) continue;
        cudaError_t q = cudaEventQuery(P->req[i].done);
        if (q == cudaSuccess) slots[k++] = (int32_t)i;
        else if (q != cudaErrorNotReady) return pcuda(q, "poll");
    }
    *n = k;
    return 0;
}

extern "C" int32_t ctsmg_pool_evict(ctsmg_pool ph, int32_t slot, const ctsmg_soilwater_io* sw,
                                    const ctsmg_soiltemp_io* st, const ctsmg_canopy_io* cio, int32_t* steps_done) {
    ctsmg_pool_request R{0, 0, 0, 0, sw, st, cio, nullptr, nullptr, nullptr, nullptr, nullptr};
    return ctsmg_pool_evict_request(ph, slot, &R, steps_done);
}

extern "C" int32_t ctsmg_pool_evict_request(ctsmg_pool ph, int32_t slot, const ctsmg_pool_request* req,
                                            int32_t* steps_done) {
    if (!ph || !req) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    const ctsmg_soilwater_io* sw = req->sw;
    const ctsmg_soiltemp_io* st = req->st;
    const ctsmg_canopy_io* cio = req->cio;
    const ctsmg_rootmoist_io* rm = req->rm;
    const ctsmg_hydrology_io* hyio = req->hy;
    if (!sw || !st) return set_error(CTSMG_E_ARG, "null argument", 0, 0);
    Pool* P = ph->P;
    if (slot < 0 || slot >= (int)P->req.size() || P->req[slot].state == R_FREE)
        return set_error(CTSMG_E_ARG, "no request in this slot", slot, 0);
    Request& r = P->req[slot];
    if (sw->ldc != r.nc || st->ldc != r.nc || st->ldp != r.np)
        return set_error(CTSMG_E_ARG, "eviction arrays must be dense like the request", slot, 0);
    if (cio && P->cfg.with_canopy && (cio->ldc != r.nc || cio->ldp != r.np || cio->ldg != r.ng))
        return set_error(CTSMG_E_ARG, "eviction canopy arrays must be dense like the request", slot, 0);
    const bool rms = rm && P->cfg.with_canopy && P->cfg.rootmoist;
    if (rms && (rm->ldc != r.nc || rm->ldp != r.np))
        return set_error(CTSMG_E_ARG, "eviction root moisture arrays must be dense like the request", slot, 0);
    const bool hyd = hyio && P->cfg.hydrology;
    if (hyd && hyio->ldc != r.nc)
        return set_error(CTSMG_E_ARG, "eviction hydrology arrays must be dense like the request", slot, 0);
    if (r.state == R_RUNNING) {                      // stop after the steps already enqueued
        PK(cudaEventRecord(r.done, P->stream), "done event");
        r.state = R_DONE;
        P->dirty = true;
    }
    PK(cudaStreamWaitEvent(P->copy, r.done, 0), "evict wait");
    std::vector<char> staged;
    auto download = [&](const FieldDesc* tab, int nf, const void* hio) -> cudaError_t {
        for (int i = 0; i < nf; ++i) {
            const FieldDesc& f = tab[i];
            void* hp = fptr(hio, f);
            const PField& u = P->fields[P->index[f.name]];
            if (!hp || (u.use == U_IN && u.name != "h2osoi_vol" && u.name != "qflx_rootsoi")) continue;
            if (!r.perm.empty() && !patch_kind(u.kind) && u.kind != K_GR) {
                // back to the request's column order
                const int lev = kind_levels(u.kind), es = u.esize, nc = r.nc;
                staged.resize((size_t)lev * nc * es);
                cudaError_t ee = copy_field(P, u, r, staged.data(), false);
                if (ee == cudaSuccess) ee = cudaStreamSynchronize(P->copy);
                if (ee != cudaSuccess) return ee;
                char* dst = static_cast<char*>(hp);
                for (int l = 0; l < lev; ++l)
                    for (int c = 0; c < nc; ++c)
                        std::memcpy(dst + ((size_t)l * nc + r.perm[c]) * es, &staged[((size_t)l * nc + c) * es], es);
                continue;
            }
            cudaError_t ee = copy_field(P, u, r, hp, false);
            if (ee != cudaSuccess) return ee;
        }
        return cudaSuccess;
    };
    cudaError_t e = download(SOILWATER_TABLE, SOILWATER_NFIELDS, sw);
    if (e == cudaSuccess) e = download(SOILTEMP_TABLE, SOILTEMP_NFIELDS, st);
    if (e == cudaSuccess && cio && P->cfg.with_canopy) e = download(CANOPY_TABLE, CANOPY_NFIELDS, cio);
    if (e == cudaSuccess && rms) e = download(ROOTMOIST_TABLE, ROOTMOIST_NFIELDS, rm);
    for (int t = 0; t < 4 && hyd && e == cudaSuccess; ++t) e = download(HYD_TABS[t], *HYD_NS[t], hyio);
    cudaError_t se = cudaStreamSynchronize(P->copy);
    if (e == cudaSuccess) e = se;
    if (e != cudaSuccess) return pcuda(e, "evict copy");
    if (steps_done) *steps_done = r.enq;
    P->cols.give(r.c0, r.nc);
    P->pats.give(r.p0, r.np);
    P->grids.give(r.g0, r.ng);
    r.state = R_FREE;
    return 0;
}

extern "C" int32_t ctsmg_pool_sync(ctsmg_pool ph) {
    if (!ph) return set_error(CTSMG_E_ARG, "null pool", 0, 0);
    Pool* P = ph->P;
    PK(cudaStreamSynchronize(P->stream), "pool sync");
    PK(cudaStreamSynchronize(P->copy), "pool sync");
    DevError h;
    PK(cudaMemcpy(&h, P->err, sizeof h, cudaMemcpyDeviceToHost), "err D2H");
    if (h.key == ~0ull) return 0;
    const int code = (int)(h.key & 0xff);
    const int pos = (int)(h.key >> 32) - 1;          // 0-based pool position
    const bool col = code == CTSMG_E_SINGULAR;
    int slot = -1, local = pos;
    for (size_t i = 0; i < P->req.size(); ++i) {
        const Request& r = P->req[i];
        if (r.state == R_FREE) continue;
        const int s0 = col ? r.c0 : r.p0, n = col ? r.nc : r.np;
        if (pos >= s0 && pos < s0 + n) {
            slot = (int)i;
            local = pos - s0;
            if (col && !r.perm.empty()) local = r.perm[local];
            local = local + 1;
            break;
        }
    }
    return set_error(code, col ? "BandDiagonal ERROR: dgbsv returned error code" : "CanopyFluxes error", slot, local);
}

extern "C" int32_t ctsmg_pool_free(ctsmg_pool ph, int32_t* cols_largest, int32_t* patches_largest,
                                   int32_t* grids_largest) {
    if (!ph) return set_error(CTSMG_E_ARG, "null pool", 0, 0);
    Pool* P = ph->P;
    if (cols_largest) *cols_largest = P->cols.largest();
    if (patches_largest) *patches_largest = P->pats.largest();
    if (grids_largest) *grids_largest = P->grids.largest();
    return 0;
}

extern "C" int32_t ctsmg_pool_destroy(ctsmg_pool ph) {
    if (!ph) return 0;
    pool_free(ph->P);
    delete ph;
    return 0;
}
