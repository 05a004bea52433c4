// capi.cu -- extern "C" entry points of libctsm_gpu.so (declared in
// include/ctsm_gpu.h).  Plain drop-in mode: every call copies the clump's
// arrays to the device, runs the kernel over the filter and copies the
// written components back, on a CUDA stream owned by the calling host thread.
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <chrono>
#include <mutex>
#include <atomic>
#include <algorithm>
#include <string>
#include <vector>
#include "ctsm_gpu.h"
#include "ctsm_device.cuh"
#include "soil_kernels.cuh"
#include "canopy_kernels.cuh"
#include "soilfluxes_kernels.cuh"
#include "rootmoist_kernels.cuh"
#include "moisture_form_kernels.cuh"
#include "surface_resistance.cuh"
#include "baregrnd_kernels.cuh"
#include "hydrology_kernels.cuh"
#include "capi_internal.h"

namespace ctsmg {

// ------------------------------------------------------------ copy accounting
// Host<->device bytes moved by the entry points of this file, for
// ctsmg_copy_bytes (every copy below goes through these three).
static std::atomic<int64_t> g_h2d_bytes{0}, g_d2h_bytes{0};
static void count_copy(cudaMemcpyKind k, size_t n) {
    if (k == cudaMemcpyHostToDevice) g_h2d_bytes += (int64_t)n;
    else if (k == cudaMemcpyDeviceToHost) g_d2h_bytes += (int64_t)n;
}
static cudaError_t copy_async(void* dst, const void* src, size_t n, cudaMemcpyKind k, cudaStream_t s) {
    count_copy(k, n);
    return cudaMemcpyAsync(dst, src, n, k, s);
}
static cudaError_t copy_2d_async(void* dst, size_t dpitch, const void* src, size_t spitch, size_t w, size_t h,
                                 cudaMemcpyKind k, cudaStream_t s) {
    count_copy(k, w * h);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, w, h, k, s);
}
static cudaError_t copy_sync(void* dst, const void* src, size_t n, cudaMemcpyKind k) {
    count_copy(k, n);
    return cudaMemcpy(dst, src, n, k);
}

// ------------------------------------------------------------ gather copy-in
// On this machine the copy engines move 2-D column slices host to device at
// about 130 GB/s while the other engine copies results back, against about
// 150-165 GB/s for a kernel that reads the same slices of the caller's
// page-locked arrays through their device-mapped addresses (and a total over
// both directions of ~275 against ~225 GB/s).  A pipelined call whose
// copied-in arrays are all page-locked therefore copies each chunk in with
// one gather kernel on the copy-in stream; other arrays take the engines.
#ifndef CTSMG_GATHER_UNROLL
#define CTSMG_GATHER_UNROLL 4          // loads in flight per thread of the gather kernel
#endif
#ifndef CTSMG_GATHER_BLOCKS_PER_SM
#define CTSMG_GATHER_BLOCKS_PER_SM 2   // its blocks of 256 threads per SM
#endif
constexpr int GATHER_MAX_FIELDS = 72;
struct GatherField {
    const char* src;        // device-mapped address of the caller's array
    char* dst;              // the device copy
    long long pitch;        // leading dimension (elements)
    int esize, row0, rows, patch;
};
struct GatherTable {
    GatherField f[GATHER_MAX_FIELDS];
    int n;
};

template <class W>
__device__ __forceinline__ void gather_rows(const GatherField& F, long long lo, long long w) {
    const long long n = w * F.rows, step = (long long)gridDim.x * blockDim.x;
    const W* __restrict__ src = reinterpret_cast<const W*>(F.src);
    W* __restrict__ dst = reinterpret_cast<W*>(F.dst);
    constexpr int U = CTSMG_GATHER_UNROLL;         // loads in flight per thread
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += U * step) {
        W v[U];
        long long o[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long e = t + u * step;
            o[u] = -1;
            if (e < n) {
                const long long r = e / w;
                o[u] = (F.row0 + r) * F.pitch + lo + (e - r * w);
                v[u] = src[o[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (o[u] >= 0) dst[o[u]] = v[u];
    }
}

// Rows row0 .. row0+rows-1, columns [c0, c1) (patches [p0, p1)) of every field.
__global__ void __launch_bounds__(256) gather_kernel(const GatherTable T, int c0, int c1, int p0, int p1) {
    for (int i = 0; i < T.n; ++i) {
        const GatherField& F = T.f[i];
        const long long lo = F.patch ? p0 : c0, w = (F.patch ? p1 : c1) - lo;
        if (w <= 0) continue;
        if (F.esize == 8) gather_rows<unsigned long long>(F, lo, w);
        else gather_rows<unsigned int>(F, lo, w);
    }
}

static std::atomic<int> g_copy_mode{0};        // 0: gather when possible, 1: copy engines only

// ------------------------------------------------------------ global state
static std::mutex g_mu;
static std::atomic<bool> g_init{false};   // read without g_mu by every entry point
static ctsmg_options g_opt;
static ctsmg_soilwater_params g_swp = {6.0};
// soil_resis_inparm and the two parameter-file values (the parameter file is
// absent here: 15 mm and 0.8 stand in until ctsmg_set_soil_resistance)
static ctsmg_soil_resistance_params g_sres = {1, 15.0, 0.8};
// SoilHydrologyMod / SaturatedExcessRunoffMod parameter-file values (absent
// here; these stand in until ctsmg_set_soilhydrology_params)
static ctsmg_soilhydrology_params g_shp = {0.01, 1.0, 1.0e-2, 1.0e-5, 6.0, 0.5, 0.4, 0.13, 1};
// soilwater_movement_inparm; defaults of the Zeng-Decker form until ctsmg_init
static ctsmg_soilwater_movement_nml g_swm = {0, 1, 4, 1, 0, 0, 60.0, 1.e-8, 1.e-1, 1.e-2};
static ctsmg_canopy_params g_cpar;
static ctsmg_pftcon g_pft;
static bool g_cpar_set = false;

// ------------------------------------------------------------ per-thread context
#ifndef CTSMG_PIPE_CHUNKS
#define CTSMG_PIPE_CHUNKS 16
#endif
constexpr int PIPE_CHUNKS = CTSMG_PIPE_CHUNKS;   // chunks of a pipelined drop-in call
constexpr int PIPE_MIN_COLUMNS = 32768;  // smaller calls run in one piece
#ifndef CTSMG_GROUP_COLUMNS
#define CTSMG_GROUP_COLUMNS 1     // heat-solve work order grouped by snow / bedrock layers
#endif
#ifndef CTSMG_PIPE_STREAMS
#define CTSMG_PIPE_STREAMS 4
#endif
constexpr int PIPE_STREAMS = CTSMG_PIPE_STREAMS; // compute streams of a pipelined call

struct ThreadCtx {
    cudaStream_t stream = nullptr;
    cudaStream_t h2d = nullptr, d2h = nullptr;      // copy streams of the pipelined calls
    cudaStream_t h2dk = nullptr;                    // copy-in stream of the gather kernel (highest priority)
    cudaStream_t xs[PIPE_STREAMS - 1] = {};         // further compute streams of a pipelined call
    cudaEvent_t ev_in[PIPE_CHUNKS] = {}, ev_done[PIPE_CHUNKS] = {};
    // per-chunk timeline of the last pipelined call (ctsmg_pipe_trace):
    // copy-in start / end, kernel start / end, copy-out end
    // device copies of time-constant inputs kept across calls
    // (ctsmg_set_time_constant_inputs): one per host array, leading
    // dimension and size, valid for the columns [lo, hi) of that array
    struct TcEntry {
        const void* host;
        int ld, esize, row0, rows;      // the rows the call copies in
        size_t bytes;
        void* dev;
        int lo, hi;
        bool valid;
    };
    std::vector<TcEntry> tc;
    unsigned tc_gen = 0;
    // copy-in of the current pipelined call by gather_kernel (page-locked arrays)
    bool gather = false;
    GatherTable gt{};
    int gather_grid = 0;
    bool trace = false;
    int trace_n = 0;
    cudaEvent_t tr[PIPE_CHUNKS][5] = {};
    // host clock: when the calling thread finished enqueuing each chunk's
    // copy-in and copy-out, from the first mark
    std::chrono::steady_clock::time_point tr_t0{};
    float trh[PIPE_CHUNKS][2] = {};
    char* arena = nullptr;
    size_t arena_cap = 0, arena_top = 0;
    int32_t* order = nullptr;                       // page-locked work order of a call
    size_t order_cap = 0;
    DevError* err = nullptr;
    std::string msg;
    int err_index = 0, err_level = 0;
    ~ThreadCtx() {
        for (auto& t : tc)
            if (t.dev) cudaFree(t.dev);
        if (arena) cudaFree(arena);
        if (order) cudaFreeHost(order);
        if (err) cudaFree(err);
        for (int k = 0; k < PIPE_CHUNKS; ++k) {
            if (ev_in[k]) cudaEventDestroy(ev_in[k]);
            if (ev_done[k]) cudaEventDestroy(ev_done[k]);
            for (cudaEvent_t t : tr[k])
                if (t) cudaEventDestroy(t);
        }
        if (h2d) cudaStreamDestroy(h2d);
        if (h2dk) cudaStreamDestroy(h2dk);
        if (d2h) cudaStreamDestroy(d2h);
        for (cudaStream_t x : xs)
            if (x) cudaStreamDestroy(x);
        if (stream) cudaStreamDestroy(stream);
    }
};
static thread_local ThreadCtx* t_ctx = nullptr;
static thread_local unsigned t_gen = 0;
static std::atomic<unsigned> g_gen{1};   // bumped by ctsmg_finalize
static std::vector<ThreadCtx*> g_ctxs;

static thread_local std::string t_msg;
static thread_local int t_idx = 0, t_lev = 0;

int set_error(int code, const char* what, int index, int level) {
    char buf[512];
    std::snprintf(buf, sizeof buf, "%s", what);
    t_msg = buf;
    t_idx = index;
    t_lev = level;
    return code;
}

static int cuda_fail(cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return set_error(CTSMG_E_CUDA, m.c_str(), 0, 0);
}

// Serialises the creation of thread contexts (streams, events, buffers):
// threads that make their first call at the same moment create them one
// after another.
static std::mutex g_ctx_create_mu;

static int ctx_get(ThreadCtx** out) {
    if (!g_init) return set_error(CTSMG_E_NOT_INIT, "ctsmg_init has not been called", 0, 0);
    if (t_gen != g_gen) t_ctx = nullptr;   // contexts were freed by ctsmg_finalize
    if (!t_ctx) {
        std::lock_guard<std::mutex> create_lock(g_ctx_create_mu);
        ThreadCtx* c = new ThreadCtx();
        cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreate"); }
        e = cudaMalloc(&c->err, sizeof(DevError));
        if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaMalloc(err)"); }
        // the gather kernel's copy-in stream at the highest priority, so its
        // blocks take SM slots ahead of the compute kernels' waiting blocks
        // (the copy engines' stream keeps the default: on a high-priority
        // stream the engine copies cost the host several ms more per call)
        int prio_least = 0, prio_greatest = 0;
        cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
        if ((e = cudaStreamCreateWithFlags(&c->h2d, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaStreamCreateWithPriority(&c->h2dk, cudaStreamNonBlocking, prio_greatest)) != cudaSuccess ||
            (e = cudaStreamCreateWithFlags(&c->d2h, cudaStreamNonBlocking)) != cudaSuccess) {
            delete c;
            return cuda_fail(e, "cudaStreamCreate");
        }
        for (cudaStream_t& x : c->xs)
            if ((e = cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking)) != cudaSuccess) {
                delete c;
                return cuda_fail(e, "cudaStreamCreate");
            }
        for (int k = 0; k < PIPE_CHUNKS && e == cudaSuccess; ++k) {
            e = cudaEventCreateWithFlags(&c->ev_in[k], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_done[k], cudaEventDisableTiming);
        }
        if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaEventCreate"); }
        t_ctx = c;
        std::lock_guard<std::mutex> lk(g_mu);
        t_gen = g_gen;
        g_ctxs.push_back(c);
    }
    *out = t_ctx;
    return 0;
}

// bump allocator over one device arena; grows (and invalidates) between calls
static int arena_reserve(ThreadCtx* c, size_t bytes) {
    if (bytes <= c->arena_cap) { c->arena_top = 0; return 0; }
    if (c->arena) { cudaStreamSynchronize(c->stream); cudaFree(c->arena); c->arena = nullptr; }
    size_t cap = bytes + bytes / 4 + (1 << 20);
    cudaError_t e = cudaMalloc(&c->arena, cap);
    if (e != cudaSuccess) { c->arena_cap = 0; return cuda_fail(e, "cudaMalloc(arena)"); }
    c->arena_cap = cap;
    c->arena_top = 0;
    return 0;
}
static void* arena_take(ThreadCtx* c, size_t bytes) {
    size_t off = (c->arena_top + 255) & ~(size_t)255;
    c->arena_top = off + bytes;
    return c->arena + off;
}

// ------------------------------------------------------------ field tables
int kind_levels(int kind) {
    switch (kind) {
        case K_C: case K_P: case K_GR: return 1;
        case K_SS: return NLEVSNO + NLEVGRND;
        case K_ZI: return NLEVSNO + NLEVGRND + 1;
        case K_G: case K_PG: return NLEVGRND;
        case K_S: case K_PS: return NLEVSOI;
        case K_SN: return NLEVSNO;
        case K_PL: return NLEVSNO + 1;
    }
    return 0;
}

// rows of a component the drop-in calls copy (FieldDesc::lev0 / nlev)
static int copy_rows(const FieldDesc& f) { return f.nlev ? f.nlev : kind_levels(f.kind); }
static size_t copy_row0(const FieldDesc& f) { return f.nlev ? (size_t)f.lev0 : 0; }
// rows of the copy-in (host to device)
static int copy_in_rows(const FieldDesc& f) { return f.in_nlev ? f.in_nlev : copy_rows(f); }
static size_t copy_in_row0(const FieldDesc& f) { return f.in_nlev ? (size_t)f.in_lev0 : copy_row0(f); }

#define FW(S, name, kind, esz, use) {offsetof(S, name), kind, esz, use, #name}
// Rows of SoilWater's (Zeng-Decker) components: levels 1..nlevsoi of the
// snow/soil and ground arrays, 1..nlevgrnd of t_soisno and zi (the frozen
// water-table search), the snow rows not at all; the fluxes and diagnostics
// it writes over levels 1..nlevsoi are not copied in.
#define FWR(S, name, kind, esz, use, lev0, nlev, no_in) {offsetof(S, name), kind, esz, use, #name, lev0, nlev, no_in}
#define SWR(name, kind, use, lev0, nlev, no_in) FWR(ctsmg_soilwater_io, name, kind, 8, use, lev0, nlev, no_in)
constexpr int SS1 = 1 - (-NLEVSNO + 1);    // row of level 1 in a [SS] array
constexpr int ZI1 = 1 + NLEVSNO;           // row of level 1 in a [ZI] array
const FieldDesc SOILWATER_TABLE[] = {
    SWR(z, K_SS, U_IN, SS1, NLEVSOI, 0), SWR(zi, K_ZI, U_IN, ZI1, NLEVGRND, 0),
    SWR(dz, K_SS, U_IN, SS1, NLEVSOI, 0), SWR(zwt, K_C, U_IN, 0, 0, 0),
    SWR(qcharge, K_C, U_OUT, 0, 0, 1), SWR(icefrac, K_G, U_OUT, 0, NLEVSOI, 1),
    SWR(qin, K_S, U_OUT, 0, 0, 1), SWR(qout, K_S, U_OUT, 0, 0, 1),
    SWR(smpmin, K_C, U_IN, 0, 0, 0), SWR(watsat, K_G, U_IN, 0, NLEVSOI, 0),
    SWR(hksat, K_G, U_IN, 0, NLEVSOI, 0), SWR(bsw, K_G, U_IN, 0, NLEVSOI, 0),
    SWR(sucsat, K_G, U_IN, 0, NLEVSOI, 0), SWR(smp_l, K_G, U_OUT, 0, NLEVSOI, 1),
    SWR(hk_l, K_G, U_OUT, 0, NLEVSOI, 1), SWR(h2osoi_ice, K_SS, U_IN, SS1, NLEVSOI, 0),
    SWR(h2osoi_liq, K_SS, U_INOUT, SS1, NLEVSOI, 0), SWR(h2osoi_vol, K_G, U_IN, 0, NLEVSOI, 0),
    SWR(qflx_deficit, K_C, U_OUT, 0, 0, 1), SWR(qflx_infl, K_C, U_IN, 0, 0, 0),
    SWR(qflx_rootsoi, K_S, U_IN, 0, 0, 0), SWR(t_soisno, K_SS, U_IN, SS1, NLEVGRND, 0),
};
const int SOILWATER_NFIELDS = sizeof(SOILWATER_TABLE) / sizeof(SOILWATER_TABLE[0]);

// soilwater_moisture_form (SoilWaterMovementMod.F90:1172-1186, 1503-1508,
// 1627-1635, 2085-2095): icefrac and eff_porosity are inputs here
const FieldDesc SOILWATER_MF_TABLE[] = {
    FW(ctsmg_soilwater_io, z, K_SS, 8, U_IN), FW(ctsmg_soilwater_io, zi, K_ZI, 8, U_IN),
    FW(ctsmg_soilwater_io, dz, K_SS, 8, U_IN), FW(ctsmg_soilwater_io, nbedrock, K_C, 4, U_IN),
    FW(ctsmg_soilwater_io, zwt, K_C, 8, U_IN), FW(ctsmg_soilwater_io, qcharge, K_C, 8, U_OUT),
    FW(ctsmg_soilwater_io, icefrac, K_G, 8, U_IN), FW(ctsmg_soilwater_io, qin, K_S, 8, U_OUT),
    FW(ctsmg_soilwater_io, qout, K_S, 8, U_OUT), FW(ctsmg_soilwater_io, smpmin, K_C, 8, U_IN),
    FW(ctsmg_soilwater_io, watsat, K_G, 8, U_IN), FW(ctsmg_soilwater_io, hksat, K_G, 8, U_IN),
    FW(ctsmg_soilwater_io, bsw, K_G, 8, U_IN), FW(ctsmg_soilwater_io, sucsat, K_G, 8, U_IN),
    FW(ctsmg_soilwater_io, smp_l, K_G, 8, U_OUT), FW(ctsmg_soilwater_io, hk_l, K_G, 8, U_OUT),
    FW(ctsmg_soilwater_io, h2osoi_liq, K_SS, 8, U_INOUT), FW(ctsmg_soilwater_io, qflx_infl, K_C, 8, U_IN),
    FW(ctsmg_soilwater_io, qflx_rootsoi, K_S, 8, U_IN), FW(ctsmg_soilwater_io, eff_porosity, K_G, 8, U_IN),
    FW(ctsmg_soilwater_io, num_substeps, K_C, 8, U_OUT),
};
const int SOILWATER_MF_NFIELDS = sizeof(SOILWATER_MF_TABLE) / sizeof(SOILWATER_MF_TABLE[0]);

// the use_flexibleCN fix after either form (SoilWaterMovementMod.F90:331-368)
const FieldDesc SOILWATER_FLEXCN_TABLE[] = {
    FW(ctsmg_soilwater_io, h2osoi_liq, K_SS, 8, U_INOUT), FW(ctsmg_soilwater_io, h2osoi_ice, K_SS, 8, U_IN),
    FW(ctsmg_soilwater_io, dz, K_SS, 8, U_IN), FW(ctsmg_soilwater_io, h2osoi_vol, K_G, 8, U_INOUT),
    FW(ctsmg_soilwater_io, wa, K_C, 8, U_INOUT),
};
const int SOILWATER_FLEXCN_NFIELDS = sizeof(SOILWATER_FLEXCN_TABLE) / sizeof(SOILWATER_FLEXCN_TABLE[0]);
// SetSoilWaterFractions: levels 1..nlevsoi of the soil components
const FieldDesc SOILWATER_FRACTIONS_TABLE[] = {
    SWR(dz, K_SS, U_IN, SS1, NLEVSOI, 0), SWR(h2osoi_ice, K_SS, U_IN, SS1, NLEVSOI, 0),
    SWR(watsat, K_G, U_IN, 0, NLEVSOI, 0), SWR(eff_porosity, K_G, U_INOUT, 0, NLEVSOI, 0),
    SWR(icefrac, K_G, U_INOUT, 0, NLEVSOI, 0),
};
const int SOILWATER_FRACTIONS_NFIELDS = sizeof(SOILWATER_FRACTIONS_TABLE) / sizeof(SOILWATER_FRACTIONS_TABLE[0]);

// calc_soilevap_resis: sl_14 (dsl, soilresis) and leepielke_1992 (soilbeta)
const FieldDesc SOILRESIS_SL14_TABLE[] = {
    FW(ctsmg_soilresis_io, dz, K_SS, 8, U_IN), FW(ctsmg_soilresis_io, t_soisno, K_SS, 8, U_IN),
    FW(ctsmg_soilresis_io, h2osoi_liq, K_SS, 8, U_IN), FW(ctsmg_soilresis_io, h2osoi_ice, K_SS, 8, U_IN),
    FW(ctsmg_soilresis_io, watsat, K_G, 8, U_IN), FW(ctsmg_soilresis_io, bsw, K_G, 8, U_IN),
    FW(ctsmg_soilresis_io, sucsat, K_G, 8, U_IN), FW(ctsmg_soilresis_io, dsl, K_C, 8, U_OUT),
    FW(ctsmg_soilresis_io, soilresis, K_C, 8, U_OUT),
};
const int SOILRESIS_SL14_NFIELDS = sizeof(SOILRESIS_SL14_TABLE) / sizeof(SOILRESIS_SL14_TABLE[0]);
const FieldDesc SOILRESIS_LP92_TABLE[] = {
    FW(ctsmg_soilresis_io, dz, K_SS, 8, U_IN), FW(ctsmg_soilresis_io, h2osoi_liq, K_SS, 8, U_IN),
    FW(ctsmg_soilresis_io, h2osoi_ice, K_SS, 8, U_IN), FW(ctsmg_soilresis_io, watfc, K_G, 8, U_IN),
    FW(ctsmg_soilresis_io, frac_sno, K_C, 8, U_IN), FW(ctsmg_soilresis_io, frac_h2osfc, K_C, 8, U_IN),
    FW(ctsmg_soilresis_io, soilbeta, K_C, 8, U_OUT),
};
const int SOILRESIS_LP92_NFIELDS = sizeof(SOILRESIS_LP92_TABLE) / sizeof(SOILRESIS_LP92_TABLE[0]);

// BareGroundFluxes (the soil resistance method adds soilresis or soilbeta)
const FieldDesc BAREGRND_TABLE[] = {
    FW(ctsmg_baregrnd_io, patch_column, K_P, 4, U_IN),
    FW(ctsmg_baregrnd_io, patch_gridcell, K_P, 4, U_IN),
    FW(ctsmg_baregrnd_io, forc_u, K_GR, 8, U_IN),
    FW(ctsmg_baregrnd_io, forc_v, K_GR, 8, U_IN),
    FW(ctsmg_baregrnd_io, forc_hgt_u, K_GR, 8, U_IN),
    FW(ctsmg_baregrnd_io, forc_hgt_t, K_GR, 8, U_IN),
    FW(ctsmg_baregrnd_io, forc_hgt_q, K_GR, 8, U_IN),
    FW(ctsmg_baregrnd_io, snl, K_C, 4, U_IN),
    FW(ctsmg_baregrnd_io, forc_t, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, forc_pbot, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, forc_q, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, forc_th, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, forc_rho, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, thv, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, t_grnd, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, qg, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, qg_snow, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, qg_soil, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, qg_h2osfc, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, dqgdT, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, htvp, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, z0mg, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, t_h2osfc, K_C, 8, U_IN),
    FW(ctsmg_baregrnd_io, t_soisno, K_SS, 8, U_IN),
    FW(ctsmg_baregrnd_io, z0hg, K_C, 8, U_INOUT),
    FW(ctsmg_baregrnd_io, z0qg, K_C, 8, U_INOUT),
    FW(ctsmg_baregrnd_io, thm, K_P, 8, U_IN),
    FW(ctsmg_baregrnd_io, forc_hgt_u_patch, K_P, 8, U_INOUT),
    FW(ctsmg_baregrnd_io, forc_hgt_t_patch, K_P, 8, U_INOUT),
    FW(ctsmg_baregrnd_io, forc_hgt_q_patch, K_P, 8, U_INOUT),
    FW(ctsmg_baregrnd_io, btran, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, t_veg, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, rssun, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, rssha, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, displa, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, z0mv, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, z0hv, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, z0qv, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, dlrad, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, ulrad, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, dhsdt_canopy, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, eflx_sh_stem, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, z0mg_patch, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, z0hg_patch, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, z0qg_patch, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, zeta, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, obu, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, ram1, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, cgrnds, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, cgrndl, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, cgrnd, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, taux, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, tauy, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, eflx_sh_grnd, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, eflx_sh_tot, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, eflx_sh_snow, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, eflx_sh_soil, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, eflx_sh_h2osfc, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, qflx_tran_veg, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, qflx_evap_veg, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, qflx_evap_soi, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, qflx_evap_tot, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, qflx_ev_snow, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, qflx_ev_soil, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, qflx_ev_h2osfc, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, t_ref2m, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, q_ref2m, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, rh_ref2m, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, kbm1, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, u10_clm, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, u10, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, va, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, vds, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, fv, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, fm, K_P, 8, U_OUT),
    FW(ctsmg_baregrnd_io, num_iter, K_P, 4, U_OUT),
    FW(ctsmg_baregrnd_io, rootr, K_PG, 8, U_OUT),
    FW(ctsmg_baregrnd_io, rresis, K_PG, 8, U_OUT),
};
const int BAREGRND_NFIELDS = sizeof(BAREGRND_TABLE) / sizeof(BAREGRND_TABLE[0]);

// SaturatedExcessRunoff, PerchedWaterTable, ThetaBasedWaterTable,
// PerchedLateralFlow, SubsurfaceLateralFlow: the components each reads or writes
const FieldDesc HYD_SAT_TABLE[] = {
    FW(ctsmg_hydrology_io, zwt, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, zwt_perched, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, frost_table, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, wtfact, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_rain_plus_snomelt, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, fsat, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, fcov, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_sat_excess_surf, K_C, 8, U_OUT),
};
const int HYD_SAT_TABLE_N = sizeof(HYD_SAT_TABLE) / sizeof(HYD_SAT_TABLE[0]);
const FieldDesc HYD_PWT_TABLE[] = {
    FW(ctsmg_hydrology_io, z, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, zi, K_ZI, 8, U_IN),
    FW(ctsmg_hydrology_io, dz, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, t_soisno, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_liq, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_ice, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_vol, K_G, 8, U_INOUT),
    FW(ctsmg_hydrology_io, zwt, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, zwt_perched, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, frost_table, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, watsat, K_G, 8, U_IN),
};
const int HYD_PWT_TABLE_N = sizeof(HYD_PWT_TABLE) / sizeof(HYD_PWT_TABLE[0]);
const FieldDesc HYD_TWT_TABLE[] = {
    FW(ctsmg_hydrology_io, nbedrock, K_C, 4, U_IN),
    FW(ctsmg_hydrology_io, z, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, zi, K_ZI, 8, U_IN),
    FW(ctsmg_hydrology_io, dz, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_liq, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_ice, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_vol, K_G, 8, U_INOUT),
    FW(ctsmg_hydrology_io, zwt, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, watsat, K_G, 8, U_IN),
};
const int HYD_TWT_TABLE_N = sizeof(HYD_TWT_TABLE) / sizeof(HYD_TWT_TABLE[0]);
const FieldDesc HYD_PLF_TABLE[] = {
    FW(ctsmg_hydrology_io, nbedrock, K_C, 4, U_IN),
    FW(ctsmg_hydrology_io, zi, K_ZI, 8, U_IN),
    FW(ctsmg_hydrology_io, dz, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_liq, K_SS, 8, U_INOUT),
    FW(ctsmg_hydrology_io, zwt_perched, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, frost_table, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, watsat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, hksat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, bsw, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, sucsat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, topo_slope, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_drain_perched, K_C, 8, U_OUT),
};
const int HYD_PLF_TABLE_N = sizeof(HYD_PLF_TABLE) / sizeof(HYD_PLF_TABLE[0]);
const FieldDesc HYD_SLF_TABLE[] = {
    FW(ctsmg_hydrology_io, nbedrock, K_C, 4, U_IN),
    FW(ctsmg_hydrology_io, zi, K_ZI, 8, U_IN),
    FW(ctsmg_hydrology_io, dz, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_liq, K_SS, 8, U_INOUT),
    FW(ctsmg_hydrology_io, h2osoi_ice, K_SS, 8, U_INOUT),
    FW(ctsmg_hydrology_io, h2osfc, K_C, 8, U_INOUT),
    FW(ctsmg_hydrology_io, zwt, K_C, 8, U_INOUT),
    FW(ctsmg_hydrology_io, frost_table, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, icefrac, K_G, 8, U_OUT),
    FW(ctsmg_hydrology_io, watsat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, bsw, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, sucsat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, eff_porosity, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, topo_slope, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_snwcp_liq, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_latflow_out, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_latflow_in, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_rsub_sat, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_drain, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_qrgwl, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_ice_runoff_xs, K_C, 8, U_OUT),
};
const int HYD_SLF_TABLE_N = sizeof(HYD_SLF_TABLE) / sizeof(HYD_SLF_TABLE[0]);
const FieldDesc HYD_INF_TABLE[] = {
    FW(ctsmg_hydrology_io, snl, K_C, 4, U_IN),
    FW(ctsmg_hydrology_io, qflx_rain_plus_snomelt, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_snow_h2osfc, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_floodc, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_liqevap_from_top_layer_col, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_ev_soil_col, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_ev_h2osfc_col, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_sat_excess_surf, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, frac_sno_eff, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, frac_h2osfc, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, frac_h2osfc_nosnow, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osfc_thresh, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, topo_slope, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, fsat, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, icefrac, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, hksat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osfc, K_C, 8, U_INOUT),
    FW(ctsmg_hydrology_io, qflx_top_soil, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_in_soil, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_top_soil_to_h2osfc, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qinmax, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_infl_excess, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_in_soil_limited, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_in_h2osfc, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_infl_excess_surf, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_h2osfc_surf, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_h2osfc_drain, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_infl, K_C, 8, U_OUT),
};
const int HYD_INF_TABLE_N = sizeof(HYD_INF_TABLE) / sizeof(HYD_INF_TABLE[0]);
const FieldDesc HYD_WT_TABLE[] = {
    FW(ctsmg_hydrology_io, z, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, zi, K_ZI, 8, U_IN),
    FW(ctsmg_hydrology_io, dz, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, t_soisno, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_liq, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_ice, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_vol, K_G, 8, U_INOUT),
    FW(ctsmg_hydrology_io, zwt, K_C, 8, U_INOUT),
    FW(ctsmg_hydrology_io, zwt_perched, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, frost_table, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, watsat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, bsw, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, sucsat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, wa, K_C, 8, U_INOUT),
    FW(ctsmg_hydrology_io, qcharge, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_drain, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_rsub_sat, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_drain_perched, K_C, 8, U_OUT),
};
const int HYD_WT_TABLE_N = sizeof(HYD_WT_TABLE) / sizeof(HYD_WT_TABLE[0]);
const FieldDesc HYD_DR_TABLE[] = {
    FW(ctsmg_hydrology_io, z, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, zi, K_ZI, 8, U_IN),
    FW(ctsmg_hydrology_io, dz, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, t_soisno, K_SS, 8, U_IN),
    FW(ctsmg_hydrology_io, h2osoi_liq, K_SS, 8, U_INOUT),
    FW(ctsmg_hydrology_io, h2osoi_ice, K_SS, 8, U_INOUT),
    FW(ctsmg_hydrology_io, h2osfc, K_C, 8, U_INOUT),
    FW(ctsmg_hydrology_io, zwt, K_C, 8, U_INOUT),
    FW(ctsmg_hydrology_io, zwt_perched, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, frost_table, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, icefrac, K_G, 8, U_OUT),
    FW(ctsmg_hydrology_io, watsat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, hksat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, bsw, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, sucsat, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, eff_porosity, K_G, 8, U_IN),
    FW(ctsmg_hydrology_io, topo_slope, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, hkdepth, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, wa, K_C, 8, U_INOUT),
    FW(ctsmg_hydrology_io, qflx_snwcp_liq, K_C, 8, U_IN),
    FW(ctsmg_hydrology_io, qflx_drain, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_rsub_sat, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_drain_perched, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_qrgwl, K_C, 8, U_OUT),
    FW(ctsmg_hydrology_io, qflx_ice_runoff_xs, K_C, 8, U_OUT),
};
const int HYD_DR_TABLE_N = sizeof(HYD_DR_TABLE) / sizeof(HYD_DR_TABLE[0]);
const FieldDesc BAREGRND_SOILRESIS[] = {FW(ctsmg_baregrnd_io, soilresis, K_C, 8, U_IN)};
const FieldDesc BAREGRND_SOILBETA[] = {FW(ctsmg_baregrnd_io, soilbeta, K_C, 8, U_IN)};

#define FT(name, kind, esz, use) FW(ctsmg_soiltemp_io, name, kind, esz, use)
const FieldDesc SOILTEMP_TABLE[] = {
    FT(snl, K_C, 4, U_IN), FT(nbedrock, K_C, 4, U_IN), FT(z, K_SS, 8, U_IN), FT(zi, K_ZI, 8, U_IN),
    FT(dz, K_SS, 8, U_IN), FT(col_patchi, K_C, 4, U_IN), FT(col_npatches, K_C, 4, U_IN),
    FT(wtcol, K_P, 8, U_IN), FT(frac_veg_nosno, K_P, 4, U_IN), FT(forc_lwrad, K_C, 8, U_IN),
    FT(sabg, K_P, 8, U_IN), FT(sabg_soil, K_P, 8, U_IN), FT(sabg_snow, K_P, 8, U_IN),
    FT(sabg_lyr, K_PL, 8, U_IN), FT(sabg_chk, K_P, 8, U_OUT), FT(htvp, K_C, 8, U_IN),
    FT(cgrnd, K_P, 8, U_IN), FT(dlrad, K_P, 8, U_IN), FT(eflx_sh_grnd, K_P, 8, U_IN),
    FT(eflx_sh_snow, K_P, 8, U_IN), FT(eflx_sh_soil, K_P, 8, U_IN), FT(eflx_sh_h2osfc, K_P, 8, U_IN),
    FT(qflx_evap_soi, K_P, 8, U_IN), FT(qflx_ev_snow, K_P, 8, U_IN), FT(qflx_ev_soil, K_P, 8, U_IN),
    FT(qflx_ev_h2osfc, K_P, 8, U_IN), FT(eflx_bot, K_C, 8, U_IN), FT(eflx_gnet, K_P, 8, U_OUT),
    FT(dgnetdT, K_P, 8, U_OUT), FT(eflx_fgr12, K_C, 8, U_OUT), FT(eflx_fgr, K_G, 8, U_OUT),
    FT(eflx_snomelt, K_C, 8, U_OUT), FT(eflx_h2osfc_to_snow, K_C, 8, U_OUT), FT(emg, K_C, 8, U_IN),
    FT(t_soisno, K_SS, 8, U_INOUT), FT(t_h2osfc, K_C, 8, U_INOUT), FT(t_grnd, K_C, 8, U_INOUT),
    FT(fact, K_SS, 8, U_OUT), FT(c_h2osfc, K_C, 8, U_OUT), FT(xmf, K_C, 8, U_OUT),
    FT(xmf_h2osfc, K_C, 8, U_OUT), FT(imelt, K_SS, 4, U_OUT), FT(watsat, K_G, 8, U_IN),
    FT(bsw, K_G, 8, U_IN), FT(sucsat, K_G, 8, U_IN), FT(tkmg, K_G, 8, U_IN), FT(tkdry, K_G, 8, U_IN),
    FT(csol, K_G, 8, U_IN), FT(thk, K_SS, 8, U_OUT), FT(h2osoi_liq, K_SS, 8, U_INOUT),
    FT(h2osoi_ice, K_SS, 8, U_INOUT), FT(h2osfc, K_C, 8, U_INOUT), FT(h2osno_no_layers, K_C, 8, U_INOUT),
    FT(int_snow, K_C, 8, U_INOUT), FT(snow_depth, K_C, 8, U_INOUT), FT(snomelt_accum, K_C, 8, U_INOUT),
    FT(frac_sno_eff, K_C, 8, U_IN), FT(frac_h2osfc, K_C, 8, U_IN), FT(bw, K_SN, 8, U_OUT),
    FT(qflx_snomelt, K_C, 8, U_OUT), FT(qflx_snofrz, K_C, 8, U_OUT), FT(qflx_snow_drain, K_C, 8, U_OUT),
    FT(qflx_snomelt_lyr, K_SN, 8, U_OUT), FT(qflx_snofrz_lyr, K_SN, 8, U_OUT),
    FT(qflx_h2osfc_to_ice, K_C, 8, U_OUT),
};
const int SOILTEMP_NFIELDS = sizeof(SOILTEMP_TABLE) / sizeof(SOILTEMP_TABLE[0]);

// The SoilTemperature table for a filter that covers every column of the
// bounds: what the heat solve writes on every filtered column is not copied
// in -- eflx_fgr (levels 1..nlevgrnd), the per-layer melt and freeze fluxes
// (every snow level), the column outputs -- and of fact, thk and
// imelt (written on levels snl+1..nlevgrnd) only the snow rows go in.
static std::vector<FieldDesc> soiltemp_dense_table() {
    std::vector<FieldDesc> t(SOILTEMP_TABLE, SOILTEMP_TABLE + SOILTEMP_NFIELDS);
    for (FieldDesc& f : t) {
        const std::string n = f.name;
        if (n == "fact" || n == "thk" || n == "imelt") { f.in_lev0 = 0; f.in_nlev = NLEVSNO; }
        else if (f.use == U_OUT && n != "bw" && f.kind != K_P) f.no_in = 1;
    }
    return t;
}

#define FC(name, kind, esz, use) FW(ctsmg_canopy_io, name, kind, esz, use)
// Compute_EffecRootFrac_And_VertTranSink_Default: levels 1..nlevsoi of rootr
// (patches) and of the two column outputs
const FieldDesc ROOTSINK_TABLE[] = {
    FW(ctsmg_rootsink_io, col_patchi, K_C, 4, U_IN), FW(ctsmg_rootsink_io, col_npatches, K_C, 4, U_IN),
    FW(ctsmg_rootsink_io, wtcol, K_P, 8, U_IN), FW(ctsmg_rootsink_io, qflx_tran_veg, K_P, 8, U_IN),
    FWR(ctsmg_rootsink_io, rootr, K_PG, 8, U_IN, 0, NLEVSOI, 0),
    FWR(ctsmg_rootsink_io, rootr_col, K_G, 8, U_INOUT, 0, NLEVSOI, 0),
    FW(ctsmg_rootsink_io, qflx_rootsoi, K_S, 8, U_INOUT),
};
const int ROOTSINK_NFIELDS = sizeof(ROOTSINK_TABLE) / sizeof(ROOTSINK_TABLE[0]);
const FieldDesc ROOTSINK_TRANCOL_TABLE[] = {FW(ctsmg_rootsink_io, qflx_tran_veg_col, K_C, 8, U_IN)};

#define FR(name, kind, esz, use) FW(ctsmg_rootmoist_io, name, kind, esz, use)
const FieldDesc ROOTMOIST_TABLE[] = {
    FR(h2osoi_liq, K_SS, 8, U_IN),
    FR(h2osoi_ice, K_SS, 8, U_IN),
    FR(dz, K_SS, 8, U_IN),
    FR(t_soisno, K_SS, 8, U_IN),
    FR(watsat, K_G, 8, U_IN),
    FR(sucsat, K_G, 8, U_IN),
    FR(bsw, K_G, 8, U_IN),
    FR(eff_porosity, K_G, 8, U_OUT),
    FR(h2osoi_liqvol, K_G, 8, U_OUT),
    FR(patch_column, K_P, 4, U_IN),
    FR(itype, K_P, 4, U_IN),
    FR(rootfr, K_PG, 8, U_IN),
    FR(btran, K_P, 8, U_OUT),
    FR(rootr, K_PG, 8, U_OUT),
    FR(rresis, K_PG, 8, U_INOUT),
};
const int ROOTMOIST_NFIELDS = sizeof(ROOTMOIST_TABLE) / sizeof(ROOTMOIST_TABLE[0]);

#define FF(name, kind, esz, use) FW(ctsmg_soilfluxes_io, name, kind, esz, use)
const FieldDesc SOILFLUXES_TABLE[] = {
    FF(snl, K_C, 4, U_IN),
    FF(col_patchi, K_C, 4, U_IN),
    FF(col_npatches, K_C, 4, U_IN),
    FF(frac_sno_eff, K_C, 8, U_IN),
    FF(frac_h2osfc, K_C, 8, U_IN),
    FF(t_grnd, K_C, 8, U_IN),
    FF(t_h2osfc, K_C, 8, U_IN),
    FF(t_h2osfc_bef, K_C, 8, U_IN),
    FF(c_h2osfc, K_C, 8, U_IN),
    FF(emg, K_C, 8, U_IN),
    FF(forc_lwrad, K_C, 8, U_IN),
    FF(htvp, K_C, 8, U_IN),
    FF(xmf, K_C, 8, U_IN),
    FF(xmf_h2osfc, K_C, 8, U_IN),
    FF(eflx_h2osfc_to_snow, K_C, 8, U_IN),
    FF(t_soisno, K_SS, 8, U_IN),
    FF(tssbef, K_SS, 8, U_IN),
    FF(fact, K_SS, 8, U_IN),
    FF(h2osoi_liq, K_SS, 8, U_IN),
    FF(h2osoi_ice, K_SS, 8, U_IN),
    FF(errsoi_col, K_C, 8, U_OUT),
    FF(patch_column, K_P, 4, U_IN),
    FF(frac_veg_nosno, K_P, 4, U_IN),
    FF(wtcol, K_P, 8, U_IN),
    FF(cgrnds, K_P, 8, U_IN),
    FF(cgrndl, K_P, 8, U_IN),
    FF(sabg_soil, K_P, 8, U_IN),
    FF(sabg_snow, K_P, 8, U_IN),
    FF(dlrad, K_P, 8, U_IN),
    FF(ulrad, K_P, 8, U_IN),
    FF(eflx_sh_veg, K_P, 8, U_IN),
    FF(qflx_evap_veg, K_P, 8, U_IN),
    FF(qflx_tran_veg, K_P, 8, U_IN),
    FF(eflx_sh_grnd, K_P, 8, U_INOUT),
    FF(qflx_evap_soi, K_P, 8, U_INOUT),
    FF(qflx_ev_snow, K_P, 8, U_INOUT),
    FF(qflx_ev_soil, K_P, 8, U_INOUT),
    FF(qflx_ev_h2osfc, K_P, 8, U_INOUT),
    FF(qflx_liqevap_from_top_layer, K_P, 8, U_OUT),
    FF(qflx_solidevap_from_top_layer, K_P, 8, U_OUT),
    FF(qflx_soliddew_to_top_layer, K_P, 8, U_OUT),
    FF(qflx_liqdew_to_top_layer, K_P, 8, U_OUT),
    FF(eflx_soil_grnd, K_P, 8, U_OUT),
    FF(eflx_sh_tot, K_P, 8, U_OUT),
    FF(qflx_evap_tot, K_P, 8, U_OUT),
    FF(eflx_lh_tot, K_P, 8, U_OUT),
    FF(qflx_evap_can, K_P, 8, U_OUT),
    FF(eflx_lh_vege, K_P, 8, U_OUT),
    FF(eflx_lh_vegt, K_P, 8, U_OUT),
    FF(eflx_lh_grnd, K_P, 8, U_OUT),
    FF(eflx_lwrad_out, K_P, 8, U_OUT),
    FF(eflx_lwrad_net, K_P, 8, U_OUT),
    FF(errsoi_patch, K_P, 8, U_OUT),
    FF(t_skin, K_P, 8, U_INOUT),
};
const int SOILFLUXES_NFIELDS = sizeof(SOILFLUXES_TABLE) / sizeof(SOILFLUXES_TABLE[0]);

const FieldDesc CANOPY_TABLE[] = {
    FC(itype, K_P, 4, U_IN),
    FC(patch_column, K_P, 4, U_IN),
    FC(patch_gridcell, K_P, 4, U_IN),
    FC(forc_u, K_GR, 8, U_IN),
    FC(forc_v, K_GR, 8, U_IN),
    FC(forc_hgt_u, K_GR, 8, U_IN),
    FC(forc_hgt_t, K_GR, 8, U_IN),
    FC(forc_hgt_q, K_GR, 8, U_IN),
    FC(forc_pco2, K_GR, 8, U_IN),
    FC(forc_po2, K_GR, 8, U_IN),
    FC(dayl, K_GR, 8, U_IN),
    FC(max_dayl, K_GR, 8, U_IN),
    FC(snl, K_C, 4, U_IN),
    FC(forc_pbot, K_C, 8, U_IN),
    FC(forc_th, K_C, 8, U_IN),
    FC(forc_q, K_C, 8, U_IN),
    FC(forc_rho, K_C, 8, U_IN),
    FC(forc_lwrad, K_C, 8, U_IN),
    FC(thv, K_C, 8, U_IN),
    FC(t_grnd, K_C, 8, U_IN),
    FC(qg, K_C, 8, U_IN),
    FC(qg_snow, K_C, 8, U_IN),
    FC(qg_soil, K_C, 8, U_IN),
    FC(qg_h2osfc, K_C, 8, U_IN),
    FC(dqgdT, K_C, 8, U_IN),
    FC(emg, K_C, 8, U_IN),
    FC(htvp, K_C, 8, U_IN),
    FC(z0mg, K_C, 8, U_IN),
    FC(snow_depth, K_C, 8, U_IN),
    FC(frac_sno_eff, K_C, 8, U_IN),
    FC(frac_h2osfc, K_C, 8, U_IN),
    FC(soilresis, K_C, 8, U_IN),
    FC(t_h2osfc, K_C, 8, U_IN),
    FC(t_soisno, K_SS, 8, U_IN),
    FC(frac_veg_nosno, K_P, 4, U_IN),
    FC(elai, K_P, 8, U_IN),
    FC(esai, K_P, 8, U_IN),
    FC(htop, K_P, 8, U_IN),
    FC(emv, K_P, 8, U_IN),
    FC(fwet, K_P, 8, U_IN),
    FC(fdry, K_P, 8, U_IN),
    FC(laisun, K_P, 8, U_IN),
    FC(laisha, K_P, 8, U_IN),
    FC(btran, K_P, 8, U_IN),
    FC(sabv, K_P, 8, U_IN),
    FC(thm, K_P, 8, U_IN),
    FC(t_a10, K_P, 8, U_IN),
    FC(parsun_z, K_P, 8, U_IN),
    FC(parsha_z, K_P, 8, U_IN),
    FC(vcmaxcintsun, K_P, 8, U_IN),
    FC(vcmaxcintsha, K_P, 8, U_IN),
    FC(displa, K_P, 8, U_INOUT),
    FC(z0mv, K_P, 8, U_INOUT),
    FC(t_veg, K_P, 8, U_INOUT),
    FC(liqcan, K_P, 8, U_INOUT),
    FC(snocan, K_P, 8, U_INOUT),
    FC(cgrnds, K_P, 8, U_INOUT),
    FC(cgrndl, K_P, 8, U_INOUT),
    FC(z0hv, K_P, 8, U_OUT),
    FC(z0qv, K_P, 8, U_OUT),
    FC(forc_hgt_u_patch, K_P, 8, U_OUT),
    FC(forc_hgt_t_patch, K_P, 8, U_OUT),
    FC(forc_hgt_q_patch, K_P, 8, U_OUT),
    FC(taf, K_P, 8, U_OUT),
    FC(qaf, K_P, 8, U_OUT),
    FC(ustar, K_P, 8, U_OUT),
    FC(um, K_P, 8, U_OUT),
    FC(obu, K_P, 8, U_OUT),
    FC(zeta, K_P, 8, U_OUT),
    FC(ram1, K_P, 8, U_OUT),
    FC(rah1, K_P, 8, U_OUT),
    FC(raw1, K_P, 8, U_OUT),
    FC(rah2, K_P, 8, U_OUT),
    FC(raw2, K_P, 8, U_OUT),
    FC(rb1, K_P, 8, U_OUT),
    FC(uaf, K_P, 8, U_OUT),
    FC(vpd, K_P, 8, U_OUT),
    FC(rhaf, K_P, 8, U_OUT),
    FC(eflx_sh_veg, K_P, 8, U_OUT),
    FC(qflx_evap_veg, K_P, 8, U_OUT),
    FC(qflx_tran_veg, K_P, 8, U_OUT),
    FC(eflx_sh_grnd, K_P, 8, U_OUT),
    FC(eflx_sh_snow, K_P, 8, U_OUT),
    FC(eflx_sh_soil, K_P, 8, U_OUT),
    FC(eflx_sh_h2osfc, K_P, 8, U_OUT),
    FC(qflx_evap_soi, K_P, 8, U_OUT),
    FC(qflx_ev_snow, K_P, 8, U_OUT),
    FC(qflx_ev_soil, K_P, 8, U_OUT),
    FC(qflx_ev_h2osfc, K_P, 8, U_OUT),
    FC(t_ref2m, K_P, 8, U_OUT),
    FC(q_ref2m, K_P, 8, U_OUT),
    FC(rh_ref2m, K_P, 8, U_OUT),
    FC(vpd_ref2m, K_P, 8, U_OUT),
    FC(dlrad, K_P, 8, U_OUT),
    FC(ulrad, K_P, 8, U_OUT),
    FC(t_skin, K_P, 8, U_OUT),
    FC(cgrnd, K_P, 8, U_OUT),
    FC(taux, K_P, 8, U_OUT),
    FC(tauy, K_P, 8, U_OUT),
    FC(err_canopy, K_P, 8, U_OUT),
    FC(rssun, K_P, 8, U_OUT),
    FC(rssha, K_P, 8, U_OUT),
    FC(psnsun, K_P, 8, U_OUT),
    FC(psnsha, K_P, 8, U_OUT),
    FC(lmrsun, K_P, 8, U_OUT),
    FC(lmrsha, K_P, 8, U_OUT),
    FC(cisun, K_P, 8, U_OUT),
    FC(cisha, K_P, 8, U_OUT),
    FC(gs_mol_sun, K_P, 8, U_OUT),
    FC(gs_mol_sha, K_P, 8, U_OUT),
    FC(rh_leaf, K_P, 8, U_OUT),
    FC(vpd_can, K_P, 8, U_OUT),
    FC(u10_clm, K_P, 8, U_OUT),
    FC(u10, K_P, 8, U_OUT),
    FC(fv, K_P, 8, U_OUT),
    FC(vds, K_P, 8, U_OUT),
    FC(fm, K_P, 8, U_OUT),
    FC(num_iter, K_P, 4, U_OUT),
};
const int CANOPY_NFIELDS = sizeof(CANOPY_TABLE) / sizeof(CANOPY_TABLE[0]);

static inline void*& field_ptr(void* io, const FieldDesc& f) {
    return *reinterpret_cast<void**>(reinterpret_cast<char*>(io) + f.offset);
}

size_t field_bytes(const FieldDesc& f, int ldc, int ldp, int ldg) {
    int ld = (f.kind == K_P || f.kind == K_PL || f.kind == K_PS || f.kind == K_PG) ? ldp : (f.kind == K_GR ? ldg : ldc);
    return (size_t)ld * kind_levels(f.kind) * f.esize;
}

// One field's levels between the caller's array and its device copy (both
// with leading dimension ld): only the n columns (patches) the call's bounds
// span of each level move, so a clump that passes a view into arrays shared
// with other clumps (c_loc(field(begc, lb)) with the processor-wide leading
// dimension) reads and writes its own columns alone.
static cudaError_t copy_field(void* dst, const void* src, const FieldDesc& f, int ld, int n, cudaMemcpyKind k,
                              cudaStream_t s) {
    const bool in = k == cudaMemcpyHostToDevice;
    const size_t es = f.esize, pitch = (size_t)ld * es, off = (in ? copy_in_row0(f) : copy_row0(f)) * pitch;
    const size_t rows = in ? copy_in_rows(f) : copy_rows(f);
    if (n >= ld) return copy_async(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off, rows * pitch, k, s);
    if (n <= 0) return cudaSuccess;
    return copy_2d_async(static_cast<char*>(dst) + off, pitch, static_cast<const char*>(src) + off, pitch,
                         (size_t)n * es, rows, k, s);
}

// Leading dimension and bounds extent of a field's kind (gridcell arrays move whole).
static void field_extent(const FieldDesc& f, int ldc, int ldp, int ldg, int nc, int np, int* ld, int* n) {
    const bool pf = f.kind == K_P || f.kind == K_PL || f.kind == K_PS || f.kind == K_PG;
    *ld = pf ? ldp : (f.kind == K_GR ? ldg : ldc);
    *n = pf ? (np < 0 ? ldp : np) : (f.kind == K_GR ? ldg : (nc < 0 ? ldc : nc));
}

// Copy the host struct's arrays into the arena; fill dio with device pointers.
// nc / np: columns / patches of the call's bounds (-1: the whole leading dimension).
static int stage_in(ThreadCtx* c, const void* hio, void* dio, size_t io_size, const FieldDesc* tab, int nf,
                    int ldc, int ldp, int ldg, int nc, int np) {
    std::memcpy(dio, hio, io_size);
    for (int i = 0; i < nf; ++i) {
        const void* hp = field_ptr(const_cast<void*>(hio), tab[i]);
        if (!hp) {
            std::string m = std::string("null pointer for component ") + tab[i].name;
            return set_error(CTSMG_E_ARG, m.c_str(), 0, 0);
        }
        size_t nb = field_bytes(tab[i], ldc, ldp, ldg);
        void* dp = arena_take(c, nb);
        if (!tab[i].no_in) {
            int ld, n;
            field_extent(tab[i], ldc, ldp, ldg, nc, np, &ld, &n);
            cudaError_t e = copy_field(dp, hp, tab[i], ld, n, cudaMemcpyHostToDevice, c->stream);
            if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync H2D");
        }
        field_ptr(dio, tab[i]) = dp;
    }
    return 0;
}

static int stage_out(ThreadCtx* c, const void* hio, const void* dio, const FieldDesc* tab, int nf,
                     int ldc, int ldp, int ldg, int nc, int np) {
    for (int i = 0; i < nf; ++i) {
        if (tab[i].use == U_IN) continue;
        void* hp = field_ptr(const_cast<void*>(hio), tab[i]);
        const void* dp = field_ptr(const_cast<void*>(dio), tab[i]);
        int ld, n;
        field_extent(tab[i], ldc, ldp, ldg, nc, np, &ld, &n);
        cudaError_t e = copy_field(hp, dp, tab[i], ld, n, cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync D2H");
    }
    return 0;
}

static size_t table_bytes(const FieldDesc* tab, int nf, int ldc, int ldp, int ldg = 0) {
    size_t s = 0;
    for (int i = 0; i < nf; ++i) s += ((field_bytes(tab[i], ldc, ldp, ldg) + 255) & ~(size_t)255);
    return s;
}

int check_filter(const ctsmg_bounds* b, int nf, const int32_t* filt) {
    if (!b) return set_error(CTSMG_E_ARG, "null bounds", 0, 0);
    if (b->endc < b->begc) return set_error(CTSMG_E_ARG, "endc < begc", 0, 0);
    if (nf < 0) return set_error(CTSMG_E_ARG, "negative filter length", 0, 0);
    if (nf > 0 && !filt) return set_error(CTSMG_E_ARG, "null filter", 0, 0);
    for (int i = 0; i < nf; ++i)
        if (filt[i] < b->begc || filt[i] > b->endc)
            return set_error(CTSMG_E_ARG, "filter index outside bounds", filt[i], 0);
    return 0;
}

// ------------------------------------------------------------ pipelined calls
// A call over an ascending filter is split into chunks of the filter; chunk k
// copies the column range (and patch range) its filter entries span, its
// kernel runs once those copies are in, and its outputs go back while later
// chunks copy in and compute.  Columns of a range that are not in the filter
// travel in and out unchanged.  Chunks whose patch ranges would overlap (a
// patch order that does not follow the columns) run the call in one piece.
struct Chunk { int f0, f1, c0, c1, p0, p1; };

// Filter entries per chunk for a kernel whose full-GPU wave is `wave`
// columns: chunks of about one wave (a chunk's kernel seldom overlaps the
// next one, whose data is still arriving, so a fraction of a wave leaves SMs
// idle and a wave and a bit costs two), at least 4 and at most PIPE_CHUNKS of
// them, rounded up to whole waves when larger than one.  wave = 0: PIPE_CHUNKS
// equal chunks.
static int chunk_columns(int num, int wave) {
    if (wave <= 0) return (num + PIPE_CHUNKS - 1) / PIPE_CHUNKS;
    long long k = ((long long)num + wave / 2) / wave;
    k = std::min<long long>(std::max<long long>(k, 4), PIPE_CHUNKS);
    long long cc = (num + k - 1) / k;
    if (cc > wave) cc = (cc + wave - 1) / wave * wave;
    return (int)cc;
}

static bool plan_chunks(const ctsmg_bounds* b, int num, const int32_t* filt, const int32_t* col_patchi,
                        const int32_t* col_npatches, int wave, std::vector<Chunk>& out) {
    if (num < PIPE_MIN_COLUMNS || !filt) return false;
    for (int i = 1; i < num; ++i)
        if (filt[i] <= filt[i - 1]) return false;
    out.clear();
    // chunk boundaries (filter positions)
    std::vector<int> fb{0};
    if (wave > 0 && num > 3 * wave && PIPE_CHUNKS >= 4) {
        // wave-sized chunks between a quarter-wave first and last chunk: the
        // pipeline's fill (the first copy-in, before any kernel) and drain
        // (the last kernel and copy-out, after the last copy-in) shrink to a
        // quarter of a wave's
        const int t = std::max(wave / 4, 1), mid = num - 2 * t;
        const int k = std::min(std::max((mid + wave - 1) / wave, 1), PIPE_CHUNKS - 2);
        const long long cc = ((long long)mid + k - 1) / k;
        fb.push_back(t);
        for (int i = 1; i < k; ++i) fb.push_back(t + (int)std::min<long long>(cc * i, mid));
        fb.push_back(num - t);
        fb.push_back(num);
    } else {
        const int cc = chunk_columns(num, wave);
        for (int k = 1; k <= PIPE_CHUNKS; ++k) {
            const int e = (int)std::min<long long>((long long)cc * k, num);
            if (e > fb.back()) fb.push_back(e);
        }
    }
    for (size_t k = 0; k + 1 < fb.size(); ++k) {
        Chunk ch;
        ch.f0 = fb[k];
        ch.f1 = fb[k + 1];
        if (ch.f1 <= ch.f0) continue;
        ch.c0 = filt[ch.f0] - b->begc;
        ch.c1 = filt[ch.f1 - 1] - b->begc + 1;
        ch.p0 = ch.p1 = 0;
        if (col_patchi) {
            int lo = 1 << 30, hi = -1;
            for (int c = ch.c0; c < ch.c1; ++c) {
                if (col_npatches[c] <= 0) continue;
                lo = std::min(lo, col_patchi[c] - b->begp);
                hi = std::max(hi, col_patchi[c] + col_npatches[c] - 1 - b->begp);
            }
            if (hi >= lo) { ch.p0 = lo; ch.p1 = hi + 1; }
            if (!out.empty() && ch.p1 > ch.p0 && out.back().p1 > out.back().p0 && ch.p0 < out.back().p1) return false;
        }
        out.push_back(ch);
    }
    return out.size() > 1;
}

// Strided copy of the [lo, hi) column (or patch) slice of every level of one
// field between the caller's array and its device copy (both with ld).
static cudaError_t copy_slice(const FieldDesc& f, void* dst, const void* src, int ld, int lo, int hi,
                              cudaMemcpyKind kind, cudaStream_t s) {
    if (hi <= lo) return cudaSuccess;
    const bool in = kind == cudaMemcpyHostToDevice;
    const size_t es = f.esize, pitch = (size_t)ld * es, w = (size_t)(hi - lo) * es;
    const size_t off = (in ? copy_in_row0(f) : copy_row0(f)) * pitch + lo * es;
    return copy_2d_async(static_cast<char*>(dst) + off, pitch, static_cast<const char*>(src) + off, pitch,
                             w, in ? copy_in_rows(f) : copy_rows(f), kind, s);
}

static bool patch_field(const FieldDesc& f) { return f.kind == K_P || f.kind == K_PL || f.kind == K_PS || f.kind == K_PG; }

// Device copies of every component (arena), no data moved yet.
static void stage_alloc(ThreadCtx* c, const void* hio, void* dio, size_t io_size, const FieldDesc* tab, int nf,
                        int ldc, int ldp) {
    std::memcpy(dio, hio, io_size);
    for (int i = 0; i < nf; ++i) field_ptr(dio, tab[i]) = arena_take(c, field_bytes(tab[i], ldc, ldp, 0));
}

// Prepares the gather copy-in of a pipelined call (c->gather) when every
// array it copies in is page-locked and mapped into the device's address
// space with its elements aligned, and the copy mode allows it; otherwise the
// call's copy-in uses the copy engines.
static void gather_setup(ThreadCtx* c, const void* hio, const void* dio, const FieldDesc* tab, int nf, int ldc,
                         int ldp) {
    c->gather = false;
    if (g_copy_mode.load() != 0) return;
    GatherTable& T = c->gt;
    T.n = 0;
    for (int i = 0; i < nf; ++i) {
        const FieldDesc& f = tab[i];
        if (f.no_in) continue;
        if (T.n == GATHER_MAX_FIELDS || (f.esize != 8 && f.esize != 4)) return;
        const void* h = field_ptr(const_cast<void*>(hio), f);
        if (!h || (reinterpret_cast<uintptr_t>(h) % f.esize) != 0) return;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        if (a.type != cudaMemoryTypeHost || !a.devicePointer ||
            (reinterpret_cast<uintptr_t>(a.devicePointer) % f.esize) != 0)
            return;
        const bool pf = patch_field(f);
        GatherField& g = T.f[T.n++];
        g.src = static_cast<const char*>(a.devicePointer);
        g.dst = static_cast<char*>(field_ptr(const_cast<void*>(dio), f));
        g.pitch = pf ? ldp : ldc;
        g.esize = f.esize;
        g.row0 = (int)copy_in_row0(f);
        g.rows = copy_in_rows(f);
        g.patch = pf ? 1 : 0;
    }
    if (!c->gather_grid) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        c->gather_grid = CTSMG_GATHER_BLOCKS_PER_SM * (sms > 0 ? sms : 1);
    }
    c->gather = true;
}

// The stream that carries a pipelined call's copy-in.
static cudaStream_t in_stream(ThreadCtx* c) { return c->gather ? c->h2dk : c->h2d; }

// ---------------------------------------------------- time-constant inputs
// With ctsmg_set_time_constant_inputs(1) a pipelined call keeps the device
// copy of each input the model never changes after initialisation (soil
// hydraulic and thermal properties, the soil-layer geometry) per host array
// and copied rows (SoilWater and SoilTemperature copy different rows of the
// same arrays, so each keeps its own), and copies it in again only when the
// call's columns are not yet covered or after
// ctsmg_invalidate_time_constant_inputs.
static std::atomic<int> g_tc_on{0};
static std::atomic<unsigned> g_tc_gen{1};

static bool time_constant(const char* name, const char* const* names) {
    for (int i = 0; names[i]; ++i)
        if (std::strcmp(name, names[i]) == 0) return true;
    return false;
}
// SoilWater's Zeng-Decker form copies levels 1..nlevsoi of z / dz and the soil
// interfaces only: the soil layers, which do not move
static const char* const TC_SOILWATER[] = {"z", "zi", "dz", "smpmin", "watsat", "hksat", "bsw", "sucsat", nullptr};
static const char* const TC_SOILTEMP[] = {"watsat", "bsw", "sucsat", "tkmg", "tkdry", "csol", nullptr};

// Points the time-constant components of a pipelined call at their kept
// device copies (dio), marks the ones already covered for [lo, hi) as not
// copied in (tab), and returns the entries this call fills.
static int tc_bind(ThreadCtx* c, const void* hio, void* dio, std::vector<FieldDesc>& tab, const char* const* names,
                   int ldc, int ldp, int lo, int hi, std::vector<ThreadCtx::TcEntry*>& fill) {
    fill.clear();
    if (!g_tc_on.load()) return 0;
    if (c->tc_gen != g_tc_gen.load()) {
        for (auto& t : c->tc)
            if (t.dev) cudaFree(t.dev);
        c->tc.clear();
        c->tc_gen = g_tc_gen.load();
    }
    c->tc.reserve(c->tc.size() + tab.size());          // the pointers in fill stay valid
    for (FieldDesc& f : tab) {
        if (!time_constant(f.name, names) || f.use != U_IN) continue;
        const void* h = field_ptr(const_cast<void*>(hio), f);
        const size_t bytes = field_bytes(f, ldc, ldp, 0);
        const int row0 = (int)copy_in_row0(f), rows = copy_in_rows(f);
        ThreadCtx::TcEntry* e = nullptr;
        for (auto& t : c->tc)
            if (t.host == h && t.ld == ldc && t.esize == f.esize && t.bytes == bytes && t.row0 == row0 &&
                t.rows == rows) {
                e = &t;
                break;
            }
        if (!e) {
            void* d = nullptr;
            cudaError_t ce = cudaMalloc(&d, bytes);
            if (ce != cudaSuccess) return cuda_fail(ce, "cudaMalloc(time-constant input)");
            c->tc.push_back(ThreadCtx::TcEntry{h, ldc, f.esize, row0, rows, bytes, d, 0, 0, false});
            e = &c->tc.back();
        }
        field_ptr(dio, f) = e->dev;
        if (e->valid && e->lo <= lo && hi <= e->hi) f.no_in = 1;
        else fill.push_back(e);
    }
    return 0;
}

// After a successful call: the entries it filled now cover [lo, hi).
static void tc_commit(std::vector<ThreadCtx::TcEntry*>& fill, int lo, int hi) {
    for (auto* e : fill) {
        e->valid = true;
        e->lo = lo;
        e->hi = hi;
    }
    fill.clear();
}

// Timeline mark `slot` of chunk k on stream s when the calling thread traces
// its pipelined calls (0 copy-in start, 1 copy-in end, 2 kernel start,
// 3 kernel end, 4 copy-out end).
static void trace_mark(ThreadCtx* c, int k, int slot, cudaStream_t s) {
    if (!c->trace || !c->tr[k][slot]) return;
    cudaEventRecord(c->tr[k][slot], s);
    const auto now = std::chrono::steady_clock::now();
    if (k == 0 && slot == 0) c->tr_t0 = now;
    const float ms = std::chrono::duration<float, std::milli>(now - c->tr_t0).count();
    if (slot == 1) c->trh[k][0] = ms;
    if (slot == 4) c->trh[k][1] = ms;
}

// Enqueue the copy-in of chunk k's components (h2d stream).
static int chunk_copies_in(ThreadCtx* c, const Chunk& ch, const void* hio, const void* dio, const FieldDesc* tab,
                           int nf, int ldc, int ldp) {
    if (c->gather) {
        size_t bytes = 0;
        for (int i = 0; i < c->gt.n; ++i) {
            const GatherField& g = c->gt.f[i];
            bytes += (size_t)g.rows * g.esize * (size_t)(g.patch ? ch.p1 - ch.p0 : ch.c1 - ch.c0);
        }
        count_copy(cudaMemcpyHostToDevice, bytes);
        gather_kernel<<<c->gather_grid, 256, 0, c->h2dk>>>(c->gt, ch.c0, ch.c1, ch.p0, ch.p1);
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? 0 : cuda_fail(e, "gather kernel launch");
    }
    for (int i = 0; i < nf; ++i) {
        const FieldDesc& f = tab[i];
        if (f.no_in) continue;
        const bool pf = patch_field(f);
        cudaError_t e = copy_slice(f, field_ptr(const_cast<void*>(dio), f), field_ptr(const_cast<void*>(hio), f),
                                   pf ? ldp : ldc, pf ? ch.p0 : ch.c0, pf ? ch.p1 : ch.c1, cudaMemcpyHostToDevice,
                                   c->h2d);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy2DAsync H2D");
    }
    return 0;
}

// Enqueue the copy-in of chunk k (h2d stream) and record ev_in[k].
static int chunk_in(ThreadCtx* c, const Chunk& ch, int k, const void* hio, const void* dio, const FieldDesc* tab,
                    int nf, int ldc, int ldp) {
    trace_mark(c, k, 0, in_stream(c));
    int rc = chunk_copies_in(c, ch, hio, dio, tab, nf, ldc, ldp);
    if (rc) return rc;
    trace_mark(c, k, 1, in_stream(c));
    cudaError_t e = cudaEventRecord(c->ev_in[k], in_stream(c));
    return e == cudaSuccess ? 0 : cuda_fail(e, "cudaEventRecord");
}

// After the kernel of chunk k (ev_done[k]), enqueue its copy-out (d2h stream).
static int chunk_out(ThreadCtx* c, const Chunk& ch, int k, const void* hio, const void* dio, const FieldDesc* tab,
                     int nf, int ldc, int ldp) {
    cudaError_t e = cudaStreamWaitEvent(c->d2h, c->ev_done[k], 0);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamWaitEvent");
    for (int i = 0; i < nf; ++i) {
        const FieldDesc& f = tab[i];
        if (f.use == U_IN) continue;
        const bool pf = patch_field(f);
        e = copy_slice(f, field_ptr(const_cast<void*>(hio), f), field_ptr(const_cast<void*>(dio), f), pf ? ldp : ldc,
                       pf ? ch.p0 : ch.c0, pf ? ch.p1 : ch.c1, cudaMemcpyDeviceToHost, c->d2h);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy2DAsync D2H");
    }
    trace_mark(c, k, 4, c->d2h);
    return 0;
}

// Compute stream of chunk k.  A chunk of a pipelined call is a fraction of a
// wave of the GPU; consecutive chunks run on PIPE_STREAMS streams in turn so
// that the kernels of chunks whose data have arrived run side by side (their
// columns are disjoint).
static cudaStream_t chunk_stream(ThreadCtx* c, int k) {
    const int i = k % PIPE_STREAMS;
    return i ? c->xs[i - 1] : c->stream;
}

// Order the further compute streams after the work already queued on
// c->stream (the status reset).
static int fork_streams(ThreadCtx* c) {
    cudaError_t e = cudaEventRecord(c->ev_done[0], c->stream);
    for (cudaStream_t x : c->xs)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(x, c->ev_done[0], 0);
    return e == cudaSuccess ? 0 : cuda_fail(e, "fork streams");
}

static cudaError_t join_streams(ThreadCtx* c) {
    cudaError_t e = cudaStreamSynchronize(c->d2h);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    for (cudaStream_t x : c->xs)
        if (e == cudaSuccess) e = cudaStreamSynchronize(x);
    return e;
}

// Page-locked host buffer of n filter entries (grown on demand).
static int32_t* order_buffer(ThreadCtx* c, size_t n) {
    if (n <= c->order_cap) return c->order;
    if (c->order) cudaFreeHost(c->order);
    c->order = nullptr;
    c->order_cap = 0;
    const size_t cap = n + n / 4 + 1024;
    if (cudaMallocHost(&c->order, cap * sizeof(int32_t)) != cudaSuccess) {
        c->order = nullptr;
        return nullptr;
    }
    c->order_cap = cap;
    return c->order;
}

// Filter entries [f0, f1) grouped by water-table depth in 0.25 m bins (a
// stable counting sort) into out[f0..f1): the Zeng-Decker solve branches on
// the level that holds the water table, so a warp whose columns share it
// runs one branch per level.
static void group_by_water_table(const int32_t* filt, int f0, int f1, const double* zwt, int begc, int32_t* out) {
    if (!CTSMG_GROUP_COLUMNS) {
        std::memcpy(out + f0, filt + f0, (size_t)(f1 - f0) * sizeof(int32_t));
        return;
    }
    constexpr int NK = 64;
    int count[NK + 1];
    std::memset(count, 0, sizeof count);
    auto key = [&](int32_t col) {
        const double z = zwt[col - begc] * 4.0;
        return (z >= 0.0 && z < (double)(NK - 1)) ? (int)z : NK - 1;    // deeper, negative or NaN: last bin
    };
    for (int i = f0; i < f1; ++i) ++count[key(filt[i]) + 1];
    for (int k = 0; k < NK; ++k) count[k + 1] += count[k];
    for (int i = f0; i < f1; ++i) out[f0 + count[key(filt[i])]++] = filt[i];
}

// Filter entries [f0, f1) grouped by snow layers, then bedrock depth (deepest
// first; a stable counting sort) into out[f0..f1): a warp of the heat-solve
// kernel then takes columns whose level loops have the same lengths, as the
// resident step's column order does.  Each column's result does not depend
// on the order, and the set of columns of [f0, f1) is unchanged.
static void group_by_layers(const int32_t* filt, int f0, int f1, const int32_t* snl, const int32_t* nbedrock,
                            int begc, int32_t* out) {
    if (!CTSMG_GROUP_COLUMNS) {
        std::memcpy(out + f0, filt + f0, (size_t)(f1 - f0) * sizeof(int32_t));
        return;
    }
    constexpr int NB = NLEVGRND + 2, NK = (NLEVSNO + 1) * NB;
    int count[NK + 1];
    std::memset(count, 0, sizeof count);
    auto key = [&](int32_t col) {
        const int cc = col - begc;
        const int sn = std::min(std::max(-snl[cc], 0), NLEVSNO);
        const int nb = nbedrock ? std::min(std::max(nbedrock[cc], 0), NB - 1) : 0;
        return (NLEVSNO - sn) * NB + (NB - 1 - nb);
    };
    for (int i = f0; i < f1; ++i) ++count[key(filt[i]) + 1];
    for (int k = 0; k < NK; ++k) count[k + 1] += count[k];
    for (int i = f0; i < f1; ++i) out[f0 + count[key(filt[i])]++] = filt[i];
}

static int read_error(ThreadCtx* c, int* code, int* index, int* level) {
    DevError h;
    cudaError_t e = copy_sync(&h, c->err, sizeof h, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(err)");
    if (h.key == ~0ull) { *code = 0; return 0; }
    *code = (int)(h.key & 0xff);
    *index = (int)(h.key >> 32);
    *level = (int)((h.key >> 8) & 0xffffff) - 1024;
    return 0;
}

ctsmg_soil_resistance_params current_soil_resistance() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_sres;
}

ctsmg_soilwater_movement_nml current_soilwater_nml() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_swm;
}

int current_snow_method() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_init ? g_opt.snow_thermal_cond_method : 0;
}

bool snow_method_if_init(int* method) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_init) return false;
    *method = g_opt.snow_thermal_cond_method;
    return true;
}

} // namespace ctsmg

using namespace ctsmg;

// ============================================================ C-ABI
extern "C" int32_t ctsmg_init(const ctsmg_options* opt) {
    if (!opt) return set_error(CTSMG_E_ARG, "null options", 0, 0);
    if (opt->nlevsno != NLEVSNO || opt->nlevsoi != NLEVSOI || opt->nlevgrnd != NLEVGRND)
        return set_error(CTSMG_E_UNSUPPORTED, "only nlevsno=12, nlevsoi=20, nlevgrnd=25 (20SL_8.5m) are built", 0, 0);
    if (opt->soilwater_movement_method != 0 && opt->soilwater_movement_method != 1)
        return set_error(CTSMG_E_UNSUPPORTED,
                         "soilwater_movement_method must be 0 (Zeng-Decker 2009) or 1 (moisture form)", 0, 0);
    if (opt->snow_thermal_cond_method != 0 && opt->snow_thermal_cond_method != 1)
        return set_error(CTSMG_E_ARG, "snow_thermal_cond_method must be 0 (Jordan1991) or 1 (Sturm1997)", 0, 0);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1) return cuda_fail(e == cudaSuccess ? cudaErrorNoDevice : e, "cudaGetDeviceCount");
    e = cudaSetDevice(0);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    std::lock_guard<std::mutex> lk(g_mu);
    g_opt = *opt;
    // the namelist defaults for this method (namelist_defaults_ctsm.xml:471-488)
    g_swm = ctsmg_soilwater_movement_nml{opt->soilwater_movement_method, 1,
                                         opt->soilwater_movement_method == 0 ? 4 : 2, 1, 0,
                                         opt->soilwater_movement_method == 0 ? 0 : 1, 60.0, 1.e-8, 1.e-1, 1.e-2};
    g_init = true;
    return 0;
}

extern "C" int32_t ctsmg_set_soilwater_movement(const ctsmg_soilwater_movement_nml* nml) {
    if (!nml) return set_error(CTSMG_E_ARG, "null namelist", 0, 0);
    const int m = nml->soilwater_movement_method, ubc = nml->upper_boundary_condition,
              lbc = nml->lower_boundary_condition;
    if (m != 0 && m != 1)
        return set_error(CTSMG_E_UNSUPPORTED, "soilwater_movement_method must be 0 or 1 (mixed and head forms are empty "
                         "in the reference)", 0, 0);
    if (m == 0 && lbc != 4)
        return set_error(CTSMG_E_ARG, "ERROR inconsistent soilwater_movement namelist: ZD09 must use bc_aquifer lbc", 0, 0);
    if (nml->use_bedrock && lbc != 2)
        return set_error(CTSMG_E_ARG, "ERROR inconsistent soilwater_movement namelist: use_bedrock requires "
                         "bc_zero_flux lbc", 0, 0);
    if (ubc != 1)
        return set_error(CTSMG_E_UNSUPPORTED, "upper_boundary_condition must be bc_flux (bc_head reads a boundary water "
                         "content the reference never sets)", 0, 0);
    if (m == 1 && (lbc < 1 || lbc > 3))
        return set_error(CTSMG_E_UNSUPPORTED, "the moisture form supports lower_boundary_condition bc_flux, "
                         "bc_zero_flux or bc_waterTable", 0, 0);
    if (m == 1 && !(nml->dtmin > 0.0 && nml->verySmall > 0.0 && nml->xTolerUpper > 0.0 && nml->xTolerLower >= 0.0))
        return set_error(CTSMG_E_ARG, "dtmin, verySmall, xTolerUpper must be positive", 0, 0);
    std::lock_guard<std::mutex> lk(g_mu);
    g_swm = *nml;
    return 0;
}

extern "C" int32_t ctsmg_set_soilwater_params(const ctsmg_soilwater_params* p) {
    if (!p) return set_error(CTSMG_E_ARG, "null params", 0, 0);
    std::lock_guard<std::mutex> lk(g_mu);
    g_swp = *p;
    return 0;
}

extern "C" int32_t ctsmg_finalize(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (ThreadCtx* c : g_ctxs) delete c;
    g_ctxs.clear();
    t_ctx = nullptr;
    ++g_gen;
    g_init = false;
    noalloc_forget_devices();
    return 0;
}

extern "C" const char* ctsmg_last_error(void) { return t_msg.c_str(); }

extern "C" int32_t ctsmg_last_error_index(int32_t* index, int32_t* level) {
    if (index) *index = t_idx;
    if (level) *level = t_lev;
    return 0;
}

// The fields one SoilWater call stages: the Zeng-Decker table, or the
// moisture form's, plus what the use_flexibleCN fix reads and writes.
static std::vector<FieldDesc> soilwater_fields(const ctsmg_soilwater_movement_nml& nml) {
    std::vector<FieldDesc> t;
    if (nml.soilwater_movement_method == 0) {
        t.assign(SOILWATER_TABLE, SOILWATER_TABLE + SOILWATER_NFIELDS);
    } else {
        t.assign(SOILWATER_MF_TABLE, SOILWATER_MF_TABLE + SOILWATER_MF_NFIELDS);
    }
    if (nml.use_flexibleCN) {
        auto put = [&](const FieldDesc& f) {
            for (auto& g : t)
                if (g.offset == f.offset) { g.use = f.use; return; }
            t.push_back(f);
        };
        for (int i = 0; i < SOILWATER_FLEXCN_NFIELDS; ++i) put(SOILWATER_FLEXCN_TABLE[i]);
    }
    return t;
}

static cudaError_t launch_soilwater_call(const ctsmg_soilwater_io& dio, int begc, int n, const int32_t* dfilt,
                                         const ctsmg_soilwater_movement_nml& nml, double e_ice, double dtime,
                                         DevError* err, cudaStream_t s, int* d_counter) {
    cudaError_t e;
    if (nml.soilwater_movement_method == 0) {
        e = launch_soilwater(dio, begc, n, dfilt, e_ice, dtime, s);
    } else {
        MoistureFormArgs P{e_ice, dtime, nml.dtmin, nml.verySmall, nml.xTolerUpper, nml.xTolerLower,
                           nml.lower_boundary_condition, nml.flux_calculation == 42 ? 1 : 0,
                           moisture_form_max_trials(dtime, nml.dtmin)};
        e = launch_moisture_form(dio, begc, n, dfilt, P, err, s, d_counter);
    }
    if (e == cudaSuccess && nml.use_flexibleCN) e = launch_flexcn(dio, begc, n, dfilt, s);
    return e;
}

static int soilwater_error(int code, int idx, int lev) {
    if (code == CTSMG_E_SINGULAR)
        return set_error(code, "soilwater_moisture_form:: problem with the lapack solver", idx, lev);
    return set_error(code, "soilwater_moisture_form:: sub-step loop did not complete the time step", idx, lev);
}

extern "C" int32_t ctsmg_soilwater(const ctsmg_bounds* bounds, int32_t num_hydrologyc,
                                   const int32_t* filter_hydrologyc, const ctsmg_soilwater_io* io,
                                   double dtime) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if ((rc = check_filter(bounds, num_hydrologyc, filter_hydrologyc))) return rc;
    const int ncol = bounds->endc - bounds->begc + 1;
    if (io->ldc < ncol) return set_error(CTSMG_E_ARG, "ldc smaller than endc-begc+1", 0, 0);
    if (!(dtime > 0.0)) return set_error(CTSMG_E_ARG, "dtime must be positive", 0, 0);
    ctsmg_soilwater_movement_nml nml;
    double e_ice;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        nml = g_swm;
        e_ice = g_swp.e_ice;
    }
    std::vector<FieldDesc> tab = soilwater_fields(nml);
    // outputs are left uncopied on the way in only when the filter covers
    // every column of the bounds (columns outside it keep their values)
    bool dense = num_hydrologyc == ncol;
    for (int i = 0; dense && i < num_hydrologyc; ++i) dense = filter_hydrologyc[i] == bounds->begc + i;
    if (!dense)
        for (auto& f : tab) f.no_in = 0;
    const FieldDesc* T = tab.data();
    const int NT = (int)tab.size();
    for (const FieldDesc& f : tab)
        if (!field_ptr(const_cast<ctsmg_soilwater_io*>(io), f)) {
            std::string m = std::string("null pointer for component ") + f.name;
            return set_error(CTSMG_E_ARG, m.c_str(), 0, 0);
        }
    if (nml.soilwater_movement_method == 1) {
        for (int i = 0; i < num_hydrologyc; ++i) {
            const int nb = io->nbedrock[filter_hydrologyc[i] - bounds->begc];
            if (nb < 2 || nb > NLEVSOI)
                return set_error(CTSMG_E_ARG, "nbedrock outside 2..nlevsoi", filter_hydrologyc[i], 0);
            if (nml.lower_boundary_condition == 3 && nb != NLEVSOI)
                return set_error(CTSMG_E_ARG, "bc_waterTable needs nbedrock = nlevsoi (use_bedrock = .false.)",
                                 filter_hydrologyc[i], 0);
        }
    }
    if (num_hydrologyc == 0) return 0;
    const int ldc = io->ldc;
    size_t need = table_bytes(T, NT, ldc, 0) + (size_t)num_hydrologyc * 4 + 4096 + 128 * PIPE_STREAMS;
    if ((rc = arena_reserve(c, need))) return rc;
    int* dcounter = (int*)arena_take(c, 128 * PIPE_STREAMS);   // one 128-byte slot per compute stream
    cudaError_t e = cudaMemsetAsync(c->err, 0xff, sizeof(DevError), c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(err)");
    std::vector<Chunk> chunks;
    // SoilWater runs in PIPE_CHUNKS equal chunks: its copies and kernels take
    // about as long as each other, and wave-sized chunks between quarter-wave
    // ends measured 0.4 ms slower per call with the gather copy-in
    if (plan_chunks(bounds, num_hydrologyc, filter_hydrologyc, nullptr, nullptr, 0, chunks)) {
        ctsmg_soilwater_io dio;
        stage_alloc(c, io, &dio, sizeof dio, T, NT, ldc, 0);
        std::vector<ThreadCtx::TcEntry*> tc_fill;
        const int tc_lo = chunks.front().c0, tc_hi = chunks.back().c1;
        if (nml.soilwater_movement_method == 0 &&
            (rc = tc_bind(c, io, &dio, tab, TC_SOILWATER, ldc, 0, tc_lo, tc_hi, tc_fill)))
            return rc;
        gather_setup(c, io, &dio, T, NT, ldc, 0);
        int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_hydrologyc * 4);
        // the Zeng-Decker form takes each chunk's columns grouped by
        // water-table depth (sorted on the host while the chunk's copies run);
        // the moisture form's persistent kernel takes them in filter order
        const bool zd = nml.soilwater_movement_method == 0;
        int32_t* hord = zd ? order_buffer(c, (size_t)num_hydrologyc) : nullptr;
        if (zd && !hord) return set_error(CTSMG_E_CUDA, "cudaMallocHost(work order)", 0, 0);
        if (!zd) {
            e = copy_async(dfilt, filter_hydrologyc, (size_t)num_hydrologyc * 4, cudaMemcpyHostToDevice,
                           in_stream(c));
            if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
        }
        auto sw_chunk_in = [&](int k) -> int {
            const Chunk& ch = chunks[k];
            if (!zd) return chunk_in(c, ch, k, io, &dio, T, NT, ldc, 0);
            trace_mark(c, k, 0, in_stream(c));
            int r = chunk_copies_in(c, ch, io, &dio, T, NT, ldc, 0);
            if (r) return r;
            group_by_water_table(filter_hydrologyc, ch.f0, ch.f1, io->zwt, bounds->begc, hord);
            cudaError_t ce = copy_async(dfilt + ch.f0, hord + ch.f0, (size_t)(ch.f1 - ch.f0) * 4,
                                        cudaMemcpyHostToDevice, in_stream(c));
            if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(filter)");
            trace_mark(c, k, 1, in_stream(c));
            ce = cudaEventRecord(c->ev_in[k], in_stream(c));
            return ce == cudaSuccess ? 0 : cuda_fail(ce, "cudaEventRecord");
        };
        const int K = (int)chunks.size();
        if ((rc = fork_streams(c))) return rc;
        if ((rc = sw_chunk_in(0))) return rc;
        for (int k = 0; k < K; ++k) {
            const Chunk& ch = chunks[k];
            cudaStream_t ks = chunk_stream(c, k);
            if ((e = cudaStreamWaitEvent(ks, c->ev_in[k], 0)) != cudaSuccess) return cuda_fail(e, "wait");
            trace_mark(c, k, 2, ks);
            // one lane-refill counter per compute stream (chunks on one stream run in order)
            e = launch_soilwater_call(dio, bounds->begc, ch.f1 - ch.f0, dfilt + ch.f0, nml, e_ice, dtime, c->err,
                                      ks, dcounter + 32 * (k % PIPE_STREAMS));
            if (e != cudaSuccess) return cuda_fail(e, "soilwater kernel launch");
            trace_mark(c, k, 3, ks);
            if ((e = cudaEventRecord(c->ev_done[k], ks)) != cudaSuccess) return cuda_fail(e, "record");
            if (k + 1 < K && (rc = sw_chunk_in(k + 1))) return rc;
            if ((rc = chunk_out(c, ch, k, io, &dio, T, NT, ldc, 0))) return rc;
        }
        c->gather = false;
        if ((e = join_streams(c)) != cudaSuccess) return cuda_fail(e, "soilwater");
        c->trace_n = c->trace ? K : 0;
        tc_commit(tc_fill, tc_lo, tc_hi);
    } else {
        ctsmg_soilwater_io dio;
        if ((rc = stage_in(c, io, &dio, sizeof dio, T, NT, ldc, 0, 0, bounds->endc - bounds->begc + 1, -1))) return rc;
        int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_hydrologyc * 4);
        e = copy_async(dfilt, filter_hydrologyc, (size_t)num_hydrologyc * 4, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
        e = launch_soilwater_call(dio, bounds->begc, num_hydrologyc, dfilt, nml, e_ice, dtime, c->err, c->stream,
                                  dcounter);
        if (e != cudaSuccess) return cuda_fail(e, "soilwater kernel launch");
        if ((rc = stage_out(c, io, &dio, T, NT, ldc, 0, 0, bounds->endc - bounds->begc + 1, -1))) return rc;
        e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "soilwater");
    }
    int code = 0, idx = 0, lev = 0;
    if ((rc = read_error(c, &code, &idx, &lev))) return rc;
    if (code) return soilwater_error(code, idx, lev);
    return 0;
}

extern "C" int32_t ctsmg_soiltemperature(const ctsmg_bounds* bounds, int32_t num_nolakec,
                                         const int32_t* filter_nolakec, const ctsmg_soiltemp_io* io,
                                         double dtime) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if ((rc = check_filter(bounds, num_nolakec, filter_nolakec))) return rc;
    const int ncol = bounds->endc - bounds->begc + 1;
    const int npat = bounds->endp - bounds->begp + 1;
    if (io->ldc < ncol || io->ldp < npat || npat < 0)
        return set_error(CTSMG_E_ARG, "ldc/ldp smaller than the bounds", 0, 0);
    if (!(dtime > 0.0)) return set_error(CTSMG_E_ARG, "dtime must be positive", 0, 0);
    for (int i = 0; i < num_nolakec; ++i) {
        const int cc = filter_nolakec[i] - bounds->begc;
        const int s = io->snl[cc], pi = io->col_patchi[cc], np = io->col_npatches[cc];
        if (s > 0 || s < -NLEVSNO) return set_error(CTSMG_E_ARG, "snl outside -nlevsno..0", filter_nolakec[i], 0);
        if (np < 0 || pi < bounds->begp || pi + np - 1 > bounds->endp)
            return set_error(CTSMG_E_ARG, "column patches outside begp..endp", filter_nolakec[i], 0);
    }
    if (num_nolakec == 0) return 0;
    const int ldc = io->ldc, ldp = io->ldp;
    // outputs the heat solve writes on every filtered column are not copied
    // in when the filter is every column of the bounds in order
    static const std::vector<FieldDesc> dense_tab = soiltemp_dense_table();
    bool dense = num_nolakec == ncol;
    for (int i = 0; dense && i < num_nolakec; ++i) dense = filter_nolakec[i] == bounds->begc + i;
    const FieldDesc* TT = dense ? dense_tab.data() : SOILTEMP_TABLE;
    const size_t ws_bytes = (size_t)SOILTEMP_WS_DOUBLES_PER_COL * num_nolakec * 8;
    size_t need = table_bytes(TT, SOILTEMP_NFIELDS, ldc, ldp) + ws_bytes + (size_t)num_nolakec * 4 + 8192;
    if ((rc = arena_reserve(c, need))) return rc;
    std::vector<Chunk> chunks;
    if (plan_chunks(bounds, num_nolakec, filter_nolakec, io->col_patchi, io->col_npatches, soiltemp_wave_columns(),
                    chunks)) {
        ctsmg_soiltemp_io dio;
        std::vector<FieldDesc> ttab;
        std::vector<ThreadCtx::TcEntry*> tc_fill;
        const int tc_lo = chunks.front().c0, tc_hi = chunks.back().c1;
        if (g_tc_on.load()) {           // a copy of the table whose no_in marks the kept components
            ttab.assign(TT, TT + SOILTEMP_NFIELDS);
            TT = ttab.data();
        }
        stage_alloc(c, io, &dio, sizeof dio, TT, SOILTEMP_NFIELDS, ldc, ldp);
        if (!ttab.empty() && (rc = tc_bind(c, io, &dio, ttab, TC_SOILTEMP, ldc, ldp, tc_lo, tc_hi, tc_fill)))
            return rc;
        gather_setup(c, io, &dio, TT, SOILTEMP_NFIELDS, ldc, ldp);
        int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_nolakec * 4);
        double* ws = (double*)arena_take(c, ws_bytes);
        int32_t* hord = order_buffer(c, (size_t)num_nolakec);
        if (!hord) return set_error(CTSMG_E_CUDA, "cudaMallocHost(work order)", 0, 0);
        // chunk k's components, then its work order (sorted on the host while
        // those copies run), then ev_in[k]
        auto stage_chunk = [&](int k) -> int {
            const Chunk& ch = chunks[k];
            trace_mark(c, k, 0, in_stream(c));
            int r = chunk_copies_in(c, ch, io, &dio, TT, SOILTEMP_NFIELDS, ldc, ldp);
            if (r) return r;
            group_by_layers(filter_nolakec, ch.f0, ch.f1, io->snl, io->nbedrock, bounds->begc, hord);
            cudaError_t ce = copy_async(dfilt + ch.f0, hord + ch.f0, (size_t)(ch.f1 - ch.f0) * 4,
                                        cudaMemcpyHostToDevice, in_stream(c));
            if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpyAsync(filter)");
            trace_mark(c, k, 1, in_stream(c));
            ce = cudaEventRecord(c->ev_in[k], in_stream(c));
            return ce == cudaSuccess ? 0 : cuda_fail(ce, "cudaEventRecord");
        };
        cudaError_t e;
        if ((e = cudaMemsetAsync(c->err, 0xff, sizeof(DevError), c->stream)) != cudaSuccess)
            return cuda_fail(e, "cudaMemsetAsync(err)");
        int snow_method;
        { std::lock_guard<std::mutex> lk(g_mu); snow_method = g_opt.snow_thermal_cond_method; }
        const int K = (int)chunks.size();
        if ((rc = fork_streams(c))) return rc;
        if ((rc = stage_chunk(0))) return rc;
        for (int k = 0; k < K; ++k) {
            const Chunk& ch = chunks[k];
            cudaStream_t ks = chunk_stream(c, k);
            if ((e = cudaStreamWaitEvent(ks, c->ev_in[k], 0)) != cudaSuccess) return cuda_fail(e, "wait");
            trace_mark(c, k, 2, ks);
            e = launch_soiltemp(dio, bounds->begc, bounds->begp, ch.f1 - ch.f0, dfilt + ch.f0, dtime, snow_method,
                                ws + ch.f0, num_nolakec, c->err, ks);
            if (e != cudaSuccess) return cuda_fail(e, "soiltemperature kernel launch");
            trace_mark(c, k, 3, ks);
            if ((e = cudaEventRecord(c->ev_done[k], ks)) != cudaSuccess) return cuda_fail(e, "record");
            if (k + 1 < K && (rc = stage_chunk(k + 1))) return rc;
            if ((rc = chunk_out(c, ch, k, io, &dio, TT, SOILTEMP_NFIELDS, ldc, ldp))) return rc;
        }
        c->gather = false;
        if ((e = join_streams(c)) != cudaSuccess) return cuda_fail(e, "soiltemperature");
        c->trace_n = c->trace ? K : 0;
        tc_commit(tc_fill, tc_lo, tc_hi);
        int code = 0, idx = 0, lev = 0;
        if ((rc = read_error(c, &code, &idx, &lev))) return rc;
        if (code) return set_error(code, "BandDiagonal ERROR: dgbsv returned error code", idx, lev);
        return 0;
    }
    ctsmg_soiltemp_io dio;
    if ((rc = stage_in(c, io, &dio, sizeof dio, TT, SOILTEMP_NFIELDS, ldc, ldp, 0, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_nolakec * 4);
    double* ws = (double*)arena_take(c, ws_bytes);
    int32_t* hord = order_buffer(c, (size_t)num_nolakec);
    if (!hord) return set_error(CTSMG_E_CUDA, "cudaMallocHost(work order)", 0, 0);
    group_by_layers(filter_nolakec, 0, num_nolakec, io->snl, io->nbedrock, bounds->begc, hord);
    cudaError_t e = copy_async(dfilt, hord, (size_t)num_nolakec * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
    e = cudaMemsetAsync(c->err, 0xff, sizeof(DevError), c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(err)");
    int snow_method;
    { std::lock_guard<std::mutex> lk(g_mu); snow_method = g_opt.snow_thermal_cond_method; }
    e = launch_soiltemp(dio, bounds->begc, bounds->begp, num_nolakec, dfilt, dtime, snow_method, ws,
                        num_nolakec, c->err, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "soiltemperature kernel launch");
    if ((rc = stage_out(c, io, &dio, TT, SOILTEMP_NFIELDS, ldc, ldp, 0, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "soiltemperature");
    int code = 0, idx = 0, lev = 0;
    if ((rc = read_error(c, &code, &idx, &lev))) return rc;
    if (code) return set_error(code, "BandDiagonal ERROR: dgbsv returned error code", idx, lev);
    return 0;
}

extern "C" int32_t ctsmg_set_canopy_params(const ctsmg_canopy_params* p, const ctsmg_pftcon* pft) {
    if (!p || !pft) return set_error(CTSMG_E_ARG, "null params", 0, 0);
    if (pft->npft < 1 || pft->npft > CTSMG_MAX_PFT) return set_error(CTSMG_E_ARG, "npft outside 1..CTSMG_MAX_PFT", 0, 0);
    for (int i = 0; i < pft->npft; ++i)
        if (pft->slatop[i] * pft->leafcn[i] <= 0.0)
            return set_error(CTSMG_E_ARG, "ERROR: slatop or leafcn is zero", i, 0);
    std::lock_guard<std::mutex> lk(g_mu);
    g_cpar = *p;
    g_pft = *pft;
    g_cpar_set = true;
    return 0;
}

extern "C" int32_t ctsmg_canopyfluxes(const ctsmg_bounds* bounds, int32_t num_exposedvegp,
                                      const int32_t* filter_exposedvegp, const ctsmg_canopy_io* io, double dtime) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if (!g_cpar_set) return set_error(CTSMG_E_NOT_INIT, "ctsmg_set_canopy_params has not been called", 0, 0);
    if (!bounds || bounds->endp < bounds->begp) return set_error(CTSMG_E_ARG, "bad patch bounds", 0, 0);
    if (num_exposedvegp < 0 || (num_exposedvegp > 0 && !filter_exposedvegp))
        return set_error(CTSMG_E_ARG, "bad patch filter", 0, 0);
    const int npat = bounds->endp - bounds->begp + 1, ncol = bounds->endc - bounds->begc + 1;
    if (io->ldp < npat || io->ldc < ncol || io->ldg < 1) return set_error(CTSMG_E_ARG, "ldp/ldc/ldg too small", 0, 0);
    if (!(dtime > 0.0)) return set_error(CTSMG_E_ARG, "dtime must be positive", 0, 0);
    for (int i = 0; i < num_exposedvegp; ++i) {
        const int pg = filter_exposedvegp[i];
        if (pg < bounds->begp || pg > bounds->endp) return set_error(CTSMG_E_ARG, "filter index outside bounds", pg, 0);
        const int p = pg - bounds->begp;
        const int cc = io->patch_column[p], gg = io->patch_gridcell[p], it = io->itype[p];
        if (cc < bounds->begc || cc > bounds->endc) return set_error(CTSMG_E_ARG, "patch column outside bounds", pg, 0);
        if (gg < io->begg || gg > io->begg + io->ldg - 1) return set_error(CTSMG_E_ARG, "patch gridcell outside ldg", pg, 0);
        if (it < 0 || it >= g_pft.npft) return set_error(CTSMG_E_ARG, "patch itype outside pftcon", pg, 0);
        const int s = io->snl[cc - bounds->begc];
        if (s > 0 || s < -NLEVSNO) return set_error(CTSMG_E_ARG, "snl outside -nlevsno..0", cc, 0);
    }
    if (num_exposedvegp == 0) return 0;
    const int ldc = io->ldc, ldp = io->ldp, ldg = io->ldg;
    size_t need = table_bytes(CANOPY_TABLE, CANOPY_NFIELDS, ldc, ldp, ldg) + (size_t)num_exposedvegp * 4 +
                  canopy_ws_bytes(num_exposedvegp) + 8192;
    if ((rc = arena_reserve(c, need))) return rc;
    CanopyArgs a;
    if ((rc = stage_in(c, io, &a.io, sizeof a.io, CANOPY_TABLE, CANOPY_NFIELDS, ldc, ldp, ldg, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_exposedvegp * 4);
    int* counter = (int*)arena_take(c, 256);
    double* cws = (double*)arena_take(c, canopy_ws_bytes(num_exposedvegp));
    cudaError_t e = copy_async(dfilt, filter_exposedvegp, (size_t)num_exposedvegp * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
    e = cudaMemsetAsync(c->err, 0xff, sizeof(DevError), c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(err)");
    {
        std::lock_guard<std::mutex> lk(g_mu);
        a.par = g_cpar;
        a.pft = g_pft;
        a.method = g_opt.stomatalcond_method;
        a.itmax = g_opt.itmax_canopy_fluxes;
    }
    a.begc = bounds->begc;
    a.begp = bounds->begp;
    a.engine = 0;
    a.medlynslope_p = nullptr;
    a.medlynintercept_p = nullptr;
    e = launch_canopy(a, num_exposedvegp, dfilt, dtime, counter, c->err, cws, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "canopy kernel launch");
    if ((rc = stage_out(c, io, &a.io, CANOPY_TABLE, CANOPY_NFIELDS, ldc, ldp, ldg, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "canopyfluxes");
    int code = 0, idx = 0, lev = 0;
    if ((rc = read_error(c, &code, &idx, &lev))) return rc;
    if (code) {
        const char* m = code == CTSMG_E_DISCRIMINANT ? "quadratic ERROR: Quadratic solution error: b^2 - 4ac is negative"
                      : code == CTSMG_E_NOT_BRACKETED ? "root must be bracketed for brent"
                      : code == CTSMG_E_FORCING_HEIGHT ? "Error: Forcing height is below canopy height for patch index"
                      : "CanopyFluxes error";
        return set_error(code, m, idx, lev);
    }
    return 0;
}

extern "C" int32_t ctsmg_soilfluxes(const ctsmg_bounds* bounds, int32_t num_nolakec, const int32_t* filter_nolakec,
                                    int32_t num_nolakep, const int32_t* filter_nolakep, const ctsmg_soilfluxes_io* io,
                                    double dtime) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if ((rc = check_filter(bounds, num_nolakec, filter_nolakec))) return rc;
    if (num_nolakep < 0 || (num_nolakep > 0 && !filter_nolakep)) return set_error(CTSMG_E_ARG, "bad patch filter", 0, 0);
    const int ncol = bounds->endc - bounds->begc + 1;
    const int npat = bounds->endp - bounds->begp + 1;
    if (io->ldc < ncol || io->ldp < npat || npat < 0)
        return set_error(CTSMG_E_ARG, "ldc/ldp smaller than the bounds", 0, 0);
    if (!(dtime > 0.0)) return set_error(CTSMG_E_ARG, "dtime must be positive", 0, 0);
    for (int i = 0; i < num_nolakep; ++i) {
        const int pg = filter_nolakep[i];
        if (pg < bounds->begp || pg > bounds->endp) return set_error(CTSMG_E_ARG, "patch filter outside bounds", pg, 0);
        const int cc = io->patch_column[pg - bounds->begp];
        if (cc < bounds->begc || cc > bounds->endc) return set_error(CTSMG_E_ARG, "patch column outside bounds", pg, 0);
        const int s = io->snl[cc - bounds->begc];
        if (s > 0 || s < -NLEVSNO) return set_error(CTSMG_E_ARG, "snl outside -nlevsno..0", cc, 0);
    }
    for (int i = 0; i < num_nolakec; ++i) {
        const int cc = filter_nolakec[i] - bounds->begc;
        const int pi = io->col_patchi[cc], np = io->col_npatches[cc];
        if (np < 0 || (np > 0 && (pi < bounds->begp || pi + np - 1 > bounds->endp)))
            return set_error(CTSMG_E_ARG, "column patches outside begp..endp", filter_nolakec[i], 0);
    }
    if (num_nolakec == 0 && num_nolakep == 0) return 0;
    const int ldc = io->ldc, ldp = io->ldp;
    size_t need = table_bytes(SOILFLUXES_TABLE, SOILFLUXES_NFIELDS, ldc, ldp) +
                  ((size_t)num_nolakec + (size_t)num_nolakep) * 4 + 8192;
    if ((rc = arena_reserve(c, need))) return rc;
    ctsmg_soilfluxes_io dio;
    if ((rc = stage_in(c, io, &dio, sizeof dio, SOILFLUXES_TABLE, SOILFLUXES_NFIELDS, ldc, ldp, 0, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    int32_t* dfc = (int32_t*)arena_take(c, (size_t)num_nolakec * 4 + 4);
    int32_t* dfp = (int32_t*)arena_take(c, (size_t)num_nolakep * 4 + 4);
    cudaError_t e = cudaSuccess;
    if (num_nolakec > 0)
        e = copy_async(dfc, filter_nolakec, (size_t)num_nolakec * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && num_nolakep > 0)
        e = copy_async(dfp, filter_nolakep, (size_t)num_nolakep * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
    e = launch_soilfluxes(dio, bounds->begc, bounds->begp, num_nolakec, dfc, num_nolakep, dfp, dtime, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "soilfluxes kernel launch");
    if ((rc = stage_out(c, io, &dio, SOILFLUXES_TABLE, SOILFLUXES_NFIELDS, ldc, ldp, 0, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "soilfluxes");
    return 0;
}

extern "C" int32_t ctsmg_root_moist_stress(const ctsmg_bounds* bounds, int32_t num_exposedvegp,
                                           const int32_t* filter_exposedvegp, const ctsmg_rootmoist_io* io) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if (!g_cpar_set) return set_error(CTSMG_E_NOT_INIT, "ctsmg_set_canopy_params has not been called", 0, 0);
    if (!bounds || bounds->endp < bounds->begp || bounds->endc < bounds->begc)
        return set_error(CTSMG_E_ARG, "bad bounds", 0, 0);
    if (num_exposedvegp < 0 || (num_exposedvegp > 0 && !filter_exposedvegp))
        return set_error(CTSMG_E_ARG, "bad patch filter", 0, 0);
    const int ncol = bounds->endc - bounds->begc + 1, npat = bounds->endp - bounds->begp + 1;
    if (io->ldc < ncol || io->ldp < npat) return set_error(CTSMG_E_ARG, "ldc/ldp smaller than the bounds", 0, 0);
    ctsmg_pftcon pft;
    { std::lock_guard<std::mutex> lk(g_mu); pft = g_pft; }
    for (int i = 0; i < num_exposedvegp; ++i) {
        const int pg = filter_exposedvegp[i];
        if (pg < bounds->begp || pg > bounds->endp) return set_error(CTSMG_E_ARG, "filter index outside bounds", pg, 0);
        const int p = pg - bounds->begp;
        const int cc = io->patch_column[p], it = io->itype[p];
        if (cc < bounds->begc || cc > bounds->endc) return set_error(CTSMG_E_ARG, "patch column outside bounds", pg, 0);
        if (it < 0 || it >= pft.npft) return set_error(CTSMG_E_ARG, "patch itype outside pftcon", pg, 0);
    }
    if (num_exposedvegp == 0) return 0;
    const int ldc = io->ldc, ldp = io->ldp;
    size_t need = table_bytes(ROOTMOIST_TABLE, ROOTMOIST_NFIELDS, ldc, ldp) + (size_t)num_exposedvegp * 4 + 4096;
    if ((rc = arena_reserve(c, need))) return rc;
    ctsmg_rootmoist_io dio;
    if ((rc = stage_in(c, io, &dio, sizeof dio, ROOTMOIST_TABLE, ROOTMOIST_NFIELDS, ldc, ldp, 0, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_exposedvegp * 4);
    cudaError_t e = copy_async(dfilt, filter_exposedvegp, (size_t)num_exposedvegp * 4, cudaMemcpyHostToDevice,
                                    c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
    e = launch_rootmoist(dio, pft, bounds->begc, bounds->begp, num_exposedvegp, dfilt, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "root moisture stress kernel launch");
    if ((rc = stage_out(c, io, &dio, ROOTMOIST_TABLE, ROOTMOIST_NFIELDS, ldc, ldp, 0, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "root moisture stress");
    return 0;
}

extern "C" int32_t ctsmg_set_soil_resistance(const ctsmg_soil_resistance_params* p) {
    if (!p) return set_error(CTSMG_E_ARG, "null params", 0, 0);
    if (p->soil_resis_method != 0 && p->soil_resis_method != 1)
        return set_error(CTSMG_E_ARG, "calc_soilevap_resis:: a soilevap resis function must be specified!", 0, 0);
    std::lock_guard<std::mutex> lk(g_mu);
    g_sres = *p;
    return 0;
}

extern "C" int32_t ctsmg_set_soil_water_fractions(const ctsmg_bounds* bounds, int32_t num_hydrologyc,
                                                  const int32_t* filter_hydrologyc, const ctsmg_soilwater_io* io) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if ((rc = check_filter(bounds, num_hydrologyc, filter_hydrologyc))) return rc;
    const int ncol = bounds->endc - bounds->begc + 1;
    if (io->ldc < ncol) return set_error(CTSMG_E_ARG, "ldc smaller than endc-begc+1", 0, 0);
    if (num_hydrologyc == 0) return 0;
    const int ldc = io->ldc;
    const FieldDesc* T = SOILWATER_FRACTIONS_TABLE;
    const int NT = SOILWATER_FRACTIONS_NFIELDS;
    if ((rc = arena_reserve(c, table_bytes(T, NT, ldc, 0) + (size_t)num_hydrologyc * 4 + 4096))) return rc;
    ctsmg_soilwater_io dio;
    if ((rc = stage_in(c, io, &dio, sizeof dio, T, NT, ldc, 0, 0, bounds->endc - bounds->begc + 1, -1))) return rc;
    int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_hydrologyc * 4);
    cudaError_t e = copy_async(dfilt, filter_hydrologyc, (size_t)num_hydrologyc * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
    e = launch_set_soil_water_fractions(dio, bounds->begc, num_hydrologyc, dfilt, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "soil water fractions kernel launch");
    if ((rc = stage_out(c, io, &dio, T, NT, ldc, 0, 0, bounds->endc - bounds->begc + 1, -1))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "soil water fractions");
    return 0;
}

extern "C" int32_t ctsmg_root_sink(const ctsmg_bounds* bounds, int32_t num_filterc, const int32_t* filterc,
                                   const ctsmg_rootsink_io* io) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if ((rc = check_filter(bounds, num_filterc, filterc))) return rc;
    if (bounds->endp < bounds->begp - 1) return set_error(CTSMG_E_ARG, "bad patch bounds", 0, 0);
    const int ncol = bounds->endc - bounds->begc + 1, npat = bounds->endp - bounds->begp + 1;
    if (io->ldc < ncol || io->ldp < npat) return set_error(CTSMG_E_ARG, "ldc/ldp smaller than the bounds", 0, 0);
    if (!io->col_patchi || !io->col_npatches) return set_error(CTSMG_E_ARG, "null col_patchi / col_npatches", 0, 0);
    for (int i = 0; i < num_filterc; ++i) {
        const int cc = filterc[i] - bounds->begc;
        const int pi = io->col_patchi[cc], np = io->col_npatches[cc];
        if (np < 0 || (np > 0 && (pi < bounds->begp || pi + np - 1 > bounds->endp)))
            return set_error(CTSMG_E_ARG, "column patches outside begp..endp", filterc[i], 0);
    }
    if (num_filterc == 0) return 0;
    const int ldc = io->ldc, ldp = io->ldp;
    const bool tc = io->qflx_tran_veg_col != nullptr;
    size_t need = table_bytes(ROOTSINK_TABLE, ROOTSINK_NFIELDS, ldc, ldp) + (size_t)num_filterc * 4 + 4096 +
                  (tc ? table_bytes(ROOTSINK_TRANCOL_TABLE, 1, ldc, ldp) : 0);
    if ((rc = arena_reserve(c, need))) return rc;
    ctsmg_rootsink_io dio;
    if ((rc = stage_in(c, io, &dio, sizeof dio, ROOTSINK_TABLE, ROOTSINK_NFIELDS, ldc, ldp, 0, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    if (tc) {
        ctsmg_rootsink_io tmp;
        if ((rc = stage_in(c, io, &tmp, sizeof tmp, ROOTSINK_TRANCOL_TABLE, 1, ldc, ldp, 0, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
        dio.qflx_tran_veg_col = tmp.qflx_tran_veg_col;
    }
    int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_filterc * 4);
    cudaError_t e = copy_async(dfilt, filterc, (size_t)num_filterc * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
    e = launch_rootsink_dropin(dio, bounds->begc, bounds->begp, num_filterc, dfilt, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "root sink kernel launch");
    if ((rc = stage_out(c, io, &dio, ROOTSINK_TABLE, ROOTSINK_NFIELDS, ldc, ldp, 0, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "root sink");
    return 0;
}

extern "C" int32_t ctsmg_soilevap_resis(const ctsmg_bounds* bounds, int32_t num_nolakec, const int32_t* filter_nolakec,
                                        const ctsmg_soilresis_io* io) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if ((rc = check_filter(bounds, num_nolakec, filter_nolakec))) return rc;
    const int ncol = bounds->endc - bounds->begc + 1;
    if (io->ldc < ncol) return set_error(CTSMG_E_ARG, "ldc smaller than endc-begc+1", 0, 0);
    const ctsmg_soil_resistance_params par = current_soil_resistance();
    const FieldDesc* T = par.soil_resis_method == 1 ? SOILRESIS_SL14_TABLE : SOILRESIS_LP92_TABLE;
    const int NT = par.soil_resis_method == 1 ? SOILRESIS_SL14_NFIELDS : SOILRESIS_LP92_NFIELDS;
    if (num_nolakec == 0) return 0;
    const int ldc = io->ldc;
    if ((rc = arena_reserve(c, table_bytes(T, NT, ldc, 0) + (size_t)num_nolakec * 4 + 4096))) return rc;
    ctsmg_soilresis_io dio;
    if ((rc = stage_in(c, io, &dio, sizeof dio, T, NT, ldc, 0, 0, bounds->endc - bounds->begc + 1, -1))) return rc;
    int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_nolakec * 4);
    cudaError_t e = copy_async(dfilt, filter_nolakec, (size_t)num_nolakec * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
    const SoilResisArgs a{par.soil_resis_method, par.d_max, par.frac_sat_soil_dsl_init};
    e = launch_soilevap_resis(dio, bounds->begc, num_nolakec, dfilt, a, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "soil resistance kernel launch");
    if ((rc = stage_out(c, io, &dio, T, NT, ldc, 0, 0, bounds->endc - bounds->begc + 1, -1))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "soil resistance");
    return 0;
}

extern "C" int32_t ctsmg_baregroundfluxes(const ctsmg_bounds* bounds, int32_t num_noexposedvegp,
                                          const int32_t* filter_noexposedvegp, const ctsmg_baregrnd_io* io) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if (!g_cpar_set) return set_error(CTSMG_E_NOT_INIT, "ctsmg_set_canopy_params has not been called", 0, 0);
    if (!bounds || bounds->endp < bounds->begp || bounds->endc < bounds->begc)
        return set_error(CTSMG_E_ARG, "bad bounds", 0, 0);
    if (num_noexposedvegp < 0 || (num_noexposedvegp > 0 && !filter_noexposedvegp))
        return set_error(CTSMG_E_ARG, "bad patch filter", 0, 0);
    const int ncol = bounds->endc - bounds->begc + 1, npat = bounds->endp - bounds->begp + 1;
    if (io->ldp < npat || io->ldc < ncol || io->ldg < 1) return set_error(CTSMG_E_ARG, "ldp/ldc/ldg too small", 0, 0);
    for (int i = 0; i < num_noexposedvegp; ++i) {
        const int pg = filter_noexposedvegp[i];
        if (pg < bounds->begp || pg > bounds->endp) return set_error(CTSMG_E_ARG, "filter index outside bounds", pg, 0);
        const int cc = io->patch_column[pg - bounds->begp], gg = io->patch_gridcell[pg - bounds->begp];
        if (cc < bounds->begc || cc > bounds->endc) return set_error(CTSMG_E_ARG, "patch column outside bounds", pg, 0);
        if (gg < io->begg || gg > io->begg + io->ldg - 1) return set_error(CTSMG_E_ARG, "patch gridcell outside ldg", pg, 0);
        const int s = io->snl[cc - bounds->begc];
        if (s > 0 || s < -NLEVSNO) return set_error(CTSMG_E_ARG, "snl outside -nlevsno..0", cc, 0);
    }
    ctsmg_canopy_params cp;
    { std::lock_guard<std::mutex> lk(g_mu); cp = g_cpar; }
    const ctsmg_soil_resistance_params sres = current_soil_resistance();
    std::vector<FieldDesc> tab(BAREGRND_TABLE, BAREGRND_TABLE + BAREGRND_NFIELDS);
    tab.push_back(sres.soil_resis_method == 1 ? BAREGRND_SOILRESIS[0] : BAREGRND_SOILBETA[0]);
    if (num_noexposedvegp == 0) return 0;
    const int ldc = io->ldc, ldp = io->ldp, ldg = io->ldg;
    const FieldDesc* T = tab.data();
    const int NT = (int)tab.size();
    size_t need = table_bytes(T, NT, ldc, ldp, ldg) + (size_t)num_noexposedvegp * 4 + (size_t)ldc * 4 + 8192;
    if ((rc = arena_reserve(c, need))) return rc;
    ctsmg_baregrnd_io dio;
    if ((rc = stage_in(c, io, &dio, sizeof dio, T, NT, ldc, ldp, ldg, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    int32_t* dfilt = (int32_t*)arena_take(c, (size_t)num_noexposedvegp * 4);
    int* dlast = (int*)arena_take(c, (size_t)ldc * 4);
    cudaError_t e = copy_async(dfilt, filter_noexposedvegp, (size_t)num_noexposedvegp * 4, cudaMemcpyHostToDevice,
                                    c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
    const BareArgs a{cp.a_coef, cp.a_exp, cp.wind_min, cp.zetamaxstable, sres.soil_resis_method};
    e = launch_baregrnd(dio, bounds->begc, bounds->begp, num_noexposedvegp, dfilt, a, dlast, ldc, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "bare ground kernel launch");
    if ((rc = stage_out(c, io, &dio, T, NT, ldc, ldp, ldg, bounds->endc - bounds->begc + 1, bounds->endp - bounds->begp + 1))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "bare ground fluxes");
    return 0;
}

extern "C" int32_t ctsmg_set_soilhydrology_params(const ctsmg_soilhydrology_params* p) {
    if (!p) return set_error(CTSMG_E_ARG, "null params", 0, 0);
    std::lock_guard<std::mutex> lk(g_mu);
    g_shp = *p;
    return 0;
}

ctsmg_soilhydrology_params ctsmg::current_soilhydrology_params() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_shp;
}

// One hydrology routine over the column filter: stage the routine's
// components, run its kernel, copy the outputs back.
static int hydrology_call(const ctsmg_bounds* bounds, int32_t n, const int32_t* filt, const ctsmg_hydrology_io* io,
                          double dtime, int which, const FieldDesc* T, int NT) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (!io) return set_error(CTSMG_E_ARG, "null io", 0, 0);
    if ((rc = check_filter(bounds, n, filt))) return rc;
    const int ncol = bounds->endc - bounds->begc + 1;
    if (io->ldc < ncol) return set_error(CTSMG_E_ARG, "ldc smaller than endc-begc+1", 0, 0);
    if (which != HYD_SAT_EXCESS && which != HYD_PERCHED_WT && which != HYD_THETA_WT && !(dtime > 0.0))
        return set_error(CTSMG_E_ARG, "dtime must be positive", 0, 0);
    for (int i = 0; i < NT; ++i)
        if (T[i].offset == offsetof(ctsmg_hydrology_io, nbedrock)) {
            for (int k = 0; k < n; ++k) {
                const int nb = io->nbedrock[filt[k] - bounds->begc];
                if (nb < 1 || nb > NLEVSOI) return set_error(CTSMG_E_ARG, "nbedrock outside 1..nlevsoi", filt[k], 0);
            }
        }
    if (n == 0) return 0;
    const int ldc = io->ldc;
    if ((rc = arena_reserve(c, table_bytes(T, NT, ldc, 0) + (size_t)n * 4 + 4096))) return rc;
    ctsmg_hydrology_io dio;
    if ((rc = stage_in(c, io, &dio, sizeof dio, T, NT, ldc, 0, 0, bounds->endc - bounds->begc + 1, -1))) return rc;
    int32_t* dfilt = (int32_t*)arena_take(c, (size_t)n * 4);
    cudaError_t e = copy_async(dfilt, filt, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(filter)");
    e = launch_hydrology(dio, bounds->begc, n, dfilt, which, current_soilhydrology_params(), dtime, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "hydrology kernel launch");
    if ((rc = stage_out(c, io, &dio, T, NT, ldc, 0, 0, bounds->endc - bounds->begc + 1, -1))) return rc;
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "hydrology");
    return 0;
}

extern "C" int32_t ctsmg_saturated_excess_runoff(const ctsmg_bounds* b, int32_t n, const int32_t* f,
                                                 const ctsmg_hydrology_io* io) {
    return hydrology_call(b, n, f, io, 0.0, HYD_SAT_EXCESS, HYD_SAT_TABLE, HYD_SAT_TABLE_N);
}
extern "C" int32_t ctsmg_perched_water_table(const ctsmg_bounds* b, int32_t n, const int32_t* f,
                                             const ctsmg_hydrology_io* io) {
    return hydrology_call(b, n, f, io, 0.0, HYD_PERCHED_WT, HYD_PWT_TABLE, HYD_PWT_TABLE_N);
}
extern "C" int32_t ctsmg_theta_based_water_table(const ctsmg_bounds* b, int32_t n, const int32_t* f,
                                                 const ctsmg_hydrology_io* io) {
    return hydrology_call(b, n, f, io, 0.0, HYD_THETA_WT, HYD_TWT_TABLE, HYD_TWT_TABLE_N);
}
extern "C" int32_t ctsmg_perched_lateral_flow(const ctsmg_bounds* b, int32_t n, const int32_t* f,
                                              const ctsmg_hydrology_io* io, double dtime) {
    return hydrology_call(b, n, f, io, dtime, HYD_PERCHED_LAT, HYD_PLF_TABLE, HYD_PLF_TABLE_N);
}
extern "C" int32_t ctsmg_subsurface_lateral_flow(const ctsmg_bounds* b, int32_t n, const int32_t* f,
                                                 const ctsmg_hydrology_io* io, double dtime) {
    return hydrology_call(b, n, f, io, dtime, HYD_SUBSURFACE_LAT, HYD_SLF_TABLE, HYD_SLF_TABLE_N);
}
extern "C" int32_t ctsmg_infiltration_chain(const ctsmg_bounds* b, int32_t n, const int32_t* f,
                                            const ctsmg_hydrology_io* io, double dtime) {
    return hydrology_call(b, n, f, io, dtime, HYD_INFIL, HYD_INF_TABLE, HYD_INF_TABLE_N);
}
extern "C" int32_t ctsmg_water_table(const ctsmg_bounds* b, int32_t n, const int32_t* f, const ctsmg_hydrology_io* io,
                                     double dtime) {
    return hydrology_call(b, n, f, io, dtime, HYD_WATER_TABLE, HYD_WT_TABLE, HYD_WT_TABLE_N);
}
extern "C" int32_t ctsmg_drainage(const ctsmg_bounds* b, int32_t n, const int32_t* f, const ctsmg_hydrology_io* io,
                                  double dtime) {
    return hydrology_call(b, n, f, io, dtime, HYD_DRAINAGE, HYD_DR_TABLE, HYD_DR_TABLE_N);
}

// Keep (1) or stop keeping (0) device copies of the time-constant inputs of
// the pipelined drop-in calls; either way the kept copies are dropped.
extern "C" int32_t ctsmg_set_time_constant_inputs(int32_t resident) {
    if (resident != 0 && resident != 1) return set_error(CTSMG_E_ARG, "resident must be 0 or 1", 0, 0);
    g_tc_on = resident;
    ++g_tc_gen;
    return 0;
}

// Drop the kept copies (a time-constant input changed on the host).
extern "C" int32_t ctsmg_invalidate_time_constant_inputs(void) {
    ++g_tc_gen;
    return 0;
}

// Copy-in mode of the pipelined drop-in calls: 0 a gather kernel when the
// arrays are page-locked (else the copy engines), 1 the copy engines always.
extern "C" int32_t ctsmg_set_copy_mode(int32_t mode) {
    if (mode != 0 && mode != 1) return set_error(CTSMG_E_ARG, "copy mode must be 0 or 1", 0, 0);
    g_copy_mode = mode;
    return 0;
}

// Per-chunk timeline of the calling thread's pipelined drop-in calls.
extern "C" int32_t ctsmg_pipe_trace(int32_t enable, float* ms_out, int32_t max_chunks, int32_t* nchunks_out) {
    ThreadCtx* c;
    int rc = ctx_get(&c);
    if (rc) return rc;
    if (ms_out && nchunks_out) {
        const int n = std::min(c->trace_n, (int)std::max(max_chunks, 0));
        for (int k = 0; k < n; ++k) {
            for (int j = 0; j < 5; ++j) {
                float ms = 0.f;
                cudaError_t e = cudaEventElapsedTime(&ms, c->tr[0][0], c->tr[k][j]);
                if (e != cudaSuccess) return cuda_fail(e, "cudaEventElapsedTime(trace)");
                ms_out[k * 7 + j] = ms;
            }
            ms_out[k * 7 + 5] = c->trh[k][0];
            ms_out[k * 7 + 6] = c->trh[k][1];
        }
        *nchunks_out = n;
    } else if (nchunks_out) {
        *nchunks_out = c->trace_n;
    }
    if (enable >= 0) {
        if (enable && !c->tr[0][0])
            for (int k = 0; k < PIPE_CHUNKS; ++k)
                for (cudaEvent_t& t : c->tr[k]) {
                    cudaError_t e = cudaEventCreate(&t);
                    if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate(trace)");
                }
        c->trace = enable != 0;
        c->trace_n = 0;
    }
    return 0;
}

extern "C" int32_t ctsmg_copy_bytes(int64_t* h2d, int64_t* d2h, int32_t reset) {
    using namespace ctsmg;
    if (h2d) *h2d = g_h2d_bytes.load();
    if (d2h) *d2h = g_d2h_bytes.load();
    if (reset) { g_h2d_bytes = 0; g_d2h_bytes = 0; }
    return 0;
}
