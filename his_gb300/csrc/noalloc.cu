// his_grid_step_noalloc: one 2-D step of one grid that allocates no device memory.
//
// Who needs it: callers that may not allocate device memory at all, such as code
// embedded in a host application that owns every device allocation through its own
// pool (and must not call cudaMalloc behind it), or a one-off step on a grid that
// should not create, keep and destroy a grid set with its own scratch.  Such callers
// pass their state and field arrays; the stage buffers, partial sums and tables the
// step needs come from one array of HIS_NOALLOC_SCRATCH_BYTES bytes compiled into
// this library, which every GPU the library runs on holds for the life of the process.
//
// The array's device address belongs to one CUDA context.  The first call in each
// context (the device's primary context, or a context the host application made
// itself and made current) looks the address up with cudaGetSymbolAddress and keeps
// it under the context's unique ID, so a later context -- after cudaDeviceReset, or a
// second context the application creates -- gets its own lookup and never an address
// of another context.  That first call per context is the set-up and should come
// before any stream capture.  Grids whose scratch would not fit the array are rejected
// with HIS_ERR_BAD_ARG before any work is queued.
//
// Every call clears the partial sums and totals it reads, so nothing in the array has
// to start at zero; the state arrays (h, hu, hv, s_filled, infil_cum) and the optional
// peak arrays are the caller's and are read and updated in place.  All calls share the
// one array: two calls whose work can overlap on the GPU (for example on two streams
// without an event between them, or from two host threads) race on it and give wrong
// results.  Order them on one stream.
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda.h>

#include "his_internal.h"
#include "swe2d_strip.cuh"

namespace his {

static __device__ __align__(256) unsigned char g_noalloc_scratch[HIS_NOALLOC_SCRATCH_BYTES];

// Current context and its process-unique ID, through the driver entry points that
// the runtime hands out (the library links the runtime only).
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
static CtxGetCurrentFn g_ctx_current = nullptr;
static CtxGetIdFn g_ctx_id = nullptr;
static std::once_flag g_ctx_once;

static void load_ctx_entry_points() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_ctx_id = reinterpret_cast<CtxGetIdFn>(f);
    cudaGetLastError();
}

// Key of the current context (0: none current yet, or the lookup is unavailable).
static unsigned long long current_ctx_key() {
    std::call_once(g_ctx_once, load_ctx_entry_points);
    if (!g_ctx_current) return 0;
    CUcontext ctx = nullptr;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    unsigned long long id = 0;
    if (g_ctx_id && g_ctx_id(ctx, &id) == CUDA_SUCCESS) return id + 1;
    return (unsigned long long)(uintptr_t)ctx;
}

constexpr int kNoallocCache = 64;
struct NoallocEntry {
    unsigned long long ctx;
    unsigned char* base;
};
static NoallocEntry g_noalloc_cache[kNoallocCache] = {};
static int g_noalloc_next = 0;
static std::mutex g_noalloc_mu;

// Device address of the scratch array in the current context, looked up once per
// context.  With no context current yet, the lookup itself brings up the device's
// primary context (as any runtime call does), and the address is kept under that
// context's key.  Without a context key (no driver entry points), the address is
// looked up on every call.
static int noalloc_base(unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    unsigned long long key = current_ctx_key();
    if (key)
        for (const NoallocEntry& e : g_noalloc_cache)
            if (e.ctx == key) {
                *out = e.base;
                return HIS_OK;
            }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "his_grid_step_noalloc: cudaGetSymbolAddress");
    if (!p) {
        set_error("his_grid_step_noalloc: cudaGetSymbolAddress returned a null address");
        return HIS_ERR_CUDA;
    }
    if (!key) key = current_ctx_key();
    if (key) {
        g_noalloc_cache[g_noalloc_next] = NoallocEntry{key, static_cast<unsigned char*>(p)};
        g_noalloc_next = (g_noalloc_next + 1) % kNoallocCache;
    }
    *out = static_cast<unsigned char*>(p);
    return HIS_OK;
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Strips of up to 58 columns and chunks of up to 48 rows (the grid set's defaults),
// then the scratch regions: three stage planes, partial sums, strip table, grid
// record, step parameters, totals.
static NoallocPlan noalloc_plan(int ny, int nx, size_t elem) {
    NoallocPlan L{};
    L.ns = (nx + 57) / 58;
    L.w = (nx + L.ns - 1) / L.ns;
    L.nch = (ny + 47) / 48;
    L.hch = (ny + L.nch - 1) / L.nch;
    L.n_strips = L.ns * L.nch;
    L.plane = align256((size_t)ny * (size_t)nx * elem);
    size_t off = 0;
    L.o_stage = off; off += 3 * L.plane;
    L.o_part = off; off += align256(sizeof(double) * NPART * (size_t)L.n_strips);
    L.o_strips = off; off += align256(sizeof(StripRef) * (size_t)L.n_strips);
    L.o_grid = off; off += 256;
    L.o_params = off; off += 256;
    L.o_out = off; off += 256;
    L.total = off;
    return L;
}

}  // namespace his

using namespace his;

extern "C" int32_t his_grid_step_noalloc(int32_t precision, const his_solver_cfg* cfg, const his_grid_desc* grid,
                                         const his_step_params* params, double* vols, void* stream) {
    int rc = check_cfg(cfg);
    if (rc) return rc;
    if (precision != HIS_PREC_F64 && precision != HIS_PREC_F32) {
        set_error("precision must be 0 (f64) or 1 (f32)");
        return HIS_ERR_BAD_ARG;
    }
    if (!grid || !params) {
        set_error("his_grid_step_noalloc: grid and params are required");
        return HIS_ERR_BAD_ARG;
    }
    const his_grid_desc& d = *grid;
    if (d.ny <= 0 || d.nx <= 0) { set_error("grid must be at least 1 x 1"); return HIS_ERR_BAD_ARG; }
    if (!(d.dx > 0) || !(d.dy > 0)) { set_error("dx and dy must be positive"); return HIS_ERR_BAD_ARG; }
    for (int e = 0; e < 4; ++e)
        if (d.bc[e] < 0 || d.bc[e] > 3) { set_error("unknown boundary kind"); return HIS_ERR_BAD_ARG; }
    if (!d.h || !d.hu || !d.hv || !d.s_filled || !d.infil_cum || !d.z || !d.manning) {
        set_error("state, bed and roughness pointers are required");
        return HIS_ERR_BAD_ARG;
    }
    const int nh = (d.f0 != nullptr) + (d.fc != nullptr) + (d.k != nullptr);
    if (nh != 0 && nh != 3) { set_error("f0, fc and k must be given together"); return HIS_ERR_BAD_ARG; }
    const size_t elem = precision == HIS_PREC_F64 ? sizeof(double) : sizeof(float);
    if ((int64_t)d.ny * d.nx > ((int64_t)HIS_NOALLOC_SCRATCH_BYTES) / (3 * (int64_t)elem)) {
        set_error("his_grid_step_noalloc: a " + std::to_string(d.ny) + " x " + std::to_string(d.nx) +
                  " grid does not fit the " + std::to_string((long long)HIS_NOALLOC_SCRATCH_BYTES) +
                  "-byte scratch; use his_grid_create for larger grids");
        return HIS_ERR_BAD_ARG;
    }
    const NoallocPlan L = noalloc_plan(d.ny, d.nx, elem);
    if (L.total > (size_t)HIS_NOALLOC_SCRATCH_BYTES) {
        set_error("his_grid_step_noalloc: a " + std::to_string(d.ny) + " x " + std::to_string(d.nx) +
                  " grid needs " + std::to_string(L.total) + " bytes of scratch, more than the " +
                  std::to_string((long long)HIS_NOALLOC_SCRATCH_BYTES) +
                  " it has; use his_grid_create for larger grids");
        return HIS_ERR_BAD_ARG;
    }
    const his_step_params& q = *params;
    if (!std::isfinite(q.dt) || !(q.dt >= 0) || !std::isfinite(q.t) || !std::isfinite(q.rain)) {
        set_error("dt, t and rain must be finite (dt >= 0)");
        return HIS_ERR_BAD_ARG;
    }
    unsigned char* base = nullptr;
    if ((rc = noalloc_base(&base))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const Consts c = to_consts(cfg);
    rc = precision == HIS_PREC_F64 ? noalloc_step_f64(c, d, *params, L, base, s)
                                   : noalloc_step_f32(c, d, *params, L, base, s);
    if (rc || !vols) return rc;
    // pageable destination: the copy returns once the five totals are on the host
    HIS_CK(cudaMemcpyAsync(vols, base + L.o_out, sizeof(double) * 5, cudaMemcpyDeviceToHost, s));
    HIS_CK(cudaStreamSynchronize(s));
    return HIS_OK;
}
