// C ABI of the flood-engine step (include/his_gb300.h): argument checks, device
// tables, host<->device parameter and result movement, precision dispatch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "his_internal.h"

namespace his {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return HIS_ERR_CUDA;
}

void* stage_acquire(HostStage& st, size_t bytes, int* slot) {
    cudaError_t e = cudaSuccess;
    if (bytes > st.bytes) {
        size_t want = (std::max(bytes, size_t(256)) + 4095) & ~size_t(4095);
        for (int k = 0; k < HostStage::SLOTS; ++k) {
            if (st.done[k]) cudaEventSynchronize(st.done[k]);
            if (st.buf[k]) cudaFreeHost(st.buf[k]);
            st.buf[k] = nullptr;
        }
        st.bytes = 0;
        for (int k = 0; k < HostStage::SLOTS && e == cudaSuccess; ++k) {
            e = cudaMallocHost(&st.buf[k], want);
            if (e == cudaSuccess) std::memset(st.buf[k], 0, want);   // recycled pinned pages hold old data
            if (e == cudaSuccess && !st.done[k]) e = cudaEventCreateWithFlags(&st.done[k], cudaEventDisableTiming);
        }
        if (e != cudaSuccess) {
            cuda_fail(e, "pinned staging buffer");
            return nullptr;
        }
        st.bytes = want;
    }
    int k = st.next;
    st.next = (k + 1) % HostStage::SLOTS;
    if ((e = cudaEventSynchronize(st.done[k])) != cudaSuccess) {
        cuda_fail(e, "pinned staging buffer: previous copy");
        return nullptr;
    }
    *slot = k;
    return st.buf[k];
}

int stage_release(HostStage& st, int slot, cudaStream_t s) {
    HIS_CK(cudaEventRecord(st.done[slot], s));
    return HIS_OK;
}

void stage_free(HostStage& st) {
    for (int k = 0; k < HostStage::SLOTS; ++k) {
        if (st.done[k]) {
            cudaEventSynchronize(st.done[k]);
            cudaEventDestroy(st.done[k]);
        }
        if (st.buf[k]) cudaFreeHost(st.buf[k]);
        st.done[k] = nullptr;
        st.buf[k] = nullptr;
    }
    st.bytes = 0;
}

// Output of an asynchronous entry point: device memory or page-locked host memory,
// which the GPU writes without the host waiting.  Pageable memory is refused: a copy
// into it would wait for the stream.  *direct is set when the kernels may store to
// the address themselves (device, managed or mapped page-locked memory); otherwise
// the results are copied there on the stream.
static int check_async_out(const void* p, const char* what, bool* direct) {
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error(std::string(what) + ": not a CUDA-visible address");
        return HIS_ERR_BAD_ARG;
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeHost && a.type != cudaMemoryTypeManaged) {
        set_error(std::string(what) + " must be device or page-locked host memory");
        return HIS_ERR_BAD_ARG;
    }
    *direct = a.type != cudaMemoryTypeHost || a.devicePointer == p;
    return HIS_OK;
}

// Work decomposition of the 2-D kernels: strips of at most tx columns (CTAs of 64,
// 128, 224 or 352 threads, see strip_threads), chunks of ty rows.
bool tile_supported(int tx, int ty) { return tx >= 1 && strip_threads(tx) > 0 && ty >= 1 && ty <= 1 << 20; }

Consts to_consts(const his_solver_cfg* c) {
    Consts k{};
    k.g = c->g; k.h_dry = c->h_dry; k.kp_eps = c->kp_eps; k.cfl = c->cfl; k.dt_min = c->dt_min; k.dt_max = c->dt_max;
    k.cfl_1d = c->cfl_1d; k.slot_width_frac = c->slot_width_frac; k.weir_cw = c->weir_cw;
    k.exchange_limit = c->exchange_limit; k.exchange_relax = c->exchange_relax;
    k.order = c->order; k.hllc = c->hllc;
    return k;
}

static int bad(const std::string& msg) {
    set_error(msg);
    return HIS_ERR_BAD_ARG;
}

int check_cfg(const his_solver_cfg* c) {
    if (!c) return bad("cfg is NULL");
    if (c->order != 1 && c->order != 2) return bad("order must be 1 or 2");
    if (c->hllc != 0 && c->hllc != 1) return bad("hllc must be 0 or 1");
    if (!(c->g > 0) || !(c->h_dry > 0) || !(c->kp_eps > 0)) return bad("g, h_dry and kp_eps must be positive");
    return HIS_OK;
}

// CSR of `key` (values in [0, n)) listing positions in increasing order.
static void build_csr(const int32_t* key, int len, int n, std::vector<int>& start, std::vector<int>& idx) {
    start.assign(n + 1, 0);
    for (int i = 0; i < len; ++i) start[key[i] + 1]++;
    for (int i = 0; i < n; ++i) start[i + 1] += start[i];
    idx.assign(len, 0);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int i = 0; i < len; ++i) idx[fill[key[i]]++] = i;
}

// Device arena built from host vectors: returns offsets, one cudaMalloc, one copy.
struct Arena {
    std::vector<char> host;
    size_t add(const void* p, size_t bytes) {
        size_t off = (host.size() + 255) & ~size_t(255);
        host.resize(off + bytes);
        if (bytes) std::memcpy(host.data() + off, p, bytes);
        return off;
    }
};

}  // namespace his

using namespace his;

extern "C" {

int32_t his_version(void) { return 100; }

const char* his_last_error(void) { return g_last_error.c_str(); }

// ------------------------------------------------------------------------- 2-D grid
int32_t his_grid_create(int32_t precision, const his_solver_cfg* cfg, int32_t n_members, const his_grid_desc* grids,
                        int32_t tile_x, int32_t tile_y, his_grid** out) {
    if (!out) return bad("out is NULL");
    *out = nullptr;
    int rc = check_cfg(cfg);
    if (rc) return rc;
    if (precision != HIS_PREC_F64 && precision != HIS_PREC_F32) return bad("precision must be 0 (f64) or 1 (f32)");
    if (n_members <= 0 || !grids) return bad("need at least one grid member");
    if (tile_x == 0) tile_x = 58;
    if (tile_y == 0) tile_y = 48;
    if (!tile_supported(tile_x, tile_y)) return bad("unsupported work decomposition (strip width 1..346, rows >= 1)");
    for (int m = 0; m < n_members; ++m) {
        const his_grid_desc& d = grids[m];
        std::string who = "member " + std::to_string(m) + ": ";
        if (d.ny <= 0 || d.nx <= 0) return bad(who + "grid must be at least 1 x 1");
        if ((int64_t)d.ny * d.nx > (int64_t)1 << 30) return bad(who + "grid too large");
        if (!(d.dx > 0) || !(d.dy > 0)) return bad(who + "dx and dy must be positive");
        for (int e = 0; e < 4; ++e)
            if (d.bc[e] < 0 || d.bc[e] > 3) return bad(who + "unknown boundary kind");
        if (!d.h || !d.hu || !d.hv || !d.s_filled || !d.infil_cum || !d.z || !d.manning)
            return bad(who + "state, bed and roughness pointers are required");
        int nh = (d.f0 != nullptr) + (d.fc != nullptr) + (d.k != nullptr);
        if (nh != 0 && nh != 3) return bad(who + "f0, fc and k must be given together");
    }
    his_grid* g = new his_grid();
    g->prec = precision;
    g->c = to_consts(cfg);
    g->n = n_members;
    g->tx = tile_x;
    g->nt = strip_threads(tile_x);
    g->ty = tile_y;
    g->desc.assign(grids, grids + n_members);
    cudaGetDevice(&g->device);
    rc = precision == HIS_PREC_F64 ? grid_init_f64(g) : grid_init_f32(g);
    if (rc == HIS_OK) {
        cudaError_t e = cudaMalloc(&g->d_params, sizeof(StepParams) * n_members);
        if (e == cudaSuccess) e = cudaMemset(g->d_params, 0, sizeof(StepParams) * n_members);
        if (e == cudaSuccess) e = cudaMalloc(&g->d_out, sizeof(double) * 8 * n_members);
        if (e == cudaSuccess) e = cudaMemset(g->d_out, 0, sizeof(double) * 8 * n_members);
        if (e == cudaSuccess) e = cudaMallocHost(&g->h_out, sizeof(double) * 8 * n_members);
        if (e != cudaSuccess) rc = cuda_fail(e, "his_grid_create: allocation");
    }
    if (rc != HIS_OK) {
        his_grid_destroy(g);
        return rc;
    }
    *out = g;
    return HIS_OK;
}

int32_t his_grid_destroy(his_grid* g) {
    if (!g) return HIS_OK;
    cudaFree(g->d_grids);
    cudaFree(g->d_tiles);
    cudaFree(g->d_params);
    cudaFree(g->d_partials);
    cudaFree(g->d_out);
    cudaFree(g->d_scratch);
    if (g->h_out) cudaFreeHost(g->h_out);
    stage_free(g->params_stage);
    for (int k = 0; k < his_grid::MAX_PARTS - 1; ++k) {
        if (g->ps[k]) {
            cudaStreamSynchronize(g->ps[k]);
            cudaStreamDestroy(g->ps[k]);
        }
        if (g->pev_join[k]) cudaEventDestroy(g->pev_join[k]);
    }
    if (g->pev_fork) cudaEventDestroy(g->pev_fork);
    if (g->ledger_exec) cudaGraphExecDestroy(g->ledger_exec);
    if (g->cap_stream) cudaStreamDestroy(g->cap_stream);
    delete g;
    return HIS_OK;
}

int64_t his_grid_scratch_bytes(const his_grid* g) {
    return g ? (int64_t)(g->scratch_bytes + g->table_bytes) : 0;
}

// Every field is set: the snapshot pointers and slot are NULL / -1 (the drop-in step
// writes no output series), which the kernels read to decide whether to write one.
extern "C" int32_t his_engine_default_chains(int32_t n_members, int32_t n_tiles);

// Parts of a grid step's stage launches (his_grid::n_parts): the engine's chain rule,
// cut at the member boundaries nearest to equal shares of the tiles; the streams and
// events are created here, on the first step.
static int grid_parts_setup(his_grid* g) {
    const int np = std::min((int)his_grid::MAX_PARTS, (int)his_engine_default_chains(g->n, g->n_tiles));
    cudaError_t e = cudaSuccess;
    if (np > 1) e = cudaEventCreateWithFlags(&g->pev_fork, cudaEventDisableTiming);
    for (int k = 0; k + 1 < np && e == cudaSuccess; ++k) {
        e = cudaStreamCreateWithFlags(&g->ps[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->pev_join[k], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        // release what was made, so that a later step retries from a clean slate
        for (int k = 0; k + 1 < his_grid::MAX_PARTS; ++k) {
            if (g->ps[k]) cudaStreamDestroy(g->ps[k]);
            if (g->pev_join[k]) cudaEventDestroy(g->pev_join[k]);
            g->ps[k] = nullptr;
            g->pev_join[k] = nullptr;
        }
        if (g->pev_fork) cudaEventDestroy(g->pev_fork);
        g->pev_fork = nullptr;
        return cuda_fail(e, "grid step: part streams");
    }
    g->part_t[0] = 0;
    int m = 0;
    for (int k = 1; k < np; ++k) {
        const long long want = (long long)g->n_tiles * k / np;
        m = std::max(m + 1, 1);
        while (m < g->n - (np - k) && g->tile0[m] < want) ++m;
        g->part_t[k] = g->tile0[m];
    }
    g->part_t[np] = g->n_tiles;
    g->n_parts = np;
    return HIS_OK;
}

static int fill_params(his_grid* g, const his_step_params* p, StepParams* sp) {
    for (int m = 0; m < g->n; ++m) {
        const his_step_params& q = p[m];
        sp[m] = StepParams{};
        sp[m].snap_k = -1;
        if (!std::isfinite(q.dt) || !(q.dt >= 0) || !std::isfinite(q.t) || !std::isfinite(q.rain))
            return bad("member " + std::to_string(m) + ": dt, t and rain must be finite (dt >= 0)");
        sp[m] = step_params_from(q);
    }
    return HIS_OK;
}

static int upload_params(his_grid* g, const his_step_params* p, cudaStream_t s) {
    std::vector<StepParams> sp(g->n);
    int rc = fill_params(g, p, sp.data());
    if (rc) return rc;
    // pageable source: returns once the data is staged, so `sp` may go out of scope
    HIS_CK(cudaMemcpyAsync(g->d_params, sp.data(), sizeof(StepParams) * g->n, cudaMemcpyHostToDevice, s));
    return HIS_OK;
}

static int upload_params_pinned(his_grid* g, const his_step_params* p, cudaStream_t s) {
    int slot = 0;
    auto* sp = (StepParams*)stage_acquire(g->params_stage, sizeof(StepParams) * g->n, &slot);
    if (!sp) return HIS_ERR_CUDA;
    int rc = fill_params(g, p, sp);
    if (rc) return rc;
    HIS_CK(cudaMemcpyAsync(g->d_params, sp, sizeof(StepParams) * g->n, cudaMemcpyHostToDevice, s));
    return stage_release(g->params_stage, slot, s);
}

static int fetch_out(his_grid* g, cudaStream_t s) {
    HIS_CK(cudaMemcpyAsync(g->h_out, g->d_out, sizeof(double) * 8 * g->n, cudaMemcpyDeviceToHost, s));
    HIS_CK(cudaStreamSynchronize(s));
    return HIS_OK;
}

int32_t his_grid_step(his_grid* g, const his_step_params* params, double* vols, void* stream) {
    if (!g || !params) return bad("grid and params are required");
    if (!g->n_parts) {
        int rc = grid_parts_setup(g);
        if (rc) return rc;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int rc = upload_params(g, params, s);
    if (rc) return rc;
    rc = g->prec == HIS_PREC_F64 ? grid_step_f64(g, s) : grid_step_f32(g, s);
    if (rc || !vols) return rc;
    if ((rc = fetch_out(g, s))) return rc;
    for (int m = 0; m < g->n; ++m)
        for (int j = 0; j < 5; ++j) vols[m * 5 + j] = g->h_out[m * 8 + j];
    return HIS_OK;
}

int32_t his_grid_step_async(his_grid* g, const his_step_params* params, double* vols, void* stream) {
    if (!g || !params) return bad("grid and params are required");
    if (!g->n_parts) {
        int rc = grid_parts_setup(g);
        if (rc) return rc;
    }
    bool direct = false;
    int rc = vols ? check_async_out(vols, "vols", &direct) : HIS_OK;
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if ((rc = upload_params_pinned(g, params, s))) return rc;
    double* ext = direct ? vols : nullptr;
    rc = g->prec == HIS_PREC_F64 ? grid_step_f64(g, s, ext) : grid_step_f32(g, s, ext);
    if (rc || !vols || direct) return rc;
    HIS_CK(cudaMemcpy2DAsync(vols, 5 * sizeof(double), g->d_out, 8 * sizeof(double), 5 * sizeof(double), g->n,
                             cudaMemcpyDefault, s));
    return HIS_OK;
}

// The caller's ledger must be device memory (the finalize kernel adds into it).
static int check_ledger(double* ledger) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, ledger) != cudaSuccess || a.type != cudaMemoryTypeDevice) {
        cudaGetLastError();
        return bad("ledger must be device memory");
    }
    return HIS_OK;
}

// The ledger step's launches (stages of every part, finalize) captured once per ledger:
// the same kernels with the same arguments every step (the step parameters are read
// from the grid's device buffer, uploaded before the graph runs).
static int capture_ledger_step(his_grid* g, double* ledger) {
    if (!g->cap_stream) HIS_CK(cudaStreamCreateWithFlags(&g->cap_stream, cudaStreamNonBlocking));
    if (g->ledger_exec) {
        HIS_CK(cudaGraphExecDestroy(g->ledger_exec));
        g->ledger_exec = nullptr;
        g->ledger_exec_for = nullptr;
    }
    HIS_CK(cudaStreamBeginCapture(g->cap_stream, cudaStreamCaptureModeThreadLocal));
    const int rc = g->prec == HIS_PREC_F64 ? grid_step_f64(g, g->cap_stream, nullptr, ledger)
                                           : grid_step_f32(g, g->cap_stream, nullptr, ledger);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(g->cap_stream, &graph);
    if (rc || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return rc ? rc : cuda_fail(e, "cudaStreamEndCapture");
    }
    const cudaError_t ei = cudaGraphInstantiate(&g->ledger_exec, graph, 0);
    cudaGraphDestroy(graph);
    HIS_CK(ei);
    g->ledger_exec_for = ledger;
    return HIS_OK;
}

int32_t his_grid_step_ledger_async(his_grid* g, const his_step_params* params, double* ledger, void* stream) {
    if (!g || !params || !ledger) return bad("grid, params and ledger are required");
    int rc = HIS_OK;
    if (ledger != g->ledger_checked) {
        if ((rc = check_ledger(ledger))) return rc;
        g->ledger_checked = ledger;
    }
    if (!g->n_parts && (rc = grid_parts_setup(g))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if ((rc = upload_params_pinned(g, params, s))) return rc;
    // a caller capturing its own graph gets the launches themselves, and so does every
    // step once a capture has failed (a capture the thread cannot open, for one)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    HIS_CK(cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusNone && !g->ledger_graph_off && g->ledger_exec_for != ledger &&
        capture_ledger_step(g, ledger) != HIS_OK) {
        cudaGetLastError();
        g->ledger_graph_off = true;
    }
    if (cs != cudaStreamCaptureStatusNone || g->ledger_graph_off)
        return g->prec == HIS_PREC_F64 ? grid_step_f64(g, s, nullptr, ledger) : grid_step_f32(g, s, nullptr, ledger);
    HIS_CK(cudaGraphLaunch(g->ledger_exec, s));
    return HIS_OK;
}

int32_t his_grid_max_rate_async(his_grid* g, double* rate, void* stream) {
    if (!g || !rate) return bad("grid and rate are required");
    bool direct = false;
    int rc = check_async_out(rate, "rate", &direct);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    double* ext = direct ? rate : nullptr;
    rc = g->prec == HIS_PREC_F64 ? grid_reduce_f64(g, s, ext, true) : grid_reduce_f32(g, s, ext, true);
    if (rc || direct) return rc;
    HIS_CK(cudaMemcpy2DAsync(rate, sizeof(double), g->d_out + 5, 8 * sizeof(double), sizeof(double), g->n,
                             cudaMemcpyDefault, s));
    return HIS_OK;
}

int32_t his_grid_step_rate_async(his_grid* g, double* rate, void* stream) {
    if (!g || !rate) return bad("grid and rate are required");
    bool direct = false;
    int rc = check_async_out(rate, "rate", &direct);
    if (rc) return rc;
    HIS_CK(cudaMemcpy2DAsync(rate, sizeof(double), g->d_out + 5, 8 * sizeof(double), sizeof(double), g->n,
                             cudaMemcpyDefault, (cudaStream_t)stream));
    return HIS_OK;
}

int32_t his_grid_max_rate(his_grid* g, double* rate, void* stream) {
    if (!g || !rate) return bad("grid and rate are required");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = g->prec == HIS_PREC_F64 ? grid_reduce_f64(g, s, nullptr, true) : grid_reduce_f32(g, s, nullptr, true);
    if (rc || (rc = fetch_out(g, s))) return rc;
    for (int m = 0; m < g->n; ++m) rate[m] = g->h_out[m * 8 + 5];
    return HIS_OK;
}

int32_t his_grid_volumes(his_grid* g, double* vols, void* stream) {
    if (!g || !vols) return bad("grid and vols are required");
    cudaStream_t s = (cudaStream_t)stream;
    int rc = g->prec == HIS_PREC_F64 ? grid_reduce_f64(g, s) : grid_reduce_f32(g, s);
    if (rc || (rc = fetch_out(g, s))) return rc;
    for (int m = 0; m < g->n; ++m) {
        vols[m * 2 + 0] = g->h_out[m * 8 + 6];
        vols[m * 2 + 1] = g->h_out[m * 8 + 7];
    }
    return HIS_OK;
}

// ------------------------------------------------------------------------ 1-D network
int32_t his_net_create(const his_solver_cfg* cfg, int32_t n_members, const his_net_desc* nets, his_net** out) {
    if (!out) return bad("out is NULL");
    *out = nullptr;
    int rc = check_cfg(cfg);
    if (rc) return rc;
    if (n_members <= 0 || !nets) return bad("need at least one network member");
    Arena ar;
    struct Offs { size_t kind, gsrc, fl, fr, gsign, ls, li, rs, ri, z, n, dx, b, m, yb, ts, fb, fm, fyb, fts;
                  size_t zf, dxf, bf, mf, ybf, tsf, nf, gsf, fbf, fmf, fybf, ftsf; };
    std::vector<Offs> offs(n_members);
    size_t smem = 0, smem_f32 = 0;
    for (int mb = 0; mb < n_members; ++mb) {
        const his_net_desc& d = nets[mb];
        std::string who = "network " + std::to_string(mb) + ": ";
        if (d.n_cells <= 0 || d.n_faces <= 0) return bad(who + "needs cells and faces");
        if (!d.kind || !d.ghost_src || !d.face_l || !d.face_r || !d.ghost_sign || !d.z || !d.manning || !d.dx ||
            !d.b || !d.m || !d.yb || !d.ts || !d.fb || !d.fm || !d.fyb || !d.fts || !d.A || !d.Q)
            return bad(who + "all arrays are required");
        for (int i = 0; i < d.n_cells; ++i) {
            if (d.kind[i] < 0 || d.kind[i] > 4) return bad(who + "cell kind out of range");
            if (d.kind[i] >= 2 && (d.ghost_src[i] < 0 || d.ghost_src[i] >= d.n_cells))
                return bad(who + "ghost cell without a valid interior neighbour");
            if (!(d.dx[i] > 0) || !(d.b[i] > 0) || !(d.ts[i] > 0)) return bad(who + "dx, b and ts must be positive");
        }
        for (int f = 0; f < d.n_faces; ++f)
            if (d.face_l[f] < 0 || d.face_l[f] >= d.n_cells || d.face_r[f] < 0 || d.face_r[f] >= d.n_cells)
                return bad(who + "face cell index out of range");
        std::vector<int> ls, li, rs, ri;
        build_csr(d.face_l, d.n_faces, d.n_cells, ls, li);
        build_csr(d.face_r, d.n_faces, d.n_cells, rs, ri);
        std::vector<int32_t> gsrc(d.ghost_src, d.ghost_src + d.n_cells);
        for (auto& x : gsrc) if (x < 0) x = 0;
        Offs& o = offs[mb];
        const size_t C = sizeof(double) * d.n_cells, F = sizeof(double) * d.n_faces;
        o.kind = ar.add(d.kind, sizeof(int32_t) * d.n_cells);
        o.gsrc = ar.add(gsrc.data(), sizeof(int32_t) * d.n_cells);
        o.fl = ar.add(d.face_l, sizeof(int32_t) * d.n_faces);
        o.fr = ar.add(d.face_r, sizeof(int32_t) * d.n_faces);
        o.gsign = ar.add(d.ghost_sign, C);
        o.ls = ar.add(ls.data(), sizeof(int) * ls.size());
        o.li = ar.add(li.data(), sizeof(int) * li.size());
        o.rs = ar.add(rs.data(), sizeof(int) * rs.size());
        o.ri = ar.add(ri.data(), sizeof(int) * ri.size());
        o.z = ar.add(d.z, C); o.n = ar.add(d.manning, C); o.dx = ar.add(d.dx, C);
        o.b = ar.add(d.b, C); o.m = ar.add(d.m, C); o.yb = ar.add(d.yb, C); o.ts = ar.add(d.ts, C);
        o.fb = ar.add(d.fb, F); o.fm = ar.add(d.fm, F); o.fyb = ar.add(d.fyb, F); o.fts = ar.add(d.fts, F);
        // float32 copies of the static geometry for the production form's exchange and
        // network substeps
        auto addf = [&](const double* a, int n) {
            std::vector<float> f(a, a + n);
            return ar.add(f.data(), sizeof(float) * f.size());
        };
        o.zf = addf(d.z, d.n_cells); o.dxf = addf(d.dx, d.n_cells); o.bf = addf(d.b, d.n_cells);
        o.mf = addf(d.m, d.n_cells); o.ybf = addf(d.yb, d.n_cells); o.tsf = addf(d.ts, d.n_cells);
        o.nf = addf(d.manning, d.n_cells); o.gsf = addf(d.ghost_sign, d.n_cells);
        o.fbf = addf(d.fb, d.n_faces); o.fmf = addf(d.fm, d.n_faces); o.fybf = addf(d.fyb, d.n_faces);
        o.ftsf = addf(d.fts, d.n_faces);
        smem = std::max(smem, net_smem_bytes(d.n_cells, d.n_faces));
        smem_f32 = std::max(smem_f32, net_smem_bytes_f32(d.n_cells, d.n_faces));
    }
    if (smem > 200 * 1024 || smem_f32 > 200 * 1024)
        return bad("network too large for one thread block's shared memory");
    his_net* N = new his_net();
    N->c = to_consts(cfg);
    N->n = n_members;
    N->smem = smem;
    N->smem_f32 = smem_f32;
    N->max_sub = 256;
    cudaGetDevice(&N->device);
    auto fail = [&](cudaError_t e, const char* w) { int r = cuda_fail(e, w); his_net_destroy(N); return r; };
    cudaError_t e = cudaMalloc(&N->d_arena, ar.host.size() ? ar.host.size() : 256);
    if (e != cudaSuccess) return fail(e, "his_net_create: arena");
    N->arena_bytes = ar.host.size();
    e = cudaMemcpy(N->d_arena, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(e, "his_net_create: copy");
    char* base = (char*)N->d_arena;
    N->h_nets.resize(n_members);
    for (int mb = 0; mb < n_members; ++mb) {
        const his_net_desc& d = nets[mb];
        const Offs& o = offs[mb];
        Net& n = N->h_nets[mb];
        n.n_cells = d.n_cells; n.n_faces = d.n_faces;
        n.kind = (const int*)(base + o.kind); n.gsrc = (const int*)(base + o.gsrc);
        n.fl = (const int*)(base + o.fl); n.fr = (const int*)(base + o.fr);
        n.gsign = (const double*)(base + o.gsign);
        n.lstart = (const int*)(base + o.ls); n.lidx = (const int*)(base + o.li);
        n.rstart = (const int*)(base + o.rs); n.ridx = (const int*)(base + o.ri);
        n.z = (const double*)(base + o.z); n.nman = (const double*)(base + o.n); n.dx = (const double*)(base + o.dx);
        n.b = (const double*)(base + o.b); n.m = (const double*)(base + o.m);
        n.yb = (const double*)(base + o.yb); n.ts = (const double*)(base + o.ts);
        n.fb = (const double*)(base + o.fb); n.fm = (const double*)(base + o.fm);
        n.fyb = (const double*)(base + o.fyb); n.fts = (const double*)(base + o.fts);
        n.zf = (const float*)(base + o.zf); n.dxf = (const float*)(base + o.dxf);
        n.bf = (const float*)(base + o.bf); n.mf = (const float*)(base + o.mf);
        n.ybf = (const float*)(base + o.ybf); n.tsf = (const float*)(base + o.tsf);
        n.nmanf = (const float*)(base + o.nf); n.gsignf = (const float*)(base + o.gsf);
        n.fbf = (const float*)(base + o.fbf); n.fmf = (const float*)(base + o.fmf);
        n.fybf = (const float*)(base + o.fybf); n.ftsf = (const float*)(base + o.ftsf);
        n.A = d.A; n.Q = d.Q;
    }
    e = cudaMalloc(&N->d_nets, sizeof(Net) * n_members);
    if (e == cudaSuccess) e = cudaMemcpy(N->d_nets, N->h_nets.data(), sizeof(Net) * n_members, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&N->d_forcing, sizeof(double) * 2 * N->max_sub * n_members);
    if (e == cudaSuccess) e = cudaMalloc(&N->d_out, sizeof(double) * 3 * n_members);
    if (e == cudaSuccess) e = cudaMallocHost(&N->h_out, sizeof(double) * 3 * n_members);
    if (e != cudaSuccess) return fail(e, "his_net_create: allocation");
    *out = N;
    return HIS_OK;
}

int32_t his_net_destroy(his_net* N) {
    if (!N) return HIS_OK;
    cudaFree(N->d_arena);
    cudaFree(N->d_nets);
    cudaFree(N->d_forcing);
    cudaFree(N->d_out);
    if (N->h_out) cudaFreeHost(N->h_out);
    stage_free(N->forcing_stage);
    delete N;
    return HIS_OK;
}

int32_t his_net_step(his_net* N, double dt, int32_t n_sub, const double* forcing, double* vols, void* stream) {
    if (!N || !forcing) return bad("network and forcing are required");
    if (n_sub < 1 || n_sub > N->max_sub) return bad("n_sub must be in [1, 256]");
    if (!std::isfinite(dt) || !(dt >= 0)) return bad("dt must be finite and >= 0");
    cudaStream_t s = (cudaStream_t)stream;
    HIS_CK(cudaMemcpyAsync(N->d_forcing, forcing, sizeof(double) * 2 * n_sub * N->n, cudaMemcpyHostToDevice, s));
    int rc = net_step_launch(N, dt, n_sub, s);
    if (rc || !vols) return rc;
    HIS_CK(cudaMemcpyAsync(N->h_out, N->d_out, sizeof(double) * 3 * N->n, cudaMemcpyDeviceToHost, s));
    HIS_CK(cudaStreamSynchronize(s));
    std::memcpy(vols, N->h_out, sizeof(double) * 3 * N->n);
    return HIS_OK;
}

int32_t his_net_step_async(his_net* N, double dt, int32_t n_sub, const double* forcing, double* vols,
                           void* stream) {
    if (!N || !forcing) return bad("network and forcing are required");
    if (n_sub < 1 || n_sub > N->max_sub) return bad("n_sub must be in [1, 256]");
    if (!std::isfinite(dt) || !(dt >= 0)) return bad("dt must be finite and >= 0");
    bool direct = false;
    int rc = vols ? check_async_out(vols, "vols", &direct) : HIS_OK;
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    size_t bytes = sizeof(double) * 2 * n_sub * N->n;
    int slot = 0;
    void* pin = stage_acquire(N->forcing_stage, bytes, &slot);
    if (!pin) return HIS_ERR_CUDA;
    std::memcpy(pin, forcing, bytes);
    HIS_CK(cudaMemcpyAsync(N->d_forcing, pin, bytes, cudaMemcpyHostToDevice, s));
    if ((rc = stage_release(N->forcing_stage, slot, s))) return rc;
    if ((rc = net_step_launch(N, dt, n_sub, s, direct ? vols : nullptr)) || !vols || direct) return rc;
    HIS_CK(cudaMemcpyAsync(vols, N->d_out, sizeof(double) * 3 * N->n, cudaMemcpyDefault, s));
    return HIS_OK;
}

int32_t his_net_step_ledger_async(his_net* N, double dt, int32_t n_sub, const double* forcing, double* ledger,
                                  void* stream) {
    if (!N || !forcing || !ledger) return bad("network, forcing and ledger are required");
    if (n_sub < 1 || n_sub > N->max_sub) return bad("n_sub must be in [1, 256]");
    if (!std::isfinite(dt) || !(dt >= 0)) return bad("dt must be finite and >= 0");
    int rc = HIS_OK;
    if (ledger != N->ledger_checked) {
        if ((rc = check_ledger(ledger))) return rc;
        N->ledger_checked = ledger;
    }
    cudaStream_t s = (cudaStream_t)stream;
    size_t bytes = sizeof(double) * 2 * n_sub * N->n;
    int slot = 0;
    void* pin = stage_acquire(N->forcing_stage, bytes, &slot);
    if (!pin) return HIS_ERR_CUDA;
    std::memcpy(pin, forcing, bytes);
    HIS_CK(cudaMemcpyAsync(N->d_forcing, pin, bytes, cudaMemcpyHostToDevice, s));
    if ((rc = stage_release(N->forcing_stage, slot, s))) return rc;
    return net_step_launch(N, dt, n_sub, s, nullptr, ledger);
}

int32_t his_net_max_rate_async(his_net* N, double* rate_wet, void* stream) {
    if (!N || !rate_wet) return bad("network and rate_wet are required");
    bool direct = false;
    int rc = check_async_out(rate_wet, "rate_wet", &direct);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if ((rc = net_reduce_launch(N, s, direct ? rate_wet : nullptr)) || direct) return rc;
    HIS_CK(cudaMemcpy2DAsync(rate_wet, 2 * sizeof(double), N->d_out, 3 * sizeof(double), 2 * sizeof(double), N->n,
                             cudaMemcpyDefault, s));
    return HIS_OK;
}

static int net_reduce(his_net* N, cudaStream_t s) {
    int rc = net_reduce_launch(N, s);
    if (rc) return rc;
    HIS_CK(cudaMemcpyAsync(N->h_out, N->d_out, sizeof(double) * 3 * N->n, cudaMemcpyDeviceToHost, s));
    HIS_CK(cudaStreamSynchronize(s));
    return HIS_OK;
}

int32_t his_net_max_rate(his_net* N, double* rate, int32_t* any_wet, void* stream) {
    if (!N || !rate || !any_wet) return bad("network, rate and any_wet are required");
    int rc = net_reduce(N, (cudaStream_t)stream);
    if (rc) return rc;
    for (int m = 0; m < N->n; ++m) {
        rate[m] = N->h_out[m * 3 + 0];
        any_wet[m] = N->h_out[m * 3 + 1] > 0.0 ? 1 : 0;
    }
    return HIS_OK;
}

int32_t his_net_volume(his_net* N, double* vol, void* stream) {
    if (!N || !vol) return bad("network and vol are required");
    int rc = net_reduce(N, (cudaStream_t)stream);
    if (rc) return rc;
    for (int m = 0; m < N->n; ++m) vol[m] = N->h_out[m * 3 + 2];
    return HIS_OK;
}

// ---------------------------------------------------------------------------- links
int32_t his_links_create(his_grid* grid, his_net* net, int32_t n_members, const his_links_desc* links,
                         his_links** out) {
    if (!out) return bad("out is NULL");
    *out = nullptr;
    if (!grid || !net || !links) return bad("grid, net and links are required");
    if (n_members != grid->n || n_members != net->n)
        return bad("links, grid and network must have the same number of members");
    Arena ar;
    struct Offs { size_t c1, inv, uq, zb, len, z2, us, ui, cs, ci, zbf, lenf, z2f; };
    std::vector<Offs> offs(n_members);
    size_t smem = 0;
    int total = 0;
    for (int mb = 0; mb < n_members; ++mb) {
        const his_links_desc& d = links[mb];
        const his_grid_desc& gd = grid->desc[mb];
        const int nc = net->h_nets[mb].n_cells;
        std::string who = "links " + std::to_string(mb) + ": ";
        if (d.n_links < 0 || d.n_unique < 0) return bad(who + "negative count");
        if (d.n_links > 0 && (!d.cell1d || !d.inv || !d.uniq || !d.zbank || !d.length || !d.z2))
            return bad(who + "all arrays are required");
        std::vector<int32_t> uq(d.n_unique);
        for (int k = 0; k < d.n_unique; ++k) {
            if (d.uniq[k] < 0 || d.uniq[k] >= (int64_t)gd.ny * gd.nx) return bad(who + "2-D cell index out of range");
            uq[k] = (int32_t)d.uniq[k];
        }
        for (int l = 0; l < d.n_links; ++l) {
            if (d.cell1d[l] < 0 || d.cell1d[l] >= nc) return bad(who + "1-D cell index out of range");
            if (d.inv[l] < 0 || d.inv[l] >= d.n_unique) return bad(who + "unique index out of range");
        }
        std::vector<int> us, ui, cs, ci;
        build_csr(d.inv, d.n_links, d.n_unique, us, ui);
        build_csr(d.cell1d, d.n_links, nc, cs, ci);
        Offs& o = offs[mb];
        const size_t L = sizeof(double) * d.n_links;
        o.c1 = ar.add(d.cell1d, sizeof(int32_t) * d.n_links);
        o.inv = ar.add(d.inv, sizeof(int32_t) * d.n_links);
        o.uq = ar.add(uq.data(), sizeof(int32_t) * uq.size());
        o.zb = ar.add(d.zbank, L); o.len = ar.add(d.length, L); o.z2 = ar.add(d.z2, L);
        auto addf = [&](const double* a) {
            std::vector<float> f(a, a + d.n_links);
            return ar.add(f.data(), sizeof(float) * f.size());
        };
        o.zbf = addf(d.zbank); o.lenf = addf(d.length); o.z2f = addf(d.z2);
        o.us = ar.add(us.data(), sizeof(int) * us.size()); o.ui = ar.add(ui.data(), sizeof(int) * ui.size());
        o.cs = ar.add(cs.data(), sizeof(int) * cs.size()); o.ci = ar.add(ci.data(), sizeof(int) * ci.size());
        smem = std::max(smem, exchange_smem_bytes(d.n_links, d.n_unique, nc));
        total += d.n_links;
    }
    if (smem > 200 * 1024) return bad("too many links for one thread block's shared memory");
    his_links* Lk = new his_links();
    Lk->grid = grid; Lk->net = net; Lk->n = n_members; Lk->total_links = total; Lk->smem = smem;
    auto fail = [&](cudaError_t e, const char* w) { int r = cuda_fail(e, w); his_links_destroy(Lk); return r; };
    cudaError_t e = cudaMalloc(&Lk->d_arena, ar.host.size() ? ar.host.size() : 256);
    if (e == cudaSuccess) e = cudaMemcpy(Lk->d_arena, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(e, "his_links_create: arena");
    char* base = (char*)Lk->d_arena;
    std::vector<Lnk> H(n_members);
    int voff = 0;
    for (int mb = 0; mb < n_members; ++mb) {
        const his_links_desc& d = links[mb];
        const Offs& o = offs[mb];
        Lnk& L = H[mb];
        L.n_links = d.n_links; L.n_unique = d.n_unique; L.v_offset = voff;
        voff += d.n_links;
        L.cell1d = (const int*)(base + o.c1); L.inv = (const int*)(base + o.inv); L.uniq = (const int*)(base + o.uq);
        L.zbank = (const double*)(base + o.zb); L.length = (const double*)(base + o.len);
        L.z2 = (const double*)(base + o.z2);
        L.zbank_f = (const float*)(base + o.zbf); L.length_f = (const float*)(base + o.lenf);
        L.z2_f = (const float*)(base + o.z2f);
        L.ustart = (const int*)(base + o.us); L.uidx = (const int*)(base + o.ui);
        L.cstart = (const int*)(base + o.cs); L.cidx = (const int*)(base + o.ci);
    }
    e = cudaMalloc(&Lk->d_links, sizeof(Lnk) * n_members);
    if (e == cudaSuccess) e = cudaMemcpy(Lk->d_links, H.data(), sizeof(Lnk) * n_members, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&Lk->d_V, sizeof(double) * std::max(total, 1));
    if (e == cudaSuccess) e = cudaMallocHost(&Lk->h_V, sizeof(double) * std::max(total, 2 * n_members));
    if (e == cudaSuccess) e = cudaMalloc(&Lk->d_exch, sizeof(double) * 2 * n_members);
    if (e == cudaSuccess) e = cudaMemset(Lk->d_exch, 0, sizeof(double) * 2 * n_members);
    if (e != cudaSuccess) return fail(e, "his_links_create: allocation");
    *out = Lk;
    return HIS_OK;
}

int32_t his_links_destroy(his_links* L) {
    if (!L) return HIS_OK;
    cudaFree(L->d_arena);
    cudaFree(L->d_links);
    cudaFree(L->d_V);
    cudaFree(L->d_exch);
    if (L->h_V) cudaFreeHost(L->h_V);
    delete L;
    return HIS_OK;
}

int32_t his_exchange(his_links* L, const his_solver_cfg* cfg, double dt, double* V, void* stream) {
    if (!L) return bad("links are required");
    if (!std::isfinite(dt) || !(dt >= 0)) return bad("dt must be finite and >= 0");
    Consts c = L->grid->c;
    if (cfg) {
        c.weir_cw = cfg->weir_cw;
        c.exchange_limit = cfg->exchange_limit;
        c.exchange_relax = cfg->exchange_relax;
    }
    cudaStream_t s = (cudaStream_t)stream;
    int rc = L->grid->prec == HIS_PREC_F64 ? exchange_f64(L, c, dt, s) : exchange_f32(L, c, dt, s);
    if (rc || !V) return rc;
    HIS_CK(cudaMemcpyAsync(L->h_V, L->d_V, sizeof(double) * std::max(L->total_links, 1), cudaMemcpyDeviceToHost, s));
    HIS_CK(cudaStreamSynchronize(s));
    std::memcpy(V, L->h_V, sizeof(double) * L->total_links);
    return HIS_OK;
}

int32_t his_exchange_async(his_links* L, const his_solver_cfg* cfg, double dt, double* V, void* stream) {
    if (!L) return bad("links are required");
    bool direct = false;
    int rc = V ? check_async_out(V, "V", &direct) : HIS_OK;
    if (rc) return rc;
    if ((rc = his_exchange(L, cfg, dt, nullptr, stream)) || !V || L->total_links == 0) return rc;
    HIS_CK(cudaMemcpyAsync(V, L->d_V, sizeof(double) * L->total_links, cudaMemcpyDefault, (cudaStream_t)stream));
    return HIS_OK;
}

int32_t his_links_exchanged(his_links* L, double* totals, int32_t reset, void* stream) {
    if (!L || !totals) return bad("links and totals are required");
    cudaStream_t s = (cudaStream_t)stream;
    HIS_CK(cudaMemcpyAsync(L->h_V, L->d_exch, sizeof(double) * 2 * L->n, cudaMemcpyDeviceToHost, s));
    HIS_CK(cudaStreamSynchronize(s));
    std::memcpy(totals, L->h_V, sizeof(double) * 2 * L->n);
    if (reset) HIS_CK(cudaMemsetAsync(L->d_exch, 0, sizeof(double) * 2 * L->n, s));
    return HIS_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------ engine
// Split the members into n chains at the member boundaries nearest to equal shares of
// the tiles (every chain at least one member); streams and events are created on
// first use, and captured graphs are dropped so that the next advance recaptures.
extern "C" int32_t his_engine_default_chains(int32_t n_members, int32_t n_tiles);

static int engine_split(his_engine* E, int n) {
    his_grid* g = E->grid;
    n = std::max(1, std::min(n, std::min(E->n, (int)his_engine::MAX_CHAINS)));
    for (int c = 1; c < n; ++c) {
        cudaError_t e = cudaSuccess;
        if (!E->cs_main[c - 1]) e = cudaStreamCreateWithFlags(&E->cs_main[c - 1], cudaStreamNonBlocking);
        if (e == cudaSuccess && !E->cs_side[c - 1])
            e = cudaStreamCreateWithFlags(&E->cs_side[c - 1], cudaStreamNonBlocking);
        for (cudaEvent_t* ev : {&E->cev_fork[c - 1], &E->cev_join[c - 1], &E->cev_out[c - 1]})
            if (e == cudaSuccess && !*ev) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(e, "engine chains: streams and events");
    }
    for (int c = 0; c < his_engine::MAX_CHAINS; ++c) {
        cudaGraphExec_t& x = E->exec_of(c);
        if (x) cudaGraphExecDestroy(x);
        x = nullptr;
        if (E->rexec[c]) cudaGraphExecDestroy(E->rexec[c]);
        E->rexec[c] = nullptr;
    }
    E->rem_steps = 0;
    E->n_chains = n;
    E->chain_m[0] = 0;
    E->chain_t[0] = 0;
    int m = 0;
    for (int c = 1; c < n; ++c) {
        const long long want = (long long)g->n_tiles * c / n;
        m = std::max(m + 1, 1);
        while (m < E->n - (n - c) && g->tile0[m] < want) ++m;
        E->chain_m[c] = m;
        E->chain_t[c] = g->tile0[m];
    }
    E->chain_m[n] = E->n;
    E->chain_t[n] = g->n_tiles;
    return HIS_OK;
}

extern "C" {

int32_t his_engine_destroy(his_engine* E) {
    if (!E) return HIS_OK;
    if (E->s0) cudaStreamSynchronize(E->s0);
    if (E->s1) cudaStreamSynchronize(E->s1);
    for (int c = 0; c < his_engine::MAX_CHAINS - 1; ++c) {
        if (E->cs_main[c]) cudaStreamSynchronize(E->cs_main[c]);
        if (E->cs_side[c]) cudaStreamSynchronize(E->cs_side[c]);
    }
    if (E->exec) cudaGraphExecDestroy(E->exec);
    for (cudaGraphExec_t x : E->cexec)
        if (x) cudaGraphExecDestroy(x);
    for (cudaGraphExec_t x : E->rexec)
        if (x) cudaGraphExecDestroy(x);
    cudaFree(E->d_em);
    cudaFree(E->d_arena);
    cudaFree(E->d_netf);
    cudaFree(E->d_vol1d);
    if (E->h_em) cudaFreeHost(E->h_em);
    for (cudaEvent_t ev : {E->ev_fork, E->ev_join, E->ev_in, E->ev_out})
        if (ev) cudaEventDestroy(ev);
    for (int c = 0; c < his_engine::MAX_CHAINS - 1; ++c) {
        for (cudaEvent_t ev : {E->cev_fork[c], E->cev_join[c], E->cev_out[c]})
            if (ev) cudaEventDestroy(ev);
        if (E->cs_main[c]) cudaStreamDestroy(E->cs_main[c]);
        if (E->cs_side[c]) cudaStreamDestroy(E->cs_side[c]);
    }
    if (E->s0) cudaStreamDestroy(E->s0);
    if (E->s1) cudaStreamDestroy(E->s1);
    delete E;
    return HIS_OK;
}

int32_t his_engine_create(his_grid* grid, his_net* net, his_links* links, int32_t n_members,
                          const his_forcing_desc* forcing, int32_t max_sub, int32_t graph_steps, his_engine** out) {
    if (!out) return bad("out is NULL");
    *out = nullptr;
    if (!grid || !forcing) return bad("grid and forcing are required");
    if (n_members != grid->n) return bad("forcing must be given for every grid member");
    if (net && net->n != n_members) return bad("network set and grid set differ in members");
    if (links && (!net || links->grid != grid || links->net != net)) return bad("links must bind this grid and network");
    if (max_sub == 0) max_sub = 64;
    if (max_sub < 1 || max_sub > 4096) return bad("max_sub must be in [1, 4096]");
    if (graph_steps == 0) graph_steps = 16;
    if (graph_steps < 1 || graph_steps > 1024) return bad("graph_steps must be in [1, 1024]");
    Arena ar;
    std::vector<size_t> orain(n_members), oq(n_members);
    std::vector<EngMember> H(n_members);
    for (int m = 0; m < n_members; ++m) {
        const his_forcing_desc& f = forcing[m];
        std::string who = "member " + std::to_string(m) + ": ";
        if (!std::isfinite(f.t0) || !std::isfinite(f.t_end) || !(f.t_end >= f.t0)) return bad(who + "need t0 <= t_end");
        if (f.rain_n < 0 || (f.rain_n > 0 && (!f.rain || !(f.rain_step > 0)))) return bad(who + "bad rain table");
        if (f.q_n < 0 || (f.q_n > 0 && (!f.q || !(f.q_step > 0)))) return bad(who + "bad inflow table");
        if (f.tide_n < 0 || f.tide_n > 4) return bad(who + "at most 4 tidal constituents");
        for (int e = 0; e < 4; ++e)
            if (f.edge_src[e] < 0 || f.edge_src[e] > 2) return bad(who + "edge value source must be 0, 1 or 2");
        orain[m] = ar.add(f.rain, sizeof(double) * std::max(f.rain_n, 0));
        oq[m] = ar.add(f.q, sizeof(double) * std::max(f.q_n, 0));
        EngMember& E = H[m];
        std::memset(&E, 0, sizeof(E));
        E.rain_t0 = f.rain_t0; E.rain_step = f.rain_step; E.rain_n = f.rain_n;
        E.tide_on = f.tide_on; E.tide_n = f.tide_n; E.tide_base = f.tide_base; E.tide_shift = f.tide_shift;
        for (int j = 0; j < 4; ++j) { E.amp[j] = f.tide_amp[j]; E.w[j] = f.tide_w[j]; E.ph[j] = f.tide_phase[j]; }
        E.q_t0 = f.q_t0; E.q_step = f.q_step; E.q_n = f.q_n;
        for (int e = 0; e < 4; ++e) { E.edge_src[e] = f.edge_src[e]; E.edge_val[e] = f.edge_val[e]; }
        E.t_end = f.t_end;
        E.t = f.t0;
        E.dt_min = INFINITY;
        E.status = f.t_end - f.t0 > 1e-9 ? ST_RUNNING : ST_DONE;
        if (f.n_out < 0) return bad(who + "n_out must be >= 0");
        if (f.n_out > 0) {
            if (!(f.out_dt > 0) || !f.snap_h || !f.snap_u || !f.snap_v || !f.snap_t)
                return bad(who + "output needs out_dt > 0 and the snap_h, snap_u, snap_v, snap_t arrays");
            if ((f.n_out - 1) * f.out_dt > f.t_end + 1e-9 * std::max(1.0, std::fabs(f.t_end)))
                return bad(who + "the last output time lies beyond t_end");
            if (net && (!f.snap_eta || !f.snap_q)) return bad(who + "output with a network needs snap_eta and snap_q");
            E.out_dt = f.out_dt;
            E.n_out = f.n_out;
            E.k_out = 1;                      // slot 0 is the initial state, written by the caller
            E.cells = grid->desc[m].ny * grid->desc[m].nx;
            E.n1d = net ? net->h_nets[m].n_cells : 0;
            E.snap_h = f.snap_h; E.snap_u = f.snap_u; E.snap_v = f.snap_v;
            E.snap_eta = net ? f.snap_eta : nullptr;
            E.snap_q = net ? f.snap_q : nullptr;
            E.snap_t = f.snap_t;
            E.snap_ledger = f.snap_ledger;
        }
    }
    his_engine* E = new his_engine();
    E->grid = grid; E->net = net; E->links = links; E->n = n_members; E->max_sub = max_sub;
    E->graph_steps = graph_steps;
    E->pre_smem = std::max<size_t>(links ? links->smem : 0, sizeof(double) * 64);
    auto fail = [&](cudaError_t e, const char* w) { int r = cuda_fail(e, w); his_engine_destroy(E); return r; };
    cudaError_t e = cudaMalloc(&E->d_arena, std::max<size_t>(ar.host.size(), 256));
    if (e == cudaSuccess && ar.host.size())
        e = cudaMemcpy(E->d_arena, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(e, "his_engine_create: forcing tables");
    for (int m = 0; m < n_members; ++m) {
        H[m].rain = forcing[m].rain_n > 0 ? (const double*)((char*)E->d_arena + orain[m]) : nullptr;
        H[m].q = forcing[m].q_n > 0 ? (const double*)((char*)E->d_arena + oq[m]) : nullptr;
    }
    e = cudaMalloc(&E->d_em, sizeof(EngMember) * n_members);
    if (e == cudaSuccess) e = cudaMemcpy(E->d_em, H.data(), sizeof(EngMember) * n_members, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMallocHost(&E->h_em, sizeof(EngMember) * n_members);
    if (e == cudaSuccess) e = cudaMalloc(&E->d_netf, sizeof(double) * 2 * (size_t)max_sub * n_members);
    if (e == cudaSuccess) e = cudaMalloc(&E->d_vol1d, sizeof(double) * 3 * n_members);
    if (e == cudaSuccess) e = cudaMemset(E->d_vol1d, 0, sizeof(double) * 3 * n_members);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&E->s0, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&E->s1, cudaStreamNonBlocking);
    for (cudaEvent_t* ev : {&E->ev_fork, &E->ev_join, &E->ev_in, &E->ev_out})
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(e, "his_engine_create: allocation");
    int rc0 = engine_split(E, his_engine_default_chains(n_members, grid->n_tiles));
    if (rc0) {
        his_engine_destroy(E);
        return rc0;
    }
    int rc = net_engine_prepare(E);
    if (rc == HIS_OK) rc = grid->prec == HIS_PREC_F64 ? engine_take_rate_f64(E) : engine_take_rate_f32(E);
    if (rc == HIS_OK) {
        e = cudaStreamSynchronize(E->s0);
        if (e != cudaSuccess) rc = cuda_fail(e, "his_engine_create: initial rate");
    }
    if (rc != HIS_OK) {
        his_engine_destroy(E);
        return rc;
    }
    *out = E;
    return HIS_OK;
}


static int engine_enqueue(his_engine* E, int chain, int n) {
    return E->grid->prec == HIS_PREC_F64 ? engine_enqueue_f64(E, chain, n) : engine_enqueue_f32(E, chain, n);
}

// One graph of n_steps steps of one chain, captured from the chain's main stream.
static int engine_capture(his_engine* E, int chain, int n_steps, cudaGraphExec_t* exec) {
    cudaStream_t s = E->main_of(chain);
    cudaGraph_t graph = nullptr;
    HIS_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = engine_enqueue(E, chain, n_steps);
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
    if (ce != cudaSuccess) return cuda_fail(ce, "his_engine_advance: capture");
    ce = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) { *exec = nullptr; return cuda_fail(ce, "his_engine_advance: instantiate"); }
    return HIS_OK;
}

// Make sure the graphs an advance of n_steps launches exist: the graph_steps graph of
// every chain (when n_steps reaches it) and the graphs of the remaining
// n_steps % graph_steps steps (one remainder size is kept; another size replaces it).
static int engine_graphs(his_engine* E, int n_steps) {
    const int nc = E->n_chains;
    if (n_steps >= E->graph_steps && !E->exec) {
        for (int c = 0; c < nc; ++c) {
            int rc = engine_capture(E, c, E->graph_steps, &E->exec_of(c));
            if (rc) return rc;
        }
    }
    const int rem = n_steps % E->graph_steps;
    if (rem && rem != E->rem_steps) {
        E->rem_steps = 0;
        for (int c = 0; c < nc; ++c) {
            if (E->rexec[c]) cudaGraphExecDestroy(E->rexec[c]);
            E->rexec[c] = nullptr;
            int rc = engine_capture(E, c, rem, &E->rexec[c]);
            if (rc) return rc;
        }
        E->rem_steps = rem;
    }
    return HIS_OK;
}

int32_t his_engine_prepare(his_engine* E, int32_t n_steps) {
    if (!E) return bad("engine is NULL");
    if (n_steps < 0) return bad("n_steps must be >= 0");
    return engine_graphs(E, n_steps);
}

int32_t his_engine_advance(his_engine* E, int32_t n_steps, void* stream) {
    if (!E) return bad("engine is NULL");
    if (n_steps < 0) return bad("n_steps must be >= 0");
    cudaStream_t caller = (cudaStream_t)stream;
    const int nc = E->n_chains;
    int rc = engine_graphs(E, n_steps);
    if (rc) return rc;
    HIS_CK(cudaEventRecord(E->ev_in, caller));
    for (int c = 0; c < nc; ++c) HIS_CK(cudaStreamWaitEvent(E->main_of(c), E->ev_in, 0));
    // the chains run independently until the end of the call, each launching its
    // graphs back to back on its own stream, so their relative phase is kept
    for (int done = 0; done + E->graph_steps <= n_steps; done += E->graph_steps)
        for (int c = 0; c < nc; ++c) HIS_CK(cudaGraphLaunch(E->exec_of(c), E->main_of(c)));
    if (n_steps % E->graph_steps)
        for (int c = 0; c < nc; ++c) HIS_CK(cudaGraphLaunch(E->rexec[c], E->main_of(c)));
    for (int c = 0; c < nc; ++c) {
        HIS_CK(cudaEventRecord(E->out_of(c), E->main_of(c)));
        HIS_CK(cudaStreamWaitEvent(caller, E->out_of(c), 0));
    }
    return HIS_OK;
}

int32_t his_engine_set_chains(his_engine* E, int32_t n_chains) {
    if (!E) return bad("engine is NULL");
    if (n_chains < 1 || n_chains > his_engine::MAX_CHAINS) return bad("n_chains must be in [1, 8]");
    for (int c = 0; c < E->n_chains; ++c) HIS_CK(cudaStreamSynchronize(E->main_of(c)));
    return engine_split(E, n_chains);
}

int32_t his_engine_chains(const his_engine* E) { return E ? E->n_chains : 0; }

// one chain per 256 strip-chunk tiles, at most 8 and at most one per member: enough
// 2-D work per chain to hide another chain's per-step kernels, without splitting
// small batches into launch-bound slivers
int32_t his_engine_default_chains(int32_t n_members, int32_t n_tiles) {
    return std::max(1, std::min(std::min((int)his_engine::MAX_CHAINS, (int)n_members), (int)(n_tiles / 256)));
}

int32_t his_engine_report(his_engine* E, his_member_report* reports, void* stream) {
    if (!E || !reports) return bad("engine and reports are required");
    cudaStream_t caller = (cudaStream_t)stream;
    HIS_CK(cudaEventRecord(E->ev_in, caller));
    HIS_CK(cudaStreamWaitEvent(E->s0, E->ev_in, 0));
    HIS_CK(cudaMemcpyAsync(E->h_em, E->d_em, sizeof(EngMember) * E->n, cudaMemcpyDeviceToHost, E->s0));
    HIS_CK(cudaStreamSynchronize(E->s0));
    for (int m = 0; m < E->n; ++m) {
        const EngMember& M = E->h_em[m];
        his_member_report& r = reports[m];
        r.t = M.t; r.dt_last = M.dt; r.dt_min = M.dt_min; r.dt_max = M.dt_max; r.rate = M.rate;
        r.steps = M.steps; r.status = M.status; r.n_sub_max = M.n_sub_max; r.n_dt_clamped = M.n_clamped;
        r.outputs = M.n_out > 0 ? M.k_out : 0;
        for (int j = 0; j < 7; ++j) r.acc[j] = M.acc[j];
    }
    return HIS_OK;
}

int32_t his_engine_resume(his_engine* E, const his_member_report* reports, const int32_t* mask, void* stream) {
    if (!E || !reports) return bad("engine and reports are required");
    for (int m = 0; m < E->n; ++m) {
        if (mask && !mask[m]) continue;
        const his_member_report& r = reports[m];
        if (!std::isfinite(r.t) || r.steps < 0 || r.status < ST_RUNNING || r.status > ST_SUBSTEPS)
            return bad("member " + std::to_string(m) + ": report has a bad clock, step count or status");
    }
    cudaStream_t caller = (cudaStream_t)stream;
    HIS_CK(cudaEventRecord(E->ev_in, caller));
    HIS_CK(cudaStreamWaitEvent(E->s0, E->ev_in, 0));
    HIS_CK(cudaMemcpyAsync(E->h_em, E->d_em, sizeof(EngMember) * E->n, cudaMemcpyDeviceToHost, E->s0));
    HIS_CK(cudaStreamSynchronize(E->s0));
    for (int m = 0; m < E->n; ++m) {
        if (mask && !mask[m]) continue;
        const his_member_report& r = reports[m];
        EngMember& M = E->h_em[m];
        M.t = r.t; M.dt = r.dt_last; M.dt_min = r.dt_min; M.dt_max = r.dt_max; M.rate = r.rate;
        M.steps = r.steps; M.status = r.status; M.n_sub_max = r.n_sub_max; M.n_clamped = r.n_dt_clamped;
        if (M.n_out > 0) M.k_out = r.outputs < 1 ? 1 : (r.outputs > M.n_out ? M.n_out : r.outputs);
        for (int j = 0; j < 7; ++j) M.acc[j] = r.acc[j];
    }
    HIS_CK(cudaMemcpyAsync(E->d_em, E->h_em, sizeof(EngMember) * E->n, cudaMemcpyHostToDevice, E->s0));
    HIS_CK(cudaStreamSynchronize(E->s0));
    return HIS_OK;
}

int32_t his_engine_profile(his_engine* E, int32_t n_steps, double* ms, void* stream) {
    if (!E || !ms) return bad("engine and ms are required");
    if (n_steps < 0) return bad("n_steps must be >= 0");
    cudaStream_t caller = (cudaStream_t)stream;
    HIS_CK(cudaEventRecord(E->ev_in, caller));
    HIS_CK(cudaStreamWaitEvent(E->s0, E->ev_in, 0));
    for (int j = 0; j < 6; ++j) ms[j] = 0.0;
    int rc = E->grid->prec == HIS_PREC_F64 ? engine_profile_f64(E, n_steps, ms) : engine_profile_f32(E, n_steps, ms);
    if (rc) return rc;
    HIS_CK(cudaStreamSynchronize(E->s0));
    return HIS_OK;
}

}  // extern "C"
