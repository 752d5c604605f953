// Host-side state behind the opaque handles of his_gb300.h (not part of the ABI).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "his_device.cuh"
#include "net1d_kernels.cuh"

// Pinned staging of host inputs for the asynchronous entry points.  A copy from
// pageable memory may wait for the stream to drain; one from a pinned slot never does.
// Slots rotate, and a slot is refilled only after the copy that last read it has
// finished (its event), which a caller that synchronises once a step never waits on.
struct HostStage {
    static constexpr int SLOTS = 4;
    void* buf[SLOTS] = {};
    cudaEvent_t done[SLOTS] = {};
    size_t bytes = 0;
    int next = 0;
};

struct his_grid {
    int prec = 0;
    his::Consts c{};
    int n = 0, tx = 58, ty = 48, nt = 64, device = 0;   // strip width, rows per chunk, threads per CTA
    std::vector<his_grid_desc> desc;
    std::vector<int> tile0, ntile;
    void* d_grids = nullptr;                 // his::Grid<R>[n]
    his::TileRef* d_tiles = nullptr;
    int n_tiles = 0;
    his::StepParams* d_params = nullptr;
    double* d_partials = nullptr;            // n_tiles x NPART
    double* d_out = nullptr;                 // n x 8
    double* h_out = nullptr;                 // pinned mirror of d_out
    void* d_scratch = nullptr;               // stage buffers of every member
    size_t scratch_bytes = 0;
    size_t table_bytes = 0;
    HostStage params_stage;                  // his_grid_step_async parameters
    // The 2-D stages of a grid step run as n_parts launches over whole members' tiles
    // [part_t[k], part_t[k + 1]), part 0 on the caller's stream and part k >= 1 on
    // ps[k - 1], forked and joined with events, so that the parts fill each other's
    // waves.  Set up on the first step (grid_parts_setup in capi.cu).
    static constexpr int MAX_PARTS = 8;
    int n_parts = 0;                         // 0: not set up yet
    int part_t[MAX_PARTS + 1] = {};
    cudaStream_t ps[MAX_PARTS - 1] = {};
    cudaEvent_t pev_fork = nullptr, pev_join[MAX_PARTS - 1] = {};
    // his_grid_step_ledger_async: the stage launches (all parts, forked and joined)
    // and the finalize as one graph, captured on cap_stream on the first call for a
    // ledger and launched on the caller's stream after the parameter upload
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t ledger_exec = nullptr;
    double* ledger_exec_for = nullptr;      // the ledger ledger_exec adds into
    double* ledger_checked = nullptr;       // the last ledger found to be device memory
    bool ledger_graph_off = false;          // capture failed once: plain launches from then on
};

struct his_net {
    his::Consts c{};
    int n = 0, device = 0;
    std::vector<his::Net> h_nets;
    his::Net* d_nets = nullptr;
    void* d_arena = nullptr;
    size_t arena_bytes = 0;
    double* d_forcing = nullptr;
    int max_sub = 0;
    double* d_out = nullptr;                 // n x 3
    double* h_out = nullptr;
    size_t smem = 0;
    size_t smem_f32 = 0;                     // the float32 substeps (staged geometry)
    HostStage forcing_stage;                 // his_net_step_async forcing
    double* ledger_checked = nullptr;        // the last ledger found to be device memory
};

struct his_links {
    his_grid* grid = nullptr;
    his_net* net = nullptr;
    int n = 0, total_links = 0;
    his::Lnk* d_links = nullptr;
    void* d_arena = nullptr;
    double* d_V = nullptr;
    double* h_V = nullptr;
    double* d_exch = nullptr;                // n x 2 running exchange totals
    size_t smem = 0;
};

struct his_engine {
    his_grid* grid = nullptr;
    his_net* net = nullptr;
    his_links* links = nullptr;
    int n = 0, max_sub = 64, graph_steps = 16;
    his::EngMember* d_em = nullptr;
    his::EngMember* h_em = nullptr;          // pinned
    void* d_arena = nullptr;
    double* d_netf = nullptr;                // n x max_sub x 2 substep forcing
    double* d_vol1d = nullptr;               // n x 3
    size_t pre_smem = 0;
    cudaStream_t s0 = nullptr, s1 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_in = nullptr, ev_out = nullptr;
    cudaGraphExec_t exec = nullptr;
    // The members run as n_chains independent chains (members [chain_m[c], chain_m[c+1]),
    // tiles [chain_t[c], chain_t[c+1])), each with its own streams and graph, so one
    // chain's latency-bound pre/post kernels overlap another's 2-D stages.  Chain 0
    // uses s0/s1, ev_fork/ev_join/ev_out and exec; chain c >= 1 the entries c - 1 of
    // the arrays below.
    static constexpr int MAX_CHAINS = 8;
    int n_chains = 1;
    int chain_m[MAX_CHAINS + 1] = {}, chain_t[MAX_CHAINS + 1] = {};
    cudaStream_t cs_main[MAX_CHAINS - 1] = {}, cs_side[MAX_CHAINS - 1] = {};
    cudaEvent_t cev_fork[MAX_CHAINS - 1] = {}, cev_join[MAX_CHAINS - 1] = {}, cev_out[MAX_CHAINS - 1] = {};
    cudaGraphExec_t cexec[MAX_CHAINS - 1] = {};
    // graphs of rem_steps < graph_steps steps, one per chain, for advances whose step
    // count is not a multiple of graph_steps (0: none captured)
    int rem_steps = 0;
    cudaGraphExec_t rexec[MAX_CHAINS] = {};
    cudaStream_t main_of(int c) const { return c == 0 ? s0 : cs_main[c - 1]; }
    cudaStream_t side_of(int c) const { return c == 0 ? s1 : cs_side[c - 1]; }
    cudaEvent_t fork_of(int c) const { return c == 0 ? ev_fork : cev_fork[c - 1]; }
    cudaEvent_t join_of(int c) const { return c == 0 ? ev_join : cev_join[c - 1]; }
    cudaEvent_t out_of(int c) const { return c == 0 ? ev_out : cev_out[c - 1]; }
    cudaGraphExec_t& exec_of(int c) { return c == 0 ? exec : cexec[c - 1]; }
};

namespace his {

void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// Pinned slot of at least `bytes` whose last copy has finished (nullptr and the
// error set on failure); stage_release records the copy that reads it on `s`.
void* stage_acquire(HostStage& st, size_t bytes, int* slot);
int stage_release(HostStage& st, int slot, cudaStream_t s);
void stage_free(HostStage& st);

#define HIS_CK(call)                                          \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return his::cuda_fail(e_, #call); \
    } while (0)

bool tile_supported(int tx, int ty);
// Threads of a strip CTA for strips of at most tx columns (a 3-column halo each side):
// 64 up to 58 columns, 128 up to 122, 224 up to 218, 352 up to 346; 0 beyond.
inline int strip_threads(int tx) {
    return tx <= 58 ? 64 : tx <= 122 ? 128 : tx <= 218 ? 224 : tx <= 346 ? 352 : 0;
}
int check_cfg(const his_solver_cfg* c);
Consts to_consts(const his_solver_cfg* c);

// Layout of the no-allocation 2-D step's scratch (noalloc.cu): one grid in strips of
// up to 58 columns and chunks of up to 48 rows, every offset a multiple of 256 bytes
// from the scratch base.
struct NoallocPlan {
    int ns, w, nch, hch, n_strips, pad;
    size_t plane;                       // one (ny, nx) plane of the compute type
    size_t o_stage, o_part, o_strips, o_grid, o_params, o_out, total;
};
int noalloc_step_f64(const Consts& c, const his_grid_desc& d, const his_step_params& p, const NoallocPlan& L,
                     unsigned char* base, cudaStream_t s);
int noalloc_step_f32(const Consts& c, const his_grid_desc& d, const his_step_params& p, const NoallocPlan& L,
                     unsigned char* base, cudaStream_t s);

// precision-specific entry points (swe2d_f64.cu / swe2d_f32.cu)
int grid_init_f64(his_grid* g);
int grid_init_f32(his_grid* g);
// ext: optional device-writable copy of the outputs (step: 5 volumes per member;
// reduce: the rate per member), written by the finalize kernel itself; rate_only:
// the CFL rate alone (d_out's volume columns are left as they were)
// ledger: optional device 8 x n float64 ledger the step's volume terms are added into
int grid_step_f64(his_grid* g, cudaStream_t s, double* ext = nullptr, double* ledger = nullptr);
int grid_step_f32(his_grid* g, cudaStream_t s, double* ext = nullptr, double* ledger = nullptr);
int grid_reduce_f64(his_grid* g, cudaStream_t s, double* ext = nullptr, bool rate_only = false);
int grid_reduce_f32(his_grid* g, cudaStream_t s, double* ext = nullptr, bool rate_only = false);
int exchange_f64(his_links* l, const Consts& c, double dt, cudaStream_t s);
int exchange_f32(his_links* l, const Consts& c, double dt, cudaStream_t s);

// n_steps engine steps of chain `chain` on its own streams
int engine_enqueue_f64(his_engine* e, int chain, int n_steps);
int engine_enqueue_f32(his_engine* e, int chain, int n_steps);
int engine_take_rate_f64(his_engine* e);
int engine_take_rate_f32(his_engine* e);
int engine_profile_f64(his_engine* e, int n_steps, double* ms);
int engine_profile_f32(his_engine* e, int n_steps, double* ms);

// net1d.cu
// vols / rate_wet: optional device-writable outputs (3 per member; rate and wet per member)
int net_step_launch(his_net* n, double dt, int n_sub, cudaStream_t s, double* vols = nullptr, double* ledger = nullptr);
int net_reduce_launch(his_net* n, cudaStream_t s, double* rate_wet = nullptr);
int net_engine_launch(his_engine* e, cudaStream_t s, int m0, int count);
int net_engine_prepare(his_engine* e);
// net1d_f32.cu: the float32 network of the production form (float32 engines)
int net_engine_launch_f32(his_engine* e, cudaStream_t s, int m0, int count);
int net_engine_prepare_f32(his_engine* e);

}  // namespace his
