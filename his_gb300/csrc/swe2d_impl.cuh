// Precision-templated host launchers of the 2-D strip kernels, the weir exchange and
// the device-resident engine.  Included once per precision by swe2d_f64.cu and
// swe2d_f32.cu.
#pragma once
#include <algorithm>
#include <vector>

#include "engine_kernels.cuh"
#include "his_internal.h"
#include "net1d_kernels.cuh"
#include "swe2d_strip.cuh"

namespace his {

template <class R, int NT>
int set_strip_attrs() {
    const int bytes = (int)StripGeom<R, NT>::smem_bytes;
    HIS_CK(cudaFuncSetAttribute(strip_kernel<R, NT, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    HIS_CK(cudaFuncSetAttribute(strip_kernel<R, NT, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    HIS_CK(cudaFuncSetAttribute(strip_kernel<R, NT, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    return HIS_OK;
}

// The 2-D stages of one step on stream s (no finalize), over tiles [t0, t0 + count)
// (default: all); a tile's partials sit at its global index.
template <class R, int NT>
int launch_stages(his_grid* g, cudaStream_t s, int t0 = 0, int count = -1) {
    using G = StripGeom<R, NT>;
    if (count < 0) count = g->n_tiles - t0;
    if (count == 0) return HIS_OK;
    auto* grids = reinterpret_cast<const Grid<R>*>(g->d_grids);
    const KC<R> kc = make_kc<R>(g->c);
    auto* strips = reinterpret_cast<const StripRef*>(g->d_tiles) + t0;
    double* part = g->d_partials + (size_t)t0 * NPART;
    if (g->c.order == 2) {
        strip_kernel<R, NT, 1><<<count, NT, G::smem_bytes, s>>>(grids, strips, g->d_params, kc, part);
        strip_kernel<R, NT, 2><<<count, NT, G::smem_bytes, s>>>(grids, strips, g->d_params, kc, part);
    } else {
        strip_kernel<R, NT, 0><<<count, NT, G::smem_bytes, s>>>(grids, strips, g->d_params, kc, part);
        stage_copy_kernel<R, NT><<<count, NT, 0, s>>>(grids, strips, g->d_params);
    }
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

// The stages over all tiles in g->n_parts parts side by side (part 0 on s), joined
// back into s.
template <class R, int NT>
int launch_stages_parted(his_grid* g, cudaStream_t s) {
    const int np = g->n_parts;
    if (np <= 1) return launch_stages<R, NT>(g, s);
    HIS_CK(cudaEventRecord(g->pev_fork, s));
    for (int k = 1; k < np; ++k) {
        HIS_CK(cudaStreamWaitEvent(g->ps[k - 1], g->pev_fork, 0));
        int rc = launch_stages<R, NT>(g, g->ps[k - 1], g->part_t[k], g->part_t[k + 1] - g->part_t[k]);
        if (rc) return rc;
        HIS_CK(cudaEventRecord(g->pev_join[k - 1], g->ps[k - 1]));
    }
    int rc = launch_stages<R, NT>(g, s, g->part_t[0], g->part_t[1] - g->part_t[0]);
    if (rc) return rc;
    for (int k = 1; k < np; ++k) HIS_CK(cudaStreamWaitEvent(s, g->pev_join[k - 1], 0));
    return HIS_OK;
}

template <class R, int NT>
int launch_step_nt(his_grid* g, cudaStream_t s, double* ext, double* ledger) {
    int rc = launch_stages_parted<R, NT>(g, s);
    if (rc) return rc;
    finalize_kernel<R><<<g->n, 32, 0, s>>>(reinterpret_cast<const Grid<R>*>(g->d_grids), g->d_params, g->c,
                                           g->d_partials, g->d_out, 0, ext, ledger);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

template <class R, int NT>
int launch_reduce_nt(his_grid* g, cudaStream_t s, double* ext, bool rate_only) {
    auto* grids = reinterpret_cast<const Grid<R>*>(g->d_grids);
    auto* strips = reinterpret_cast<const StripRef*>(g->d_tiles);
    if (rate_only)
        strip_rate_kernel<R, NT><<<g->n_tiles, NT, 0, s>>>(grids, strips, make_kc<R>(g->c), g->d_partials);
    else
        strip_reduce_kernel<R, NT><<<g->n_tiles, NT, 0, s>>>(grids, strips, make_kc<R>(g->c), g->d_partials);
    finalize_kernel<R><<<g->n, 32, 0, s>>>(grids, g->d_params, g->c, g->d_partials, g->d_out, rate_only ? 2 : 1,
                                           ext);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

#define HIS_NT_DISPATCH(FN, R, g, ...)                           \
    do {                                                         \
        if (g->nt == 64) return FN<R, 64>(g, __VA_ARGS__);       \
        if (g->nt == 128) return FN<R, 128>(g, __VA_ARGS__);     \
        if (g->nt == 224) return FN<R, 224>(g, __VA_ARGS__);     \
        if (g->nt == 352) return FN<R, 352>(g, __VA_ARGS__);     \
        set_error("unsupported strip width (threads per CTA)");  \
        return HIS_ERR_BAD_ARG;                                  \
    } while (0)

// Strip decomposition of every member: columns in ceil(nx / (NT - 6)) strips of equal
// width, rows in chunks of `ty` rows; the work units are listed member by member.
template <class R>
int grid_init_impl(his_grid* g) {
    int rc;
    if ((rc = set_strip_attrs<R, 64>()) != HIS_OK) return rc;
    if ((rc = set_strip_attrs<R, 128>()) != HIS_OK) return rc;
    if ((rc = set_strip_attrs<R, 224>()) != HIS_OK) return rc;
    if ((rc = set_strip_attrs<R, 352>()) != HIS_OK) return rc;
    const int n = g->n;
    std::vector<Grid<R>> H(n);
    std::vector<StripRef> strips;
    g->tile0.assign(n, 0);
    g->ntile.assign(n, 0);
    std::vector<size_t> off(n);
    size_t total = 0;
    for (int m = 0; m < n; ++m) {
        const his_grid_desc& d = g->desc[m];
        size_t plane = ((size_t)d.ny * d.nx * sizeof(R) + 255) & ~size_t(255);
        off[m] = total;
        total += 3 * plane;
    }
    g->scratch_bytes = total;
    HIS_CK(cudaMalloc(&g->d_scratch, total > 0 ? total : 256));
    const int wmax = g->tx;
    for (int m = 0; m < n; ++m) {
        const his_grid_desc& d = g->desc[m];
        Grid<R>& G = H[m];
        G.ny = d.ny;
        G.nx = d.nx;
        for (int e = 0; e < 4; ++e) G.bc[e] = d.bc[e];
        G.dx = d.dx;
        G.dy = d.dy;
        G.area = d.dx * d.dy;
        G.t0 = d.horton_t0;
        G.rdx = R(d.dx);
        G.rdy = R(d.dy);
        G.rt0 = R(d.horton_t0);
        G.idx = R(1.0 / d.dx);
        G.idy = R(1.0 / d.dy);
        const int ns = (d.nx + wmax - 1) / wmax;
        const int w = (d.nx + ns - 1) / ns;
        const int nch = (d.ny + g->ty - 1) / g->ty;
        const int hch = (d.ny + nch - 1) / nch;          // balanced chunk height <= ty
        G.tiles_x = ns;
        G.tiles_y = nch;
        G.n_tiles = ns * nch;
        G.tile0 = (int)strips.size();
        g->tile0[m] = G.tile0;
        g->ntile[m] = G.n_tiles;
        for (int cy = 0; cy < nch; ++cy)
            for (int sx = 0; sx < ns; ++sx) {
                const int x0 = sx * w, y0 = cy * hch;
                strips.push_back(StripRef{m, x0, std::min(w, d.nx - x0), y0, std::min(y0 + hch, d.ny), 0});
            }
        G.h = (R*)d.h; G.hu = (R*)d.hu; G.hv = (R*)d.hv; G.sf = (R*)d.s_filled; G.ic = (R*)d.infil_cum;
        size_t plane = ((size_t)d.ny * d.nx * sizeof(R) + 255) & ~size_t(255);
        char* base = (char*)g->d_scratch + off[m];
        G.h1 = (R*)base; G.hu1 = (R*)(base + plane); G.hv1 = (R*)(base + 2 * plane);
        G.z = (const R*)d.z; G.n = (const R*)d.manning; G.S = (const R*)d.storage;
        G.f0 = (const R*)d.f0; G.fc = (const R*)d.fc; G.k = (const R*)d.k; G.rw = (const R*)d.rain_weight;
        G.pk = (R*)d.peak_h; G.ps = (R*)d.peak_speed;
    }
    g->n_tiles = (int)strips.size();
    HIS_CK(cudaMalloc(&g->d_grids, sizeof(Grid<R>) * n));
    HIS_CK(cudaMemcpy(g->d_grids, H.data(), sizeof(Grid<R>) * n, cudaMemcpyHostToDevice));
    HIS_CK(cudaMalloc(&g->d_tiles, sizeof(StripRef) * strips.size()));
    HIS_CK(cudaMemcpy(g->d_tiles, strips.data(), sizeof(StripRef) * strips.size(), cudaMemcpyHostToDevice));
    HIS_CK(cudaMalloc(&g->d_partials, sizeof(double) * NPART * (size_t)g->n_tiles));
    HIS_CK(cudaMemset(g->d_partials, 0, sizeof(double) * NPART * (size_t)g->n_tiles));
    g->table_bytes = sizeof(Grid<R>) * n + sizeof(StripRef) * strips.size() + sizeof(double) * NPART * g->n_tiles;
    return HIS_OK;
}

template <class R>
int grid_step_impl(his_grid* g, cudaStream_t s, double* ext, double* ledger) {
    HIS_NT_DISPATCH(launch_step_nt, R, g, s, ext, ledger);
}

template <class R>
int grid_reduce_impl(his_grid* g, cudaStream_t s, double* ext, bool rate_only) {
    HIS_NT_DISPATCH(launch_reduce_nt, R, g, s, ext, rate_only);
}

template <class R>
int exchange_impl(his_links* l, const Consts& c, double dt, cudaStream_t s) {
    if (l->smem > 48 * 1024)
        HIS_CK(cudaFuncSetAttribute(exchange_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)l->smem));
    exchange_kernel<R><<<l->n, EXCHANGE_THREADS, l->smem, s>>>(l->d_links, l->net->d_nets,
                                                  reinterpret_cast<const Grid<R>*>(l->grid->d_grids), c, dt, l->d_V,
                                                  l->d_exch);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

// One device-resident step for every member of one chain (see engine_kernels.cuh)
// on the chain's main stream; the 1-D substeps run on its side stream between a
// fork and a join event, concurrently with the 2-D stages.
template <class R, int NT>
int eng_enqueue_nt(his_grid* g, his_engine* E, int chain, int n_steps) {
    auto* grids = reinterpret_cast<const Grid<R>*>(g->d_grids);
    const Net* nets = E->net ? E->net->d_nets : nullptr;
    const Lnk* links = E->links ? E->links->d_links : nullptr;
    double* exch = E->links ? E->links->d_exch : nullptr;
    const int m0 = E->chain_m[chain], mc = E->chain_m[chain + 1] - m0;
    const int t0 = E->chain_t[chain], tc = E->chain_t[chain + 1] - t0;
    cudaStream_t s_main = E->main_of(chain), s_side = E->side_of(chain);
    cudaEvent_t fork = E->fork_of(chain), join = E->join_of(chain);
    if (mc == 0) return HIS_OK;
    for (int k = 0; k < n_steps; ++k) {
        eng_pre_kernel<R><<<mc, ENG_PRE_THREADS, E->pre_smem, s_main>>>(E->d_em, g->d_params, grids, nets, links, g->c,
                                                                        E->d_netf, E->max_sub, exch, m0);
        if (E->net) {
            HIS_CK(cudaEventRecord(fork, s_main));
            HIS_CK(cudaStreamWaitEvent(s_side, fork, 0));
            int rc = net_engine_launch(E, s_side, m0, mc);
            if (rc) return rc;
            HIS_CK(cudaEventRecord(join, s_side));
        }
        int rc = launch_stages<R, NT>(g, s_main, t0, tc);
        if (rc) return rc;
        if (E->net) HIS_CK(cudaStreamWaitEvent(s_main, join, 0));
        eng_post_kernel<R><<<mc, 32, 0, s_main>>>(E->d_em, g->d_params, grids, g->c, g->d_partials,
                                                  E->net ? E->d_vol1d : nullptr, g->d_out, m0);
        HIS_CK(cudaGetLastError());
    }
    return HIS_OK;
}

template <class R>
int engine_enqueue_impl(his_engine* E, int chain, int n_steps) {
    his_grid* g = E->grid;
    HIS_NT_DISPATCH(eng_enqueue_nt, R, g, E, chain, n_steps);
}

template <class R>
int engine_take_rate_impl(his_engine* E) {
    // kernel attributes are set here, outside any stream capture
    if (E->pre_smem > 48 * 1024)
        HIS_CK(cudaFuncSetAttribute(eng_pre_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)E->pre_smem));
    int rc = grid_reduce_impl<R>(E->grid, E->s0, nullptr, false);
    if (rc) return rc;
    eng_take_rate_kernel<<<(E->n + 127) / 128, 128, 0, E->s0>>>(E->d_em, E->grid->d_out, E->n);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

// Same step sequence as eng_enqueue_nt, uncaptured, with CUDA events around each
// kernel class on its own stream; accumulates device milliseconds into ms[6].
template <class R, int NT>
int eng_profile_nt(his_grid* g, his_engine* E, int n_steps, double* ms) {
    using G = StripGeom<R, NT>;
    auto* grids = reinterpret_cast<const Grid<R>*>(g->d_grids);
    const Net* nets = E->net ? E->net->d_nets : nullptr;
    const Lnk* links = E->links ? E->links->d_links : nullptr;
    double* exch = E->links ? E->links->d_exch : nullptr;
    const KC<R> kc = make_kc<R>(g->c);
    auto* strips = reinterpret_cast<const StripRef*>(g->d_tiles);
    cudaEvent_t ev[7];
    for (auto& e : ev) HIS_CK(cudaEventCreate(&e));
    int rc = HIS_OK;
    for (int k = 0; k < n_steps && rc == HIS_OK; ++k) {
        cudaEventRecord(ev[0], E->s0);
        eng_pre_kernel<R><<<E->n, ENG_PRE_THREADS, E->pre_smem, E->s0>>>(E->d_em, g->d_params, grids, nets, links, g->c,
                                                             E->d_netf, E->max_sub, exch, 0);
        cudaEventRecord(ev[1], E->s0);
        if (E->net) {
            cudaStreamWaitEvent(E->s1, ev[1], 0);
            cudaEventRecord(ev[4], E->s1);
            rc = net_engine_launch(E, E->s1, 0, E->n);
            cudaEventRecord(ev[5], E->s1);
        }
        if (g->c.order == 2) {
            strip_kernel<R, NT, 1><<<g->n_tiles, NT, G::smem_bytes, E->s0>>>(grids, strips, g->d_params, kc,
                                                                            g->d_partials);
            cudaEventRecord(ev[2], E->s0);
            strip_kernel<R, NT, 2><<<g->n_tiles, NT, G::smem_bytes, E->s0>>>(grids, strips, g->d_params, kc,
                                                                            g->d_partials);
        } else {
            cudaEventRecord(ev[2], E->s0);
            strip_kernel<R, NT, 0><<<g->n_tiles, NT, G::smem_bytes, E->s0>>>(grids, strips, g->d_params, kc,
                                                                            g->d_partials);
            stage_copy_kernel<R, NT><<<g->n_tiles, NT, 0, E->s0>>>(grids, strips, g->d_params);
        }
        cudaEventRecord(ev[3], E->s0);
        if (E->net) cudaStreamWaitEvent(E->s0, ev[5], 0);
        eng_post_kernel<R><<<E->n, 32, 0, E->s0>>>(E->d_em, g->d_params, grids, g->c, g->d_partials,
                                                   E->net ? E->d_vol1d : nullptr, g->d_out, 0);
        cudaEventRecord(ev[6], E->s0);
        cudaError_t ce = cudaEventSynchronize(ev[6]);
        if (ce != cudaSuccess) { rc = cuda_fail(ce, "his_engine_profile"); break; }
        float t;
        cudaEventElapsedTime(&t, ev[0], ev[1]); ms[0] += t;
        cudaEventElapsedTime(&t, ev[1], ev[2]); ms[1] += t;
        cudaEventElapsedTime(&t, ev[2], ev[3]); ms[2] += t;
        if (E->net) { cudaEventElapsedTime(&t, ev[4], ev[5]); ms[3] += t; }
        cudaEventElapsedTime(&t, ev[3], ev[6]); ms[4] += t;
        cudaEventElapsedTime(&t, ev[0], ev[6]); ms[5] += t;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (rc == HIS_OK) HIS_CK(cudaGetLastError());
    return rc;
}

template <class R>
int engine_profile_impl(his_engine* E, int n_steps, double* ms) {
    his_grid* g = E->grid;
    HIS_NT_DISPATCH(eng_profile_nt, R, g, E, n_steps, ms);
}

// ---------------------------------------------------------------- no-allocation step
// Writes the grid record, the step parameters and the strip table of one grid into
// the caller's scratch and clears its partial sums and totals.  The records arrive
// as kernel arguments, so no host buffer has to outlive the call.
template <class R>
__global__ void noalloc_setup_kernel(Grid<R> G, StepParams P, NoallocPlan L, unsigned char* __restrict__ base) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    auto* strips = reinterpret_cast<StripRef*>(base + L.o_strips);
    auto* part = reinterpret_cast<double*>(base + L.o_part);
    for (int b = i; b < L.n_strips; b += stride) {
        const int sx = b % L.ns, cy = b / L.ns;
        const int x0 = sx * L.w, y0 = cy * L.hch;
        strips[b] = StripRef{0, x0, min(L.w, G.nx - x0), y0, min(y0 + L.hch, G.ny), 0};
    }
    for (int j = i; j < NPART * L.n_strips; j += stride) part[j] = 0.0;
    if (i < 8) reinterpret_cast<double*>(base + L.o_out)[i] = 0.0;
    if (i == 0) {
        *reinterpret_cast<Grid<R>*>(base + L.o_grid) = G;
        *reinterpret_cast<StepParams*>(base + L.o_params) = P;
    }
}

// One step of one grid with every table and stage buffer in the scratch at `base`
// (laid out by L): the same strip kernels, decomposition (58-column strips, 48-row
// chunks) and fixed-order totals as a one-member set created with default tiles.
template <class R>
int noalloc_step_impl(const Consts& c, const his_grid_desc& d, const his_step_params& p, const NoallocPlan& L,
                      unsigned char* base, cudaStream_t s) {
    constexpr int NT = 64;
    static_assert(sizeof(Grid<R>) <= 256 && sizeof(StepParams) <= 256, "records exceed their scratch slots");
    int rc = set_strip_attrs<R, NT>();
    if (rc) return rc;
    Grid<R> G{};
    G.ny = d.ny;
    G.nx = d.nx;
    for (int e = 0; e < 4; ++e) G.bc[e] = d.bc[e];
    G.dx = d.dx;
    G.dy = d.dy;
    G.area = d.dx * d.dy;
    G.t0 = d.horton_t0;
    G.rdx = R(d.dx);
    G.rdy = R(d.dy);
    G.rt0 = R(d.horton_t0);
    G.idx = R(1.0 / d.dx);
    G.idy = R(1.0 / d.dy);
    G.tile0 = 0;
    G.tiles_x = L.ns;
    G.tiles_y = L.nch;
    G.n_tiles = L.n_strips;
    G.h = (R*)d.h; G.hu = (R*)d.hu; G.hv = (R*)d.hv; G.sf = (R*)d.s_filled; G.ic = (R*)d.infil_cum;
    unsigned char* st = base + L.o_stage;
    G.h1 = (R*)st; G.hu1 = (R*)(st + L.plane); G.hv1 = (R*)(st + 2 * L.plane);
    G.z = (const R*)d.z; G.n = (const R*)d.manning; G.S = (const R*)d.storage;
    G.f0 = (const R*)d.f0; G.fc = (const R*)d.fc; G.k = (const R*)d.k; G.rw = (const R*)d.rain_weight;
    G.pk = (R*)d.peak_h; G.ps = (R*)d.peak_speed;
    const StepParams P = step_params_from(p);
    const int work = std::max(L.n_strips * (int)NPART, 8);
    noalloc_setup_kernel<R><<<(work + 255) / 256, 256, 0, s>>>(G, P, L, base);
    auto* grid = reinterpret_cast<const Grid<R>*>(base + L.o_grid);
    auto* params = reinterpret_cast<const StepParams*>(base + L.o_params);
    auto* strips = reinterpret_cast<const StripRef*>(base + L.o_strips);
    auto* part = reinterpret_cast<double*>(base + L.o_part);
    auto* out = reinterpret_cast<double*>(base + L.o_out);
    const KC<R> kc = make_kc<R>(c);
    const size_t smem = StripGeom<R, NT>::smem_bytes;
    if (c.order == 2) {
        strip_kernel<R, NT, 1><<<L.n_strips, NT, smem, s>>>(grid, strips, params, kc, part);
        strip_kernel<R, NT, 2><<<L.n_strips, NT, smem, s>>>(grid, strips, params, kc, part);
    } else {
        strip_kernel<R, NT, 0><<<L.n_strips, NT, smem, s>>>(grid, strips, params, kc, part);
        stage_copy_kernel<R, NT><<<L.n_strips, NT, 0, s>>>(grid, strips, params);
    }
    finalize_kernel<R><<<1, 32, 0, s>>>(grid, params, c, part, out, 0, nullptr);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

}  // namespace his
