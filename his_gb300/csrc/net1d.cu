// Launchers of the 1-D network kernels (float64, built with -fmad=false); float32
// engines run the production form's network (net1d_f32.cu).
#include "his_internal.h"
#include "net1d_kernels.cuh"

namespace his {

// n_sub substeps of dt/n_sub each for every member; forcing: per member, per
// substep (inflow, stage); vols: 3 per member.
// ledger (optional): 8 x members float64 ledger; the substeps' boundary volumes and
// clip are added into its 1-D rows.
__global__ void net_step_kernel(const Net* __restrict__ nets, Consts c, double dt_total, int n_sub,
                                const double* __restrict__ forcing, double* __restrict__ vols,
                                double* __restrict__ ledger) {
    extern __shared__ double sm[];
    __shared__ double v[3];
    net_substeps_dev(nets[blockIdx.x], c, dt_total, n_sub, forcing + (size_t)blockIdx.x * n_sub * 2,
                     (vols || ledger) ? v : nullptr, sm);
    if (threadIdx.x == 0) {
        if (vols)
            for (int j = 0; j < 3; ++j) vols[blockIdx.x * 3 + j] = v[j];
        if (ledger) {
            const size_t B = gridDim.x;
            ledger[LG_BND1_IN * B + blockIdx.x] += v[0];
            ledger[LG_BND1_OUT * B + blockIdx.x] += v[1];
            ledger[LG_CLIP1 * B + blockIdx.x] += v[2];
        }
    }
}

// 1-D CFL rate over wet interior cells, the any-wet flag and the channel volume.
// out: 3 per member (rate, any_wet, volume).
__global__ void net_reduce_kernel(const Net* __restrict__ nets, Consts c, double* __restrict__ out,
                                  double* __restrict__ rate_wet) {
    __shared__ double red[32 * 3];
    const Net& N = nets[blockIdx.x];
    const Sec s{N.b, N.m, N.yb, N.ts};
    double rate = 0.0, wet_any = 0.0, vol = 0.0;
    for (int i = threadIdx.x; i < N.n_cells; i += blockDim.x) {
        if (N.kind[i] > 1) continue;
        const double A = N.A[i];
        vol += A * N.dx[i];
        const double y = sec_depth(s, i, A);
        if (!(y > c.h_dry)) continue;
        wet_any = 1.0;
        const double cc = sqrt(c.g * A / sec_top(s, i, y));
        const double u = vel1d(c, s, i, A, N.Q[i]);
        rate = fmax(rate, (fabs(u) + cc) / N.dx[i]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    rate = warp_max(rate);
    wet_any = warp_max(wet_any);
    vol = warp_sum(vol);
    if (lane == 0) { red[warp * 3] = rate; red[warp * 3 + 1] = wet_any; red[warp * 3 + 2] = vol; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = red[0], w = red[1], v = red[2];
        for (int k = 1; k < nw; ++k) { r = fmax(r, red[k * 3]); w = fmax(w, red[k * 3 + 1]); v += red[k * 3 + 2]; }
        out[blockIdx.x * 3 + 0] = r;
        out[blockIdx.x * 3 + 1] = w;
        out[blockIdx.x * 3 + 2] = v;
        if (rate_wet) {
            rate_wet[blockIdx.x * 2 + 0] = r;
            rate_wet[blockIdx.x * 2 + 1] = w;
        }
    }
}

// Engine form: each member's dt, substep count and substep forcing come from the
// device (written by the engine's pre kernel); members not stepping are skipped.
__global__ void net_engine_kernel(const Net* __restrict__ nets, Consts c, const EngMember* __restrict__ em,
                                  const StepParams* __restrict__ params, const double* __restrict__ netf, int max_sub,
                                  double* __restrict__ vol1d, int m0) {
    extern __shared__ double sm[];
    const int m = m0 + blockIdx.x;
    if (!params[m].active) return;
    const EngMember& E = em[m];
    const StepParams& P = params[m];
    net_substeps_dev(nets[m], c, E.dt, E.n_sub, netf + (size_t)m * max_sub * 2, vol1d + m * 3, sm, P.snap_eta,
                     P.snap_q, P.snap_ledger ? P.snap_ledger + L_V1D : nullptr);
}

int net_engine_prepare(his_engine* e) {
    if (e->grid->prec == HIS_PREC_F32) return net_engine_prepare_f32(e);
    if (e->net && e->net->smem > 48 * 1024)
        HIS_CK(cudaFuncSetAttribute(net_engine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)e->net->smem));
    return HIS_OK;
}

int net_engine_launch(his_engine* e, cudaStream_t s, int m0, int count) {
    if (e->grid->prec == HIS_PREC_F32) return net_engine_launch_f32(e, s, m0, count);
    his_net* n = e->net;
    net_engine_kernel<<<count, 128, n->smem, s>>>(n->d_nets, n->c, e->d_em, e->grid->d_params, e->d_netf, e->max_sub,
                                                  e->d_vol1d, m0);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

int net_step_launch(his_net* n, double dt, int n_sub, cudaStream_t s, double* vols, double* ledger) {
    if (n->smem > 48 * 1024)
        HIS_CK(cudaFuncSetAttribute(net_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)n->smem));
    net_step_kernel<<<n->n, 128, n->smem, s>>>(n->d_nets, n->c, dt, n_sub, n->d_forcing,
                                               vols ? vols : (ledger ? nullptr : n->d_out), ledger);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

int net_reduce_launch(his_net* n, cudaStream_t s, double* rate_wet) {
    net_reduce_kernel<<<n->n, 128, 0, s>>>(n->d_nets, n->c, n->d_out, rate_wet);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

}  // namespace his
