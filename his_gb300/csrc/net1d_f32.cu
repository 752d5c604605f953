// Launcher of the float32 network substeps of the production form (float32 engines),
// built with fused multiply-add and fast float32 intrinsics like the float32 2-D
// kernels.  The float64 network (net1d.cu) serves float64 engines and the drop-in
// SWE1D.
#include "his_internal.h"
#include "net1d_kernels.cuh"

namespace his {

__global__ void net_engine_kernel_f32(const Net* __restrict__ nets, Consts c, const EngMember* __restrict__ em,
                                      const StepParams* __restrict__ params, const double* __restrict__ netf,
                                      int max_sub, double* __restrict__ vol1d, int m0) {
    extern __shared__ double sm[];
    const int m = m0 + blockIdx.x;
    if (!params[m].active) return;
    const EngMember& E = em[m];
    const StepParams& P = params[m];
    net_substeps_f32_dev(nets[m], c, E.dt, E.n_sub, netf + (size_t)m * max_sub * 2, vol1d + m * 3, sm, P.snap_eta,
                         P.snap_q, P.snap_ledger ? P.snap_ledger + L_V1D : nullptr);
}

int net_engine_prepare_f32(his_engine* e) {
    if (e->net && e->net->smem_f32 > 48 * 1024)
        HIS_CK(cudaFuncSetAttribute(net_engine_kernel_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)e->net->smem_f32));
    return HIS_OK;
}

int net_engine_launch_f32(his_engine* e, cudaStream_t s, int m0, int count) {
    his_net* n = e->net;
    net_engine_kernel_f32<<<count, 128, n->smem_f32, s>>>(n->d_nets, n->c, e->d_em, e->grid->d_params, e->d_netf,
                                                      e->max_sub, e->d_vol1d, m0);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

}  // namespace his
