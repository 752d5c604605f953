// Production form: 2-D state, fluxes and updates in float32 (float64 volume sums and
// exchange volumes).  Built with fused multiply-add enabled.
#include "swe2d_impl.cuh"

namespace his {
int grid_init_f32(his_grid* g) { return grid_init_impl<float>(g); }
int grid_step_f32(his_grid* g, cudaStream_t s, double* ext, double* ledger) {
    return grid_step_impl<float>(g, s, ext, ledger);
}
int grid_reduce_f32(his_grid* g, cudaStream_t s, double* ext, bool rate_only) {
    return grid_reduce_impl<float>(g, s, ext, rate_only);
}
int exchange_f32(his_links* l, const Consts& c, double dt, cudaStream_t s) { return exchange_impl<float>(l, c, dt, s); }
int engine_enqueue_f32(his_engine* e, int chain, int n) { return engine_enqueue_impl<float>(e, chain, n); }
int engine_take_rate_f32(his_engine* e) { return engine_take_rate_impl<float>(e); }
int engine_profile_f32(his_engine* e, int n, double* ms) { return engine_profile_impl<float>(e, n, ms); }
int noalloc_step_f32(const Consts& c, const his_grid_desc& d, const his_step_params& p, const NoallocPlan& L,
                     unsigned char* base, cudaStream_t s) {
    return noalloc_step_impl<float>(c, d, p, L, base, s);
}
}  // namespace his
