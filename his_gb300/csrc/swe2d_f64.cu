// Plain method: every 2-D kernel instantiated in float64.  Built with -fmad=false so
// products and sums round separately, as in the reference's float64 torch ops.
#include "swe2d_impl.cuh"

namespace his {
int grid_init_f64(his_grid* g) { return grid_init_impl<double>(g); }
int grid_step_f64(his_grid* g, cudaStream_t s, double* ext, double* ledger) {
    return grid_step_impl<double>(g, s, ext, ledger);
}
int grid_reduce_f64(his_grid* g, cudaStream_t s, double* ext, bool rate_only) {
    return grid_reduce_impl<double>(g, s, ext, rate_only);
}
int exchange_f64(his_links* l, const Consts& c, double dt, cudaStream_t s) { return exchange_impl<double>(l, c, dt, s); }
int engine_enqueue_f64(his_engine* e, int chain, int n) { return engine_enqueue_impl<double>(e, chain, n); }
int engine_take_rate_f64(his_engine* e) { return engine_take_rate_impl<double>(e); }
int engine_profile_f64(his_engine* e, int n, double* ms) { return engine_profile_impl<double>(e, n, ms); }
int noalloc_step_f64(const Consts& c, const his_grid_desc& d, const his_step_params& p, const NoallocPlan& L,
                     unsigned char* base, cudaStream_t s) {
    return noalloc_step_impl<double>(c, d, p, L, base, s);
}
}  // namespace his
