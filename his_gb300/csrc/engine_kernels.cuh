// Device-resident coupled time loop: every member advances with its own dt, chosen,
// forced and accounted for on the GPU, so K steps run as one CUDA graph with no
// host round trip.  The per-member kernels take the first member m0 of the chain
// they serve (block b works on member m0 + b).  One step is
//
//   eng_pre   (one CTA per member)  2-D CFL dt from the rate of the current state,
//             1-D CFL and substep count, weir exchange, forcing at t, t+dt and at the
//             1-D substep starts                          (coupling.py:201-212)
//   stage 1, stage 2 (tiles of every member)              (swe2d.py:305-371)
//   net substeps (one CTA per member, concurrent with the 2-D stages)
//                                                         (coupling.py:216-221)
//   eng_post  (one warp per member)  step volumes summed in tile order into the
//             float64 accumulators, t += dt, plausibility (coupling.py:213-227, :169-192)
#pragma once
#include "net1d_kernels.cuh"
#include "swe2d_strip.cuh"

namespace his {

// threads of the per-member pre-step CTA.  1024 cut the pre kernel of a 400 x 325
// member from 38.6 to 28.7 us, but a CTA that size holds a whole SM's registers while
// it runs, and with member chains side by side the step got slower (0.509 against
// 0.466 ms); threads 32..40 evaluate the step parameters
constexpr int ENG_PRE_THREADS = 512;
static_assert(ENG_PRE_THREADS >= 64 && ENG_PRE_THREADS <= 1024, "pre-step CTA size");

__host__ __device__ inline size_t eng_pre_smem_bytes(size_t exchange_bytes) {
    size_t r = sizeof(double) * 64;
    return exchange_bytes > r ? exchange_bytes : r;
}

template <class R>
__global__ void eng_pre_kernel(EngMember* __restrict__ em, StepParams* __restrict__ params,
                               const Grid<R>* __restrict__ grids, const Net* __restrict__ nets,
                               const Lnk* __restrict__ links, Consts c, double* __restrict__ netf, int max_sub,
                               double* __restrict__ exch, int m0) {
    extern __shared__ double sm[];
    __shared__ int s_go, s_nsub, s_snap;
    __shared__ double s_dt;
    const int m = m0 + blockIdx.x;
    EngMember& E = em[m];
    if (threadIdx.x == 0) {
        s_go = E.status == ST_RUNNING;
        if (!s_go) params[m].active = 0;
        double rate = E.rate;
        double dt = rate > 0.0 ? c.cfl / rate : c.dt_max;
        if (dt < c.dt_min || dt > c.dt_max) {
            if (dt < c.dt_min && s_go) E.n_clamped++;
            dt = fmin(fmax(dt, c.dt_min), c.dt_max);
        }
        // the step ends at the member's end or its next output time (coupling.py:255-262)
        double limit = E.t_end;
        const bool out_on = E.n_out > 0 && E.k_out < E.n_out;
        const double t_next = out_on ? E.out_dt * E.k_out : 0.0;
        if (out_on) limit = fmin(limit, t_next);
        s_dt = fmin(dt, limit - E.t);
        s_snap = out_on && E.t + s_dt >= t_next - 1e-9 ? E.k_out : -1;
        s_nsub = 0;
    }
    __syncthreads();
    if (!s_go) return;
    const double dt = s_dt;
    if (nets) {
        double r1 = 0.0;
        bool wet = false;
        if constexpr (sizeof(R) == 4) net_rate_dev_f32(nets[m], c, r1, wet, sm);
        else net_rate_dev(nets[m], c, r1, wet, sm);
        if (threadIdx.x == 0) {
            const double dt1 = wet ? fmin(c.cfl_1d / r1, c.dt_max) : c.dt_max;
            const double ns = ceil(dt / dt1 - 1e-9);
            s_nsub = ns < 1.0 ? 1 : (ns > (double)max_sub ? max_sub + 1 : (int)ns);
        }
        __syncthreads();
        if (s_nsub > max_sub) {
            if (threadIdx.x == 0) {
                E.status = ST_SUBSTEPS;
                params[m].active = 0;
            }
            return;
        }
        if (links) exchange_dev<R>(links[m], nets[m], grids[m], c, dt, nullptr, exch, m, sm);
        const double sub = dt / s_nsub;
        for (int k = threadIdx.x; k < s_nsub; k += blockDim.x) {
            const double tk = E.t + k * sub;
            netf[((size_t)m * max_sub + k) * 2 + 0] = eng_inflow(E, tk);
            netf[((size_t)m * max_sub + k) * 2 + 1] = eng_tide(E, tk);
        }
    }
    // the step's parameters, spread over threads that each write their own fields, so
    // the float64 forcing (harmonic tides) is evaluated side by side rather than by
    // one thread: threads 32..35 the edge values at t, 36..39 at t + dt, 40 the rain
    // (a warp apart from the substep forcing above), thread 0 the rest
    StepParams& P = params[m];
    const int tid = threadIdx.x;
    if (tid >= 32 && tid < 40) {
        const int e = tid & 3;
        if (tid < 36) {
            const double v = eng_edge(E, e, E.t);
            P.bc0[e] = v;
            P.bc0_f[e] = (float)v;
        } else {
            const double v = eng_edge(E, e, E.t + dt);
            P.bc1[e] = v;
            P.bc1_f[e] = (float)v;
        }
    } else if (tid == 40) {
        const double r = eng_rain(E, E.t);
        P.rain = r;
        P.rain_f = (float)r;
    } else if (tid == 0) {
        P.dt = dt;
        P.t = E.t;
        P.dt_f = (float)dt;
        P.t_f = (float)E.t;
        P.active = 1;
        const int k = s_snap;
        P.snap_k = k;
        P.snap_h = k >= 0 ? E.snap_h + (size_t)k * E.cells : nullptr;
        P.snap_u = k >= 0 ? E.snap_u + (size_t)k * E.cells : nullptr;
        P.snap_v = k >= 0 ? E.snap_v + (size_t)k * E.cells : nullptr;
        P.snap_eta = k >= 0 && E.snap_eta ? E.snap_eta + (size_t)k * E.n1d : nullptr;
        P.snap_q = k >= 0 && E.snap_q ? E.snap_q + (size_t)k * E.n1d : nullptr;
        P.snap_ledger = k >= 0 && E.snap_ledger ? E.snap_ledger + (size_t)k * LEDGER_N : nullptr;
        E.dt = dt;
        E.n_sub = s_nsub;
    }
}

template <class R>
__global__ void eng_post_kernel(EngMember* __restrict__ em, const StepParams* __restrict__ params,
                                const Grid<R>* __restrict__ grids, Consts c, const double* __restrict__ partials,
                                const double* __restrict__ vol1d, double* __restrict__ out, int m0) {
    const int m = m0 + blockIdx.x, lane = threadIdx.x;
    if (!params[m].active) return;
    const Grid<R>& gd = grids[m];
    double s[NPART];
#pragma unroll
    for (int j = 0; j < NPART; ++j) s[j] = 0.0;
    for (int t = lane; t < gd.n_tiles; t += 32) {
        const double* p = partials + (size_t)(gd.tile0 + t) * NPART;
#pragma unroll
        for (int j = 0; j < NPART; ++j) s[j] = (j == P_RATE || j == P_HMAX) ? fmax(s[j], p[j]) : s[j] + p[j];
    }
#pragma unroll
    for (int j = 0; j < NPART; ++j) s[j] = (j == P_RATE || j == P_HMAX) ? warp_max(s[j]) : warp_sum(s[j]);
    if (lane != 0) return;
    EngMember& E = em[m];
    const StepParams& pr = params[m];
    const double dt = (double)R(pr.dt);
    double qin = s[P_XIN1] * gd.dy + s[P_YIN1] * gd.dx;
    double qout = s[P_XOUT1] * gd.dy + s[P_YOUT1] * gd.dx;
    double clip = s[P_CLIP1] * gd.area;
    if (c.order == 2) {
        qin = 0.5 * (qin + (s[P_XIN2] * gd.dy + s[P_YIN2] * gd.dx));
        qout = 0.5 * (qout + (s[P_XOUT2] * gd.dy + s[P_YOUT2] * gd.dx));
        clip = clip + s[P_CLIP2] * gd.area;
    }
    const double rain = gd.rw ? s[P_RAINW] * gd.area
                              : (double)(R(pr.rain) * R(pr.dt)) * ((double)((long long)gd.nx * gd.ny) * gd.area);
    const double infil = s[P_INFIL] * gd.area;
    E.acc[0] += rain;
    E.acc[1] += infil;
    E.acc[2] += qin * dt;
    E.acc[3] += qout * dt;
    E.acc[6] += clip;
    if (vol1d && E.n_sub > 0) {
        E.acc[4] += vol1d[m * 3 + 0];
        E.acc[5] += vol1d[m * 3 + 1];
        E.acc[6] += vol1d[m * 3 + 2];
    }
    E.rate = s[P_RATE];
    E.t = E.t + E.dt;
    if (pr.snap_k >= 0) {
        E.snap_t[pr.snap_k] = E.t;
        E.k_out = pr.snap_k + 1;
        if (double* L = pr.snap_ledger) {        // the 1-D kernel writes L[L_V1D]
            L[L_V2D] = s[P_HSUM] * gd.area;
            L[L_STORE] = s[P_SSUM] * gd.area;
            L[L_RAIN] = E.acc[0]; L[L_INFIL] = E.acc[1]; L[L_BND2_IN] = E.acc[2]; L[L_BND2_OUT] = E.acc[3];
            L[L_BND1_IN] = E.acc[4]; L[L_BND1_OUT] = E.acc[5]; L[L_CLIP] = E.acc[6];
        }
    }
    E.steps += 1;
    E.dt_min = fmin(E.dt_min, E.dt);
    E.dt_max = fmax(E.dt_max, E.dt);
    E.n_sub_max = max(E.n_sub_max, E.n_sub);
    double* o = out + (size_t)m * 8;
    o[0] = qin * dt; o[1] = qout * dt; o[2] = rain; o[3] = infil; o[4] = clip;
    o[5] = s[P_RATE]; o[6] = s[P_HSUM] * gd.area; o[7] = s[P_SSUM] * gd.area;
    if (!isfinite(s[P_HSUM]) || !isfinite(s[P_RATE])) E.status = ST_NONFINITE;
    else if (s[P_HMAX] > MAX_PLAUSIBLE_DEPTH_2D) E.status = ST_IMPLAUSIBLE;
    else if (E.t >= E.t_end - 1e-9) E.status = ST_DONE;
}

// Copy the rate of the current state (finalize output, mode 1) into the engine records.
static __global__ void eng_take_rate_kernel(EngMember* __restrict__ em, const double* __restrict__ out, int n) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < n) em[m].rate = out[(size_t)m * 8 + 5];
}

}  // namespace his
