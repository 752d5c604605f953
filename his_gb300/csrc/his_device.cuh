// Device-side building blocks of the flood-engine step: constants, member and
// tile descriptors, ghost cells, MUSCL/hydrostatic reconstruction, HLLC/HLL flux,
// Kurganov-Petrova velocities and block reductions.
//
// Everything is templated on the storage/arithmetic type R (double for the plain
// method, float for the production form).  The float64 translation unit is built
// with -fmad=false so its arithmetic rounds after every operation, like the
// reference solver's float64 torch ops (hydrointel/solver/swe2d.py).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/his_gb300.h"

namespace his {

enum : int { BC_CLOSED = 0, BC_TRANSMISSIVE = 1, BC_STAGE = 2, BC_DISCHARGE = 3 };
enum : int { EDGE_W = 0, EDGE_E = 1, EDGE_S = 2, EDGE_N = 3 };

// Per-tile partial sums written by the stage kernels (one slot per tile, summed in
// tile order by the finalize kernel: deterministic and independent of the batch).
enum : int {
    P_CLIP1 = 0, P_XIN1, P_XOUT1, P_YIN1, P_YOUT1,
    P_CLIP2, P_XIN2, P_XOUT2, P_YIN2, P_YOUT2,
    P_INFIL, P_RAINW, P_RATE, P_HSUM, P_SSUM, P_HMAX,
    NPART
};

// Rows of the coupled step's float64 volume ledger (8 x members, row-major), in the
// reference's term order with the clip of each model in its own row, so that the 2-D
// and 1-D kernels of a step, which run on two streams, never add to the same element
enum : int { LG_RAIN = 0, LG_INFIL, LG_BND2_IN, LG_BND2_OUT, LG_BND1_IN, LG_BND1_OUT, LG_CLIP2, LG_CLIP1, LEDGER_ROWS };

// Member status in the device-resident engine
enum : int { ST_RUNNING = 0, ST_DONE = 1, ST_NONFINITE = 2, ST_IMPLAUSIBLE = 3, ST_SUBSTEPS = 4 };
constexpr double MAX_PLAUSIBLE_DEPTH_2D = 10.0;   // coupling.py:39

// One member of the device-resident engine: its forcing tables and its evolving
// clock, step statistics and float64 volume accumulators, in the reference's term
// order (rain, infiltration, bnd2d_in, bnd2d_out, bnd1d_in, bnd1d_out, clip).
struct EngMember {
    double rain_t0, rain_step;
    const double* rain;          // m/s per block
    int rain_n, tide_on, tide_n, q_n;
    double tide_base, tide_shift;
    double amp[4], w[4], ph[4];
    double q_t0, q_step;
    const double* q;             // inflow hydrograph, m^3/s
    int edge_src[4];             // 0 constant, 1 tide(t), 2 inflow(t) x edge_val
    double edge_val[4];
    double t_end;
    double t, dt, dt_min, dt_max, rate;
    long long steps;
    int status, n_sub, n_sub_max, n_clamped;
    double acc[7];
    // output times k * out_dt, k = 1 .. n_out - 1 (k = 0, the initial state, is written
    // by the host); k_out is the next one.  Snapshot slots: 2-D depth and KP velocities
    // (n_out x cells), 1-D level and discharge (n_out x n1d), and the times reached.
    double out_dt;
    int n_out, k_out, cells, n1d;
    float *snap_h, *snap_u, *snap_v, *snap_eta, *snap_q;
    double *snap_t, *snap_ledger;    // ledger: LEDGER_N values per output (below)
};

// Volume ledger at an output time, in the order of the reference's snapshot ledger
// (coupling.py:229-242): 2-D surface, 1-D channel and retained volume, then the
// accumulated source terms.
enum : int { L_V2D = 0, L_V1D, L_STORE, L_RAIN, L_INFIL, L_BND2_IN, L_BND2_OUT, L_BND1_IN, L_BND1_OUT, L_CLIP,
             LEDGER_N };

// Piecewise-constant rain, harmonic tide and linearly interpolated inflow, as the
// reference evaluates them (engine.py:145-166, hyetograph.py:42-46, tide.py:29-31,
// catchment.py:32-40).
__device__ __forceinline__ double eng_rain(const EngMember& E, double t) {
    if (E.rain_n <= 0) return 0.0;
    const double k = floor((t - E.rain_t0) / E.rain_step + 1e-9);
    if (k < 0.0 || k >= (double)E.rain_n) return 0.0;
    return E.rain[(int)k];
}
__device__ __forceinline__ double eng_tide(const EngMember& E, double t) {
    const double tt = t + E.tide_shift;
    double eta = 0.0;
    for (int j = 0; j < E.tide_n; ++j) eta = eta + E.amp[j] * cos(E.w[j] * tt - E.ph[j]);
    return E.tide_base + (E.tide_on ? eta : 0.0);
}
__device__ __forceinline__ double eng_inflow(const EngMember& E, double t) {
    if (E.q_n <= 0) return 0.0;
    const double x = (t - E.q_t0) / E.q_step;
    if (x <= 0.0) return E.q[0];
    if (x >= (double)(E.q_n - 1)) return E.q[E.q_n - 1];
    const int k = (int)x;
    const double w = x - k;
    return (1.0 - w) * E.q[k] + w * E.q[k + 1];
}
__device__ __forceinline__ double eng_edge(const EngMember& E, int e, double t) {
    if (E.edge_src[e] == 1) return eng_tide(E, t);
    if (E.edge_src[e] == 2) return eng_inflow(E, t) * E.edge_val[e];
    return E.edge_val[e];
}

struct Consts {
    double g, h_dry, kp_eps, cfl, dt_min, dt_max;
    double cfl_1d, slot_width_frac, weir_cw, exchange_limit, exchange_relax;
    int order, hllc;
};

template <class R>
struct Grid {
    int ny, nx;
    int bc[4];
    double dx, dy, area, t0;
    int tile0, tiles_x, tiles_y, n_tiles;
    R *h, *hu, *hv, *sf, *ic;        // state: depth, momenta, retained water, infiltrated depth
    R *h1, *hu1, *hv1;               // stage-1 state (library scratch)
    const R *z, *n, *S, *f0, *fc, *k, *rw;
    R *pk, *ps;                      // optional running peak depth and speed
    R rdx, rdy, rt0;                 // dx, dy, Horton t0 in the compute type
    R idx, idy;                      // 1/dx, 1/dy (the float32 kernels multiply instead of dividing)
};

// Per-member step parameters, in float64 and (for the float32 kernels, which must not
// convert on GB300's slow FP64 pipe) as float32 copies written by the same producer.
struct StepParams {
    double dt, t, rain;
    double bc0[4], bc1[4];
    int active, snap_k;              // snap_k: output slot written by this step, or -1
    float dt_f, t_f, rain_f, pad_f;
    float bc0_f[4], bc1_f[4];
    // this step's snapshot slots (NULL: no output at the end of this step)
    float *snap_h, *snap_u, *snap_v, *snap_eta, *snap_q;
    double* snap_ledger;
};

__host__ __device__ inline void params_set_f32(StepParams& p) {
    p.dt_f = (float)p.dt;
    p.t_f = (float)p.t;
    p.rain_f = (float)p.rain;
    for (int e = 0; e < 4; ++e) {
        p.bc0_f[e] = (float)p.bc0[e];
        p.bc1_f[e] = (float)p.bc1[e];
    }
}

// The step record of one member from the ABI's step parameters: every field set
// (snapshot slot -1 and no snapshot pointers: no output at the end of this step), the
// float32 copies formed here.  Every producer of records on the host uses it.
inline StepParams step_params_from(const his_step_params& q) {
    StepParams sp{};
    sp.snap_k = -1;
    sp.dt = q.dt;
    sp.t = q.t;
    sp.rain = q.rain;
    for (int e = 0; e < 4; ++e) {
        sp.bc0[e] = q.bc_t[e];
        sp.bc1[e] = q.bc_t_dt[e];
    }
    sp.active = 1;
    params_set_f32(sp);
    return sp;
}

struct TileRef {
    int member, x0, y0, local;
};

// The solver constants in the compute type R, converted on the host and passed by
// value: converting float64 constants inside the kernels put the float32 kernels on
// GB300's FP64 pipe (a small fraction of the float32 rate).
template <class R>
struct KC {
    R g, hg, nhg, h_dry, kp_eps;
    int order, hllc;
};

template <class R>
inline KC<R> make_kc(const Consts& c) {
    KC<R> k;
    k.g = R(c.g);
    k.hg = R(0.5 * c.g);
    k.nhg = R(-0.5 * c.g);
    k.h_dry = R(c.h_dry);
    k.kp_eps = R(c.kp_eps);
    k.order = c.order;
    k.hllc = c.hllc;
    return k;
}

// Step parameters in the compute type (no conversion in the float32 kernels)
template <class R> __device__ __forceinline__ R par_dt(const StepParams& p);
template <> __device__ __forceinline__ double par_dt<double>(const StepParams& p) { return p.dt; }
template <> __device__ __forceinline__ float par_dt<float>(const StepParams& p) { return p.dt_f; }
template <class R> __device__ __forceinline__ R par_t(const StepParams& p);
template <> __device__ __forceinline__ double par_t<double>(const StepParams& p) { return p.t; }
template <> __device__ __forceinline__ float par_t<float>(const StepParams& p) { return p.t_f; }
template <class R> __device__ __forceinline__ R par_rain(const StepParams& p);
template <> __device__ __forceinline__ double par_rain<double>(const StepParams& p) { return p.rain; }
template <> __device__ __forceinline__ float par_rain<float>(const StepParams& p) { return p.rain_f; }
template <class R> __device__ __forceinline__ R par_bc(const StepParams& p, int stage2, int e);
template <> __device__ __forceinline__ double par_bc<double>(const StepParams& p, int stage2, int e) {
    return stage2 ? p.bc1[e] : p.bc0[e];
}
template <> __device__ __forceinline__ float par_bc<float>(const StepParams& p, int stage2, int e) {
    return stage2 ? p.bc1_f[e] : p.bc0_f[e];
}

// ------------------------------------------------------------------ scalar helpers
// float64: the selections of the reference's torch.maximum/minimum/clamp on finite
// values, spelled out; float32: the native min/max instructions.
template <class R> __device__ __forceinline__ R rmax(R a, R b) {
    if constexpr (sizeof(R) == 4) return fmaxf(a, b);
    else return a > b ? a : (b > a ? b : a);
}
template <class R> __device__ __forceinline__ R rmin(R a, R b) {
    if constexpr (sizeof(R) == 4) return fminf(a, b);
    else return a < b ? a : (b < a ? b : a);
}
template <class R> __device__ __forceinline__ R relu(R x) {
    if constexpr (sizeof(R) == 4) return fmaxf(x, 0.0f);
    else return x > R(0) ? x : R(0);
}
template <class R> __device__ __forceinline__ R clamp0(R x) {
    if constexpr (sizeof(R) == 4) return fmaxf(x, 0.0f);
    else return x < R(0) ? R(0) : x;
}
// x / d for a cell spacing d: float64 divides as the reference does; float32
// multiplies by the reciprocal formed once on the host.
template <class R> __device__ __forceinline__ R per_len(R x, R d, R inv_d) {
    if constexpr (sizeof(R) == 4) return x * inv_d;
    else return x / d;
}

__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }

// h**4 as the reference computes it (a power call), in each precision.
__device__ __forceinline__ double pow4(double h) { return pow(h, 4.0); }
__device__ __forceinline__ float pow4(float h) { float h2 = h * h; return h2 * h2; }
// hf**(4/3)
__device__ __forceinline__ double pow43(double x) { return pow(x, 4.0 / 3.0); }
__device__ __forceinline__ float pow43(float x) { return powf(x, 4.0f / 3.0f); }
__device__ __forceinline__ double rexp(double x) { return exp(x); }
__device__ __forceinline__ float rexp(float x) { return expf(x); }
__device__ __forceinline__ double cbrt_pow(double x) { return pow(x, 1.0 / 3.0); }
__device__ __forceinline__ float cbrt_pow(float x) { return powf(x, 1.0f / 3.0f); }

// Kurganov-Petrova desingularised velocity (swe2d.py:161-167)
template <class R>
__device__ __forceinline__ void kp_velocity(const KC<R>& c, R h, R hu, R hv, R& u, R& v) {
    const R SQRT2 = R(1.4142135623730951);
    if constexpr (sizeof(R) == 4) {
        const float h2 = h * h, h4 = h2 * h2;
        const float s = SQRT2 * h * rsqrtf(h4 + fmaxf(h4, c.kp_eps));
        const bool wet = h >= c.h_dry;
        u = wet ? hu * s : 0.0f;
        v = wet ? hv * s : 0.0f;
        return;
    }
    R h4 = pow4(h);
    R den = dsqrt(h4 + rmax(h4, c.kp_eps));
    if (h >= c.h_dry) {
        u = SQRT2 * h * hu / den;
        v = SQRT2 * h * hv / den;
    } else {
        u = R(0);
        v = R(0);
    }
}

// Ghost states of stage and discharge edges from the adjacent interior cell
// (boundaries.py:63-78).  un is that cell's outward-normal velocity; the ghost's
// depth, outward-normal and tangential velocity are returned (its bed is the cell's).
template <class R>
__device__ __forceinline__ void stage_ghost(const KC<R>& c, R val, R h, R un, R ut, R z, R& hg_o, R& un_o, R& ut_o) {
    const R g = c.g, hd = c.h_dry;
    R hg = clamp0(val - z);
    R ci = dsqrt(g * h), cg = dsqrt(g * hg);
    bool wet_i = h >= hd;
    R ung = wet_i ? un + R(2) * (ci - cg) : R(0);
    bool sup = wet_i && (un > ci);
    if (sup) { ung = un; hg = h; }
    if (!(hg >= hd)) ung = R(0);
    hg_o = hg;
    un_o = ung;
    ut_o = ung > R(0) ? ut : R(0);
}

template <class R>
__device__ __forceinline__ void discharge_ghost(const KC<R>& c, R val, R h, R& hg_o, R& un_o, R& ut_o) {
    const R g = c.g, hd = c.h_dry;
    R hc = rmax(cbrt_pow(val * val / g), hd);
    R hg = h >= hd ? h : hc;
    hg_o = hg;
    un_o = -val / hg;
    ut_o = R(0);
}

template <class R>
__device__ __forceinline__ R minmod(R a, R b) {
    // float32: the median of (a, b, 0) from four min/max (for finite a, b: the smaller
    // magnitude with the common sign, zero when the signs differ)
    if constexpr (sizeof(R) == 4) return fmaxf(fminf(a, b), fminf(fmaxf(a, b), 0.0f));
    if (a * b > R(0)) {
        R m = rmin(fabs(a), fabs(b));
        return a > R(0) ? m : -m;
    }
    return R(0);
}

// MUSCL face states of one cell along one axis (swe2d.py:205-219).  Inputs are the
// cell and its two neighbours along the axis; outputs the minus (left face) and
// plus (right face) reconstructions of h, normal and tangential velocity, and the
// recovered bed z = eta - h.
//
// float64 (plain method): the reference's own formulation, eta = h + z formed per
// cell and the bed recovered as Zm = Em - Hm, Zp = Ep - Hp.
// float32 (production form): the same reconstruction in difference form.  The
// surface-elevation differences are dE = dh + dz (never forming eta = h + z, whose
// float32 rounding would be ulp(z) ~ 1e-6 m at tens of metres of terrain) and the
// reconstructed bed enters only through the in-cell bed slope d = sE - sH
// (Zp - Zm = d, Zm = z - d/2, Zp = z + d/2), so the hydrostatic reconstruction
// and the bed source keep their exact cancellation at rest.
template <class R>
struct Recon {
    R Hm, Hp, Um, Up, Vm, Vp, Zm, Zp;   // Zm/Zp: float64 path
    R z, d, h0, sE;                     // float32 path: cell bed, in-cell bed slope, depth, eta slope
};

template <class R>
__device__ __forceinline__ Recon<R> reconstruct(const KC<R>& c, R hm, R h0, R hp, R um, R u0, R up, R vm, R v0, R vp,
                                                R zm, R z0, R zp) {
    Recon<R> r;
    r.z = z0;
    r.h0 = h0;
    r.sE = R(0);
    if (c.order == 2) {
        R hmin = rmin(rmin(hm, h0), hp);
        R ok = (hmin >= c.h_dry) ? R(1) : R(0);
        R sH = minmod(h0 - hm, hp - h0) * ok;
        R sU = minmod(u0 - um, up - u0) * ok;
        R sV = minmod(v0 - vm, vp - v0) * ok;
        r.Hm = h0 - R(0.5) * sH;
        r.Hp = h0 + R(0.5) * sH;
        r.Um = u0 - R(0.5) * sU;
        r.Up = u0 + R(0.5) * sU;
        r.Vm = v0 - R(0.5) * sV;
        r.Vp = v0 + R(0.5) * sV;
        if constexpr (sizeof(R) == 8) {
            R em = hm + zm, e0 = h0 + z0, ep = hp + zp;
            R sE = minmod(e0 - em, ep - e0) * ok;
            R Em = e0 - R(0.5) * sE, Ep = e0 + R(0.5) * sE;
            r.Zm = Em - r.Hm;
            r.Zp = Ep - r.Hp;
            r.d = R(0);
        } else {
            R sE = minmod((h0 - hm) + (z0 - zm), (hp - h0) + (zp - z0)) * ok;
            r.d = sE - sH;
            r.sE = sE;
            r.Zm = r.Zp = R(0);
        }
    } else {
        r.Hm = r.Hp = h0;
        r.Um = r.Up = u0;
        r.Vm = r.Vp = v0;
        r.Zm = r.Zp = z0;
        r.d = R(0);
    }
    return r;
}

// HLLC / HLL flux with two-rarefaction wave speeds and dry-bed fixes (swe2d.py:61-101)
template <class R>
__device__ __forceinline__ void riemann(const KC<R>& c, R hL, R uL, R vL, R hR, R uR, R vR, R& F1o, R& F2o,
                                        R& F3o) {
    const R g = c.g, tiny = R(1e-14);
    R cL = dsqrt(g * hL), cR = dsqrt(g * hR);
    bool dryL = hL <= tiny, dryR = hR <= tiny;
    R u_s = R(0.5) * (uL + uR) + cL - cR;
    R c_s = R(0.5) * (cL + cR) + R(0.25) * (uL - uR);
    R SL = rmin(uL - cL, u_s - c_s);
    R SR = rmax(uR + cR, u_s + c_s);
    if (dryL) { SL = uR - R(2) * cR; SR = uR + cR; }
    if (dryR) { SL = uL - cL; SR = uL + R(2) * cL; }
    const R hg = c.hg;
    R qL = hL * uL, qR = hR * uR;
    R FL1 = qL, FR1 = qR;
    R FL2 = qL * uL + hg * hL * hL, FR2 = qR * uR + hg * hR * hR;
    R den = SR - SL;
    if (fabs(den) < tiny) den = R(1);
    bool left = SL >= R(0), right = SR <= R(0);
    R F1, F2, F3;
    if (left) {
        F1 = FL1; F2 = FL2;
    } else if (right) {
        F1 = FR1; F2 = FR2;
    } else {
        F1 = (SR * FL1 - SL * FR1 + SL * SR * (hR - hL)) / den;
        F2 = (SR * FL2 - SL * FR2 + SL * SR * (qR - qL)) / den;
    }
    if (c.hllc) {
        R num = SL * hR * (uR - SR) - SR * hL * (uL - SL);
        R dd = hR * (uR - SR) - hL * (uL - SL);
        R SM = fabs(dd) < tiny ? R(0.5) * (uL + uR) : num / dd;
        F3 = F1 * (SM >= R(0) ? vL : vR);
    } else {
        R FL3 = qL * vL, FR3 = qR * vR;
        F3 = left ? FL3 : (right ? FR3 : (SR * FL3 - SL * FR3 + SL * SR * (hR * vR - hL * vL)) / den);
    }
    if (dryL && dryR) { F1 = R(0); F2 = R(0); F3 = R(0); }
    F1o = F1; F2o = F2; F3o = F3;
}

// The same HLLC/HLL flux in well-balanced deviation form (float32 production form).
// Instead of the momentum flux F2 it returns, for each side s in {L, R},
//     D_s = F2 + corr_s - g/2 h_s^2 = F2 - g/2 h*_s^2
// (corr_s = g/2 (h_s^2 - h*_s^2) is the hydrostatic-reconstruction correction), so
// that the cell update -[(F2 + corrL)_east - (F2 + corrR)_west] + bed source becomes
// -[D_L,east - D_R,west] - g/2 (H+ + H-) sE: every term is small at rest and no
// O(g h^2 / 2) quantities cancel in float32.  The pressure difference across the face
// is formed from the depth difference, dp = g/2 (h*_R - h*_L)(h*_R + h*_L).
template <class R>
__device__ __forceinline__ void riemann_wb(const KC<R>& c, R hL, R uL, R vL, R hR, R uR, R vR, R jump, R& F1o,
                                           R& DLo, R& DRo, R& F3o) {
    const R g = c.g, tiny = R(1e-14);
    R cL = dsqrt(g * hL), cR = dsqrt(g * hR);
    bool dryL = hL <= tiny, dryR = hR <= tiny;
    R u_s = R(0.5) * (uL + uR) + cL - cR;
    R c_s = R(0.5) * (cL + cR) + R(0.25) * (uL - uR);
    R SL = rmin(uL - cL, u_s - c_s);
    R SR = rmax(uR + cR, u_s + c_s);
    if (dryL) { SL = uR - R(2) * cR; SR = uR + cR; }
    if (dryR) { SL = uL - cL; SR = uL + R(2) * cL; }
    const R hg = c.hg;
    R qL = hL * uL, qR = hR * uR;
    R dp = hg * jump * (hR + hL);
    R den = SR - SL;
    if (fabs(den) < tiny) den = R(1);
    bool left = SL >= R(0), right = SR <= R(0);
    R F1, DL, DR, F3;
    if (left) {
        F1 = qL; DL = qL * uL; DR = qL * uL - dp;
    } else if (right) {
        F1 = qR; DL = qR * uR + dp; DR = qR * uR;
    } else {
        R inv = R(1) / den;
        F1 = (SR * qL - SL * qR + SL * SR * jump) * inv;
        R dyn = (SR * qL * uL - SL * qR * uR + SL * SR * (qR - qL)) * inv;
        DL = dyn - SL * dp * inv;
        DR = dyn - SR * dp * inv;
    }
    if (c.hllc) {
        R num = SL * hR * (uR - SR) - SR * hL * (uL - SL);
        R dd = hR * (uR - SR) - hL * (uL - SL);
        R SM = fabs(dd) < tiny ? R(0.5) * (uL + uR) : num / dd;
        F3 = F1 * (SM >= R(0) ? vL : vR);
    } else {
        R FL3 = qL * vL, FR3 = qR * vR;
        F3 = left ? FL3 : (right ? FR3 : (SR * FL3 - SL * FR3 + SL * SR * (hR * vR - hL * vL)) / den);
    }
    if (dryL && dryR) { F1 = R(0); DL = R(0); DR = R(0); F3 = R(0); }
    F1o = F1; DLo = DL; DRo = DR; F3o = F3;
}

// Face flux between two reconstructed cells (swe2d.py:226-234): hydrostatic
// reconstruction z* = max(zL, zR), h* = max(0, h + z - z*); returns the mass flux,
// the momentum flux plus the left and right pressure corrections, and the
// tangential flux.
template <class R>
__device__ __forceinline__ void face_flux(const KC<R>& c, const Recon<R>& L, const Recon<R>& Rr, R& F1, R& F2L,
                                          R& F2R, R& F3) {
    R hL = L.Hp, uL = L.Up, vL = L.Vp;
    R hR = Rr.Hm, uR = Rr.Um, vR = Rr.Vm;
    R hLs, hRs;
    if constexpr (sizeof(R) == 8) {
        R zL = L.Zp, zR = Rr.Zm;
        R zf = rmax(zL, zR);
        hLs = clamp0(hL + zL - zf);
        hRs = clamp0(hR + zR - zf);
    } else {
        // z* - zL = max(0, zR - zL), z* - zR = max(0, zL - zR), with
        // zR - zL = (z_R - z_L) - (d_L + d_R) / 2 formed from the cell-bed difference
        R dz = (Rr.z - L.z) - R(0.5) * (L.d + Rr.d);
        R aL = hL - clamp0(dz), aR = hR - clamp0(-dz);
        hLs = clamp0(aL);
        hRs = clamp0(aR);
        // surface jump h*_R - h*_L = (eta_R - eta_L) - (sE_L + sE_R)/2 when neither side is
        // clamped, formed from cell differences rather than from two rounded depths
        R jump = (aL > R(0) && aR > R(0))
                     ? ((Rr.h0 - L.h0) + (Rr.z - L.z)) - R(0.5) * (L.sE + Rr.sE)
                     : hRs - hLs;
        riemann_wb(c, hLs, uL, vL, hRs, uR, vR, jump, F1, F2L, F2R, F3);
        return;
    }
    if constexpr (sizeof(R) == 8) {
        R F2;
        riemann(c, hLs, uL, vL, hRs, uR, vR, F1, F2, F3);
        const R hg = c.hg;
        R corrL = hg * (hL * hL - hLs * hLs);
        R corrR = hg * (hR * hR - hRs * hRs);
        F2L = F2 + corrL;
        F2R = F2 + corrR;
    }
}

// ------------------------------------------------------------ block reductions
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace his
