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
    P_INFIL, P_RAINW, P_RATE, P_HSUM, P_SSUM, P_SPARE,
    NPART
};

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
};

struct StepParams {
    double dt, t, rain;
    double bc0[4], bc1[4];
    int active, pad;
};

struct TileRef {
    int member, x0, y0, local;
};

// ------------------------------------------------------------------ scalar helpers
template <class R> __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : (b > a ? b : a); }
template <class R> __device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : (b < a ? b : a); }
template <class R> __device__ __forceinline__ R relu(R x) { return x > R(0) ? x : R(0); }
template <class R> __device__ __forceinline__ R clamp0(R x) { return x < R(0) ? R(0) : x; }

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
__device__ __forceinline__ void kp_velocity(const Consts& c, R h, R hu, R hv, R& u, R& v) {
    const R SQRT2 = R(1.4142135623730951);
    R h4 = pow4(h);
    R den = dsqrt(h4 + rmax(h4, R(c.kp_eps)));
    if (h >= R(c.h_dry)) {
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
__device__ __forceinline__ void stage_ghost(const Consts& c, R val, R h, R un, R ut, R z, R& hg_o, R& un_o, R& ut_o) {
    const R g = R(c.g), hd = R(c.h_dry);
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
__device__ __forceinline__ void discharge_ghost(const Consts& c, R val, R h, R& hg_o, R& un_o, R& ut_o) {
    const R g = R(c.g), hd = R(c.h_dry);
    R hc = rmax(cbrt_pow(val * val / g), hd);
    R hg = h >= hd ? h : hc;
    hg_o = hg;
    un_o = -val / hg;
    ut_o = R(0);
}

template <class R>
__device__ __forceinline__ R minmod(R a, R b) {
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
template <class R>
struct Recon {
    R Hm, Hp, Um, Up, Vm, Vp, Zm, Zp;
};

template <class R>
__device__ __forceinline__ Recon<R> reconstruct(const Consts& c, R hm, R h0, R hp, R um, R u0, R up, R vm, R v0, R vp,
                                                R zm, R z0, R zp) {
    Recon<R> r;
    if (c.order == 2) {
        R hmin = rmin(rmin(hm, h0), hp);
        R ok = (hmin >= R(c.h_dry)) ? R(1) : R(0);
        R em = hm + zm, e0 = h0 + z0, ep = hp + zp;
        R sH = minmod(h0 - hm, hp - h0) * ok;
        R sE = minmod(e0 - em, ep - e0) * ok;
        R sU = minmod(u0 - um, up - u0) * ok;
        R sV = minmod(v0 - vm, vp - v0) * ok;
        r.Hm = h0 - R(0.5) * sH;
        r.Hp = h0 + R(0.5) * sH;
        R Em = e0 - R(0.5) * sE, Ep = e0 + R(0.5) * sE;
        r.Um = u0 - R(0.5) * sU;
        r.Up = u0 + R(0.5) * sU;
        r.Vm = v0 - R(0.5) * sV;
        r.Vp = v0 + R(0.5) * sV;
        r.Zm = Em - r.Hm;
        r.Zp = Ep - r.Hp;
    } else {
        r.Hm = r.Hp = h0;
        r.Um = r.Up = u0;
        r.Vm = r.Vp = v0;
        r.Zm = r.Zp = z0;
    }
    return r;
}

// HLLC / HLL flux with two-rarefaction wave speeds and dry-bed fixes (swe2d.py:61-101)
template <class R>
__device__ __forceinline__ void riemann(const Consts& c, R hL, R uL, R vL, R hR, R uR, R vR, R& F1o, R& F2o,
                                        R& F3o) {
    const R g = R(c.g), tiny = R(1e-14);
    R cL = dsqrt(g * hL), cR = dsqrt(g * hR);
    bool dryL = hL <= tiny, dryR = hR <= tiny;
    R u_s = R(0.5) * (uL + uR) + cL - cR;
    R c_s = R(0.5) * (cL + cR) + R(0.25) * (uL - uR);
    R SL = rmin(uL - cL, u_s - c_s);
    R SR = rmax(uR + cR, u_s + c_s);
    if (dryL) { SL = uR - R(2) * cR; SR = uR + cR; }
    if (dryR) { SL = uL - cL; SR = uL + R(2) * cL; }
    const R hg = R(0.5 * c.g);
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

// Face flux between two reconstructed cells (swe2d.py:226-234): hydrostatic
// reconstruction z* = max(zL, zR), h* = max(0, h + z - z*); returns the mass flux,
// the momentum flux plus the left and right pressure corrections, and the
// tangential flux.
template <class R>
__device__ __forceinline__ void face_flux(const Consts& c, const Recon<R>& L, const Recon<R>& Rr, R& F1, R& F2L,
                                          R& F2R, R& F3) {
    R hL = L.Hp, uL = L.Up, vL = L.Vp, zL = L.Zp;
    R hR = Rr.Hm, uR = Rr.Um, vR = Rr.Vm, zR = Rr.Zm;
    R zf = rmax(zL, zR);
    R hLs = clamp0(hL + zL - zf), hRs = clamp0(hR + zR - zf);
    R F2;
    riemann(c, hLs, uL, vL, hRs, uR, vR, F1, F2, F3);
    const R hg = R(0.5 * c.g);
    R corrL = hg * (hL * hL - hLs * hLs);
    R corrR = hg * (hR * hR - hRs * hRs);
    F2L = F2 + corrL;
    F2R = F2 + corrR;
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
