// 2-D finite-volume step kernels (one tile of TX x TY cells per CTA).
//
// One SSP-RK2 step is two launches over every tile of every member:
//   STAGE 1: rhs at (h, hu, hv) with the edge values at t  -> Euler -> clip -> stage buffers
//   STAGE 2: rhs at the stage buffers with the values at t+dt -> RK average -> clip
//            -> rain -> Horton -> retention store -> friction -> state, CFL rate
// (first order: STAGE 0 does Euler, clip, sources and friction in one launch).
//
// The rhs of a tile needs the fluxes of the faces of the tile plus a one-cell ring
// (the positivity limiter scales a face by the theta of its upwind cell, and theta
// needs all four faces of that cell), and a face needs two cells either side
// (MUSCL): the CTA stages a (TX+6) x (TY+6) halo tile of (h, u, v, z) in shared
// memory, builds ghost cells at domain edges on the fly, computes every needed
// face flux once, then theta, then the update of its own cells.
//
// Reference: hydrointel/solver/swe2d.py:196-371, boundaries.py:56-128.
#pragma once
#include "his_device.cuh"

namespace his {

template <class R, int TX, int TY>
struct TileGeom {
    static constexpr int NT = TX * TY;
    static constexpr int RX = TX + 6, RY = TY + 6, NR = RX * RY;       // halo tile
    static constexpr int XW = TX + 3, XH = TY + 2, NXF = XW * XH;      // x faces -1..TX+1, rows -1..TY
    static constexpr int YW = TX + 2, YH = TY + 3, NYF = YW * YH;      // y faces -1..TY+1, cols -1..TX
    static constexpr int TW = TX + 2, TH = TY + 2, NTH = TW * TH;      // theta ring
    static constexpr int NRED = 11;
    static constexpr size_t smem_bytes =
        sizeof(R) * (4 * NR + 4 * NXF + 4 * NYF + NTH) + sizeof(double) * 32 * NRED + 16;
};

// Bed source and reconstructed bed of one cell along one axis (swe2d.py:220).
// (float32: Zp - Zm is the in-cell bed slope d = sE - sH, see reconstruct())
template <class R>
__device__ __forceinline__ R bed_source(const KC<R>& c, R hm, R h0, R hp, R zm, R z0, R zp) {
    R hmin = rmin(rmin(hm, h0), hp);
    R ok = (hmin >= c.h_dry) ? R(1) : R(0);
    R sH = minmod(h0 - hm, hp - h0) * ok;
    R Hm = h0 - R(0.5) * sH, Hp = h0 + R(0.5) * sH;
    if constexpr (sizeof(R) == 8) {
        R em = hm + zm, e0 = h0 + z0, ep = hp + zp;
        R sE = minmod(e0 - em, ep - e0) * ok;
        R Em = e0 - R(0.5) * sE, Ep = e0 + R(0.5) * sE;
        R Zm = Em - Hm, Zp = Ep - Hp;
        return c.nhg * (Hm + Hp) * (Zp - Zm);
    } else {
        // float32: the bed source plus the hydrostatic part of the face momentum fluxes,
        // -g/2 (H+ + H-)(H+ - H- + Zp - Zm) = -g/2 (H+ + H-) sE (see riemann_wb)
        R sE = minmod((h0 - hm) + (z0 - zm), (hp - h0) + (zp - z0)) * ok;
        return c.nhg * (Hm + Hp) * sE;
    }
}

// Load one halo-tile position: an interior cell, or the ghost that the x-sweep (for
// cells outside in x) or the y-sweep (outside in y) would see (boundaries.py:81-128).
template <class R>
__device__ __forceinline__ void load_halo(const KC<R>& c, const Grid<R>& gd, const R* bcv, const R* __restrict__ H,
                                          const R* __restrict__ HU, const R* __restrict__ HV, int gx, int gy, R& hh,
                                          R& uu, R& vv, R& zz) {
    const int nx = gd.nx, ny = gd.ny;
    const int ng = c.order == 1 ? 1 : 2;
    const bool inx = (unsigned)gx < (unsigned)nx, iny = (unsigned)gy < (unsigned)ny;
    if (inx && iny) {
        size_t i = (size_t)gy * nx + gx;
        hh = H[i];
        kp_velocity(c, hh, HU[i], HV[i], uu, vv);
        zz = gd.z[i];
        return;
    }
    if (!inx && !iny) { hh = uu = vv = zz = R(0); return; }
    const bool alongx = !inx;                       // ghost of the x-sweep
    const int n = alongx ? nx : ny;
    const int gpos = alongx ? gx : gy;
    const bool lo = gpos < 0;
    const int side = alongx ? (lo ? EDGE_W : EDGE_E) : (lo ? EDGE_S : EDGE_N);
    const int k = lo ? (-gpos - 1) : (gpos - n);
    const int kind = gd.bc[side];
    int layer;
    if (kind == BC_CLOSED || kind == BC_TRANSMISSIVE) {
        if (n < ng) layer = lo ? 0 : n - 1;
        else layer = lo ? k : n - 1 - k;
    } else {
        layer = lo ? 0 : n - 1;
    }
    layer = layer < 0 ? 0 : (layer > n - 1 ? n - 1 : layer);
    size_t i = alongx ? (size_t)gy * nx + layer : (size_t)layer * nx + gx;
    R h0 = H[i], u0, v0;
    kp_velocity(c, h0, HU[i], HV[i], u0, v0);
    R z0 = gd.z[i];
    const R sgn = lo ? R(-1) : R(1);
    R un = sgn * (alongx ? u0 : v0);
    R ut = alongx ? v0 : u0;
    R hg, ung, utg;
    if (kind == BC_CLOSED) { hg = h0; ung = -un; utg = ut; }
    else if (kind == BC_TRANSMISSIVE) { hg = h0; ung = un; utg = ut; }
    else if (kind == BC_STAGE) stage_ghost(c, bcv[side], h0, un, ut, z0, hg, ung, utg);
    else discharge_ghost(c, bcv[side], h0, hg, ung, utg);
    hh = hg;
    zz = z0;
    if (alongx) { uu = sgn * ung; vv = utg; }
    else { vv = sgn * ung; uu = utg; }
}

template <class T>
__device__ __forceinline__ T warp_sum_t(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
template <class T>
__device__ __forceinline__ T warp_max_t(T v) {
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// Block reduction of NV per-thread values in the compute type T: within each warp by
// shuffles, then across warps by lane j of warp 0 for value j (warps in order), which
// converts its result once and writes it to out[slots[j]] (the float64 tile partial).
template <int NV, class T>
__device__ __forceinline__ void block_reduce_store(T (&v)[NV], const bool* is_max, T* red, double* out,
                                                   const int* slots, int nthreads) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = nthreads >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = is_max[j] ? warp_max_t(v[j]) : warp_sum_t(v[j]);
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) red[warp * NV + j] = v[j];
    }
    __syncthreads();
    if (warp == 0 && lane < NV) {
        const bool mx = is_max[lane];
        T a = red[lane];
        for (int w = 1; w < nw; ++w) {
            const T b = red[w * NV + lane];
            a = mx ? (b > a ? b : a) : a + b;
        }
        out[slots[lane]] = (double)a;
    }
}

// STAGE: 0 = first-order full step, 1 = RK stage 1, 2 = RK stage 2 + sources.
template <class R, int TX, int TY, int STAGE>
__global__ void __launch_bounds__(TX * TY) stage_kernel(const Grid<R>* __restrict__ grids,
                                                         const TileRef* __restrict__ tiles,
                                                         const StepParams* __restrict__ params, const KC<R> c,
                                                         double* __restrict__ partials) {
    using G = TileGeom<R, TX, TY>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sh_h = reinterpret_cast<R*>(smem_raw);
    R* sh_u = sh_h + G::NR;
    R* sh_v = sh_u + G::NR;
    R* sh_z = sh_v + G::NR;
    R* xF1 = sh_z + G::NR;
    R* xF2L = xF1 + G::NXF;
    R* xF2R = xF2L + G::NXF;
    R* xF3 = xF2R + G::NXF;
    R* yF1 = xF3 + G::NXF;
    R* yF2L = yF1 + G::NYF;
    R* yF2R = yF2L + G::NYF;
    R* yF3 = yF2R + G::NYF;
    R* thS = yF3 + G::NYF;
    R* red = reinterpret_cast<R*>((reinterpret_cast<uintptr_t>(thS + G::NTH) + 15) & ~uintptr_t(15));
    __shared__ R bcv[4];

    const TileRef tr = tiles[blockIdx.x];
    const Grid<R>& gd = grids[tr.member];
    const StepParams& pr = params[tr.member];
    if (!pr.active) return;
    const int nx = gd.nx, ny = gd.ny, x0 = tr.x0, y0 = tr.y0;
    const int tid = threadIdx.x;
    const R dt = par_dt<R>(pr);
    if (tid < 4) bcv[tid] = par_bc<R>(pr, STAGE == 2, tid);
    __syncthreads();
    const R* __restrict__ H = STAGE == 2 ? gd.h1 : gd.h;
    const R* __restrict__ HU = STAGE == 2 ? gd.hu1 : gd.hu;
    const R* __restrict__ HV = STAGE == 2 ? gd.hv1 : gd.hv;

    // ---- A: halo tile of (h, u, v, z)
    for (int p = tid; p < G::NR; p += G::NT) {
        int ry = p / G::RX, rx = p - ry * G::RX;
        R hh, uu, vv, zz;
        load_halo(c, gd, bcv, H, HU, HV, x0 + rx - 3, y0 + ry - 3, hh, uu, vv, zz);
        sh_h[p] = hh; sh_u[p] = uu; sh_v[p] = vv; sh_z[p] = zz;
    }
    __syncthreads();

    // ---- B: face fluxes (x faces: normal u; y faces: normal v)
    for (int p = tid; p < G::NXF; p += G::NT) {
        int fyi = p / G::XW, fxi = p - fyi * G::XW;
        int fx = fxi - 1, y = fyi - 1;
        int gfx = x0 + fx, gy = y0 + y;
        R F1 = R(0), F2L = R(0), F2R = R(0), F3 = R(0);
        if ((unsigned)gy < (unsigned)ny && gfx >= 0 && gfx <= nx) {
            const int b = (y + 3) * G::RX + fx + 2;    // left cell of the face
            Recon<R> L = reconstruct(c, sh_h[b - 1], sh_h[b], sh_h[b + 1], sh_u[b - 1], sh_u[b], sh_u[b + 1],
                                     sh_v[b - 1], sh_v[b], sh_v[b + 1], sh_z[b - 1], sh_z[b], sh_z[b + 1]);
            Recon<R> Rr = reconstruct(c, sh_h[b], sh_h[b + 1], sh_h[b + 2], sh_u[b], sh_u[b + 1], sh_u[b + 2],
                                      sh_v[b], sh_v[b + 1], sh_v[b + 2], sh_z[b], sh_z[b + 1], sh_z[b + 2]);
            face_flux(c, L, Rr, F1, F2L, F2R, F3);
        }
        xF1[p] = F1; xF2L[p] = F2L; xF2R[p] = F2R; xF3[p] = F3;
    }
    for (int p = tid; p < G::NYF; p += G::NT) {
        int fyi = p / G::YW, xi = p - fyi * G::YW;
        int fy = fyi - 1, x = xi - 1;
        int gfy = y0 + fy, gx = x0 + x;
        R F1 = R(0), F2L = R(0), F2R = R(0), F3 = R(0);
        if ((unsigned)gx < (unsigned)nx && gfy >= 0 && gfy <= ny) {
            const int RX = G::RX;
            const int b = (fy + 2) * RX + x + 3;       // lower cell of the face
            Recon<R> L = reconstruct(c, sh_h[b - RX], sh_h[b], sh_h[b + RX], sh_v[b - RX], sh_v[b], sh_v[b + RX],
                                     sh_u[b - RX], sh_u[b], sh_u[b + RX], sh_z[b - RX], sh_z[b], sh_z[b + RX]);
            Recon<R> U = reconstruct(c, sh_h[b], sh_h[b + RX], sh_h[b + 2 * RX], sh_v[b], sh_v[b + RX],
                                     sh_v[b + 2 * RX], sh_u[b], sh_u[b + RX], sh_u[b + 2 * RX], sh_z[b],
                                     sh_z[b + RX], sh_z[b + 2 * RX]);
            face_flux(c, L, U, F1, F2L, F2R, F3);
        }
        yF1[p] = F1; yF2L[p] = F2L; yF2R[p] = F2R; yF3[p] = F3;
    }
    __syncthreads();

    // ---- C: positivity-limiter theta on the tile plus a one-cell ring (swe2d.py:259-264)
    const R rdx = gd.rdx, rdy = gd.rdy;
    for (int p = tid; p < G::NTH; p += G::NT) {
        int ti = p / G::TW, tj = p - ti * G::TW;
        int x = tj - 1, y = ti - 1;
        int gx = x0 + x, gy = y0 + y;
        R th = R(1);
        if ((unsigned)gx < (unsigned)nx && (unsigned)gy < (unsigned)ny) {
            R Fw = xF1[(y + 1) * G::XW + x + 1], Fe = xF1[(y + 1) * G::XW + x + 2];
            R Gs = yF1[(y + 1) * G::YW + x + 1], Gn = yF1[(y + 2) * G::YW + x + 1];
            R out = (relu(Fe) + relu(-Fw)) / rdx + (relu(Gn) + relu(-Gs)) / rdy;
            R need = out * dt;
            R hh = sh_h[(y + 3) * G::RX + x + 3];
            th = need > hh ? hh / (need > R(0) ? need : R(1)) : R(1);
        }
        thS[p] = th;
    }
    __syncthreads();

    // ---- D: update of the tile's own cells
    // per-cell contributions in the compute type; the block sums them per warp in R and
    // across warps (and the finalize kernel across tiles) in float64
    R acc_clip = 0, xin = 0, xout = 0, yin = 0, yout = 0, infil = 0, rainw = 0, rate = 0, hsum = 0, ssum = 0;
    R hmax = 0;
    const R rdt = par_rain<R>(pr) * dt;
    const R tt = clamp0(par_t<R>(pr) - gd.rt0);
    const int x = tid % TX, y = tid / TX;
    const int gx = x0 + x, gy = y0 + y;
    if (gx < nx && gy < ny) {
        const R thC = thS[(y + 1) * G::TW + x + 1];
        const R thW = thS[(y + 1) * G::TW + x], thE = thS[(y + 1) * G::TW + x + 2];
        const R thSo = thS[y * G::TW + x + 1], thN = thS[(y + 2) * G::TW + x + 1];
        const int w = (y + 1) * G::XW + x + 1, e = w + 1;
        const int s = (y + 1) * G::YW + x + 1, nn = s + G::YW;
        const R Fw = xF1[w], Fe = xF1[e], Gs = yF1[s], Gn = yF1[nn];
        const R sw = Fw > R(0) ? thW : thC, se = Fe > R(0) ? thC : thE;
        const R ss = Gs > R(0) ? thSo : thC, sn = Gn > R(0) ? thC : thN;
        const R F1w = Fw * sw, F1e = Fe * se, G1s = Gs * ss, G1n = Gn * sn;
        R a1 = -(F1e - F1w) / rdx;
        R a2 = -(xF2L[e] - xF2R[w]) / rdx;
        R a3 = -(xF3[e] * se - xF3[w] * sw) / rdx;
        R b1 = -(G1n - G1s) / rdy;
        R b2 = -(yF2L[nn] - yF2R[s]) / rdy;
        R b3 = -(yF3[nn] * sn - yF3[s] * ss) / rdy;
        const int cc = (y + 3) * G::RX + x + 3;
        if (c.order == 2) {
            R scx = bed_source(c, sh_h[cc - 1], sh_h[cc], sh_h[cc + 1], sh_z[cc - 1], sh_z[cc], sh_z[cc + 1]);
            R scy = bed_source(c, sh_h[cc - G::RX], sh_h[cc], sh_h[cc + G::RX], sh_z[cc - G::RX], sh_z[cc],
                               sh_z[cc + G::RX]);
            a2 = a2 + scx / rdx;
            b2 = b2 + scy / rdy;
        }
        const R dh = a1 + b1, dhu = a2 + b3, dhv = a3 + b2;
        if (gx == 0) { xin += relu(F1w); xout += relu(-F1w); }
        if (gx == nx - 1) { xin += relu(-F1e); xout += relu(F1e); }
        if (gy == 0) { yin += relu(G1s); yout += relu(-G1s); }
        if (gy == ny - 1) { yin += relu(-G1n); yout += relu(G1n); }

        const size_t i = (size_t)gy * nx + gx;
        R hn, hun, hvn;
        if (STAGE == 2) {
            const R h1 = sh_h[cc], hu1 = gd.hu1[i], hv1 = gd.hv1[i];
            hn = R(0.5) * (gd.h[i] + h1 + dt * dh);
            hun = R(0.5) * (gd.hu[i] + hu1 + dt * dhu);
            hvn = R(0.5) * (gd.hv[i] + hv1 + dt * dhv);
        } else {
            hn = sh_h[cc] + dt * dh;
            hun = gd.hu[i] + dt * dhu;
            hvn = gd.hv[i] + dt * dhv;
        }
        R neg = clamp0(-hn);
        acc_clip = neg;
        hn = hn + neg;
        if (STAGE == 1) {
            gd.h1[i] = hn; gd.hu1[i] = hun; gd.hv1[i] = hvn;
        } else {
            // ---- sources after the RK update (swe2d.py:330-360)
            R sf = gd.S ? gd.sf[i] : R(0);
            R icum = gd.f0 ? gd.ic[i] : R(0);
            if (gd.rw) {
                R add = rdt * gd.rw[i];
                hn = hn + add;
                rainw = add;
            } else {
                hn = hn + rdt;
            }
            if (gd.f0) {
                R f0 = gd.f0[i], fc = gd.fc[i], kk = gd.k[i];
                R rate_f = fc + (f0 - fc) * rexp(-kk * tt);
                R pot = rate_f * dt;
                R take = rmin(pot, hn);
                R safe = hn > R(0) ? hn : R(1);
                R scale = hn > R(0) ? (hn - take) / safe : R(0);
                hn = hn - take;
                hun = hun * scale;
                hvn = hvn * scale;
                R taken = take;
                if (gd.S) {
                    R tks = rmin(pot - take, sf);
                    sf = sf - tks;
                    taken = taken + tks;
                }
                icum = icum + taken;
                infil = taken;
                gd.ic[i] = icum;
            }
            if (gd.S) {
                R room = clamp0(gd.S[i] - sf);
                R fill = rmin(room, hn);
                R safe = hn > R(0) ? hn : R(1);
                R scale = hn > R(0) ? (hn - fill) / safe : R(0);
                hn = hn - fill;
                hun = hun * scale;
                hvn = hvn * scale;
                sf = sf + fill;
                gd.sf[i] = sf;
            }
            // ---- semi-implicit Manning friction (swe2d.py:362-370)
            R u, v;
            kp_velocity(c, hn, hun, hvn, u, v);
            R speed = dsqrt(u * u + v * v);
            R hf = rmax(hn, c.h_dry);
            R nm = gd.n[i];
            R denom = R(1) + dt * c.g * nm * nm * speed / pow43(hf);
            u = u / denom;
            v = v / denom;
            bool wet = hn >= c.h_dry;
            hun = wet ? hn * u : R(0);
            hvn = wet ? hn * v : R(0);
            gd.h[i] = hn; gd.hu[i] = hun; gd.hv[i] = hvn;
            if (gd.pk) gd.pk[i] = rmax(gd.pk[i], hn);
            if (gd.ps) gd.ps[i] = rmax(gd.ps[i], wet ? dsqrt(u * u + v * v) : R(0));
            // ---- CFL rate of the new state for the next step (swe2d.py:179-184)
            R u2, v2;
            kp_velocity(c, hn, hun, hvn, u2, v2);
            R cw = dsqrt(c.g * hn);
            R r = hn > c.h_dry ? (fabs(u2) + cw) / rdx + (fabs(v2) + cw) / rdy : R(0);
            rate = r;
            hsum = hn;
            ssum = sf;
            hmax = hn;
        }
    }
    __syncthreads();
    double* out = partials + (size_t)blockIdx.x * NPART;
    if (STAGE == 1) {
        R v[5] = {acc_clip, xin, xout, yin, yout};
        const bool mx[5] = {false, false, false, false, false};
        const int sl[5] = {P_CLIP1, P_XIN1, P_XOUT1, P_YIN1, P_YOUT1};
        block_reduce_store<5>(v, mx, red, out, sl, G::NT);
    } else {
        const int b = STAGE == 2 ? P_CLIP2 : P_CLIP1;
        R v[11] = {acc_clip, xin, xout, yin, yout, infil, rainw, rate, hsum, ssum, hmax};
        const bool mx[11] = {false, false, false, false, false, false, false, true, false, false, true};
        const int sl[11] = {b, b + 1, b + 2, b + 3, b + 4, P_INFIL, P_RAINW, P_RATE, P_HSUM, P_SSUM, P_HMAX};
        block_reduce_store<11>(v, mx, red, out, sl, G::NT);
    }
}

// Per-tile CFL rate, surface and retained water of the current state (no halo).
template <class R, int TX, int TY>
__global__ void __launch_bounds__(TX * TY) cell_reduce_kernel(const Grid<R>* __restrict__ grids,
                                                               const TileRef* __restrict__ tiles, const KC<R> c,
                                                               double* __restrict__ partials) {
    __shared__ double red[32 * 3];   // volumes are summed in float64 (this kernel is not on the step path)
    const TileRef tr = tiles[blockIdx.x];
    const Grid<R>& gd = grids[tr.member];
    const int x = threadIdx.x % TX, y = threadIdx.x / TX;
    const int gx = tr.x0 + x, gy = tr.y0 + y;
    double rate = 0, hs = 0, ss = 0;
    if (gx < gd.nx && gy < gd.ny) {
        size_t i = (size_t)gy * gd.nx + gx;
        R h = gd.h[i], u, v;
        kp_velocity(c, h, gd.hu[i], gd.hv[i], u, v);
        R cw = dsqrt(c.g * h);
        R r = h > c.h_dry ? (fabs(u) + cw) / gd.rdx + (fabs(v) + cw) / gd.rdy : R(0);
        rate = (double)r;
        hs = (double)h;
        ss = gd.sf ? (double)gd.sf[i] : 0.0;
    }
    double v[3] = {rate, hs, ss};
    const bool mx[3] = {true, false, false};
    const int sl[3] = {P_RATE, P_HSUM, P_SSUM};
    block_reduce_store<3>(v, mx, red, partials + (size_t)blockIdx.x * NPART, sl, TX * TY);
}

// Per-member totals from the tile partials, in tile order.  out: 8 per member =
// bnd_in, bnd_out, rain, infil, clip (m^3), rate (1/s), surface and retained volume.
// mode 0: after a step; mode 1: rate and volumes only.
template <class R>
__global__ void finalize_kernel(const Grid<R>* __restrict__ grids, const StepParams* __restrict__ params, Consts c,
                                const double* __restrict__ partials, double* __restrict__ out, int mode) {
    const int m = blockIdx.x, lane = threadIdx.x;
    const Grid<R>& gd = grids[m];
    if (mode == 0 && !params[m].active) return;
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
    double* o = out + (size_t)m * 8;
    o[5] = s[P_RATE];
    o[6] = s[P_HSUM] * gd.area;
    o[7] = s[P_SSUM] * gd.area;
    if (mode != 0) return;
    const StepParams& pr = params[m];
    const double dt = (double)R(pr.dt);
    double qin = s[P_XIN1] * gd.dy + s[P_YIN1] * gd.dx;
    double qout = s[P_XOUT1] * gd.dy + s[P_YOUT1] * gd.dx;
    double clip = s[P_CLIP1] * gd.area;
    if (c.order == 2) {
        double qin2 = s[P_XIN2] * gd.dy + s[P_YIN2] * gd.dx;
        double qout2 = s[P_XOUT2] * gd.dy + s[P_YOUT2] * gd.dx;
        qin = 0.5 * (qin + qin2);
        qout = 0.5 * (qout + qout2);
        clip = clip + s[P_CLIP2] * gd.area;
    }
    o[0] = qin * dt;
    o[1] = qout * dt;
    if (gd.rw) o[2] = s[P_RAINW] * gd.area;
    else o[2] = (double)(R(pr.rain) * R(pr.dt)) * ((double)((long long)gd.nx * gd.ny) * gd.area);
    o[3] = s[P_INFIL] * gd.area;
    o[4] = clip;
}

}  // namespace his
