// 2-D finite-volume step kernels: row-marching strips.
//
// A CTA of NT threads owns a strip of W <= NT - 6 columns of one member and marches
// up a chunk of rows [y0, y1).  Thread t works on column cx = x0 - 3 + t.  Per new
// row r, with two barriers (StripPipe::row below):
//   A  builds row r of (h, u, v, z) into a four-row shared ring (ghost cells at the
//      domain edges, boundaries.py:81-128), prefetches row r+1 and the update inputs
//      of row r-3, forms the y-reconstruction of row r-1 and the x-reconstruction of
//      row r-2 (swe2d.py:205-219) and publishes the latter's plus side;
//   B  forms the y-face between rows r-2 and r-1 and the x-face west of its cell in
//      row r-2 (swe2d.py:61-101, 226-234), two independent chains side by side;
//   C  forms the positivity-limiter theta of row r-2 (swe2d.py:259-264);
//   D  updates row r-3: divergence of the donor-scaled fluxes, bed source, RK stage,
//      then in the last stage rain, infiltration, retention, friction, CFL rate and
//      peaks (swe2d.py:305-371).
// Every cell is loaded once (plus a 3-column halo each side) and every face flux,
// reconstruction and theta is computed once.  Per-thread partial sums (clip,
// boundary flux, infiltration, rain, rate, volumes) are reduced once per strip-chunk
// into one float64 slot set, summed in a fixed order per member by the finalize
// kernel, so results do not depend on the batch a member runs in.
#pragma once
#include "his_device.cuh"

namespace his {

struct StripRef {
    int member, x0, w, y0, y1, pad;
};

// Four values of one cell or face kept together in shared memory, so that one
// vector access moves them: cells {h, u, v, z}, faces {F1, F2L, F2R, F3}, and the
// x-reconstruction as {Hm, Hp, Um, Up} and {Vm, Vp, Zm, Zp} (float32: {Vm, Vp, d, sE}).
template <class R>
struct alignas(4 * sizeof(R)) Q4 {
    R a, b, c, d;
};

// Shared-memory layout of one CTA.  Rings of the last rows' cells, x- and y-faces and
// thetas: a thread publishes each value once and reads both its neighbours' entries
// and its own earlier rows from them, so no row-to-row state is shifted through
// registers.  Every row of entries has one padding slot on each side: thread t's
// entry is at t + 1, so the neighbours of the first and last thread are in bounds
// (their values are never used).
template <class R, int NT>
struct StripGeom {
    static constexpr int RING = 4;                 // rows kept per ring (slot = row & 3)
    static constexpr int P = NT + 2;               // padded row of entries
    static constexpr int NRED = 11;                // reduced values (the reduction reuses the cell ring)
    // cells [RING][P], x-recon plus side [P], x-faces [2][P], y-faces [RING][P]; then
    // the plus-side surface slope [P] and theta [RING][P]
    static constexpr size_t quads = (size_t)(RING + 1 + 2 + RING) * P;
    static constexpr size_t scalars = (size_t)(1 + RING) * P;
    static_assert((size_t)4 * RING * P >= (size_t)(NT / 32) * NRED, "reduction scratch must fit in the cell ring");
    static constexpr size_t smem_bytes = sizeof(Q4<R>) * quads + sizeof(R) * scalars;
    // resident CTAs per SM the float32 kernels are register-capped for; float64 keeps
    // the compiler's choice (one CTA of any width must fit the register file)
    static constexpr int min_ctas(int stage) {
        return sizeof(R) == 4 ? ((stage == 1 ? 768 : 640) / NT > 0 ? (stage == 1 ? 768 : 640) / NT : 1) : 1;
    }
};

// Centred bed source of one cell along one axis (swe2d.py:220), from the cell's own
// reconstruction: -g/2 (H- + H+)(Z+ - Z-).  float32: Z+ - Z- is the in-cell surface
// slope sE (the hydrostatic part of the face momentum fluxes is carried by riemann_wb).
// The row loop computes it where the reconstruction is formed and carries it in
// registers to the update of that cell.
template <class R>
__device__ __forceinline__ R bed_term(const KC<R>& c, const Recon<R>& r) {
    if constexpr (sizeof(R) == 8) return c.nhg * (r.Hm + r.Hp) * (r.Zp - r.Zm);
    else return c.nhg * (r.Hm + r.Hp) * r.sE;
}

// One halo position: an interior cell, or the ghost that the x-sweep (outside in x)
// or the y-sweep (outside in y) would see (boundaries.py:81-128), in two parts for
// software pipelining: halo_fetch issues the loads of the source cell (the cell
// itself, or the layer a ghost copies) rows ahead; halo_build turns the fetched raw
// values into (h, u, v, z) when the row is due.
template <class R>
struct HaloRaw {
    R h, hu, hv, z;
};

template <class R>
__device__ __forceinline__ HaloRaw<R> halo_fetch(const KC<R>& c, const Grid<R>& gd, const R* __restrict__ H,
                                                 const R* __restrict__ HU, const R* __restrict__ HV, int gx, int gy) {
    const int nx = gd.nx, ny = gd.ny;
    const bool inx = (unsigned)gx < (unsigned)nx, iny = (unsigned)gy < (unsigned)ny;
    HaloRaw<R> a;
    if (!inx && !iny) { a.h = a.hu = a.hv = a.z = R(0); return a; }
    // 32-bit cell indices (a grid holds at most 2^30 cells): one wide multiply-add forms
    // each address
    unsigned i;
    if (inx && iny) {
        i = (unsigned)gy * (unsigned)nx + (unsigned)gx;
    } else {
        const int ng = c.order == 1 ? 1 : 2;
        const bool alongx = !inx;
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
        i = alongx ? (unsigned)gy * (unsigned)nx + (unsigned)layer : (unsigned)layer * (unsigned)nx + (unsigned)gx;
    }
    a.h = H[i];
    a.hu = HU[i];
    a.hv = HV[i];
    a.z = gd.z[i];
    return a;
}

template <class R>
__device__ __forceinline__ void halo_build(const KC<R>& c, const Grid<R>& gd, const R* bcv, const HaloRaw<R>& a,
                                           int gx, int gy, R& hh, R& uu, R& vv, R& zz) {
    const int nx = gd.nx, ny = gd.ny;
    const bool inx = (unsigned)gx < (unsigned)nx, iny = (unsigned)gy < (unsigned)ny;
    if (!inx && !iny) { hh = uu = vv = zz = R(0); return; }
    R u0, v0;
    kp_velocity(c, a.h, a.hu, a.hv, u0, v0);
    zz = a.z;
    if (inx && iny) { hh = a.h; uu = u0; vv = v0; return; }
    const bool alongx = !inx;
    const int n = alongx ? nx : ny;
    const int gpos = alongx ? gx : gy;
    const bool lo = gpos < 0;
    const int side = alongx ? (lo ? EDGE_W : EDGE_E) : (lo ? EDGE_S : EDGE_N);
    const int kind = gd.bc[side];
    (void)n;
    const R sgn = lo ? R(-1) : R(1);
    R un = sgn * (alongx ? u0 : v0);
    R ut = alongx ? v0 : u0;
    R hg, ung, utg;
    if (kind == BC_CLOSED) { hg = a.h; ung = -un; utg = ut; }
    else if (kind == BC_TRANSMISSIVE) { hg = a.h; ung = un; utg = ut; }
    else if (kind == BC_STAGE) stage_ghost(c, bcv[side], a.h, un, ut, a.z, hg, ung, utg);
    else discharge_ghost(c, bcv[side], a.h, hg, ung, utg);
    hh = hg;
    if (alongx) { uu = sgn * ung; vv = utg; }
    else { vv = sgn * ung; uu = utg; }
}

// Per-cell inputs of the update (row orow), fetched one row ahead.
template <class R>
struct CellIn {
    R h0, hu0, hv0, hu1, hv1, sf, ic, f0, fc, k, S, n, rw;
};

// Optional fields of a member, tested once per CTA: the row loop reads a bit of a
// register instead of re-reading a 64-bit pointer from the shared record and
// comparing it with null.
enum : unsigned { FEAT_STORE = 1u, FEAT_HORTON = 2u, FEAT_RAINW = 4u, FEAT_PEAK = 8u, FEAT_PSPEED = 16u, FEAT_SNAP = 32u };
template <class R>
__device__ __forceinline__ unsigned grid_features(const Grid<R>& gd) {
    return (gd.S ? FEAT_STORE : 0u) | (gd.f0 ? FEAT_HORTON : 0u) | (gd.rw ? FEAT_RAINW : 0u) |
           (gd.pk ? FEAT_PEAK : 0u) | (gd.ps ? FEAT_PSPEED : 0u);
}

template <class R, int STAGE>
__device__ __forceinline__ CellIn<R> cell_fetch(const Grid<R>& gd, unsigned i, unsigned feat) {
    CellIn<R> a;
    a.hu0 = gd.hu[i];
    a.hv0 = gd.hv[i];
    if (STAGE == 2) {
        a.h0 = gd.h[i];
        a.hu1 = gd.hu1[i];
        a.hv1 = gd.hv1[i];
    } else {
        a.h0 = a.hu1 = a.hv1 = R(0);
    }
    if (STAGE != 1) {
        const bool hs = feat & FEAT_STORE, hf = feat & FEAT_HORTON;
        a.sf = hs ? gd.sf[i] : R(0);
        a.S = hs ? gd.S[i] : R(0);
        a.ic = hf ? gd.ic[i] : R(0);
        a.f0 = hf ? gd.f0[i] : R(0);
        a.fc = hf ? gd.fc[i] : R(0);
        a.k = hf ? gd.k[i] : R(0);
        a.n = gd.n[i];
        a.rw = (feat & FEAT_RAINW) ? gd.rw[i] : R(0);
    } else {
        a.sf = a.S = a.ic = a.f0 = a.fc = a.k = a.n = a.rw = R(0);
    }
    return a;
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

// Block reduction of NV per-thread values in the compute type T (warps by shuffles,
// then lane j of warp 0 over the warps in order), one float64 store per value.
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

// One side of a reconstructed cell as a face sees it: depth, normal and tangential
// velocity, and X = the recovered bed (float64) or the in-cell bed slope d (float32),
// S = the in-cell surface slope sE (float32).  The cell's own bed z and depth h0 (the
// float32 flux's difference form) come with the cell record.
template <class R>
struct Side {
    R H, U, V, X, S;
};
template <class R>
__device__ __forceinline__ Side<R> side_plus(const Recon<R>& r) {
    if constexpr (sizeof(R) == 8) return Side<R>{r.Hp, r.Up, r.Vp, r.Zp, R(0)};
    else return Side<R>{r.Hp, r.Up, r.Vp, r.d, r.sE};
}
template <class R>
__device__ __forceinline__ Side<R> side_minus(const Recon<R>& r) {
    if constexpr (sizeof(R) == 8) return Side<R>{r.Hm, r.Um, r.Vm, r.Zm, R(0)};
    else return Side<R>{r.Hm, r.Um, r.Vm, r.d, r.sE};
}

// Face flux from the plus side of the cell below / west of the face (bed zl, depth hl)
// and the minus side of the cell above / east of it: face_flux's arithmetic exactly.
template <class R>
__device__ __forceinline__ Q4<R> side_flux(const KC<R>& c, const Side<R>& L, R zl, R hl, const Side<R>& Rt, R zr,
                                           R hr) {
    Recon<R> a, b;
    a.Hp = L.H; a.Up = L.U; a.Vp = L.V;
    b.Hm = Rt.H; b.Um = Rt.U; b.Vm = Rt.V;
    if constexpr (sizeof(R) == 8) {
        a.Zp = L.X; b.Zm = Rt.X;
    } else {
        a.d = L.X; a.sE = L.S; a.z = zl; a.h0 = hl;
        b.d = Rt.X; b.sE = Rt.S; b.z = zr; b.h0 = hr;
    }
    (void)zl; (void)hl; (void)zr; (void)hr;
    Q4<R> f;
    face_flux(c, a, b, f.a, f.b, f.c, f.d);
    return f;
}

// The row-marching pipeline of one strip chunk (see the head of this file).  Row r is
// the newest row built; per row two barriers separate the phases:
//   A  build row r into the cell ring, prefetch row r+1 and the update inputs of row
//      r-3; y-reconstruction of row r-1 and the y-face between rows r-2 and r-1;
//      x-reconstruction of row r-2 from its neighbours' cells, plus side published
//   -- barrier --
//   B  x-face between columns cx-1 and cx of row r-2, published
//   -- barrier --
//   C  theta of row r-2, published
//   D  update of row r-3 from the rings' entries of rows r-4 .. r-2
// row<true> is the steady state: every row touched lies inside the grid, so the
// range tests, y-ghosts and domain-edge terms drop out; row<false> handles the
// pipeline fill at the chunk's start, the drain at its end and the grid's edges.
template <class R, int NT, int STAGE>
struct StripPipe {
    using G = StripGeom<R, NT>;
    static constexpr int P = G::P;
    static constexpr int RM = G::RING - 1;
    Q4<R>* s_cell;
    Q4<R>* s_rp;
    Q4<R>* s_xf;
    Q4<R>* s_yf;
    R* s_rs;
    R* s_th;
    const Grid<R>& gd;
    const KC<R>& c;
    const R* bcv;
    float* const* s_snap;
    const R* __restrict__ H;
    const R* __restrict__ HU;
    const R* __restrict__ HV;
    int ts, cx, cxc, nx, ny, y0, y1, scol, xside, xkind;
    unsigned feat;                     // FEAT_* bits of the member's optional fields
    bool col_in, do_out, west, east;
    R dt, rdx, rdy, idx, idy, rdt, tt;
    // carried state of this thread's column
    HaloRaw<R> ra;                     // raw row r (prefetched one row ahead)
    Side<R> ylow;                      // plus side of the y-reconstruction of row r-2
    R by1, by2, bx1;                   // bed terms: y of rows r-2, r-3; x of row r-3
    CellIn<R> cin;
    R acc_clip, xin, xout, yin, yout, infil, rainw, rate, hsum, ssum, hmax;

    // Raw values of an interior row at this thread's source column (its own column, or
    // the layer an x-ghost copies)
    __device__ __forceinline__ HaloRaw<R> fetch_in(int gy) const {
        const unsigned i = (unsigned)gy * (unsigned)nx + (unsigned)scol;
        return HaloRaw<R>{H[i], HU[i], HV[i], gd.z[i]};
    }
    // halo_build for a row inside the grid: an interior cell, or the x-ghost that the
    // x-sweep would see (boundaries.py:81-128)
    __device__ __forceinline__ Q4<R> build_in(const HaloRaw<R>& a) const {
        R u0, v0;
        kp_velocity(c, a.h, a.hu, a.hv, u0, v0);
        if (xkind < 0) return Q4<R>{a.h, u0, v0, a.z};
        const R sgn = xside == EDGE_W ? R(-1) : R(1);
        const R un = sgn * u0, ut = v0;
        R hg, ung, utg;
        if (xkind == BC_CLOSED) { hg = a.h; ung = -un; utg = ut; }
        else if (xkind == BC_TRANSMISSIVE) { hg = a.h; ung = un; utg = ut; }
        else if (xkind == BC_STAGE) stage_ghost(c, bcv[xside], a.h, un, ut, a.z, hg, ung, utg);
        else discharge_ghost(c, bcv[xside], a.h, hg, ung, utg);
        return Q4<R>{hg, sgn * ung, utg, a.z};
    }

    template <bool FULL>
    __device__ __forceinline__ void row(const int r) {
        const int k0 = (r & RM) * P, k1 = ((r - 1) & RM) * P, k2 = ((r - 2) & RM) * P, k3 = ((r - 3) & RM) * P,
                  k4 = ((r - 4) & RM) * P;
        const int xo = ((r - 2) & 1) * P, xp = ((r - 3) & 1) * P;
        const int orow = r - 3, row = r - 2;
        const bool upd = FULL || (orow >= y0 && orow < y1);
        // ---- A: row r, prefetches, y-face r-1, x-reconstruction of row r-2
        Q4<R> c0;
        if (FULL) {
            c0 = build_in(ra);
        } else {
            halo_build(c, gd, bcv, ra, cx, r, c0.a, c0.b, c0.c, c0.d);
        }
        s_cell[k0 + ts] = c0;
        ra = FULL ? fetch_in(r + 1) : halo_fetch(c, gd, H, HU, HV, cx, r + 1);
        if (upd) cin = cell_fetch<R, STAGE>(gd, (unsigned)orow * (unsigned)nx + (unsigned)cxc, feat);
        R by0 = R(0), bx0 = R(0);
        const Q4<R> c2 = s_cell[k2 + ts];           // own cells of rows r-2 and r-1
        const Q4<R> c1 = s_cell[k1 + ts];
        // y-reconstruction of row r-1 (normal velocity v, tangential u); its face with
        // row r-2 is formed in phase B beside the x-face, two independent chains
        const bool yact = FULL || r >= y0 - 1;
        Side<R> ylo = ylow, yum;
        if (yact) {
            const Recon<R> yup = reconstruct(c, c2.a, c1.a, c0.a, c2.c, c1.c, c0.c, c2.b, c1.b, c0.b, c2.d, c1.d, c0.d);
            yum = side_minus(yup);
            ylow = side_plus(yup);
            if (c.order == 2) by0 = bed_term(c, yup);
        }
        const bool xact = FULL || (r >= y0 + 1 && (unsigned)row < (unsigned)ny);
        Q4<R> cl;
        Side<R> xm;
        if (xact) {
            cl = s_cell[k2 + ts - 1];
            const Q4<R> cr = s_cell[k2 + ts + 1];
            const Recon<R> xr = reconstruct(c, cl.a, c2.a, cr.a, cl.b, c2.b, cr.b, cl.c, c2.c, cr.c, cl.d, c2.d, cr.d);
            const Side<R> xp_ = side_plus(xr);
            s_rp[ts] = Q4<R>{xp_.H, xp_.U, xp_.V, xp_.X};
            if constexpr (sizeof(R) == 4) s_rs[ts] = xp_.S;
            xm = side_minus(xr);
            if (c.order == 2) bx0 = bed_term(c, xr);
        }
        __syncthreads();
        // ---- B: y-face between rows r-2 and r-1; x-face between columns cx-1 and cx of row r-2
        Q4<R> yf0{R(0), R(0), R(0), R(0)};
        if (yact) {
            const int fy = r - 1;
            if (FULL || (r >= y0 && fy >= 0 && fy <= ny)) yf0 = side_flux(c, ylo, c2.d, c2.a, yum, c1.d, c1.a);
            if (FULL || r >= y0) s_yf[k1 + ts] = yf0;
        }
        Q4<R> xf0{R(0), R(0), R(0), R(0)};
        if (xact) {
            const Q4<R> lp = s_rp[ts - 1];
            Side<R> L{lp.a, lp.b, lp.c, lp.d, R(0)};
            if constexpr (sizeof(R) == 4) L.S = s_rs[ts - 1];
            xf0 = side_flux(c, L, cl.d, cl.a, xm, c2.d, c2.a);
            s_xf[xo + ts] = xf0;
        }
        __syncthreads();
        // ---- C: theta of row r-2 (swe2d.py:259-264); 1 outside the grid
        R th0 = R(1);
        Q4<R> yn{R(0), R(0), R(0), R(0)};          // y-face r-2: south of row r-2, north of row r-3
        if (FULL || r >= y0 + 1) {
            yn = s_yf[k2 + ts];
            if (FULL || (unsigned)row < (unsigned)ny) {
                const R Fw = xf0.a, Fe = s_xf[xo + ts + 1].a, Gs = yn.a, Gn = yf0.a;
                const R out = per_len(relu(Fe) + relu(-Fw), rdx, idx) + per_len(relu(Gn) + relu(-Gs), rdy, idy);
                const R need = out * dt;
                const R hh = c2.a;
                const R th = need > hh ? hh / (need > R(0) ? need : R(1)) : R(1);
                th0 = col_in ? th : R(1);
            }
            s_th[k2 + ts] = th0;
        }
        // ---- D: update of row r-3
        if (upd) update<FULL>(orow, xp, k3, k4, th0, yn);
        by2 = by1;
        by1 = by0;
        bx1 = bx0;
    }

    template <bool FULL>
    __device__ __forceinline__ void update(const int orow, const int xp, const int k3, const int k4, const R thN,
                                           const Q4<R>& yn) {
        const R thC = s_th[k3 + ts], thS = s_th[k4 + ts];
        const R thW = s_th[k3 + ts - 1], thE = s_th[k3 + ts + 1];
        const Q4<R> xw = s_xf[xp + ts], xe = s_xf[xp + ts + 1], ys = s_yf[k3 + ts];
        const R h3 = s_cell[k3 + ts].a;
        const R Fw = xw.a, Fe = xe.a, Gs = ys.a, Gn = yn.a;
        const R sw = Fw > R(0) ? thW : thC, se = Fe > R(0) ? thC : thE;
        const R ss = Gs > R(0) ? thS : thC, sn = Gn > R(0) ? thC : thN;
        const R F1w = Fw * sw, F1e = Fe * se, G1s = Gs * ss, G1n = Gn * sn;
        R a1 = per_len(-(F1e - F1w), rdx, idx);
        R a2 = per_len(-(xe.b - xw.c), rdx, idx);
        R a3 = per_len(-(xe.d * se - xw.d * sw), rdx, idx);
        R b1 = per_len(-(G1n - G1s), rdy, idy);
        R b2 = per_len(-(yn.b - ys.c), rdy, idy);
        R b3 = per_len(-(yn.d * sn - ys.d * ss), rdy, idy);
        if (c.order == 2) {
            a2 = a2 + per_len(bx1, rdx, idx);
            b2 = b2 + per_len(by2, rdy, idy);
        }
        const R dh = a1 + b1, dhu = a2 + b3, dhv = a3 + b2;
        if (!do_out) return;
        if (west) { xin += relu(F1w); xout += relu(-F1w); }
        if (east) { xin += relu(-F1e); xout += relu(F1e); }
        if (!FULL) {
            if (orow == 0) { yin += relu(G1s); yout += relu(-G1s); }
            if (orow == ny - 1) { yin += relu(-G1n); yout += relu(G1n); }
        }
        const unsigned i = (unsigned)orow * (unsigned)nx + (unsigned)cx;
        R hn, hun, hvn;
        if (STAGE == 2) {
            hn = R(0.5) * (cin.h0 + h3 + dt * dh);
            hun = R(0.5) * (cin.hu0 + cin.hu1 + dt * dhu);
            hvn = R(0.5) * (cin.hv0 + cin.hv1 + dt * dhv);
        } else {
            hn = h3 + dt * dh;
            hun = cin.hu0 + dt * dhu;
            hvn = cin.hv0 + dt * dhv;
        }
        const R neg = clamp0(-hn);
        acc_clip += neg;
        hn = hn + neg;
        if (STAGE == 1) {
            gd.h1[i] = hn; gd.hu1[i] = hun; gd.hv1[i] = hvn;
            return;
        }
        // ---- rain, Horton infiltration, retention store (swe2d.py:330-360)
        R sf = cin.sf;
        if (feat & FEAT_RAINW) {
            const R add = rdt * cin.rw;
            hn = hn + add;
            rainw += add;
        } else {
            hn = hn + rdt;
        }
        if (feat & FEAT_HORTON) {
            const R rate_f = cin.fc + (cin.f0 - cin.fc) * rexp(-cin.k * tt);
            const R pot = rate_f * dt;
            const R take = rmin(pot, hn);
            const R safe = hn > R(0) ? hn : R(1);
            const R scale = hn > R(0) ? (hn - take) / safe : R(0);
            hn = hn - take;
            hun = hun * scale;
            hvn = hvn * scale;
            R taken = take;
            if (feat & FEAT_STORE) {
                const R tks = rmin(pot - take, sf);
                sf = sf - tks;
                taken = taken + tks;
            }
            infil += taken;
            gd.ic[i] = cin.ic + taken;
        }
        if (feat & FEAT_STORE) {
            const R room = clamp0(cin.S - sf);
            const R fill = rmin(room, hn);
            const R safe = hn > R(0) ? hn : R(1);
            const R scale = hn > R(0) ? (hn - fill) / safe : R(0);
            hn = hn - fill;
            hun = hun * scale;
            hvn = hvn * scale;
            sf = sf + fill;
            gd.sf[i] = sf;
        }
        // ---- semi-implicit Manning friction (swe2d.py:362-370)
        R u, v, ks = R(0);
        if constexpr (sizeof(R) == 4) {
            // KP factor of the new depth, kept for the CFL velocity below
            const float h2 = hn * hn, h4 = h2 * h2;
            ks = hn >= c.h_dry ? 1.4142135623730951f * hn * rsqrtf(h4 + fmaxf(h4, c.kp_eps)) : 0.0f;
            u = hun * ks;
            v = hvn * ks;
        } else {
            kp_velocity(c, hn, hun, hvn, u, v);
        }
        const R speed = dsqrt(u * u + v * v);
        const R hf = rmax(hn, c.h_dry);
        const R nm = cin.n;
        const R denom = R(1) + dt * c.g * nm * nm * speed / pow43(hf);
        u = u / denom;
        v = v / denom;
        const bool wet = hn >= c.h_dry;
        hun = wet ? hn * u : R(0);
        hvn = wet ? hn * v : R(0);
        if (STAGE == 2) {
            gd.h[i] = hn; gd.hu[i] = hun; gd.hv[i] = hvn;
        } else {
            gd.h1[i] = hn; gd.hu1[i] = hun; gd.hv1[i] = hvn;
        }
        if (feat & FEAT_PEAK) gd.pk[i] = rmax(gd.pk[i], hn);
        // ---- CFL rate of the new state for the next step (swe2d.py:179-184)
        R u2, v2;
        if constexpr (sizeof(R) == 4) {
            u2 = hun * ks;
            v2 = hvn * ks;
        } else {
            kp_velocity(c, hn, hun, hvn, u2, v2);
        }
        // running peak speed and output use the KP velocities of the new state, as the
        // reference's snapshots do (swe2d.py:161-167, coupling.py:229-242)
        if (feat & FEAT_PSPEED) gd.ps[i] = rmax(gd.ps[i], dsqrt(u2 * u2 + v2 * v2));
        if (feat & FEAT_SNAP) {
            s_snap[0][i] = (float)hn;
            s_snap[1][i] = (float)u2;
            s_snap[2][i] = (float)v2;
        }
        const R cw = dsqrt(c.g * hn);
        const R rr = hn > c.h_dry ? per_len(fabs(u2) + cw, rdx, idx) + per_len(fabs(v2) + cw, rdy, idy) : R(0);
        rate = rmax(rate, rr);
        hsum += hn;
        ssum += sf;
        hmax = rmax(hmax, hn);
    }
};

// Source column of an x-ghost: the layer of the grid it copies (boundaries.py:104-116),
// as halo_fetch picks it; the column itself inside the grid.
template <class R>
__device__ __forceinline__ int ghost_source_column(const KC<R>& c, const Grid<R>& gd, int cx) {
    const int nx = gd.nx;
    if ((unsigned)cx < (unsigned)nx) return cx;
    const int ng = c.order == 1 ? 1 : 2;
    const bool lo = cx < 0;
    const int k = lo ? (-cx - 1) : (cx - nx);
    const int kind = gd.bc[lo ? EDGE_W : EDGE_E];
    int layer;
    if (kind == BC_CLOSED || kind == BC_TRANSMISSIVE) layer = nx < ng ? (lo ? 0 : nx - 1) : (lo ? k : nx - 1 - k);
    else layer = lo ? 0 : nx - 1;
    return layer < 0 ? 0 : (layer > nx - 1 ? nx - 1 : layer);
}

// STAGE: 0 = first-order full step, 1 = RK stage 1, 2 = RK stage 2 + sources.
// Stage 1 writes the stage buffers; stage 2 reads them in its halo and writes the
// state.  The first-order step reads the state in its halo, so it writes its result
// to the stage buffers and stage_copy_kernel moves it back (no CTA overwrites cells
// that another CTA may still read).
template <class R, int NT, int STAGE>
__global__ void __launch_bounds__(NT, StripGeom<R, NT>::min_ctas(STAGE)) strip_kernel(const Grid<R>* __restrict__ grids,
                                                    const StripRef* __restrict__ strips,
                                                    const StepParams* __restrict__ params, const KC<R> kc,
                                                    double* __restrict__ partials) {
    using G = StripGeom<R, NT>;
    // the stages of the second-order method (1, 2) and the first-order step (0) are
    // launched for their order only, so the order is a constant of the instantiation
    KC<R> c = kc;
    c.order = STAGE == 0 ? 1 : 2;
    constexpr int P = G::P;
    extern __shared__ __align__(32) unsigned char smem_raw[];
    __shared__ R bcv[4];
    __shared__ float* s_snap[3];                      // output slots of this step (stage 0 / 2)
    // the member's record, staged once: its field pointers are re-read every row, and
    // from global memory those reads stall the row loop
    __shared__ __align__(16) Grid<R> s_gd;

    const StripRef sr = strips[blockIdx.x];
    const StepParams& pr = params[sr.member];
    if (!pr.active) return;
    const int t = threadIdx.x;
    {
        static_assert(sizeof(Grid<R>) % 4 == 0, "record copied as 32-bit words");
        const unsigned* src = reinterpret_cast<const unsigned*>(grids + sr.member);
        unsigned* dst = reinterpret_cast<unsigned*>(&s_gd);
        for (int k = t; k < (int)(sizeof(Grid<R>) / 4); k += NT) dst[k] = src[k];
    }
    if (t < 4) bcv[t] = par_bc<R>(pr, STAGE == 2, t);
    if (t == 0) {
        s_snap[0] = STAGE != 1 ? pr.snap_h : nullptr;
        s_snap[1] = pr.snap_u;
        s_snap[2] = pr.snap_v;
    }
    __syncthreads();
    const Grid<R>& gd = s_gd;
    Q4<R>* s_cell = reinterpret_cast<Q4<R>*>(smem_raw);
    Q4<R>* s_rp = s_cell + G::RING * P;
    Q4<R>* s_xf = s_rp + P;
    Q4<R>* s_yf = s_xf + 2 * P;
    R* s_rs = reinterpret_cast<R*>(s_yf + G::RING * P);
    R* s_th = s_rs + P;
    StripPipe<R, NT, STAGE> pp{s_cell, s_rp, s_xf, s_yf, s_rs, s_th, gd, c, bcv, s_snap,
                               STAGE == 2 ? gd.h1 : gd.h, STAGE == 2 ? gd.hu1 : gd.hu, STAGE == 2 ? gd.hv1 : gd.hv};
    const int nx = gd.nx, ny = gd.ny;
    const int x0 = sr.x0, W = sr.w, y0 = sr.y0, y1 = sr.y1;
    const int cx = x0 - 3 + t;                        // this thread's column
    const int q = cx - x0;                            // column relative to the strip
    pp.ts = t + 1;
    pp.feat = grid_features(gd) | (s_snap[0] ? FEAT_SNAP : 0u);      // FEAT_SNAP: outputs due this step
    pp.cx = cx;
    pp.cxc = cx < 0 ? 0 : (cx > nx - 1 ? nx - 1 : cx);
    pp.nx = nx;
    pp.ny = ny;
    pp.y0 = y0;
    pp.y1 = y1;
    pp.col_in = (unsigned)cx < (unsigned)nx;
    pp.do_out = q >= 0 && q < W && pp.col_in;
    pp.west = cx == 0;
    pp.east = cx == nx - 1;
    pp.scol = ghost_source_column(c, gd, cx);
    pp.xside = cx < 0 ? EDGE_W : EDGE_E;
    pp.xkind = pp.col_in ? -1 : gd.bc[pp.xside];
    pp.dt = par_dt<R>(pr);
    pp.rdx = gd.rdx;
    pp.rdy = gd.rdy;
    pp.idx = gd.idx;
    pp.idy = gd.idy;
    pp.rdt = par_rain<R>(pr) * pp.dt;
    pp.tt = clamp0(par_t<R>(pr) - gd.rt0);
    pp.acc_clip = pp.xin = pp.xout = pp.yin = pp.yout = pp.infil = pp.rainw = pp.rate = pp.hsum = pp.ssum = R(0);
    pp.hmax = R(0);
    pp.by1 = pp.by2 = pp.bx1 = R(0);
    // software pipeline: raw rows are fetched one row ahead
    pp.ra = halo_fetch(c, gd, pp.H, pp.HU, pp.HV, cx, y0 - 3);
    static_assert((G::RING & (G::RING - 1)) == 0, "ring slots are row & (RING - 1)");
    // steady-state rows: every row touched (r-4 .. r+1) inside the grid, the update row
    // neither the first nor the last row of the grid
    const int r_lo = max(y0 + 3, 4), r_hi = min(y1 + 2, ny - 2);
    int r = y0 - 3;
    for (; r <= y1 + 2 && r < r_lo; ++r) pp.template row<false>(r);
    // (not unrolled: four copies of the row body ran 1.75x slower, the hot loop no
    // longer fitting the instruction cache beside the other member chains' kernels)
    for (; r <= r_hi; ++r) pp.template row<true>(r);
    for (; r <= y1 + 2; ++r) pp.template row<false>(r);
    __syncthreads();
    R* red = reinterpret_cast<R*>(smem_raw);
    double* out = partials + (size_t)blockIdx.x * NPART;
    if (STAGE == 1) {
        R v[5] = {pp.acc_clip, pp.xin, pp.xout, pp.yin, pp.yout};
        const bool mx[5] = {false, false, false, false, false};
        const int sl[5] = {P_CLIP1, P_XIN1, P_XOUT1, P_YIN1, P_YOUT1};
        block_reduce_store<5>(v, mx, red, out, sl, NT);
    } else {
        const int b = STAGE == 2 ? P_CLIP2 : P_CLIP1;
        R v[11] = {pp.acc_clip, pp.xin, pp.xout, pp.yin, pp.yout, pp.infil, pp.rainw, pp.rate, pp.hsum, pp.ssum,
                   pp.hmax};
        const bool mx[11] = {false, false, false, false, false, false, false, true, false, false, true};
        const int sl[11] = {b, b + 1, b + 2, b + 3, b + 4, P_INFIL, P_RAINW, P_RATE, P_HSUM, P_SSUM, P_HMAX};
        block_reduce_store<11>(v, mx, red, out, sl, NT);
    }
}

// First-order step: move the result from the stage buffers back to the state.
template <class R, int NT>
__global__ void __launch_bounds__(NT) stage_copy_kernel(const Grid<R>* __restrict__ grids,
                                                         const StripRef* __restrict__ strips,
                                                         const StepParams* __restrict__ params) {
    const StripRef sr = strips[blockIdx.x];
    const Grid<R>& gd = grids[sr.member];
    if (!params[sr.member].active) return;
    const int cx = sr.x0 + threadIdx.x;
    if ((int)threadIdx.x >= sr.w || cx >= gd.nx) return;
    for (int y = sr.y0; y < sr.y1; ++y) {
        const size_t i = (size_t)y * gd.nx + cx;
        gd.h[i] = gd.h1[i];
        gd.hu[i] = gd.hu1[i];
        gd.hv[i] = gd.hv1[i];
    }
}

// Per strip-chunk CFL rate, surface and retained water of the current state (float64 sums).
template <class R, int NT>
__global__ void __launch_bounds__(NT) strip_reduce_kernel(const Grid<R>* __restrict__ grids,
                                                           const StripRef* __restrict__ strips, const KC<R> c,
                                                           double* __restrict__ partials) {
    __shared__ double red[32 * 3];
    const StripRef sr = strips[blockIdx.x];
    const Grid<R>& gd = grids[sr.member];
    double rate = 0, hs = 0, ss = 0;
    const int cx = sr.x0 + threadIdx.x;
    if ((int)threadIdx.x < sr.w && cx < gd.nx) {
        for (int y = sr.y0; y < sr.y1 && y < gd.ny; ++y) {
            const size_t i = (size_t)y * gd.nx + cx;
            R h = gd.h[i], u, v;
            kp_velocity(c, h, gd.hu[i], gd.hv[i], u, v);
            const R cw = dsqrt(c.g * h);
            const R r = h > c.h_dry ? per_len(fabs(u) + cw, gd.rdx, gd.idx) + per_len(fabs(v) + cw, gd.rdy, gd.idy)
                                    : R(0);
            rate = fmax(rate, (double)r);
            hs += (double)h;
            ss += (double)gd.sf[i];
        }
    }
    double v[3] = {rate, hs, ss};
    const bool mx[3] = {true, false, false};
    const int sl[3] = {P_RATE, P_HSUM, P_SSUM};
    block_reduce_store<3>(v, mx, red, partials + (size_t)blockIdx.x * NPART, sl, NT);
}

// Per strip-chunk CFL rate alone (swe2d.py:179-184), for the step's dt: the maximum
// is exact in the compute type, so the cells need no float64 work (slow on this GPU)
// and the result equals strip_reduce_kernel's; rows are unrolled to keep loads in
// flight.  Writes only the P_RATE partial.
template <class R, int NT>
__global__ void __launch_bounds__(NT) strip_rate_kernel(const Grid<R>* __restrict__ grids,
                                                         const StripRef* __restrict__ strips, const KC<R> c,
                                                         double* __restrict__ partials) {
    __shared__ R red[32];
    const StripRef sr = strips[blockIdx.x];
    const Grid<R>& gd = grids[sr.member];
    R rate = R(0);
    const int cx = sr.x0 + threadIdx.x;
    if ((int)threadIdx.x < sr.w && cx < gd.nx) {
        const int y1 = min(sr.y1, gd.ny);
#pragma unroll 4
        for (int y = sr.y0; y < y1; ++y) {
            const size_t i = (size_t)y * gd.nx + cx;
            R h = gd.h[i], u, v;
            kp_velocity(c, h, gd.hu[i], gd.hv[i], u, v);
            const R cw = dsqrt(c.g * h);
            const R r = h > c.h_dry ? per_len(fabs(u) + cw, gd.rdx, gd.idx) + per_len(fabs(v) + cw, gd.rdy, gd.idy)
                                    : R(0);
            rate = rmax(rate, r);
        }
    }
    R v[1] = {rate};
    const bool mx[1] = {true};
    const int sl[1] = {P_RATE};
    block_reduce_store<1>(v, mx, red, partials + (size_t)blockIdx.x * NPART, sl, NT);
}

// Per-member totals from the strip-chunk partials, in a fixed order.  out: 8 per
// member = bnd_in, bnd_out, rain, infil, clip (m^3), rate (1/s), surface and retained
// volume.  mode 0: after a step; mode 1: rate and volumes only; mode 2: rate only
// (after strip_rate_kernel).  ext (optional, device-writable): mode 0 the 5 volumes,
// modes 1 and 2 the rate, per member.  ledger (optional, mode 0): an 8 x n_members
// float64 ledger (rows LG_*) the step's rain, infiltration, boundary and clip volumes
// are added into.
template <class R>
__global__ void finalize_kernel(const Grid<R>* __restrict__ grids, const StepParams* __restrict__ params, Consts c,
                                const double* __restrict__ partials, double* __restrict__ out, int mode,
                                double* __restrict__ ext, double* __restrict__ ledger = nullptr) {
    const int m = blockIdx.x, lane = threadIdx.x;
    const Grid<R>& gd = grids[m];
    if (mode == 0 && !params[m].active) return;
    if (mode == 2) {
        double r = 0.0;
        for (int t = lane; t < gd.n_tiles; t += 32) r = fmax(r, partials[(size_t)(gd.tile0 + t) * NPART + P_RATE]);
        r = warp_max(r);
        if (lane == 0) {
            out[(size_t)m * 8 + 5] = r;
            if (ext) ext[m] = r;
        }
        return;
    }
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
    if (mode != 0) {
        if (ext) ext[m] = s[P_RATE];
        return;
    }
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
    if (ext) {
#pragma unroll
        for (int j = 0; j < 5; ++j) ext[(size_t)m * 5 + j] = o[j];
    }
    if (ledger) {
        const size_t B = gridDim.x;
        ledger[LG_RAIN * B + m] += o[2];
        ledger[LG_INFIL * B + m] += o[3];
        ledger[LG_BND2_IN * B + m] += o[0];
        ledger[LG_BND2_OUT * B + m] += o[1];
        ledger[LG_CLIP2 * B + m] += o[4];
    }
}

}  // namespace his
