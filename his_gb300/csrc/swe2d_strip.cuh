// 2-D finite-volume step kernels: row-marching strips.
//
// A CTA of NT threads owns a strip of W <= NT - 6 columns of one member and marches
// up a chunk of rows [y0, y1).  Thread t works on column cx = x0 - 3 + t.  Per new
// row r it
//   P1  loads row r of (h, u, v, z) into a ring of 8 rows (ghost cells built at the
//       domain edges, boundaries.py:81-128),
//   P2  computes the y-face between rows r-2 and r-1 (the lower cell's
//       y-reconstruction is carried in registers from the previous row) and the
//       x-reconstruction of row r-2,
//   P3  computes the x-faces of row r-2,
//   P4  computes the positivity-limiter theta of row r-2 (swe2d.py:259-264),
//   P5  updates row r-3 (divergence of the donor-scaled fluxes, bed source, RK
//       stage, then in the last stage rain, infiltration, retention, friction, CFL
//       rate and peaks; swe2d.py:305-371).
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

// Shared-memory layout of one CTA
template <class R, int NT>
struct StripGeom {
    static constexpr int RING = 4;                 // cell rows kept (rows r-3 .. r are live)
    static constexpr int FR = 4;                   // y-face and theta rows kept (3 live)
    static constexpr int FRX = 2;                  // x-face rows kept (2 live)
    static constexpr int NRED = 11;                // reduced values (the reduction reuses the cell ring)
    static constexpr size_t quads = (size_t)(RING + 2 + FRX + FR) * NT;
    static constexpr size_t th = (size_t)FR * NT;
    static_assert((size_t)4 * RING * NT >= (size_t)32 * NRED, "reduction scratch must fit in the cell ring");
    static constexpr size_t smem_bytes = sizeof(Q4<R>) * quads + sizeof(R) * th;
    // resident CTAs per SM the float32 kernels are register-capped for (shared memory
    // allows 14 of 64 threads): about 768 threads' worth for stage 1 and 640 for the
    // larger stage-2 body, so that they keep their live values in registers.  With the
    // engine's member chains running side by side this beat tighter caps (896 / 768:
    // 0.474 against 0.466 ms per step at 64 x 400 x 325) and looser ones (640 / 512:
    // 0.502 ms).  float64 keeps the compiler's choice (one CTA of any width must fit
    // the register file)
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
    size_t i;
    if (inx && iny) {
        i = (size_t)gy * nx + gx;
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
        i = alongx ? (size_t)gy * nx + layer : (size_t)layer * nx + gx;
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

template <class R, int STAGE>
__device__ __forceinline__ CellIn<R> cell_fetch(const Grid<R>& gd, size_t i) {
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
        a.sf = gd.S ? gd.sf[i] : R(0);
        a.S = gd.S ? gd.S[i] : R(0);
        a.ic = gd.f0 ? gd.ic[i] : R(0);
        a.f0 = gd.f0 ? gd.f0[i] : R(0);
        a.fc = gd.f0 ? gd.fc[i] : R(0);
        a.k = gd.f0 ? gd.k[i] : R(0);
        a.n = gd.n[i];
        a.rw = gd.rw ? gd.rw[i] : R(0);
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

// x-reconstruction of one cell in shared memory (two records at xr[t] and xr[NT + t]);
// the float32 form's cell depth and bed come from the cell record (h0, z).
template <class R>
__device__ __forceinline__ void store_recon(Q4<R>* xr, int t, int nt, const Recon<R>& r) {
    xr[t] = Q4<R>{r.Hm, r.Hp, r.Um, r.Up};
    if constexpr (sizeof(R) == 8) xr[nt + t] = Q4<R>{r.Vm, r.Vp, r.Zm, r.Zp};
    else xr[nt + t] = Q4<R>{r.Vm, r.Vp, r.d, r.sE};
}

template <class R>
__device__ __forceinline__ Recon<R> load_recon(const Q4<R>* xr, int t, int nt, R h0, R z) {
    const Q4<R> p = xr[t], q = xr[nt + t];
    Recon<R> r;
    r.Hm = p.a; r.Hp = p.b; r.Um = p.c; r.Up = p.d;
    r.Vm = q.a; r.Vp = q.b;
    if constexpr (sizeof(R) == 8) {
        r.Zm = q.c; r.Zp = q.d;
        r.z = r.d = r.h0 = r.sE = R(0);
    } else {
        r.d = q.c; r.sE = q.d;
        r.z = z; r.h0 = h0;
        r.Zm = r.Zp = R(0);
    }
    return r;
}

// STAGE: 0 = first-order full step, 1 = RK stage 1, 2 = RK stage 2 + sources.
// Stage 1 writes the stage buffers; stage 2 reads them in its halo and writes the
// state.  The first-order step reads the state in its halo, so it writes its result
// to the stage buffers and stage_copy_kernel moves it back (no CTA overwrites cells
// that another CTA may still read).
template <class R, int NT, int STAGE>
__global__ void __launch_bounds__(NT, StripGeom<R, NT>::min_ctas(STAGE)) strip_kernel(const Grid<R>* __restrict__ grids,
                                                    const StripRef* __restrict__ strips,
                                                    const StepParams* __restrict__ params, const KC<R> c,
                                                    double* __restrict__ partials) {
    using G = StripGeom<R, NT>;
    extern __shared__ __align__(32) unsigned char smem_raw[];
    Q4<R>* s_cell = reinterpret_cast<Q4<R>*>(smem_raw);   // [RING][NT] {h, u, v, z}
    Q4<R>* s_xr = s_cell + G::RING * NT;                  // [2][NT] x-reconstruction
    Q4<R>* s_xf = s_xr + 2 * NT;                          // [FRX][NT] x-faces {F1, F2L, F2R, F3}
    Q4<R>* s_yf = s_xf + G::FRX * NT;                     // [FR][NT] y-faces
    R* s_th = reinterpret_cast<R*>(s_yf + G::FR * NT);    // [FR][NT] theta
    R* red = reinterpret_cast<R*>(smem_raw);              // after the row loop
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
    __syncthreads();
    const Grid<R>& gd = s_gd;
    const int nx = gd.nx, ny = gd.ny;
    const int x0 = sr.x0, W = sr.w, y0 = sr.y0, y1 = sr.y1;
    const int cx = x0 - 3 + t;                        // this thread's column
    const R dt = par_dt<R>(pr);
    if (t < 4) bcv[t] = par_bc<R>(pr, STAGE == 2, t);
    if (t == 0) {
        s_snap[0] = STAGE != 1 ? pr.snap_h : nullptr;
        s_snap[1] = pr.snap_u;
        s_snap[2] = pr.snap_v;
    }
    const R* __restrict__ H = STAGE == 2 ? gd.h1 : gd.h;
    const R* __restrict__ HU = STAGE == 2 ? gd.hu1 : gd.hu;
    const R* __restrict__ HV = STAGE == 2 ? gd.hv1 : gd.hv;
    const R rdx = gd.rdx, rdy = gd.rdy, idx = gd.idx, idy = gd.idy;
    const R rdt = par_rain<R>(pr) * dt;
    const R tt = clamp0(par_t<R>(pr) - gd.rt0);
    const bool col_in = (unsigned)cx < (unsigned)nx;
    const int q = cx - x0;                                      // column relative to the strip
    const bool do_yface = q >= -1 && q <= W && col_in;
    const bool do_xrec = q >= -2 && q <= W + 1;
    const bool do_xface = q >= -1 && q <= W + 1 && cx >= 0 && cx <= nx;
    const bool do_theta = q >= -1 && q <= W;                    // theta = 1 outside the domain
    const bool do_out = q >= 0 && q < W && col_in;

    R acc_clip = 0, xin = 0, xout = 0, yin = 0, yout = 0, infil = 0, rainw = 0, rate = 0, hsum = 0, ssum = 0;
    R hmax = 0;
    Recon<R> ylow;                                   // y-reconstruction of row r-2 (carried)
    R by1 = R(0), by2 = R(0);                        // y bed terms of rows r-2 and r-3
    R bxc = R(0);                                    // x bed term of row r-3
    R h_r3 = R(0);                                   // depth of this column in row r-3
    // software pipeline: halo rows are fetched two rows ahead, update inputs at the start
    // of the iteration that uses them
    HaloRaw<R> ra = halo_fetch(c, gd, H, HU, HV, cx, y0 - 3);
    HaloRaw<R> rb = halo_fetch(c, gd, H, HU, HV, cx, y0 - 2);
    CellIn<R> cin;
    static_assert((G::RING & (G::RING - 1)) == 0, "ring slots are row & (RING - 1)");
    __syncthreads();

    for (int r = y0 - 3; r <= y1 + 2; ++r) {
        const int s0 = r & (G::RING - 1), s1 = (r - 1) & (G::RING - 1);   // ring slots of rows r, r-1,
        const int s2 = (r - 2) & (G::RING - 1), s3 = (r - 3) & (G::RING - 1);  // r-2 and r-3
        // ---- P1: build row r from values fetched two rows ago; fetch row r + 2 and the
        //      update inputs of row r - 2
        const int sl = s0;
        const HaloRaw<R> rnext = halo_fetch(c, gd, H, HU, HV, cx, r + 2);
        // update inputs of row r-3, consumed after three barriers of this iteration
        if (do_out && r - 3 >= y0 && r - 3 < y1) cin = cell_fetch<R, STAGE>(gd, (size_t)(r - 3) * nx + cx);
        {
            R hh, uu, vv, zz;
            halo_build(c, gd, bcv, ra, cx, r, hh, uu, vv, zz);
            s_cell[sl * NT + t] = Q4<R>{hh, uu, vv, zz};
        }
        ra = rb;
        rb = rnext;
        __syncthreads();
        // ---- P2: y-face between rows r-2 and r-1 (face index r-1), x-reconstruction of row r-2
        R by_new = R(0), bx_new = R(0);
        Q4<R> cm2{};                                 // cell (row r-2, this column)
        if (r >= y0 - 1) {
            cm2 = s_cell[s2 * NT + t];
            if (do_yface) {
                // y-reconstruction of row r-1: normal v, tangential u
                const Q4<R> cb = s_cell[s1 * NT + t], cc = s_cell[s0 * NT + t];
                Recon<R> yup = reconstruct(c, cm2.a, cb.a, cc.a, cm2.c, cb.c, cc.c, cm2.b, cb.b, cc.b,
                                           cm2.d, cb.d, cc.d);
                const int fy = r - 1;
                if (r >= y0 && fy >= y0 - 1 && fy <= y1 + 1) {
                    R F1 = R(0), F2L = R(0), F2R = R(0), F3 = R(0);
                    if (fy >= 0 && fy <= ny) face_flux(c, ylow, yup, F1, F2L, F2R, F3);
                    s_yf[(fy & (G::FR - 1)) * NT + t] = Q4<R>{F1, F2L, F2R, F3};
                }
                ylow = yup;
                if (c.order == 2) by_new = bed_term(c, yup);
            }
            if (r >= y0 + 1 && do_xrec) {
                const Q4<R> cl = s_cell[s2 * NT + t - 1], cr = s_cell[s2 * NT + t + 1];
                Recon<R> xr = reconstruct(c, cl.a, cm2.a, cr.a, cl.b, cm2.b, cr.b, cl.c, cm2.c, cr.c,
                                          cl.d, cm2.d, cr.d);
                store_recon(s_xr, t, NT, xr);
                if (c.order == 2) bx_new = bed_term(c, xr);
            }
        }
        __syncthreads();
        if (r >= y0 + 1) {
            const int row = r - 2;
            // ---- P3: x-faces of row r-2 (face cx between columns cx-1 and cx)
            if (do_xface && (unsigned)row < (unsigned)ny) {
                const Q4<R> cl = s_cell[s2 * NT + t - 1];
                Recon<R> L = load_recon(s_xr, t - 1, NT, cl.a, cl.d), Rr = load_recon(s_xr, t, NT, cm2.a, cm2.d);
                R F1, F2L, F2R, F3;
                face_flux(c, L, Rr, F1, F2L, F2R, F3);
                s_xf[(row & (G::FRX - 1)) * NT + t] = Q4<R>{F1, F2L, F2R, F3};
            }
            __syncthreads();
            // ---- P4: theta of row r-2
            if (do_theta) {
                R th = R(1);
                if ((unsigned)row < (unsigned)ny && col_in) {
                    const int fr = (row & (G::FR - 1)) * NT, frx = (row & (G::FRX - 1)) * NT;
                    const R Fw = s_xf[frx + t].a, Fe = s_xf[frx + t + 1].a;
                    const R Gs = s_yf[fr + t].a, Gn = s_yf[((row + 1) & (G::FR - 1)) * NT + t].a;
                    const R out = per_len(relu(Fe) + relu(-Fw), rdx, idx) + per_len(relu(Gn) + relu(-Gs), rdy, idy);
                    const R need = out * dt;
                    const R hh = cm2.a;
                    th = need > hh ? hh / (need > R(0) ? need : R(1)) : R(1);
                }
                s_th[(row & (G::FR - 1)) * NT + t] = th;
            }
            __syncthreads();
        }
        // ---- P5: update row r-3
        const int orow = r - 3;
        if (orow >= y0 && orow < y1 && do_out) {
            const int f0 = (orow & (G::FR - 1)) * NT, f1 = ((orow + 1) & (G::FR - 1)) * NT;
            const int fx = (orow & (G::FRX - 1)) * NT;
            const int tc = f0 + t;
            const R thC = s_th[tc], thW = s_th[tc - 1], thE = s_th[tc + 1];
            const R thS = s_th[((orow - 1) & (G::FR - 1)) * NT + t], thN = s_th[f1 + t];
            const Q4<R> xw = s_xf[fx + t], xe = s_xf[fx + t + 1], ys = s_yf[f0 + t], yn = s_yf[f1 + t];
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
                a2 = a2 + per_len(bxc, rdx, idx);
                b2 = b2 + per_len(by2, rdy, idy);
            }
            const R dh = a1 + b1, dhu = a2 + b3, dhv = a3 + b2;
            if (cx == 0) { xin += relu(F1w); xout += relu(-F1w); }
            if (cx == nx - 1) { xin += relu(-F1e); xout += relu(F1e); }
            if (orow == 0) { yin += relu(G1s); yout += relu(-G1s); }
            if (orow == ny - 1) { yin += relu(-G1n); yout += relu(G1n); }
            const size_t i = (size_t)orow * nx + cx;
            R hn, hun, hvn;
            if (STAGE == 2) {
                const R h1 = h_r3;
                hn = R(0.5) * (cin.h0 + h1 + dt * dh);
                hun = R(0.5) * (cin.hu0 + cin.hu1 + dt * dhu);
                hvn = R(0.5) * (cin.hv0 + cin.hv1 + dt * dhv);
            } else {
                hn = h_r3 + dt * dh;
                hun = cin.hu0 + dt * dhu;
                hvn = cin.hv0 + dt * dhv;
            }
            const R neg = clamp0(-hn);
            acc_clip += neg;
            hn = hn + neg;
            if (STAGE == 1) {
                gd.h1[i] = hn; gd.hu1[i] = hun; gd.hv1[i] = hvn;
            } else {
                // ---- rain, Horton infiltration, retention store (swe2d.py:330-360)
                R sf = cin.sf;
                if (gd.rw) {
                    const R add = rdt * cin.rw;
                    hn = hn + add;
                    rainw += add;
                } else {
                    hn = hn + rdt;
                }
                if (gd.f0) {
                    const R rate_f = cin.fc + (cin.f0 - cin.fc) * rexp(-cin.k * tt);
                    const R pot = rate_f * dt;
                    const R take = rmin(pot, hn);
                    const R safe = hn > R(0) ? hn : R(1);
                    const R scale = hn > R(0) ? (hn - take) / safe : R(0);
                    hn = hn - take;
                    hun = hun * scale;
                    hvn = hvn * scale;
                    R taken = take;
                    if (gd.S) {
                        const R tks = rmin(pot - take, sf);
                        sf = sf - tks;
                        taken = taken + tks;
                    }
                    infil += taken;
                    gd.ic[i] = cin.ic + taken;
                }
                if (gd.S) {
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
                if (gd.pk) gd.pk[i] = rmax(gd.pk[i], hn);
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
                if (gd.ps) gd.ps[i] = rmax(gd.ps[i], dsqrt(u2 * u2 + v2 * v2));
                if (float* sh = s_snap[0]) {
                    sh[i] = (float)hn;
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
        }
        by2 = by1;
        by1 = by_new;
        bxc = bx_new;
        h_r3 = cm2.a;
    }
    __syncthreads();
    double* out = partials + (size_t)blockIdx.x * NPART;
    if (STAGE == 1) {
        R v[5] = {acc_clip, xin, xout, yin, yout};
        const bool mx[5] = {false, false, false, false, false};
        const int sl[5] = {P_CLIP1, P_XIN1, P_XOUT1, P_YIN1, P_YOUT1};
        block_reduce_store<5>(v, mx, red, out, sl, NT);
    } else {
        const int b = STAGE == 2 ? P_CLIP2 : P_CLIP1;
        R v[11] = {acc_clip, xin, xout, yin, yout, infil, rainw, rate, hsum, ssum, hmax};
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
// modes 1 and 2 the rate, per member.
template <class R>
__global__ void finalize_kernel(const Grid<R>* __restrict__ grids, const StepParams* __restrict__ params, Consts c,
                                const double* __restrict__ partials, double* __restrict__ out, int mode,
                                double* __restrict__ ext) {
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
}

}  // namespace his
