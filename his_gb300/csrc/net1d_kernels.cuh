// 1-D St. Venant network step and 1-D <-> 2-D weir exchange (one CTA per member).
//
// The channel network is small (10^2 - 10^3 cells): a member's whole network lives
// in shared memory for all of its substeps.  Scatter-adds of the reference
// (torch index_add over faces / links) become per-cell gathers over CSR lists kept
// in the reference's index order, so every sum has the reference's association
// and the result does not depend on thread scheduling.
//
// All arithmetic is float64 in both precisions (the 1-D network, its junction level
// pool and the exchange volumes are the float64 islands of the production form).
//
// Reference: hydrointel/solver/swe1d.py:51-107, :253-368; coupling.py:73-124.
#pragma once
#include "his_device.cuh"

namespace his {

struct Net {
    int n_cells, n_faces;
    const int *kind, *gsrc, *fl, *fr;
    const double* gsign;
    const int *lstart, *lidx, *rstart, *ridx;      // faces where the cell is left / right (face order)
    const double *z, *nman, *dx;
    const double *b, *m, *yb, *ts;                 // cell sections
    const double *fb, *fm, *fyb, *fts;             // face sections
    double *A, *Q;
};

struct Lnk {
    int n_links, n_unique, v_offset, pad;
    const int *cell1d, *inv, *uniq;
    const double *zbank, *length, *z2;
    const int *ustart, *uidx;                      // unique 2-D cell -> links (link order)
    const int *cstart, *cidx;                      // 1-D cell -> links (link order)
};

// ---------------------------------------------------------------- sections (swe1d.py:51-84)
struct Sec {
    const double *b, *m, *yb, *ts;
};

__device__ __forceinline__ double sec_area(const Sec& s, int i, double y) {
    double yt = fmin(y, s.yb[i]);
    double at = yt * (s.b[i] + s.m[i] * yt);
    return at + s.ts[i] * clamp0(y - s.yb[i]);
}
__device__ __forceinline__ double sec_top(const Sec& s, int i, double y) {
    return y <= s.yb[i] ? s.b[i] + 2.0 * s.m[i] * y : s.ts[i];
}
__device__ __forceinline__ double sec_i1(const Sec& s, int i, double y) {
    double yt = fmin(y, s.yb[i]);
    double above = clamp0(y - s.yb[i]);
    double it = s.b[i] * yt * yt / 2.0 + s.m[i] * (yt * yt * yt) / 3.0;
    double at = yt * (s.b[i] + s.m[i] * yt);
    return it + at * above + s.ts[i] * above * above / 2.0;
}
__device__ __forceinline__ double sec_perim(const Sec& s, int i, double y) {
    double yt = fmin(y, s.yb[i]);
    return s.b[i] + 2.0 * yt * sqrt(1.0 + s.m[i] * s.m[i]);
}
__device__ __forceinline__ double sec_bank_area(const Sec& s, int i) { return s.yb[i] * (s.b[i] + s.m[i] * s.yb[i]); }
__device__ __forceinline__ double sec_depth(const Sec& s, int i, double A) {
    A = clamp0(A);
    double ab = sec_bank_area(s, i);
    double b = s.b[i];
    double y_t = 2.0 * A / (b + sqrt(b * b + 4.0 * s.m[i] * A));
    return A <= ab ? y_t : s.yb[i] + (A - ab) / s.ts[i];
}
__device__ __forceinline__ double vel1d(const Consts& c, const Sec& s, int i, double A, double Q) {
    double y = sec_depth(s, i, A);
    return y >= c.h_dry ? Q / fmax(A, 1e-12) : 0.0;
}

// HLL flux of the 1-D equations (swe1d.py:87-107)
__device__ __forceinline__ void hll_1d(double AL, double QL, double pL, double cL, double AR, double QR, double pR,
                                       double cR, double uL, double uR, double& F1o, double& F2o) {
    const double tiny = 1e-14;
    bool dryL = AL <= tiny, dryR = AR <= tiny;
    double SL = rmin(uL - cL, uR - cR);
    double SR = rmax(uL + cL, uR + cR);
    if (dryL) { SL = uR - 2.0 * cR; SR = uR + cR; }
    if (dryR) { SL = uL - cL; SR = uL + 2.0 * cL; }
    double FL1 = QL, FR1 = QR;
    double FL2 = QL * uL + pL, FR2 = QR * uR + pR;
    double den = SR - SL;
    if (fabs(den) < tiny) den = 1.0;
    bool left = SL >= 0.0, right = SR <= 0.0;
    double F1, F2;
    if (left) { F1 = FL1; F2 = FL2; }
    else if (right) { F1 = FR1; F2 = FR2; }
    else {
        F1 = (SR * FL1 - SL * FR1 + SL * SR * (AR - AL)) / den;
        F2 = (SR * FL2 - SL * FR2 + SL * SR * (QR - QL)) / den;
    }
    if (dryL && dryR) { F1 = 0.0; F2 = 0.0; }
    F1o = F1;
    F2o = F2;
}

// Deterministic block sum of NV doubles; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = warp_sum(v[j]);
    if (lane == 0)
        for (int j = 0; j < NV; ++j) red[warp * NV + j] = v[j];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int j = 0; j < NV; ++j) {
            double a = red[j];
            for (int w = 1; w < nw; ++w) a += red[w * NV + j];
            v[j] = a;
        }
    __syncthreads();
}

__host__ __device__ inline size_t net_smem_bytes(int n_cells, int n_faces) {
    return sizeof(double) * (7 * (size_t)n_cells + 4 * (size_t)n_faces + 32 * 4);
}

__host__ __device__ inline size_t exchange_smem_bytes(int n_links, int n_unique, int n_cells) {
    return sizeof(double) * (2 * (size_t)n_links + 2 * (size_t)n_unique + (size_t)n_cells + 32 * 2);
}

// Weir exchange for one member per CTA (coupling.py:73-124).  dt is per member
// (params) when params is non-NULL, else dt_host.  V: per-link volumes at
// lnk.v_offset; exch: per member (2-D -> 1-D total, 1-D -> 2-D total).
template <class R>
__global__ void exchange_kernel(const Lnk* __restrict__ links, const Net* __restrict__ nets,
                                const Grid<R>* __restrict__ grids, const StepParams* __restrict__ params, Consts c,
                                double dt_host, double* __restrict__ Vout, double* __restrict__ exch) {
    extern __shared__ double sm[];
    const int mb = blockIdx.x;
    const Lnk& L = links[mb];
    const Net& N = nets[mb];
    const Grid<R>& gd = grids[mb];
    if (params && !params[mb].active) return;
    const double dt = params ? params[mb].dt : dt_host;
    const int nl = L.n_links, nu = L.n_unique, nc = N.n_cells, tid = threadIdx.x, nt = blockDim.x;
    double *V = sm, *sg = V + nl, *hu_ = sg + nl, *f2 = hu_ + nu, *f1 = f2 + nu, *red = f1 + nc;
    const Sec s{N.b, N.m, N.yb, N.ts};
    const double area2 = gd.area;
    for (int k = tid; k < nu; k += nt) hu_[k] = (double)gd.h[L.uniq[k]];
    __syncthreads();
    for (int l = tid; l < nl; l += nt) {
        const int c1 = L.cell1d[l];
        const double h2 = hu_[L.inv[l]];
        const double eta2 = L.z2[l] + h2;
        const double y1 = sec_depth(s, c1, N.A[c1]);
        const double eta1 = N.z[c1] + y1;
        const double zb = L.zbank[l];
        const double up = rmax(eta1, eta2), dn = rmin(eta1, eta2);
        const double d_up = clamp0(up - zb), d_dn = clamp0(dn - zb);
        const double ratio = d_up > 0.0 ? d_dn / d_up : 0.0;
        const double q = c.weir_cw * L.length[l] * pow(d_up, 1.5) * pow(clamp0(1.0 - pow(ratio, 1.5)), 0.385);
        sg[l] = eta2 > eta1 ? 1.0 : -1.0;
        double v = q * dt;
        const double plan1 = (y1 <= N.yb[c1] ? N.b[c1] + 2.0 * N.m[c1] * y1 : N.ts[c1]) * N.dx[c1];
        const double v_eq = (up - dn) / (1.0 / area2 + 1.0 / plan1);
        V[l] = rmin(v, c.exchange_relax * v_eq);
    }
    __syncthreads();
    // donor limits, aggregated per donor in link order (coupling.py:98-107)
    for (int k = tid; k < nu; k += nt) {
        double tot = 0.0;
        for (int j = L.ustart[k]; j < L.ustart[k + 1]; ++j) { int l = L.uidx[j]; tot += sg[l] > 0.0 ? V[l] : 0.0; }
        const double avail = c.exchange_limit * hu_[k] * area2;
        f2[k] = tot > avail ? avail / (tot > 0.0 ? tot : 1.0) : 1.0;
    }
    for (int i = tid; i < nc; i += nt) {
        double tot = 0.0;
        for (int j = L.cstart[i]; j < L.cstart[i + 1]; ++j) { int l = L.cidx[j]; tot += sg[l] < 0.0 ? V[l] : 0.0; }
        const double avail = c.exchange_limit * clamp0(N.A[i] - sec_bank_area(s, i)) * N.dx[i];
        f1[i] = tot > avail ? avail / (tot > 0.0 ? tot : 1.0) : 1.0;
    }
    __syncthreads();
    double ex[2] = {0.0, 0.0};
    for (int l = tid; l < nl; l += nt) {
        const double v = (sg[l] > 0.0 ? V[l] * f2[L.inv[l]] : V[l] * f1[L.cell1d[l]]) * sg[l];
        V[l] = v;
        if (Vout) Vout[L.v_offset + l] = v;
        ex[0] += clamp0(v);
        ex[1] += clamp0(-v);
    }
    __syncthreads();
    // apply: 2-D through the unique cells, momentum kept only for water that stays
    for (int k = tid; k < nu; k += nt) {
        double d = 0.0;
        for (int j = L.ustart[k]; j < L.ustart[k + 1]; ++j) d += V[L.uidx[j]];
        const double hu0 = hu_[k];
        const double hn = hu0 - d / area2;
        const double keep = hu0 > 0.0 ? fmin(hn / (hu0 > 0.0 ? hu0 : 1.0), 1.0) : 0.0;
        const int idx = L.uniq[k];
        const R kr = R(keep);
        gd.h[idx] = R(hn);
        gd.hu[idx] = gd.hu[idx] * kr;
        gd.hv[idx] = gd.hv[idx] * kr;
    }
    for (int i = tid; i < nc; i += nt) {
        double d = 0.0;
        for (int j = L.cstart[i]; j < L.cstart[i + 1]; ++j) d += V[L.cidx[j]];
        N.A[i] = N.A[i] + d / N.dx[i];
    }
    block_sum<2>(ex, red);
    if (tid == 0 && exch) {
        exch[mb * 2 + 0] += ex[0];
        exch[mb * 2 + 1] += ex[1];
    }
}

}  // namespace his
