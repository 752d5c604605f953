// 1-D St. Venant network step and 1-D <-> 2-D weir exchange (one CTA per member).
//
// The channel network is small (10^2 - 10^3 cells): a member's whole network lives
// in shared memory for all of its substeps.  Scatter-adds of the reference
// (torch index_add over faces / links) become per-cell gathers over CSR lists kept
// in the reference's index order, so every sum has the reference's association
// and the result does not depend on thread scheduling.
//
// The drop-in 1-D step (net_step_kernel) is float64 in both precisions.  The
// device-resident engine's float32 form (net_engine_kernel_f32) computes section
// geometry, wave speeds, HLL fluxes, limiter and friction in float32 over float64
// area and discharge state, float64 updates and tallies, and float64 junction depths
// (the level-pool solve); its float64 form (net_engine_kernel) is float64 throughout.
// The weir exchange is float64 in the plain method; in the production form its
// per-link arithmetic is float32 (GB300's float64 pipe runs at a small fraction of the
// float32 rate and this work sits on every step's critical path), with the 1-D area
// update and the exchanged-volume tallies kept in float64.
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
    const float *zf, *dxf, *bf, *mf, *ybf, *tsf;   // float32 copies of z, dx and the cell sections
    const float *nmanf, *gsignf;                   // float32 roughness and ghost signs
    const float *fbf, *fmf, *fybf, *ftsf;          // float32 face sections
    double *A, *Q;
};

struct Lnk {
    int n_links, n_unique, v_offset, pad;
    const int *cell1d, *inv, *uniq;
    const double *zbank, *length, *z2;
    const float *zbank_f, *length_f, *z2_f;        // float32 copies for the production form
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

// n_sub substeps of dt/n_sub each for the network N, run by the whole CTA.
// forcing: per substep (inflow, stage).  vols (thread 0, if non-NULL): bnd_in,
// bnd_out, clip summed over the substeps.  sm: net_smem_bytes() of shared memory.
__device__ __forceinline__ void net_substeps_dev(const Net& N, const Consts& c, double dt_total, int n_sub,
                                                 const double* __restrict__ forcing, double* vols, double* sm,
                                                 float* snap_eta = nullptr, float* snap_q = nullptr,
                                                 double* snap_v1d = nullptr) {
    const int nc = N.n_cells, nf = N.n_faces, tid = threadIdx.x, nt = blockDim.x;
    double *A = sm, *Q = A + nc, *Ag = Q + nc, *Qg = Ag + nc, *yv = Qg + nc, *uv = yv + nc, *th = uv + nc;
    double *F1 = th + nc, *F2 = F1 + nf, *pL = F2 + nf, *pR = pL + nf, *red = pR + nf;
    const Sec s{N.b, N.m, N.yb, N.ts}, fs{N.fb, N.fm, N.fyb, N.fts};
    const double g = c.g, dt = dt_total / n_sub;
    for (int i = tid; i < nc; i += nt) { A[i] = N.A[i]; Q[i] = N.Q[i]; }
    __syncthreads();
    double tot_in = 0.0, tot_out = 0.0, tot_clip = 0.0;
    for (int k = 0; k < n_sub; ++k) {
        const double q_in = forcing[2 * k + 0];
        const double eta = forcing[2 * k + 1];
        // ghost cells from the interior neighbour (swe1d.py:265-294)
        for (int i = tid; i < nc; i += nt) {
            const int kd = N.kind[i];
            if (kd < 2) { Ag[i] = A[i]; Qg[i] = Q[i]; continue; }
            const int src = N.gsrc[i];
            const double As = A[src], Qs = Q[src], sg = N.gsign[i];
            const double ys = sec_depth(s, i, As);
            const double un = sg * vel1d(c, s, i, As, Qs);
            const bool wet_i = ys >= c.h_dry;
            double An, Qn;
            if (kd == 3) {
                double yst = clamp0(eta - N.z[i]);
                double Ast = sec_area(s, i, yst);
                double ci = sqrt(g * As / sec_top(s, i, ys));
                double cg = sqrt(g * Ast / sec_top(s, i, yst));
                double un_st = wet_i ? un + 2.0 * (ci - cg) : 0.0;
                if (wet_i && (un > ci)) { un_st = un; Ast = As; }
                if (!(sec_depth(s, i, Ast) >= c.h_dry)) un_st = 0.0;
                An = Ast;
                Qn = sg * Ast * un_st;
            } else if (kd == 2) {
                double yc = fmax(pow(q_in * q_in / (g * N.b[i] * N.b[i]), 1.0 / 3.0), c.h_dry);
                An = wet_i ? As : sec_area(s, i, yc);
                Qn = -sg * q_in;
            } else {
                An = As;
                Qn = -Qs;
            }
            Ag[i] = An;
            Qg[i] = Qn;
        }
        __syncthreads();
        for (int i = tid; i < nc; i += nt) {
            yv[i] = sec_depth(s, i, Ag[i]);
            uv[i] = vel1d(c, s, i, Ag[i], Qg[i]);
        }
        __syncthreads();
        // face fluxes with hydrostatic reconstruction (swe1d.py:326-336)
        for (int f = tid; f < nf; f += nt) {
            const int l = N.fl[f], r = N.fr[f];
            const double zL = N.z[l], zR = N.z[r], zf = rmax(zL, zR);
            const double yL = clamp0(zL + yv[l] - zf), yR = clamp0(zR + yv[r] - zf);
            const double AL = sec_area(fs, f, yL), AR = sec_area(fs, f, yR);
            const double uL = uv[l], uR = uv[r];
            pL[f] = g * sec_i1(fs, f, yL);
            pR[f] = g * sec_i1(fs, f, yR);
            const double cL = sqrt(g * AL / sec_top(fs, f, yL));
            const double cR = sqrt(g * AR / sec_top(fs, f, yR));
            hll_1d(AL, AL * uL, pL[f], cL, AR, AR * uR, pR[f], cR, uL, uR, F1[f], F2[f]);
        }
        __syncthreads();
        // outflow limiter; ghosts unlimited (swe1d.py:337-344)
        for (int i = tid; i < nc; i += nt) {
            double out = 0.0;
            for (int j = N.lstart[i]; j < N.lstart[i + 1]; ++j) out += relu(F1[N.lidx[j]]);
            for (int j = N.rstart[i]; j < N.rstart[i + 1]; ++j) out += relu(-F1[N.ridx[j]]);
            const double vol = Ag[i] * N.dx[i];
            const double need = out * dt;
            const double t = need > vol ? vol / (need > 0.0 ? need : 1.0) : 1.0;
            th[i] = N.kind[i] >= 2 ? 1.0 : t;
        }
        __syncthreads();
        double bsum[3] = {0.0, 0.0, 0.0};
        for (int f = tid; f < nf; f += nt) {
            const double sc = F1[f] > 0.0 ? th[N.fl[f]] : th[N.fr[f]];
            const double Fs = F1[f] * sc;
            F1[f] = Fs;
            if (N.kind[N.fl[f]] >= 2) { bsum[0] += relu(Fs); bsum[1] += relu(-Fs); }
            if (N.kind[N.fr[f]] >= 2) { bsum[0] += relu(-Fs); bsum[1] += relu(Fs); }
        }
        __syncthreads();
        // update, clip, semi-implicit friction; ghosts keep their filled state (swe1d.py:345-368)
        for (int i = tid; i < nc; i += nt) {
            double dA = 0.0, dQ = 0.0;
            for (int j = N.lstart[i]; j < N.lstart[i + 1]; ++j) dA += -F1[N.lidx[j]];
            for (int j = N.rstart[i]; j < N.rstart[i + 1]; ++j) dA += F1[N.ridx[j]];
            for (int j = N.lstart[i]; j < N.lstart[i + 1]; ++j) { int f = N.lidx[j]; dQ += -(F2[f] - pL[f]); }
            for (int j = N.rstart[i]; j < N.rstart[i + 1]; ++j) { int f = N.ridx[j]; dQ += F2[f] - pR[f]; }
            const int kd = N.kind[i];
            double A1 = Ag[i] + dt * dA / N.dx[i];
            double Q1 = Qg[i] + dt * dQ / N.dx[i];
            const double neg = clamp0(-A1);
            bsum[2] += neg * N.dx[i] * (kd >= 2 ? 0.0 : 1.0);
            A1 = A1 + neg;
            const double y1 = sec_depth(s, i, A1);
            const double Ac = fmax(A1, 1e-12);
            const double R = Ac / sec_perim(s, i, y1);
            const double nm = N.nman[i];
            const double denom = 1.0 + dt * g * (nm * nm) * fabs(Q1) / (Ac * pow(fmax(R, c.h_dry), 4.0 / 3.0));
            Q1 = Q1 / denom;
            if (!((y1 >= c.h_dry) && kd != 1)) Q1 = 0.0;
            if (kd >= 2) { A1 = Ag[i]; Q1 = Qg[i]; }
            A[i] = A1;
            Q[i] = Q1;
        }
        block_sum<3>(bsum, red);
        if (tid == 0) {
            tot_in += bsum[0] * dt;
            tot_out += bsum[1] * dt;
            tot_clip += bsum[2];
        }
    }
    __syncthreads();
    for (int i = tid; i < nc; i += nt) { N.A[i] = A[i]; N.Q[i] = Q[i]; }
    if (snap_eta) {                         // output: level z + depth and discharge (coupling.py:229-242)
        double v1 = 0.0;
        for (int i = tid; i < nc; i += nt) {
            snap_eta[i] = (float)(N.z[i] + sec_depth(s, i, A[i]));
            snap_q[i] = (float)Q[i];
            if (N.kind[i] <= 1) v1 += A[i] * N.dx[i];
        }
        if (snap_v1d) {                     // channel volume over the interior cells (swe1d.py:245-247)
            double vv[1] = {v1};
            block_sum<1>(vv, red);
            if (tid == 0) *snap_v1d = vv[0];
        }
    }
    if (tid == 0 && vols) {
        vols[0] = tot_in;
        vols[1] = tot_out;
        vols[2] = tot_clip;
    }
}


// ---------------------------------------------------------- float32 substeps
// The production form of the network step: section geometry, wave speeds, fluxes,
// the outflow limiter and friction in float32 arithmetic; the state (cross-section
// area A and discharge Q), its per-substep update, the clip and boundary tallies, and
// the depth of the junction level pools in float64.  GB300 runs float64 at a small
// fraction of its float32 rate, and the float64 network filled one SM's float64 pipe.
struct SecF {
    const float *b, *m, *yb, *ts;
};
__device__ __forceinline__ float secf_area(const SecF& s, int i, float y) {
    const float yt = fminf(y, s.yb[i]);
    return yt * (s.b[i] + s.m[i] * yt) + s.ts[i] * fmaxf(y - s.yb[i], 0.0f);
}
__device__ __forceinline__ float secf_top(const SecF& s, int i, float y) {
    return y <= s.yb[i] ? s.b[i] + 2.0f * s.m[i] * y : s.ts[i];
}
__device__ __forceinline__ float secf_i1(const SecF& s, int i, float y) {
    const float yt = fminf(y, s.yb[i]);
    const float above = fmaxf(y - s.yb[i], 0.0f);
    const float it = s.b[i] * yt * yt * 0.5f + s.m[i] * (yt * yt * yt) * (1.0f / 3.0f);
    const float at = yt * (s.b[i] + s.m[i] * yt);
    return it + at * above + s.ts[i] * above * above * 0.5f;
}
__device__ __forceinline__ float secf_perim(const SecF& s, int i, float y) {
    const float yt = fminf(y, s.yb[i]);
    return s.b[i] + 2.0f * yt * sqrtf(1.0f + s.m[i] * s.m[i]);
}
__device__ __forceinline__ float secf_depth(const SecF& s, int i, float A) {
    A = fmaxf(A, 0.0f);
    const float b = s.b[i], yb = s.yb[i];
    const float ab = yb * (b + s.m[i] * yb);
    return A <= ab ? 2.0f * A / (b + sqrtf(b * b + 4.0f * s.m[i] * A)) : yb + (A - ab) / s.ts[i];
}

__device__ __forceinline__ void hll_1d_f32(float AL, float QL, float pL, float cL, float AR, float QR, float pR,
                                           float cR, float uL, float uR, float& F1o, float& F2o) {
    const float tiny = 1e-14f;
    const bool dryL = AL <= tiny, dryR = AR <= tiny;
    float SL = fminf(uL - cL, uR - cR);
    float SR = fmaxf(uL + cL, uR + cR);
    if (dryL) { SL = uR - 2.0f * cR; SR = uR + cR; }
    if (dryR) { SL = uL - cL; SR = uL + 2.0f * cL; }
    const float FL2 = QL * uL + pL, FR2 = QR * uR + pR;
    float den = SR - SL;
    if (fabsf(den) < tiny) den = 1.0f;
    float F1, F2;
    if (SL >= 0.0f) { F1 = QL; F2 = FL2; }
    else if (SR <= 0.0f) { F1 = QR; F2 = FR2; }
    else {
        const float inv = 1.0f / den;
        F1 = (SR * QL - SL * QR + SL * SR * (AR - AL)) * inv;
        F2 = (SR * FL2 - SL * FR2 + SL * SR * (QR - QL)) * inv;
    }
    if (dryL && dryR) { F1 = 0.0f; F2 = 0.0f; }
    F1o = F1;
    F2o = F2;
}

// Shared memory of the float32 substeps: the state in float64 (A, Q and their
// ghost-filled copies), a reduction slot, the per-substep float32 work arrays, and the
// network's static geometry and connectivity staged once per launch, so that no phase
// waits on a global load (a lone CTA per network has no other warps to hide it).
__host__ __device__ inline size_t net_smem_bytes_f32(int n_cells, int n_faces) {
    const size_t nc = (size_t)n_cells, nf = (size_t)n_faces;
    return sizeof(double) * (4 * nc + 32 * 4) + sizeof(float) * (4 * nc + 4 * nf) +   // state, red; work
           sizeof(float) * (8 * nc + 4 * nf) +                                       // cell and face geometry
           sizeof(int) * (2 * nc + 2 * nf + 2 * (nc + 1) + 2 * nf) + 16;             // kinds, faces, CSR
}

// n_sub substeps of dt/n_sub each for the network N (the arguments of net_substeps_dev).
__device__ __forceinline__ void net_substeps_f32_dev(const Net& N, const Consts& c, double dt_total, int n_sub,
                                                     const double* __restrict__ forcing, double* vols, double* sm,
                                                     float* snap_eta = nullptr, float* snap_q = nullptr,
                                                     double* snap_v1d = nullptr) {
    const int nc = N.n_cells, nf = N.n_faces, tid = threadIdx.x, nt = blockDim.x;
    double *A = sm, *Q = A + nc, *Ag = Q + nc, *Qg = Ag + nc, *red = Qg + nc;      // red: 128 doubles
    float *Af = reinterpret_cast<float*>(red + 32 * 4), *yv = Af + nc, *uv = yv + nc, *th = uv + nc;
    float *F1 = th + nc, *F2 = F1 + nf, *pL = F2 + nf, *pR = pL + nf;
    // staged geometry
    float *zs = pR + nf, *dxs = zs + nc, *bs = dxs + nc, *ms = bs + nc, *ybs = ms + nc, *tss = ybs + nc,
          *nms = tss + nc, *gss = nms + nc;
    float *fbs = gss + nc, *fms = fbs + nf, *fybs = fms + nf, *ftss = fybs + nf;
    int *kind = reinterpret_cast<int*>(ftss + nf), *gsrc = kind + nc, *fl = gsrc + nc, *fr = fl + nf;
    int *lst = fr + nf, *rst = lst + nc + 1, *lix = rst + nc + 1, *rix = lix + nf;
    for (int i = tid; i < nc; i += nt) {
        A[i] = N.A[i]; Q[i] = N.Q[i];
        zs[i] = N.zf[i]; dxs[i] = N.dxf[i]; bs[i] = N.bf[i]; ms[i] = N.mf[i]; ybs[i] = N.ybf[i]; tss[i] = N.tsf[i];
        nms[i] = N.nmanf[i]; gss[i] = N.gsignf[i];
        kind[i] = N.kind[i]; gsrc[i] = N.gsrc[i];
    }
    for (int i = tid; i <= nc; i += nt) { lst[i] = N.lstart[i]; rst[i] = N.rstart[i]; }
    for (int f = tid; f < nf; f += nt) {
        fbs[f] = N.fbf[f]; fms[f] = N.fmf[f]; fybs[f] = N.fybf[f]; ftss[f] = N.ftsf[f];
        fl[f] = N.fl[f]; fr[f] = N.fr[f];
        lix[f] = N.lidx[f]; rix[f] = N.ridx[f];
    }
    const SecF s{bs, ms, ybs, tss}, fs{fbs, fms, fybs, ftss};
    const Sec sd{N.b, N.m, N.yb, N.ts};
    __shared__ float s_k[3];
    if (tid == 0) {
        s_k[0] = (float)c.g;
        s_k[1] = (float)c.h_dry;
        s_k[2] = (float)(dt_total / n_sub);
    }
    __syncthreads();
    const float g = s_k[0], h_dry = s_k[1], dt = s_k[2];
    double tot_in = 0.0, tot_out = 0.0, tot_clip = 0.0;
    for (int k = 0; k < n_sub; ++k) {
        const float q_in = (float)forcing[2 * k + 0];
        const float eta = (float)forcing[2 * k + 1];
        // ghost cells from the interior neighbour (swe1d.py:265-294)
        for (int i = tid; i < nc; i += nt) {
            const int kd = kind[i];
            if (kd < 2) {
                Ag[i] = A[i];
                Qg[i] = Q[i];
                Af[i] = (float)A[i];
                continue;
            }
            const int src = gsrc[i];
            const float As = (float)A[src], Qs = (float)Q[src], sg = gss[i];
            const float ys = secf_depth(s, i, As);
            const float un = sg * (ys >= h_dry ? Qs / fmaxf(As, 1e-12f) : 0.0f);
            const bool wet_i = ys >= h_dry;
            float An, Qn;
            if (kd == 3) {
                const float yst = fmaxf(eta - zs[i], 0.0f);
                float Ast = secf_area(s, i, yst);
                const float ci = sqrtf(g * As / secf_top(s, i, ys));
                const float cg = sqrtf(g * Ast / secf_top(s, i, yst));
                float un_st = wet_i ? un + 2.0f * (ci - cg) : 0.0f;
                if (wet_i && (un > ci)) { un_st = un; Ast = As; }
                if (!(secf_depth(s, i, Ast) >= h_dry)) un_st = 0.0f;
                An = Ast;
                Qn = sg * Ast * un_st;
            } else if (kd == 2) {
                const float b = bs[i];
                const float yc = fmaxf(cbrtf(q_in * q_in / (g * b * b)), h_dry);
                An = wet_i ? As : secf_area(s, i, yc);
                Qn = -sg * q_in;
            } else {
                An = As;
                Qn = -Qs;
            }
            Ag[i] = (double)An;
            Qg[i] = (double)Qn;
            Af[i] = An;
        }
        __syncthreads();
        // depth and velocity; a junction's level-pool depth in float64
        for (int i = tid; i < nc; i += nt) {
            const float y = kind[i] == 1 ? (float)sec_depth(sd, i, Ag[i]) : secf_depth(s, i, Af[i]);
            yv[i] = y;
            uv[i] = y >= h_dry ? (float)Qg[i] / fmaxf(Af[i], 1e-12f) : 0.0f;
        }
        __syncthreads();
        // face fluxes with hydrostatic reconstruction (swe1d.py:326-336)
        for (int f = tid; f < nf; f += nt) {
            const int l = fl[f], r = fr[f];
            const float zL = zs[l], zR = zs[r], zfc = fmaxf(zL, zR);
            const float yL = fmaxf(zL + yv[l] - zfc, 0.0f), yR = fmaxf(zR + yv[r] - zfc, 0.0f);
            const float AL = secf_area(fs, f, yL), AR = secf_area(fs, f, yR);
            const float uL = uv[l], uR = uv[r];
            const float pl = g * secf_i1(fs, f, yL), pr = g * secf_i1(fs, f, yR);
            pL[f] = pl;
            pR[f] = pr;
            const float cL = sqrtf(g * AL / secf_top(fs, f, yL));
            const float cR = sqrtf(g * AR / secf_top(fs, f, yR));
            hll_1d_f32(AL, AL * uL, pl, cL, AR, AR * uR, pr, cR, uL, uR, F1[f], F2[f]);
        }
        __syncthreads();
        // outflow limiter; ghosts unlimited (swe1d.py:337-344)
        for (int i = tid; i < nc; i += nt) {
            float out = 0.0f;
            for (int j = lst[i]; j < lst[i + 1]; ++j) out += fmaxf(F1[lix[j]], 0.0f);
            for (int j = rst[i]; j < rst[i + 1]; ++j) out += fmaxf(-F1[rix[j]], 0.0f);
            const float vol = Af[i] * dxs[i];
            const float need = out * dt;
            const float t = need > vol ? vol / (need > 0.0f ? need : 1.0f) : 1.0f;
            th[i] = kind[i] >= 2 ? 1.0f : t;
        }
        __syncthreads();
        double bsum[3] = {0.0, 0.0, 0.0};
        for (int f = tid; f < nf; f += nt) {
            const float sc = F1[f] > 0.0f ? th[fl[f]] : th[fr[f]];
            const float Fs = F1[f] * sc;
            F1[f] = Fs;
            if (kind[fl[f]] >= 2) { bsum[0] += fmaxf(Fs, 0.0f); bsum[1] += fmaxf(-Fs, 0.0f); }
            if (kind[fr[f]] >= 2) { bsum[0] += fmaxf(-Fs, 0.0f); bsum[1] += fmaxf(Fs, 0.0f); }
        }
        __syncthreads();
        // update in float64, clip, semi-implicit friction; ghosts keep their filled state
        // (swe1d.py:345-368)
        for (int i = tid; i < nc; i += nt) {
            float dA = 0.0f, dQ = 0.0f;
            for (int j = lst[i]; j < lst[i + 1]; ++j) { const int f = lix[j]; dA -= F1[f]; dQ -= F2[f] - pL[f]; }
            for (int j = rst[i]; j < rst[i + 1]; ++j) { const int f = rix[j]; dA += F1[f]; dQ += F2[f] - pR[f]; }
            const int kd = kind[i];
            const float rdx = 1.0f / dxs[i];
            double A1 = Ag[i] + (double)(dt * dA * rdx);
            double Q1 = Qg[i] + (double)(dt * dQ * rdx);
            const double neg = clamp0(-A1);
            if (neg > 0.0 && kd < 2) bsum[2] += neg * N.dx[i];
            A1 = A1 + neg;
            const float A1f = (float)A1;
            const float y1 = secf_depth(s, i, A1f);
            const float Ac = fmaxf(A1f, 1e-12f);
            const float R = Ac / secf_perim(s, i, y1);
            const float nm = nms[i];
            const float denom = 1.0f + dt * g * (nm * nm) * fabsf((float)Q1) / (Ac * powf(fmaxf(R, h_dry), 4.0f / 3.0f));
            Q1 = Q1 / (double)denom;
            if (!((y1 >= h_dry) && kd != 1)) Q1 = 0.0;
            if (kd >= 2) { A1 = Ag[i]; Q1 = Qg[i]; }
            A[i] = A1;
            Q[i] = Q1;
        }
        bsum[0] *= (double)dt;
        bsum[1] *= (double)dt;
        block_sum<3>(bsum, red);
        if (tid == 0) {
            tot_in += bsum[0];
            tot_out += bsum[1];
            tot_clip += bsum[2];
        }
    }
    __syncthreads();
    for (int i = tid; i < nc; i += nt) { N.A[i] = A[i]; N.Q[i] = Q[i]; }
    if (snap_eta) {                         // output: level z + depth and discharge (coupling.py:229-242)
        double v1 = 0.0;
        for (int i = tid; i < nc; i += nt) {
            snap_eta[i] = (float)(N.z[i] + sec_depth(sd, i, A[i]));
            snap_q[i] = (float)Q[i];
            if (kind[i] <= 1) v1 += A[i] * N.dx[i];
        }
        if (snap_v1d) {                     // channel volume over the interior cells (swe1d.py:245-247)
            double vv[1] = {v1};
            block_sum<1>(vv, red);
            if (tid == 0) *snap_v1d = vv[0];
        }
    }
    if (tid == 0 && vols) {
        vols[0] = tot_in;
        vols[1] = tot_out;
        vols[2] = tot_clip;
    }
}

__host__ __device__ inline size_t exchange_smem_bytes(int n_links, int n_unique, int n_cells) {
    const size_t f64 = sizeof(double) * (2 * (size_t)n_links + 2 * (size_t)n_unique + (size_t)n_cells + 32 * 2);
    const size_t f32 = sizeof(float) * (2 * (size_t)n_links + 2 * (size_t)n_unique + 4 * (size_t)n_cells) +
                       sizeof(double) * 32 * 2;
    return f64 > f32 ? f64 : f32;
}

// Production-form exchange (2-D state in float32): the same steps as the float64
// form below, in float32 arithmetic from float32 copies of the static link and
// section tables.  Per 1-D cell the level, plan width and donor volume are formed
// once; the 1-D area update and the tallies accumulate in float64.
__device__ __forceinline__ void exchange_dev_f32(const Lnk& L, const Net& N, const Grid<float>& gd, const Consts& c,
                                                 double dt, double* __restrict__ Vout, double* __restrict__ exch,
                                                 int mb, double* sm) {
    const int nl = L.n_links, nu = L.n_unique, nc = N.n_cells, tid = threadIdx.x, nt = blockDim.x;
    double* red = sm;                                   // 64 doubles
    float* V = reinterpret_cast<float*>(sm + 64);
    float *sg = V + nl, *hu_ = sg + nl, *f2 = hu_ + nu, *eta1 = f2 + nu, *plan1 = eta1 + nc, *f1 = plan1 + nc,
          *avail1 = f1 + nc;
    __shared__ float s_k[6];
    if (tid == 0) {
        s_k[0] = (float)dt;
        s_k[1] = (float)c.weir_cw;
        s_k[2] = (float)c.exchange_relax;
        s_k[3] = (float)c.exchange_limit;
        s_k[4] = (float)gd.area;
        s_k[5] = (float)(1.0 / gd.area);
    }
    for (int k = tid; k < nu; k += nt) hu_[k] = gd.h[L.uniq[k]];
    for (int i = tid; i < nc; i += nt) {
        const float A = fmaxf((float)N.A[i], 0.0f);
        const float b = N.bf[i], m = N.mf[i], yb = N.ybf[i], ts = N.tsf[i];
        const float ab = yb * (b + m * yb);
        const float y = A <= ab ? 2.0f * A / (b + sqrtf(b * b + 4.0f * m * A)) : yb + (A - ab) / ts;
        eta1[i] = N.zf[i] + y;
        plan1[i] = (y <= yb ? b + 2.0f * m * y : ts) * N.dxf[i];
        avail1[i] = fmaxf(A - ab, 0.0f) * N.dxf[i];
    }
    __syncthreads();
    const float dtf = s_k[0], cw = s_k[1], relax = s_k[2], limit = s_k[3], area2 = s_k[4], rarea2 = s_k[5];
    for (int l = tid; l < nl; l += nt) {
        const int c1 = L.cell1d[l];
        const float eta2 = L.z2_f[l] + hu_[L.inv[l]];
        const float e1 = eta1[c1];
        const float zb = L.zbank_f[l];
        const float up = fmaxf(e1, eta2), dn = fminf(e1, eta2);
        const float d_up = fmaxf(up - zb, 0.0f), d_dn = fmaxf(dn - zb, 0.0f);
        const float ratio = d_up > 0.0f ? d_dn / d_up : 0.0f;
        const float sub = powf(fmaxf(1.0f - ratio * sqrtf(ratio), 0.0f), 0.385f);
        const float q = cw * L.length_f[l] * (d_up * sqrtf(d_up)) * sub;
        sg[l] = eta2 > e1 ? 1.0f : -1.0f;
        const float v_eq = (up - dn) / (rarea2 + 1.0f / plan1[c1]);
        V[l] = fminf(q * dtf, relax * v_eq);
    }
    __syncthreads();
    // donor limits, aggregated per donor in link order (coupling.py:98-107)
    for (int k = tid; k < nu; k += nt) {
        float tot = 0.0f;
        for (int j = L.ustart[k]; j < L.ustart[k + 1]; ++j) { int l = L.uidx[j]; tot += sg[l] > 0.0f ? V[l] : 0.0f; }
        const float avail = limit * hu_[k] * area2;
        f2[k] = tot > avail ? avail / (tot > 0.0f ? tot : 1.0f) : 1.0f;
    }
    for (int i = tid; i < nc; i += nt) {
        float tot = 0.0f;
        for (int j = L.cstart[i]; j < L.cstart[i + 1]; ++j) { int l = L.cidx[j]; tot += sg[l] < 0.0f ? V[l] : 0.0f; }
        const float avail = limit * avail1[i];
        f1[i] = tot > avail ? avail / (tot > 0.0f ? tot : 1.0f) : 1.0f;
    }
    __syncthreads();
    float ex0 = 0.0f, ex1 = 0.0f;
    for (int l = tid; l < nl; l += nt) {
        const float v = (sg[l] > 0.0f ? V[l] * f2[L.inv[l]] : V[l] * f1[L.cell1d[l]]) * sg[l];
        V[l] = v;
        if (Vout) Vout[L.v_offset + l] = (double)v;
        ex0 += fmaxf(v, 0.0f);
        ex1 += fmaxf(-v, 0.0f);
    }
    __syncthreads();
    // apply: 2-D through the unique cells, momentum kept only for water that stays
    for (int k = tid; k < nu; k += nt) {
        float d = 0.0f;
        for (int j = L.ustart[k]; j < L.ustart[k + 1]; ++j) d += V[L.uidx[j]];
        const float hu0 = hu_[k];
        const float hn = hu0 - d * rarea2;
        const float keep = hu0 > 0.0f ? fminf(hn / hu0, 1.0f) : 0.0f;
        const int idx = L.uniq[k];
        gd.h[idx] = hn;
        gd.hu[idx] = gd.hu[idx] * keep;
        gd.hv[idx] = gd.hv[idx] * keep;
    }
    for (int i = tid; i < nc; i += nt) {
        float d = 0.0f;
        for (int j = L.cstart[i]; j < L.cstart[i + 1]; ++j) d += V[L.cidx[j]];
        if (d != 0.0f) N.A[i] = N.A[i] + (double)(d / N.dxf[i]);
    }
    double ex[2] = {(double)ex0, (double)ex1};
    block_sum<2>(ex, red);
    if (tid == 0 && exch) {
        exch[mb * 2 + 0] += ex[0];
        exch[mb * 2 + 1] += ex[1];
    }
    __syncthreads();
}

// Weir exchange for one member per CTA, float64 plain method (coupling.py:73-124).
// V: per-link volumes at lnk.v_offset; exch: per member (2-D -> 1-D total,
// 1-D -> 2-D total).
__device__ __forceinline__ void exchange_dev_f64(const Lnk& L, const Net& N, const Grid<double>& gd, const Consts& c,
                                                 double dt, double* __restrict__ Vout, double* __restrict__ exch,
                                                 int mb, double* sm) {
    using R = double;
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
    __syncthreads();
}

template <class R>
__device__ __forceinline__ void exchange_dev(const Lnk& L, const Net& N, const Grid<R>& gd, const Consts& c, double dt,
                                             double* __restrict__ Vout, double* __restrict__ exch, int mb, double* sm) {
    if constexpr (sizeof(R) == 4) exchange_dev_f32(L, N, gd, c, dt, Vout, exch, mb, sm);
    else exchange_dev_f64(L, N, gd, c, dt, Vout, exch, mb, sm);
}

// One CTA of EXCHANGE_THREADS per member.  The drop-in step runs it alone between
// its CFL wait and the 2-D stages, so more threads (fewer dependent rounds over the
// ~1,200 links per phase) shorten the step directly.
constexpr int EXCHANGE_THREADS = 1024;

template <class R>
__global__ void __launch_bounds__(EXCHANGE_THREADS) exchange_kernel(const Lnk* __restrict__ links, const Net* __restrict__ nets,
                                const Grid<R>* __restrict__ grids, Consts c, double dt, double* __restrict__ Vout,
                                double* __restrict__ exch) {
    extern __shared__ double sm[];
    const int mb = blockIdx.x;
    exchange_dev(links[mb], nets[mb], grids[mb], c, dt, Vout, exch, mb, sm);
}

// 1-D CFL rate over wet interior cells and whether any is wet (swe1d.py:253-262);
// results valid in thread 0.  red: 64 doubles of shared memory.
__device__ __forceinline__ void net_rate_dev(const Net& N, const Consts& c, double& rate_o, bool& wet_o, double* red) {
    const Sec s{N.b, N.m, N.yb, N.ts};
    double rate = 0.0, wet_any = 0.0;
    for (int i = threadIdx.x; i < N.n_cells; i += blockDim.x) {
        if (N.kind[i] > 1) continue;
        const double A = N.A[i];
        const double y = sec_depth(s, i, A);
        if (!(y > c.h_dry)) continue;
        wet_any = 1.0;
        const double cc = sqrt(c.g * A / sec_top(s, i, y));
        const double u = vel1d(c, s, i, A, N.Q[i]);
        rate = fmax(rate, (fabs(u) + cc) / N.dx[i]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    rate = warp_max(rate);
    wet_any = warp_max(wet_any);
    if (lane == 0) { red[warp * 2] = rate; red[warp * 2 + 1] = wet_any; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = red[0], w = red[1];
        for (int k = 1; k < nw; ++k) { r = fmax(r, red[k * 2]); w = fmax(w, red[k * 2 + 1]); }
        rate_o = r;
        wet_o = w > 0.0;
    }
    __syncthreads();
}

// The same rate in float32 arithmetic (production form: it only sets the substep count).
__device__ __forceinline__ void net_rate_dev_f32(const Net& N, const Consts& c, double& rate_o, bool& wet_o,
                                                 double* red) {
    __shared__ float s_c[2];
    if (threadIdx.x == 0) {
        s_c[0] = (float)c.g;
        s_c[1] = (float)c.h_dry;
    }
    __syncthreads();
    const float g = s_c[0], h_dry = s_c[1];
    float rate = 0.0f, wet_any = 0.0f;
    for (int i = threadIdx.x; i < N.n_cells; i += blockDim.x) {
        if (N.kind[i] > 1) continue;
        const float A = fmaxf((float)N.A[i], 0.0f);
        const float b = N.bf[i], m = N.mf[i], yb = N.ybf[i], ts = N.tsf[i];
        const float ab = yb * (b + m * yb);
        const float y = A <= ab ? 2.0f * A / (b + sqrtf(b * b + 4.0f * m * A)) : yb + (A - ab) / ts;
        if (!(y > h_dry)) continue;
        wet_any = 1.0f;
        const float top = y <= yb ? b + 2.0f * m * y : ts;
        const float cc = sqrtf(g * A / top);
        const float u = (float)N.Q[i] / fmaxf(A, 1e-12f);
        rate = fmaxf(rate, (fabsf(u) + cc) / N.dxf[i]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        rate = fmaxf(rate, __shfl_xor_sync(0xffffffffu, rate, o));
        wet_any = fmaxf(wet_any, __shfl_xor_sync(0xffffffffu, wet_any, o));
    }
    float* redf = reinterpret_cast<float*>(red);
    if (lane == 0) { redf[warp * 2] = rate; redf[warp * 2 + 1] = wet_any; }
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = redf[0], w = redf[1];
        for (int k = 1; k < nw; ++k) { r = fmaxf(r, redf[k * 2]); w = fmaxf(w, redf[k * 2 + 1]); }
        rate_o = (double)r;
        wet_o = w > 0.0f;
    }
    __syncthreads();
}

}  // namespace his
