// Launchers of the 1-D network kernels (float64, built with -fmad=false).
#include "his_internal.h"
#include "net1d_kernels.cuh"

namespace his {

// n_sub substeps of dt/n_sub each.  forcing: per member, per substep (inflow, stage).
// vols: 3 per member (bnd_in, bnd_out, clip) summed over the substeps.
__global__ void net_step_kernel(const Net* __restrict__ nets, Consts c, double dt_total, int n_sub,
                                const double* __restrict__ forcing, double* __restrict__ vols) {
    extern __shared__ double sm[];
    const Net& N = nets[blockIdx.x];
    const int nc = N.n_cells, nf = N.n_faces, tid = threadIdx.x, nt = blockDim.x;
    double *A = sm, *Q = A + nc, *Ag = Q + nc, *Qg = Ag + nc, *yv = Qg + nc, *uv = yv + nc, *th = uv + nc;
    double *F1 = th + nc, *F2 = F1 + nf, *pL = F2 + nf, *pR = pL + nf, *red = pR + nf;
    const Sec s{N.b, N.m, N.yb, N.ts}, fs{N.fb, N.fm, N.fyb, N.fts};
    const double g = c.g, dt = dt_total / n_sub;
    for (int i = tid; i < nc; i += nt) { A[i] = N.A[i]; Q[i] = N.Q[i]; }
    __syncthreads();
    double tot_in = 0.0, tot_out = 0.0, tot_clip = 0.0;
    for (int k = 0; k < n_sub; ++k) {
        const double q_in = forcing[((size_t)blockIdx.x * n_sub + k) * 2 + 0];
        const double eta = forcing[((size_t)blockIdx.x * n_sub + k) * 2 + 1];
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
    if (tid == 0 && vols) {
        vols[blockIdx.x * 3 + 0] = tot_in;
        vols[blockIdx.x * 3 + 1] = tot_out;
        vols[blockIdx.x * 3 + 2] = tot_clip;
    }
}

// 1-D CFL rate over wet interior cells, the any-wet flag and the channel volume.
// out: 3 per member (rate, any_wet, volume).
__global__ void net_reduce_kernel(const Net* __restrict__ nets, Consts c, double* __restrict__ out) {
    __shared__ double red[32 * 3];
    const Net& N = nets[blockIdx.x];
    const Sec s{N.b, N.m, N.yb, N.ts};
    double rate = 0.0, wet_any = 0.0, vol = 0.0;
    for (int i = threadIdx.x; i < N.n_cells; i += blockDim.x) {
        if (N.kind[i] > 1) continue;
        const double A = N.A[i];
        vol += A * N.dx[i];
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
    vol = warp_sum(vol);
    if (lane == 0) { red[warp * 3] = rate; red[warp * 3 + 1] = wet_any; red[warp * 3 + 2] = vol; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = red[0], w = red[1], v = red[2];
        for (int k = 1; k < nw; ++k) { r = fmax(r, red[k * 3]); w = fmax(w, red[k * 3 + 1]); v += red[k * 3 + 2]; }
        out[blockIdx.x * 3 + 0] = r;
        out[blockIdx.x * 3 + 1] = w;
        out[blockIdx.x * 3 + 2] = v;
    }
}

int net_step_launch(his_net* n, double dt, int n_sub, cudaStream_t s) {
    if (n->smem > 48 * 1024)
        HIS_CK(cudaFuncSetAttribute(net_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)n->smem));
    net_step_kernel<<<n->n, 128, n->smem, s>>>(n->d_nets, n->c, dt, n_sub, n->d_forcing, n->d_out);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

int net_reduce_launch(his_net* n, cudaStream_t s) {
    net_reduce_kernel<<<n->n, 128, 0, s>>>(n->d_nets, n->c, n->d_out);
    HIS_CK(cudaGetLastError());
    return HIS_OK;
}

}  // namespace his
