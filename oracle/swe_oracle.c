/*
 * ORACLE -- test infrastructure only.
 *
 * A plain-C, cell-loop restatement of the time step of the coupled 1-D/2-D
 * flood engine in Elciiid/HIS (hydrointel/solver).  It exists to check the CUDA
 * path: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it, always as the checker and never as the thing measured or shipped.
 *
 * Parity is pinned: tests/golden/make_golden.py runs the reference solver itself
 * (float64, torch CPU) on small seeded cases and tests/test_oracle_golden.py
 * checks this file against those vectors.
 *
 * Every routine follows the reference's expression order (left-to-right
 * evaluation of the Python expressions, no contraction: build with
 * -ffp-contract=off) so that float64 results agree with the reference to the
 * last bits wherever the reference's own arithmetic is deterministic.
 *
 * Reference map (file:line in the reference project):
 *   orc_velocities          hydrointel/solver/swe2d.py:161-167  (Kurganov-Petrova)
 *   orc_max_rate            hydrointel/solver/swe2d.py:179-184
 *   ghost / pad_line        hydrointel/solver/boundaries.py:56-128
 *   sweep_line              hydrointel/solver/swe2d.py:196-234
 *   riemann                 hydrointel/solver/swe2d.py:61-101
 *   orc_rhs                 hydrointel/solver/swe2d.py:252-279
 *   orc_swe2d_step          hydrointel/solver/swe2d.py:305-371, infiltration.py:34-37
 *   sec_*                   hydrointel/solver/swe1d.py:51-84
 *   hll_1d                  hydrointel/solver/swe1d.py:87-107
 *   orc_swe1d_step          hydrointel/solver/swe1d.py:265-294, :320-368
 *   orc_swe1d_max_rate      hydrointel/solver/swe1d.py:253-262
 *   orc_exchange            hydrointel/solver/coupling.py:73-124
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    double g, h_dry, kp_eps, cfl, dt_min, dt_max;
    double cfl_1d, slot_width_frac, weir_cw, exchange_limit, exchange_relax;
    int32_t order, hllc;
} orc_cfg;

enum { BC_CLOSED = 0, BC_TRANSMISSIVE = 1, BC_STAGE = 2, BC_DISCHARGE = 3 };
enum { EDGE_W = 0, EDGE_E = 1, EDGE_S = 2, EDGE_N = 3 };

static const double SQRT2 = 1.4142135623730951;  /* math.sqrt(2.0) */

static inline double relu(double x) { return x > 0.0 ? x : 0.0; }
static inline double maxd(double a, double b) { return a > b ? a : (b > a ? b : a); }
static inline double mind(double a, double b) { return a < b ? a : (b < a ? b : a); }
static inline double clamp0(double x) { return x < 0.0 ? 0.0 : x; }

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ 2-D */

static inline void kp_velocity(const orc_cfg* c, double h, double hu, double hv, double* u, double* v) {
    double h4 = pow(h, 4.0);
    double den = sqrt(h4 + maxd(h4, c->kp_eps));
    if (h >= c->h_dry) {
        *u = SQRT2 * h * hu / den;
        *v = SQRT2 * h * hv / den;
    } else {
        *u = 0.0;
        *v = 0.0;
    }
}

void orc_velocities(const orc_cfg* c, int64_t n, const double* h, const double* hu, const double* hv,
                    double* u, double* v) {
    for (int64_t i = 0; i < n; ++i) kp_velocity(c, h[i], hu[i], hv[i], &u[i], &v[i]);
}

double orc_max_rate(const orc_cfg* c, int ny, int nx, double dx, double dy,
                    const double* h, const double* hu, const double* hv) {
    double m = 0.0;
    for (int64_t i = 0; i < (int64_t)ny * nx; ++i) {
        double u, v;
        kp_velocity(c, h[i], hu[i], hv[i], &u, &v);
        double cc = sqrt(c->g * h[i]);
        double r = (h[i] > c->h_dry) ? (fabs(u) + cc) / dx + (fabs(v) + cc) / dy : 0.0;
        if (r > m) m = r;
    }
    return m;
}

/* Ghost state of one edge for a one-cell layer (boundaries.py:56-78).  un is the
   outward-normal velocity of the layer; returns ghost (h, un, ut, z). */
static void edge_ghost(const orc_cfg* c, int kind, double val, double h, double un, double ut, double z,
                       double* hg_o, double* un_o, double* ut_o, double* zg_o) {
    const double g = c->g;
    if (kind == BC_CLOSED) { *hg_o = h; *un_o = -un; *ut_o = ut; *zg_o = z; return; }
    if (kind == BC_TRANSMISSIVE) { *hg_o = h; *un_o = un; *ut_o = ut; *zg_o = z; return; }
    if (kind == BC_STAGE) {
        double hg = clamp0(val - z);
        double ci = sqrt(g * h), cg = sqrt(g * hg);
        int wet_i = h >= c->h_dry;
        double ung = wet_i ? un + 2.0 * (ci - cg) : 0.0;
        int sup = wet_i && (un > ci);
        if (sup) { ung = un; hg = h; }
        if (!(hg >= c->h_dry)) ung = 0.0;
        *hg_o = hg; *un_o = ung; *ut_o = (ung > 0.0) ? ut : 0.0; *zg_o = z;
        return;
    }
    /* discharge */
    double hc = maxd(pow(val * val / g, 1.0 / 3.0), c->h_dry);
    double hg = (h >= c->h_dry) ? h : hc;
    *hg_o = hg; *un_o = -val / hg; *ut_o = 0.0; *zg_o = z;
}

/* Fill a padded line (length n + 2 ng) from interior values taken with stride
   (boundaries.py:81-128).  `lo`/`hi` are BC kinds of the low and high edge. */
static void pad_line(const orc_cfg* c, int n, int ng, int lo, int hi, double vlo, double vhi,
                     const double* h, const double* un_c, const double* ut_c, const double* z, int64_t stride,
                     double* ph, double* pn, double* pt, double* pz) {
    for (int i = 0; i < n; ++i) {
        ph[ng + i] = h[i * stride]; pn[ng + i] = un_c[i * stride];
        pt[ng + i] = ut_c[i * stride]; pz[ng + i] = z[i * stride];
    }
    for (int side = 0; side < 2; ++side) {
        int kind = side == 0 ? lo : hi;
        double sgn = side == 0 ? -1.0 : 1.0;
        double val = side == 0 ? vlo : vhi;
        for (int k = 0; k < ng; ++k) {
            int layer;
            int pos = side == 0 ? ng - 1 - k : ng + n + k;
            if (kind == BC_CLOSED || kind == BC_TRANSMISSIVE) {
                if (n < ng) layer = side == 0 ? 0 : n - 1;
                else layer = side == 0 ? k : n - 1 - k;
            } else {
                layer = side == 0 ? 0 : n - 1;
            }
            double hh = h[layer * stride], zz = z[layer * stride];
            double un = sgn * un_c[layer * stride], ut = ut_c[layer * stride];
            double hg, ung, utg, zg;
            edge_ghost(c, kind, val, hh, un, ut, zz, &hg, &ung, &utg, &zg);
            ph[pos] = hg; pn[pos] = sgn * ung; pt[pos] = utg; pz[pos] = zg;
        }
    }
}

static inline double minmod(double a, double b) {
    if (a * b > 0.0) {
        double m = mind(fabs(a), fabs(b));
        return a > 0.0 ? m : -m;
    }
    return 0.0;
}

/* HLLC / HLL flux (swe2d.py:61-101) */
static void riemann(const orc_cfg* c, double hL, double uL, double vL, double hR, double uR, double vR,
                    double* F1o, double* F2o, double* F3o) {
    const double g = c->g, tiny = 1e-14;
    double cL = sqrt(g * hL), cR = sqrt(g * hR);
    int dryL = hL <= tiny, dryR = hR <= tiny;
    double u_s = 0.5 * (uL + uR) + cL - cR;
    double c_s = 0.5 * (cL + cR) + 0.25 * (uL - uR);
    double SL = mind(uL - cL, u_s - c_s);
    double SR = maxd(uR + cR, u_s + c_s);
    if (dryL) { SL = uR - 2.0 * cR; SR = uR + cR; }
    if (dryR) { SL = uL - cL; SR = uL + 2.0 * cL; }
    double qL = hL * uL, qR = hR * uR;
    double FL1 = qL, FR1 = qR;
    double FL2 = qL * uL + 0.5 * g * hL * hL, FR2 = qR * uR + 0.5 * g * hR * hR;
    double den = SR - SL;
    if (fabs(den) < tiny) den = 1.0;
    double H1 = (SR * FL1 - SL * FR1 + SL * SR * (hR - hL)) / den;
    double H2 = (SR * FL2 - SL * FR2 + SL * SR * (qR - qL)) / den;
    int left = SL >= 0.0, right = SR <= 0.0;
    double F1 = left ? FL1 : (right ? FR1 : H1);
    double F2 = left ? FL2 : (right ? FR2 : H2);
    double F3;
    if (c->hllc) {
        double num = SL * hR * (uR - SR) - SR * hL * (uL - SL);
        double dd = hR * (uR - SR) - hL * (uL - SL);
        double SM = fabs(dd) < tiny ? 0.5 * (uL + uR) : num / dd;
        F3 = F1 * (SM >= 0.0 ? vL : vR);
    } else {
        double FL3 = qL * vL, FR3 = qR * vR;
        double H3 = (SR * FL3 - SL * FR3 + SL * SR * (hR * vR - hL * vL)) / den;
        F3 = left ? FL3 : (right ? FR3 : H3);
    }
    if (dryL && dryR) { F1 = 0.0; F2 = 0.0; F3 = 0.0; }
    *F1o = F1; *F2o = F2; *F3o = F3;
}

/* Face fluxes along one padded line (swe2d.py:196-234).  Outputs on n+1 faces:
   F1, F2, F3, cL, cR; Sc on n cells (order 2 only). work: 8*(n+2) doubles. */
static void sweep_line(const orc_cfg* c, int n, int ng, const double* h, const double* un, const double* ut,
                       const double* z, double* F1, double* F2, double* F3, double* cLo, double* cRo, double* Sc,
                       double* work) {
    const double g = c->g;
    int m = n + 2;
    double *Hm = work, *Hp = work + m, *Um = work + 2 * m, *Up = work + 3 * m;
    double *Vm = work + 4 * m, *Vp = work + 5 * m, *Zm = work + 6 * m, *Zp = work + 7 * m;
    for (int s = 0; s < m; ++s) {
        int k = s + ng - 1;
        if (c->order == 2) {
            double hmin = mind(mind(h[k - 1], h[k]), h[k + 1]);
            double ok = (hmin >= c->h_dry) ? 1.0 : 0.0;
            double em1 = h[k - 1] + z[k - 1], e0 = h[k] + z[k], ep1 = h[k + 1] + z[k + 1];
            double sH = minmod(h[k] - h[k - 1], h[k + 1] - h[k]) * ok;
            double sE = minmod(e0 - em1, ep1 - e0) * ok;
            double sU = minmod(un[k] - un[k - 1], un[k + 1] - un[k]) * ok;
            double sV = minmod(ut[k] - ut[k - 1], ut[k + 1] - ut[k]) * ok;
            double E = h[k] + z[k];
            Hm[s] = h[k] - 0.5 * sH; Hp[s] = h[k] + 0.5 * sH;
            double Em = E - 0.5 * sE, Ep = E + 0.5 * sE;
            Um[s] = un[k] - 0.5 * sU; Up[s] = un[k] + 0.5 * sU;
            Vm[s] = ut[k] - 0.5 * sV; Vp[s] = ut[k] + 0.5 * sV;
            Zm[s] = Em - Hm[s]; Zp[s] = Ep - Hp[s];
        } else {
            Hm[s] = Hp[s] = h[k]; Um[s] = Up[s] = un[k]; Vm[s] = Vp[s] = ut[k]; Zm[s] = Zp[s] = z[k];
        }
    }
    for (int f = 0; f <= n; ++f) {
        double hL = Hp[f], uL = Up[f], vL = Vp[f], zL = Zp[f];
        double hR = Hm[f + 1], uR = Um[f + 1], vR = Vm[f + 1], zR = Zm[f + 1];
        double zf = maxd(zL, zR);
        double hLs = clamp0(hL + zL - zf), hRs = clamp0(hR + zR - zf);
        riemann(c, hLs, uL, vL, hRs, uR, vR, &F1[f], &F2[f], &F3[f]);
        cLo[f] = 0.5 * g * (hL * hL - hLs * hLs);
        cRo[f] = 0.5 * g * (hR * hR - hRs * hRs);
    }
    if (c->order == 2 && Sc) {
        for (int i = 0; i < n; ++i) {
            int s = i + 1;
            Sc[i] = -0.5 * g * (Hm[s] + Hp[s]) * (Zp[s] - Zm[s]);
        }
    }
}

/* Right-hand side (swe2d.py:252-279).  q[0] = gross boundary inflow rate,
   q[1] = outflow rate (m^3/s), both from the limited boundary face fluxes. */
void orc_rhs(const orc_cfg* c, int ny, int nx, double dx, double dy, const int32_t* bc, const double* vals,
             const double* z, const double* h, const double* hu, const double* hv, double dt,
             double* dh, double* dhu, double* dhv, double* q) {
    const int ng = c->order == 1 ? 1 : 2;
    const int64_t N = (int64_t)ny * nx;
    double* u = (double*)malloc(sizeof(double) * N);
    double* v = (double*)malloc(sizeof(double) * N);
    orc_velocities(c, N, h, hu, hv, u, v);
    /* x faces: (ny, nx+1); y faces stored per column: (nx, ny+1) */
    int64_t NXF = (int64_t)ny * (nx + 1), NYF = (int64_t)nx * (ny + 1);
    double *X1 = malloc(sizeof(double) * NXF), *X2 = malloc(sizeof(double) * NXF), *X3 = malloc(sizeof(double) * NXF);
    double *XL = malloc(sizeof(double) * NXF), *XR = malloc(sizeof(double) * NXF);
    double *Y1 = malloc(sizeof(double) * NYF), *Y2 = malloc(sizeof(double) * NYF), *Y3 = malloc(sizeof(double) * NYF);
    double *YL = malloc(sizeof(double) * NYF), *YR = malloc(sizeof(double) * NYF);
    double *SCX = malloc(sizeof(double) * N), *SCY = malloc(sizeof(double) * N);
    double* theta = malloc(sizeof(double) * N);

#pragma omp parallel
    {
        int L = (nx > ny ? nx : ny) + 2 * ng;
        double* buf = (double*)malloc(sizeof(double) * (4 * L + 8 * (L + 2)));
        double *ph = buf, *pn = buf + L, *pt = buf + 2 * L, *pz = buf + 3 * L, *work = buf + 4 * L;
#pragma omp for schedule(static)
        for (int j = 0; j < ny; ++j) {
            const int64_t o = (int64_t)j * nx;
            pad_line(c, nx, ng, bc[EDGE_W], bc[EDGE_E], vals[EDGE_W], vals[EDGE_E], h + o, u + o, v + o, z + o, 1,
                     ph, pn, pt, pz);
            int64_t f = (int64_t)j * (nx + 1);
            sweep_line(c, nx, ng, ph, pn, pt, pz, X1 + f, X2 + f, X3 + f, XL + f, XR + f,
                       c->order == 2 ? SCX + o : NULL, work);
        }
#pragma omp for schedule(static)
        for (int i = 0; i < nx; ++i) {
            pad_line(c, ny, ng, bc[EDGE_S], bc[EDGE_N], vals[EDGE_S], vals[EDGE_N], h + i, v + i, u + i, z + i, nx,
                     ph, pn, pt, pz);
            int64_t f = (int64_t)i * (ny + 1);
            sweep_line(c, ny, ng, ph, pn, pt, pz, Y1 + f, Y2 + f, Y3 + f, YL + f, YR + f,
                       c->order == 2 ? SCY + (int64_t)i * ny : NULL, work);
        }
        free(buf);
    }
    /* positivity limiter: theta per cell (swe2d.py:259-264) */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) {
            double Fe = X1[(int64_t)j * (nx + 1) + i + 1], Fw = X1[(int64_t)j * (nx + 1) + i];
            double Gn = Y1[(int64_t)i * (ny + 1) + j + 1], Gs = Y1[(int64_t)i * (ny + 1) + j];
            double out = (relu(Fe) + relu(-Fw)) / dx + (relu(Gn) + relu(-Gs)) / dy;
            double need = out * dt;
            double hh = h[(int64_t)j * nx + i];
            theta[(int64_t)j * nx + i] = need > hh ? hh / (need > 0.0 ? need : 1.0) : 1.0;
        }
    }
    /* donor-scaled fluxes and assembly (swe2d.py:236-250, :265-271) */
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) {
            int64_t c0 = (int64_t)j * nx + i;
            int64_t fw = (int64_t)j * (nx + 1) + i, fe = fw + 1;
            double tw = i > 0 ? theta[c0 - 1] : 1.0, tc = theta[c0], te = i < nx - 1 ? theta[c0 + 1] : 1.0;
            double sw = X1[fw] > 0.0 ? tw : tc;
            double se = X1[fe] > 0.0 ? tc : te;
            double F1w = X1[fw] * sw, F1e = X1[fe] * se;
            double F3w = X3[fw] * sw, F3e = X3[fe] * se;
            double a1 = -(F1e - F1w) / dx;
            double a2 = -((X2[fe] + XL[fe]) - (X2[fw] + XR[fw])) / dx;
            if (c->order == 2) a2 = a2 + SCX[c0] / dx;
            double a3 = -(F3e - F3w) / dx;
            int64_t gs = (int64_t)i * (ny + 1) + j, gn = gs + 1;
            double ts_ = j > 0 ? theta[c0 - nx] : 1.0, tn = j < ny - 1 ? theta[c0 + nx] : 1.0;
            double ss = Y1[gs] > 0.0 ? ts_ : tc;
            double sn = Y1[gn] > 0.0 ? tc : tn;
            double G1s = Y1[gs] * ss, G1n = Y1[gn] * sn;
            double G3s = Y3[gs] * ss, G3n = Y3[gn] * sn;
            double b1 = -(G1n - G1s) / dy;
            double b2 = -((Y2[gn] + YL[gn]) - (Y2[gs] + YR[gs])) / dy;
            if (c->order == 2) b2 = b2 + SCY[(int64_t)i * ny + j] / dy;
            double b3 = -(G3n - G3s) / dy;
            dh[c0] = a1 + b1;
            dhu[c0] = a2 + b3;
            dhv[c0] = a3 + b2;
        }
    }
    /* boundary rates from the limited edge fluxes (swe2d.py:272-278) */
    double w_in = 0, e_in = 0, s_in = 0, n_in = 0, w_out = 0, e_out = 0, s_out = 0, n_out = 0;
    for (int j = 0; j < ny; ++j) {
        int64_t c0 = (int64_t)j * nx;
        double Fw = X1[(int64_t)j * (nx + 1)], Fe = X1[(int64_t)j * (nx + 1) + nx];
        double Fws = Fw * (Fw > 0.0 ? 1.0 : theta[c0]);
        double Fes = Fe * (Fe > 0.0 ? theta[c0 + nx - 1] : 1.0);
        w_in += relu(Fws); e_in += relu(-Fes); w_out += relu(-Fws); e_out += relu(Fes);
    }
    for (int i = 0; i < nx; ++i) {
        double Gs = Y1[(int64_t)i * (ny + 1)], Gn = Y1[(int64_t)i * (ny + 1) + ny];
        double Gss = Gs * (Gs > 0.0 ? 1.0 : theta[i]);
        double Gns = Gn * (Gn > 0.0 ? theta[(int64_t)(ny - 1) * nx + i] : 1.0);
        s_in += relu(Gss); n_in += relu(-Gns); s_out += relu(-Gss); n_out += relu(Gns);
    }
    q[0] = (w_in + e_in) * dy + (s_in + n_in) * dx;
    q[1] = (w_out + e_out) * dy + (s_out + n_out) * dx;
    free(u); free(v); free(X1); free(X2); free(X3); free(XL); free(XR);
    free(Y1); free(Y2); free(Y3); free(YL); free(YR); free(SCX); free(SCY); free(theta);
}

/* One full step for one member (swe2d.py:305-371).
   vals0 / vals1: BC values (W, E, S, N) at t and t + dt.
   Optional fields (NULL to disable): storage, horton (f0, fc, k), rain_weight.
   vol out: [bnd_in, bnd_out, rain, infil, clip] (m^3). */
void orc_swe2d_step(const orc_cfg* c, int ny, int nx, double dx, double dy, const int32_t* bc,
                    const double* vals0, const double* vals1, const double* z, const double* nman,
                    const double* storage, const double* f0, const double* fc, const double* kk, double t0,
                    const double* rain_weight, double dt, double t, double rain,
                    double* h, double* hu, double* hv, double* s_filled, double* infil_cum, double* vol) {
    const int64_t N = (int64_t)ny * nx;
    const double area = dx * dy, g = c->g;
    double* h1 = malloc(sizeof(double) * N);
    double* hu1 = malloc(sizeof(double) * N);
    double* hv1 = malloc(sizeof(double) * N);
    double* d0 = malloc(sizeof(double) * N);
    double* d1 = malloc(sizeof(double) * N);
    double* d2 = malloc(sizeof(double) * N);
    double q[2], q2[2];
    orc_rhs(c, ny, nx, dx, dy, bc, vals0, z, h, hu, hv, dt, d0, d1, d2, q);
    double clip = 0.0, clip_s;
    clip_s = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        h1[i] = h[i] + dt * d0[i];
        hu1[i] = hu[i] + dt * d1[i];
        hv1[i] = hv[i] + dt * d2[i];
        double neg = clamp0(-h1[i]);
        clip_s += neg;
        h1[i] = h1[i] + neg;
    }
    clip = clip_s * area;
    double qin = q[0], qout = q[1];
    if (c->order == 2) {
        orc_rhs(c, ny, nx, dx, dy, bc, vals1, z, h1, hu1, hv1, dt, d0, d1, d2, q2);
        clip_s = 0.0;
        for (int64_t i = 0; i < N; ++i) {
            h1[i] = 0.5 * (h[i] + h1[i] + dt * d0[i]);
            hu1[i] = 0.5 * (hu[i] + hu1[i] + dt * d1[i]);
            hv1[i] = 0.5 * (hv[i] + hv1[i] + dt * d2[i]);
            double neg = clamp0(-h1[i]);
            clip_s += neg;
            h1[i] = h1[i] + neg;
        }
        qin = 0.5 * (qin + q2[0]);
        qout = 0.5 * (qout + q2[1]);
        clip = clip + clip_s * area;
    }
    vol[0] = qin * dt;
    vol[1] = qout * dt;
    /* rain (swe2d.py:331-337) */
    double rdt = rain * dt;
    if (rain_weight) {
        double s = 0.0;
        for (int64_t i = 0; i < N; ++i) {
            double add = rdt * rain_weight[i];
            h1[i] = h1[i] + add;
            s += add;
        }
        vol[2] = s * area;
    } else {
        for (int64_t i = 0; i < N; ++i) h1[i] = h1[i] + rdt;
        vol[2] = rdt * ((double)((int64_t)nx * ny) * area);
    }
    /* Horton infiltration from the surface, then from the store (swe2d.py:339-352) */
    double inf_s = 0.0;
    if (f0) {
        double tt = clamp0(t - t0);
        for (int64_t i = 0; i < N; ++i) {
            double rate = fc[i] + (f0[i] - fc[i]) * exp(-kk[i] * tt);
            double pot = rate * dt;
            double take = mind(pot, h1[i]);
            double safe = h1[i] > 0.0 ? h1[i] : 1.0;
            double scale = h1[i] > 0.0 ? (h1[i] - take) / safe : 0.0;
            h1[i] = h1[i] - take;
            hu1[i] = hu1[i] * scale;
            hv1[i] = hv1[i] * scale;
            double taken = take;
            if (storage) {
                double ts_ = mind(pot - take, s_filled[i]);
                s_filled[i] = s_filled[i] - ts_;
                taken = taken + ts_;
            }
            infil_cum[i] = infil_cum[i] + taken;
            inf_s += taken;
        }
    }
    vol[3] = inf_s * area;
    /* retention store fill (swe2d.py:353-360) */
    if (storage) {
        for (int64_t i = 0; i < N; ++i) {
            double room = clamp0(storage[i] - s_filled[i]);
            double fill = mind(room, h1[i]);
            double safe = h1[i] > 0.0 ? h1[i] : 1.0;
            double scale = h1[i] > 0.0 ? (h1[i] - fill) / safe : 0.0;
            h1[i] = h1[i] - fill;
            hu1[i] = hu1[i] * scale;
            hv1[i] = hv1[i] * scale;
            s_filled[i] = s_filled[i] + fill;
        }
    }
    /* semi-implicit Manning friction (swe2d.py:362-370) */
    for (int64_t i = 0; i < N; ++i) {
        double u, v;
        kp_velocity(c, h1[i], hu1[i], hv1[i], &u, &v);
        double speed = sqrt(u * u + v * v);
        double hf = maxd(h1[i], c->h_dry);
        double denom = 1.0 + dt * g * nman[i] * nman[i] * speed / pow(hf, 4.0 / 3.0);
        u = u / denom;
        v = v / denom;
        int wet = h1[i] >= c->h_dry;
        h[i] = h1[i];
        hu[i] = wet ? h1[i] * u : 0.0;
        hv[i] = wet ? h1[i] * v : 0.0;
    }
    vol[4] = clip;
    free(h1); free(hu1); free(hv1); free(d0); free(d1); free(d2);
}

/* ------------------------------------------------------------------ 1-D */

/* Section geometry (swe1d.py:51-84) on arrays b, m, yb, ts at index i */
typedef struct { const double *b, *m, *yb, *ts; } orc_sec;

static inline double sec_area(const orc_sec* s, int64_t i, double y) {
    double yt = mind(y, s->yb[i]);
    double at = yt * (s->b[i] + s->m[i] * yt);
    return at + s->ts[i] * clamp0(y - s->yb[i]);
}
static inline double sec_top(const orc_sec* s, int64_t i, double y) {
    return y <= s->yb[i] ? s->b[i] + 2.0 * s->m[i] * y : s->ts[i];
}
static inline double sec_i1(const orc_sec* s, int64_t i, double y) {
    double yt = mind(y, s->yb[i]);
    double above = clamp0(y - s->yb[i]);
    double it = s->b[i] * yt * yt / 2.0 + s->m[i] * (yt * yt * yt) / 3.0;
    double at = yt * (s->b[i] + s->m[i] * yt);
    return it + at * above + s->ts[i] * above * above / 2.0;
}
static inline double sec_perim(const orc_sec* s, int64_t i, double y) {
    double yt = mind(y, s->yb[i]);
    return s->b[i] + 2.0 * yt * sqrt(1.0 + s->m[i] * s->m[i]);
}
static inline double sec_bank_area(const orc_sec* s, int64_t i) {
    return s->yb[i] * (s->b[i] + s->m[i] * s->yb[i]);
}
static inline double sec_depth(const orc_sec* s, int64_t i, double A) {
    A = clamp0(A);
    double ab = sec_bank_area(s, i);
    double b = s->b[i];
    double y_t = 2.0 * A / (b + sqrt(b * b + 4.0 * s->m[i] * A));
    return A <= ab ? y_t : s->yb[i] + (A - ab) / s->ts[i];
}
static inline double vel1d(const orc_cfg* c, const orc_sec* s, int64_t i, double A, double Q) {
    double y = sec_depth(s, i, A);
    return y >= c->h_dry ? Q / (A > 1e-12 ? A : 1e-12) : 0.0;
}

/* 1-D CFL rate max over wet interior cells (swe1d.py:253-262); returns 0 if none */
double orc_swe1d_max_rate(const orc_cfg* c, int n_cells, const int32_t* kind, const double* b, const double* m,
                          const double* yb, const double* ts, const double* dx, const double* A, const double* Q,
                          int32_t* any_wet) {
    orc_sec s = {b, m, yb, ts};
    double mx = 0.0;
    int wet_any = 0;
    for (int i = 0; i < n_cells; ++i) {
        double y = sec_depth(&s, i, A[i]);
        int wet = (y > c->h_dry) && kind[i] <= 1;
        if (!wet) continue;
        wet_any = 1;
        double cc = sqrt(c->g * A[i] / sec_top(&s, i, y));
        double u = vel1d(c, &s, i, A[i], Q[i]);
        double r = (fabs(u) + cc) / dx[i];
        if (r > mx) mx = r;
    }
    *any_wet = wet_any;
    return mx;
}

static inline void hll_1d(double AL, double QL, double pL, double cL, double AR, double QR, double pR, double cR,
                          double uL, double uR, double* F1o, double* F2o) {
    const double tiny = 1e-14;
    int dryL = AL <= tiny, dryR = AR <= tiny;
    double SL = mind(uL - cL, uR - cR);
    double SR = maxd(uL + cL, uR + cR);
    if (dryL) { SL = uR - 2.0 * cR; SR = uR + cR; }
    if (dryR) { SL = uL - cL; SR = uL + 2.0 * cL; }
    double FL1 = QL, FR1 = QR;
    double FL2 = QL * uL + pL, FR2 = QR * uR + pR;
    double den = SR - SL;
    if (fabs(den) < tiny) den = 1.0;
    double H1 = (SR * FL1 - SL * FR1 + SL * SR * (AR - AL)) / den;
    double H2 = (SR * FL2 - SL * FR2 + SL * SR * (QR - QL)) / den;
    int left = SL >= 0.0, right = SR <= 0.0;
    double F1 = left ? FL1 : (right ? FR1 : H1);
    double F2 = left ? FL2 : (right ? FR2 : H2);
    if (dryL && dryR) { F1 = 0.0; F2 = 0.0; }
    *F1o = F1; *F2o = F2;
}

/* One 1-D step (swe1d.py:320-368) for one member.
   kind: 0 reach, 1 junction, 2 ghost-inflow, 3 ghost-stage, 4 ghost-closed.
   gsrc / gsign: interior neighbour and +-1 for ghosts.
   Cell sections b, m, yb, ts (n_cells); face sections fb, fm, fyb, fts (n_faces).
   out: [bnd_in, bnd_out, clip] (m^3). */
void orc_swe1d_step(const orc_cfg* c, int n_cells, int n_faces, const int32_t* kind, const int32_t* gsrc,
                    const double* gsign, const int32_t* fl, const int32_t* fr, const double* z, const double* nman,
                    const double* dx, const double* b, const double* m, const double* yb, const double* ts,
                    const double* fb, const double* fm, const double* fyb, const double* fts,
                    double q_in, double eta, double dt, double* A, double* Q, double* out) {
    const double g = c->g;
    orc_sec s = {b, m, yb, ts}, fs = {fb, fm, fyb, fts};
    double* Ag = malloc(sizeof(double) * n_cells);
    double* Qg = malloc(sizeof(double) * n_cells);
    double* y = malloc(sizeof(double) * n_cells);
    double* u = malloc(sizeof(double) * n_cells);
    double* theta = malloc(sizeof(double) * n_cells);
    double* acc = malloc(sizeof(double) * n_cells);
    double* accQ = malloc(sizeof(double) * n_cells);
    double* F1 = malloc(sizeof(double) * n_faces);
    double* F2 = malloc(sizeof(double) * n_faces);
    double* pL = malloc(sizeof(double) * n_faces);
    double* pR = malloc(sizeof(double) * n_faces);
    memcpy(Ag, A, sizeof(double) * n_cells);
    memcpy(Qg, Q, sizeof(double) * n_cells);
    /* ghosts (swe1d.py:265-294), computed from the pre-step interior state */
    for (int gi = 0; gi < n_cells; ++gi) {
        if (kind[gi] < 2) continue;
        int src = gsrc[gi];
        double As = A[src], Qs = Q[src], sg = gsign[gi];
        double ys = sec_depth(&s, gi, As);
        double zg = z[gi];
        double un = sg * vel1d(c, &s, gi, As, Qs);
        int wet_i = ys >= c->h_dry;
        double Anew, Qnew;
        if (kind[gi] == 3) {
            double yst = clamp0(eta - zg);
            double Ast = sec_area(&s, gi, yst);
            double ci = sqrt(g * As / sec_top(&s, gi, ys));
            double cg = sqrt(g * Ast / sec_top(&s, gi, yst));
            double un_st = wet_i ? un + 2.0 * (ci - cg) : 0.0;
            int sup = wet_i && (un > ci);
            if (sup) { un_st = un; Ast = As; }
            if (!(sec_depth(&s, gi, Ast) >= c->h_dry)) un_st = 0.0;
            Anew = Ast;
            Qnew = sg * Ast * un_st;
        } else if (kind[gi] == 2) {
            double yc = maxd(pow(q_in * q_in / (g * b[gi] * b[gi]), 1.0 / 3.0), c->h_dry);
            Anew = wet_i ? As : sec_area(&s, gi, yc);
            Qnew = -sg * q_in;
        } else {
            Anew = As;
            Qnew = -Qs;
        }
        Ag[gi] = Anew;
        Qg[gi] = Qnew;
    }
    for (int i = 0; i < n_cells; ++i) {
        y[i] = sec_depth(&s, i, Ag[i]);
        u[i] = vel1d(c, &s, i, Ag[i], Qg[i]);
    }
    for (int f = 0; f < n_faces; ++f) {
        int l = fl[f], r = fr[f];
        double zL = z[l], zR = z[r];
        double zf = maxd(zL, zR);
        double yL = clamp0(zL + y[l] - zf), yR = clamp0(zR + y[r] - zf);
        double AL = sec_area(&fs, f, yL), AR = sec_area(&fs, f, yR);
        double uL = u[l], uR = u[r];
        pL[f] = g * sec_i1(&fs, f, yL);
        pR[f] = g * sec_i1(&fs, f, yR);
        double cL = sqrt(g * AL / sec_top(&fs, f, yL));
        double cR = sqrt(g * AR / sec_top(&fs, f, yR));
        hll_1d(AL, AL * uL, pL[f], cL, AR, AR * uR, pR[f], cR, uL, uR, &F1[f], &F2[f]);
    }
    /* conservative outflow limiter (swe1d.py:337-344); index_add order: all fl, then all fr */
    for (int i = 0; i < n_cells; ++i) acc[i] = 0.0;
    for (int f = 0; f < n_faces; ++f) acc[fl[f]] += relu(F1[f]);
    for (int f = 0; f < n_faces; ++f) acc[fr[f]] += relu(-F1[f]);
    for (int i = 0; i < n_cells; ++i) {
        double vol = Ag[i] * dx[i];
        double need = acc[i] * dt;
        double th = need > vol ? vol / (need > 0.0 ? need : 1.0) : 1.0;
        theta[i] = kind[i] >= 2 ? 1.0 : th;
    }
    for (int f = 0; f < n_faces; ++f) {
        double sc = F1[f] > 0.0 ? theta[fl[f]] : theta[fr[f]];
        F1[f] = F1[f] * sc;
    }
    for (int i = 0; i < n_cells; ++i) { acc[i] = 0.0; accQ[i] = 0.0; }
    for (int f = 0; f < n_faces; ++f) acc[fl[f]] += -F1[f];
    for (int f = 0; f < n_faces; ++f) acc[fr[f]] += F1[f];
    for (int f = 0; f < n_faces; ++f) accQ[fl[f]] += -(F2[f] - pL[f]);
    for (int f = 0; f < n_faces; ++f) accQ[fr[f]] += F2[f] - pR[f];
    double clip = 0.0;
    for (int i = 0; i < n_cells; ++i) {
        double A1 = Ag[i] + dt * acc[i] / dx[i];
        double Q1 = Qg[i] + dt * accQ[i] / dx[i];
        double neg = clamp0(-A1);
        clip += neg * dx[i] * (kind[i] >= 2 ? 0.0 : 1.0);
        A1 = A1 + neg;
        /* semi-implicit friction (swe1d.py:358-364) */
        double y1 = sec_depth(&s, i, A1);
        double Ac = A1 > 1e-12 ? A1 : 1e-12;
        double R = Ac / sec_perim(&s, i, y1);
        double denom = 1.0 + dt * g * (nman[i] * nman[i]) * fabs(Q1) / (Ac * pow(maxd(R, c->h_dry), 4.0 / 3.0));
        Q1 = Q1 / denom;
        if (!((y1 >= c->h_dry) && kind[i] != 1)) Q1 = 0.0;
        if (kind[i] >= 2) { A1 = Ag[i]; Q1 = Qg[i]; }
        A[i] = A1;
        Q[i] = Q1;
    }
    double bi = 0.0, bo = 0.0, bi2 = 0.0, bo2 = 0.0;
    for (int f = 0; f < n_faces; ++f) {
        if (kind[fl[f]] >= 2) { bi += relu(F1[f]); bo += relu(-F1[f]); }
    }
    for (int f = 0; f < n_faces; ++f) {
        if (kind[fr[f]] >= 2) { bi2 += relu(-F1[f]); bo2 += relu(F1[f]); }
    }
    out[0] = (bi + bi2) * dt;
    out[1] = (bo + bo2) * dt;
    out[2] = clip;
    free(Ag); free(Qg); free(y); free(u); free(theta); free(acc); free(accQ); free(F1); free(F2); free(pL); free(pR);
}

/* ------------------------------------------------------------ exchange */

/* 1-D <-> 2-D weir exchange for one member (coupling.py:73-124).
   Links: cell1d, zbank, length, z2, inv (-> unique 2-D cell), uniq (flat 2-D index).
   Updates h, hu, hv (2-D, flat) and A (1-D) in place; V out per link (+ = 2-D -> 1-D). */
void orc_exchange(const orc_cfg* c, int n_links, int n_unique, int n_cells, const int32_t* cell1d,
                  const double* zbank, const double* length, const double* z2, const int32_t* inv,
                  const int64_t* uniq, const double* z1, const double* dx1, const double* b, const double* m,
                  const double* yb, const double* ts, double area2, double dt,
                  double* h, double* hu, double* hv, double* A, double* V) {
    orc_sec s = {b, m, yb, ts};
    double* h_u = malloc(sizeof(double) * n_unique);
    double* tot2 = malloc(sizeof(double) * n_unique);
    double* f2 = malloc(sizeof(double) * n_unique);
    double* tot1 = malloc(sizeof(double) * n_cells);
    double* f1 = malloc(sizeof(double) * n_cells);
    double* sign = malloc(sizeof(double) * n_links);
    for (int k = 0; k < n_unique; ++k) h_u[k] = h[uniq[k]];
    for (int l = 0; l < n_links; ++l) {
        int c1 = cell1d[l];
        double h2 = h_u[inv[l]];
        double eta2 = z2[l] + h2;
        double y1 = sec_depth(&s, c1, A[c1]);
        double eta1 = z1[c1] + y1;
        double zb = zbank[l];
        double up = maxd(eta1, eta2), dn = mind(eta1, eta2);
        double d_up = clamp0(up - zb), d_dn = clamp0(dn - zb);
        double ratio = d_up > 0.0 ? d_dn / d_up : 0.0;
        double q = c->weir_cw * length[l] * pow(d_up, 1.5) * pow(clamp0(1.0 - pow(ratio, 1.5)), 0.385);
        sign[l] = eta2 > eta1 ? 1.0 : -1.0;
        double v = q * dt;
        double plan1 = (y1 <= yb[c1] ? b[c1] + 2.0 * m[c1] * y1 : ts[c1]) * dx1[c1];
        double v_eq = (up - dn) / (1.0 / area2 + 1.0 / plan1);
        v = mind(v, c->exchange_relax * v_eq);
        V[l] = v;
    }
    for (int k = 0; k < n_unique; ++k) tot2[k] = 0.0;
    for (int l = 0; l < n_links; ++l) tot2[inv[l]] += sign[l] > 0.0 ? V[l] : 0.0;
    for (int k = 0; k < n_unique; ++k) {
        double avail = c->exchange_limit * h_u[k] * area2;
        f2[k] = tot2[k] > avail ? avail / (tot2[k] > 0.0 ? tot2[k] : 1.0) : 1.0;
    }
    for (int i = 0; i < n_cells; ++i) tot1[i] = 0.0;
    for (int l = 0; l < n_links; ++l) tot1[cell1d[l]] += sign[l] < 0.0 ? V[l] : 0.0;
    for (int i = 0; i < n_cells; ++i) {
        double avail = c->exchange_limit * clamp0(A[i] - sec_bank_area(&s, i)) * dx1[i];
        f1[i] = tot1[i] > avail ? avail / (tot1[i] > 0.0 ? tot1[i] : 1.0) : 1.0;
    }
    for (int l = 0; l < n_links; ++l) {
        double v = sign[l] > 0.0 ? V[l] * f2[inv[l]] : V[l] * f1[cell1d[l]];
        V[l] = v * sign[l];
    }
    for (int k = 0; k < n_unique; ++k) tot2[k] = 0.0;
    for (int l = 0; l < n_links; ++l) tot2[inv[l]] += V[l];
    for (int k = 0; k < n_unique; ++k) {
        double hn = h_u[k] - tot2[k] / area2;
        double keep = h_u[k] > 0.0 ? mind(hn / (h_u[k] > 0.0 ? h_u[k] : 1.0), 1.0) : 0.0;
        int64_t idx = uniq[k];
        h[idx] = hn;
        hu[idx] = hu[idx] * keep;
        hv[idx] = hv[idx] * keep;
    }
    for (int i = 0; i < n_cells; ++i) tot1[i] = 0.0;
    for (int l = 0; l < n_links; ++l) tot1[cell1d[l]] += V[l];
    for (int i = 0; i < n_cells; ++i) A[i] = A[i] + tot1[i] / dx1[i];
    free(h_u); free(tot2); free(f2); free(tot1); free(f1); free(sign);
}
