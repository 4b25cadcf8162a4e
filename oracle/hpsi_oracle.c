/*
 * hpsi_oracle.c — CPU restatement (FP64) of the reference's H|psi> path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline legs of bench.py load this library, and only as the checker or
 * as the timed CPU baseline — never as the product path.
 *
 * Each function follows the reference (bzzlfd/effmass) step by step; the
 * citations are file:line in that project.  Its pins are the reference's own
 * outputs on the same inputs (tests/golden, made by oracle/ref_driver.cpp from
 * the reference sources) and the known-answer tests of the reference's unit
 * tests (test/math/test_fft.cpp, test/math/test_sph_harmonics.cpp,
 * test/H_psi/test_structure_factor.cpp), restated in tests/test_oracle.py.
 *
 * Built with -ffp-contract=off so that no fused multiply-add changes the
 * rounding relative to the reference's scalar C++.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../include/hpsi_gb300.h"
#include "mrfft.h"

#define PI_D 3.141592653589793238462643383279502884

/* ------------------------------------------------------------------------ */
/* spherical coordinates of K (src/io/GKK.cppm:431-449)                      */
/* ------------------------------------------------------------------------ */
void oracle_spherical(int ng, const double* K, double* q, double* theta, double* phi)
{
    for (int ig = 0; ig < ng; ++ig) {
        double kx = K[3 * ig], ky = K[3 * ig + 1], kz = K[3 * ig + 2];
        double qq = sqrt(kx * kx + ky * ky + kz * kz);
        q[ig] = qq;
        theta[ig] = (qq > 0.0) ? acos(kz / qq) : 0.0;
        phi[ig] = atan2(ky, kx);
    }
}

/* ------------------------------------------------------------------------ */
/* real Y_lm and angular gradients                                           */
/*  trig tables        src/math/sph_harmonics.cppm:489-502                   */
/*  Q recurrence       :120-170 (seed/step1/advance), used by setLMax :643-696 */
/*  R = Q/sin(theta)   :188-243, filled by :789-828                          */
/*  dQ/dtheta          :268-335, filled by :877-916                          */
/*  assembly get()     :702-735; get_ang_grad_phi :737-787;                  */
/*                     get_ang_grad_theta :830-875                           */
/* Output layout: y[(l*l + l + m)*ng + ig] (the reference's flat (l,m) index  */
/* of RealSphericalHarmonicsData::get, :1001).  dth/dph may be NULL.          */
/* ------------------------------------------------------------------------ */
static double seed_coeff(int m)
{
    double Q0 = 0.5 / sqrt(PI_D);
    double coeff = Q0;
    if (m % 2 != 0) coeff = -coeff;
    for (int k = 1; k <= m; ++k) coeff *= sqrt((double)(2 * k + 1) / (2 * k));
    return coeff;
}

static void rec_coeffs(int l, int m, double* r1, double* r2, double* denom)
{
    *r1 = (2.0 * l - 1.0) * sqrt(((2.0 * l + 1.0) * (l - m)) / ((2.0 * l - 1.0) * (l + m)));
    *r2 = (l + m - 1.0) * sqrt(((2.0 * l + 1.0) * (l - m) * (l - m - 1)) /
                               ((2.0 * l - 3.0) * (l + m) * (l + m - 1)));
    *denom = 1.0 / (l - m);
}

void oracle_ylm(int lmax, int ng, const double* theta, const double* phi, double* y, double* dth, double* dph)
{
    const int ntri = (lmax + 1) * (lmax + 2) / 2;
    double* ct = (double*)malloc(sizeof(double) * ng * 4);
    double* st = ct + ng;
    double* cp = st + ng;
    double* sp = cp + ng;
    for (int i = 0; i < ng; ++i) { ct[i] = cos(theta[i]); st[i] = sin(theta[i]); }
    for (int i = 0; i < ng; ++i) { cp[i] = cos(phi[i]); sp[i] = sin(phi[i]); }

    double* Q = (double*)calloc((size_t)ntri * ng, sizeof(double));   /* Q[l(l+1)/2+m] */
    double* R = (double*)calloc((size_t)ntri * ng, sizeof(double));   /* Q/sin(theta) */
    double* dQ = (double*)calloc((size_t)ntri * ng, sizeof(double));  /* dQ/dtheta */
    double* cm = (double*)malloc(sizeof(double) * (lmax + 1) * ng);
    double* sm = (double*)malloc(sizeof(double) * (lmax + 1) * ng);
    double* prev = (double*)malloc(sizeof(double) * ng);
    double* curr = (double*)malloc(sizeof(double) * ng);
#define TRI(l, m) ((size_t)((l) * ((l) + 1) / 2 + (m)) * ng)

    /* Q_l^m and cos(m phi), sin(m phi) */
    for (int i = 0; i < ng; ++i) { cm[i] = 1.0; sm[i] = 0.0; }
    double* cmw = (double*)malloc(sizeof(double) * ng);
    double* smw = (double*)malloc(sizeof(double) * ng);
    for (int i = 0; i < ng; ++i) { cmw[i] = 1.0; smw[i] = 0.0; }
    for (int m = 0; m <= lmax; ++m) {
        if (m == 0) {
            double Q0 = 0.5 / sqrt(PI_D);
            for (int i = 0; i < ng; ++i) curr[i] = Q0;
        } else {
            double c = seed_coeff(m);
            for (int i = 0; i < ng; ++i) curr[i] = c * pow(st[i], m);
        }
        memcpy(Q + TRI(m, m), curr, sizeof(double) * ng);
        if (m < lmax) {
            double f = sqrt(2.0 * m + 3.0);
            for (int i = 0; i < ng; ++i) { prev[i] = curr[i]; curr[i] = f * ct[i] * curr[i]; }
            memcpy(Q + TRI(m + 1, m), curr, sizeof(double) * ng);
            for (int l = m + 2; l <= lmax; ++l) {
                double r1, r2, dn;
                rec_coeffs(l, m, &r1, &r2, &dn);
                for (int i = 0; i < ng; ++i) {
                    double nx = (ct[i] * r1 * curr[i] - r2 * prev[i]) * dn;
                    prev[i] = curr[i];
                    curr[i] = nx;
                }
                memcpy(Q + TRI(l, m), curr, sizeof(double) * ng);
            }
        }
        memcpy(cm + (size_t)m * ng, cmw, sizeof(double) * ng);
        memcpy(sm + (size_t)m * ng, smw, sizeof(double) * ng);
        if (m < lmax) {
            for (int i = 0; i < ng; ++i) {
                double old = cmw[i];
                cmw[i] = cmw[i] * cp[i] - smw[i] * sp[i];
                smw[i] = smw[i] * cp[i] + old * sp[i];
            }
        }
    }
    free(cmw);
    free(smw);

    /* R_l^m = Q_l^m / sin(theta), m >= 1 */
    for (int m = 1; m <= lmax; ++m) {
        double c = seed_coeff(m);
        if (m == 1) for (int i = 0; i < ng; ++i) curr[i] = c;
        else for (int i = 0; i < ng; ++i) curr[i] = c * pow(st[i], m - 1);
        memcpy(R + TRI(m, m), curr, sizeof(double) * ng);
        if (m < lmax) {
            double f = sqrt(2.0 * m + 3.0);
            for (int i = 0; i < ng; ++i) { prev[i] = curr[i]; curr[i] = f * ct[i] * curr[i]; }
            memcpy(R + TRI(m + 1, m), curr, sizeof(double) * ng);
            for (int l = m + 2; l <= lmax; ++l) {
                double r1, r2, dn;
                rec_coeffs(l, m, &r1, &r2, &dn);
                for (int i = 0; i < ng; ++i) {
                    double nx = (ct[i] * r1 * curr[i] - r2 * prev[i]) * dn;
                    prev[i] = curr[i];
                    curr[i] = nx;
                }
                memcpy(R + TRI(l, m), curr, sizeof(double) * ng);
            }
        }
    }

    /* dQ_l^m / dtheta */
    for (int m = 0; m <= lmax; ++m) {
        if (m == 0) {
            for (int i = 0; i < ng; ++i) curr[i] = 0.0;
        } else {
            double c = seed_coeff(m);
            if (m == 1) for (int i = 0; i < ng; ++i) curr[i] = c * ct[i];
            else {
                double f = (double)m * c;
                for (int i = 0; i < ng; ++i) curr[i] = f * pow(st[i], m - 1) * ct[i];
            }
        }
        memcpy(dQ + TRI(m, m), curr, sizeof(double) * ng);
        if (m < lmax) {
            double f = sqrt(2.0 * m + 3.0);
            const double* Qmm = Q + TRI(m, m);
            for (int i = 0; i < ng; ++i) { prev[i] = curr[i]; curr[i] = f * (-st[i] * Qmm[i] + ct[i] * curr[i]); }
            memcpy(dQ + TRI(m + 1, m), curr, sizeof(double) * ng);
            for (int l = m + 2; l <= lmax; ++l) {
                double r1, r2, dn;
                rec_coeffs(l, m, &r1, &r2, &dn);
                const double* Ql1 = Q + TRI(l - 1, m);
                for (int i = 0; i < ng; ++i) {
                    double nx = (ct[i] * r1 * curr[i] - st[i] * r1 * Ql1[i] - r2 * prev[i]) * dn;
                    prev[i] = curr[i];
                    curr[i] = nx;
                }
                memcpy(dQ + TRI(l, m), curr, sizeof(double) * ng);
            }
        }
    }

    const double sf = sqrt(2.0);
    for (int l = 0; l <= lmax; ++l) {
        for (int m = -l; m <= l; ++m) {
            int ma = m < 0 ? -m : m;
            double* yo = y + (size_t)(l * l + l + m) * ng;
            const double* Qv = Q + TRI(l, ma);
            const double* c_ = cm + (size_t)ma * ng;
            const double* s_ = sm + (size_t)ma * ng;
            for (int i = 0; i < ng; ++i) {
                if (m == 0) yo[i] = Qv[i];
                else {
                    double val = sf * Qv[i];
                    yo[i] = (m > 0) ? val * c_[i] : val * s_[i];
                }
            }
            if (dph) {
                double* po = dph + (size_t)(l * l + l + m) * ng;
                const double* Rv = R + TRI(l, ma);
                if (m == 0) for (int i = 0; i < ng; ++i) po[i] = 0.0;
                else if (m > 0) {
                    double fac = -(double)m * sf;
                    for (int i = 0; i < ng; ++i) po[i] = fac * Rv[i] * s_[i];
                } else {
                    double fac = (double)ma * sf;
                    for (int i = 0; i < ng; ++i) po[i] = fac * Rv[i] * c_[i];
                }
            }
            if (dth) {
                double* to = dth + (size_t)(l * l + l + m) * ng;
                const double* dv = dQ + TRI(l, ma);
                if (m == 0) for (int i = 0; i < ng; ++i) to[i] = dv[i];
                else if (m > 0) for (int i = 0; i < ng; ++i) to[i] = sf * dv[i] * c_[i];
                else for (int i = 0; i < ng; ++i) to[i] = sf * dv[i] * s_[i];
            }
        }
    }
#undef TRI
    free(ct); free(Q); free(R); free(dQ); free(cm); free(sm); free(prev); free(curr);
}

/* ------------------------------------------------------------------------ */
/* beta(q) interpolation: BetaqTables::interpolate                           */
/* (src/pseudo/ncpp_advance.cppm:644-674) with lagrangeCubic                 */
/* (src/math/numerical.cppm:93-104).  Returns HPSI_ERR_RANGE for q > q_max.  */
/* ------------------------------------------------------------------------ */
static double lagrange_cubic(double f0, double f1, double f2, double f3, double px)
{
    double ux = 1.0 - px, vx = 2.0 - px, wx = 3.0 - px;
    return f0 * ux * vx * wx / 6.0 + f1 * px * vx * wx / 2.0 - f2 * px * ux * wx / 2.0 +
           f3 * px * ux * vx / 6.0;
}

int oracle_beta_interp(const double* t, int nq, double dq, double q_max, double norm, double q, double* out)
{
    if (q < 0.0 || q > q_max) return HPSI_ERR_RANGE;
    if (q == 0.0) { *out = t[0] * norm; return HPSI_OK; }
    double s = q / dq;
    int i0 = (int)floor(s) - 1;
    double px = s - (double)i0;
    if (i0 < 0) { i0 = 0; px = s; }
    if (i0 + 3 >= nq) return HPSI_ERR_RANGE;
    *out = lagrange_cubic(t[i0], t[i0 + 1], t[i0 + 2], t[i0 + 3], px) * norm;
    return HPSI_OK;
}

/* ------------------------------------------------------------------------ */
/* structure factor S(g,k) = exp(-i 2 pi (k+g).tau), separable mode          */
/* (src/H_psi/structure_factor.cppm:92-123, cache :136-159).                 */
/* out: [ng] interleaved complex.                                            */
/* ------------------------------------------------------------------------ */
static inline void cmul(double ar, double ai, double br, double bi, double* cr, double* ci)
{
    *cr = ar * br - ai * bi;
    *ci = ar * bi + ai * br;
}

int oracle_structure_factor(int ng, const int* g, const double* kf, const double* tau, int n1, int n2, int n3, double* out)
{
    const double kd = -2.0 * PI_D * (kf[0] * tau[0] + kf[1] * tau[1] + kf[2] * tau[2]);
    const double kpr = cos(kd), kpi = sin(kd);
    const int n[3] = {n1, n2, n3};
    for (int ig = 0; ig < ng; ++ig) {
        double pr[3], pi_[3];
        for (int d = 0; d < 3; ++d) {
            int gd = g[3 * ig + d];
            /* cache index g + n/2 + 4 must lie in [0, n+8) */
            int idx = gd + n[d] / 2 + 4;
            if (idx < 0 || idx >= n[d] + 8) return HPSI_ERR_RANGE;
            double a = -2.0 * PI_D * gd * tau[d];
            pr[d] = cos(a);
            pi_[d] = sin(a);
        }
        double r, i, r2, i2;
        cmul(kpr, kpi, pr[0], pi_[0], &r, &i);
        cmul(r, i, pr[1], pi_[1], &r2, &i2);
        cmul(r2, i2, pr[2], pi_[2], &r, &i);
        out[2 * ig] = r;
        out[2 * ig + 1] = i;
    }
    return HPSI_OK;
}

/* ------------------------------------------------------------------------ */
/* FFT3D (src/math/fft.cppm:60-85): 1-D lines along n3, then n2, then n1.     */
/* dir = +1: G2R (backward, factor 1); dir = -1: R2G (forward, 1/n per axis).  */
/* ------------------------------------------------------------------------ */
void oracle_fft3d(double* grid, int n1, int n2, int n3, int dir)
{
    int nmax = n1 > n2 ? n1 : n2;
    if (n3 > nmax) nmax = n3;
    double* line = (double*)malloc(sizeof(double) * 2 * nmax);
    int ns[3] = {n1, n2, n3};
    mrfft_plan_s* pl[3];
    for (int d = 0; d < 3; ++d) pl[d] = mrfft_make(ns[d]);
    const int sign = dir > 0 ? +1 : -1;
    size_t s23 = (size_t)n2 * n3;
    for (int i = 0; i < n1; ++i)
        for (int j = 0; j < n2; ++j) {
            double* p = grid + 2 * ((size_t)i * s23 + (size_t)j * n3);
            if (n3 > 1) mrfft_exec(pl[2], p, sign, dir > 0 ? 1.0 : 1.0 / n3);
        }
    if (n2 > 1)
        for (int i = 0; i < n1; ++i)
            for (int k = 0; k < n3; ++k) {
                for (int j = 0; j < n2; ++j) {
                    size_t o = 2 * ((size_t)i * s23 + (size_t)j * n3 + k);
                    line[2 * j] = grid[o]; line[2 * j + 1] = grid[o + 1];
                }
                mrfft_exec(pl[1], line, sign, dir > 0 ? 1.0 : 1.0 / n2);
                for (int j = 0; j < n2; ++j) {
                    size_t o = 2 * ((size_t)i * s23 + (size_t)j * n3 + k);
                    grid[o] = line[2 * j]; grid[o + 1] = line[2 * j + 1];
                }
            }
    if (n1 > 1)
        for (int j = 0; j < n2; ++j)
            for (int k = 0; k < n3; ++k) {
                for (int i = 0; i < n1; ++i) {
                    size_t o = 2 * ((size_t)i * s23 + (size_t)j * n3 + k);
                    line[2 * i] = grid[o]; line[2 * i + 1] = grid[o + 1];
                }
                mrfft_exec(pl[0], line, sign, dir > 0 ? 1.0 : 1.0 / n1);
                for (int i = 0; i < n1; ++i) {
                    size_t o = 2 * ((size_t)i * s23 + (size_t)j * n3 + k);
                    grid[o] = line[2 * i]; grid[o + 1] = line[2 * i + 1];
                }
            }
    for (int d = 0; d < 3; ++d) mrfft_free(pl[d]);
    free(line);
}

/* ------------------------------------------------------------------------ */
/* per-k preparation shared by H and dH/dk                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    int ng, lmax;
    double *q, *theta, *phi;
    double *ct, *st, *cp, *sp;
    double *y, *yth, *yph;  /* [(lmax+1)^2][ng] */
} kprep;

static int species_lmax(const hpsi_system* sys)
{
    int lmax = 0;
    for (int s = 0; s < sys->n_species; ++s)
        for (int i = 0; i < sys->species[s].n_proj; ++i)
            if (sys->species[s].proj_l[i] > lmax) lmax = sys->species[s].proj_l[i];
    return lmax;
}

static void kprep_init(kprep* P, const hpsi_system* sys, const hpsi_kpoint* kp, int grads)
{
    int ng = kp->npw;
    P->ng = ng;
    P->lmax = species_lmax(sys);
    int nlm = (P->lmax + 1) * (P->lmax + 1);
    P->q = (double*)malloc(sizeof(double) * ng * 7);
    P->theta = P->q + ng; P->phi = P->theta + ng;
    P->ct = P->phi + ng; P->st = P->ct + ng; P->cp = P->st + ng; P->sp = P->cp + ng;
    oracle_spherical(ng, kp->kvec, P->q, P->theta, P->phi);
    for (int i = 0; i < ng; ++i) {
        P->ct[i] = cos(P->theta[i]); P->st[i] = sin(P->theta[i]);
        P->cp[i] = cos(P->phi[i]); P->sp[i] = sin(P->phi[i]);
    }
    P->y = (double*)malloc(sizeof(double) * (size_t)nlm * ng * (grads ? 3 : 1));
    P->yth = grads ? P->y + (size_t)nlm * ng : NULL;
    P->yph = grads ? P->y + (size_t)2 * nlm * ng : NULL;
    oracle_ylm(P->lmax, ng, P->theta, P->phi, P->y, P->yth, P->yph);
}

static void kprep_free(kprep* P)
{
    free(P->q);
    free(P->y);
}

/* ------------------------------------------------------------------------ */
/* H|psi> for one band (src/H_psi/hamiltonian_callable.cpp:94-356)           */
/* ------------------------------------------------------------------------ */
static int hpsi_one(const hpsi_system* sys, const hpsi_kpoint* kp, const kprep* P, const double* psi,
                    double* hpsi, double* grid)
{
    const int ng = kp->npw, n1 = sys->n1, n2 = sys->n2, n3 = sys->n3;
    const double norm = 1.0 / sqrt(sys->omega);

    /* kinetic :119-126 */
    for (int ig = 0; ig < ng; ++ig) {
        hpsi[2 * ig] += kp->kinetic[ig] * psi[2 * ig];
        hpsi[2 * ig + 1] += kp->kinetic[ig] * psi[2 * ig + 1];
    }

    /* local :138-182 */
    size_t n123 = (size_t)n1 * n2 * n3;
    memset(grid, 0, sizeof(double) * 2 * n123);
    for (int ig = 0; ig < ng; ++ig) {
        int i = ((kp->g_idx[3 * ig] % n1) + n1) % n1;
        int j = ((kp->g_idx[3 * ig + 1] % n2) + n2) % n2;
        int k = ((kp->g_idx[3 * ig + 2] % n3) + n3) % n3;
        size_t idx = (size_t)i * n2 * n3 + (size_t)j * n3 + k;
        grid[2 * idx] = psi[2 * ig];
        grid[2 * idx + 1] = psi[2 * ig + 1];
    }
    oracle_fft3d(grid, n1, n2, n3, +1);
    for (size_t r = 0; r < n123; ++r) {
        grid[2 * r] *= sys->v_loc[r];
        grid[2 * r + 1] *= sys->v_loc[r];
    }
    oracle_fft3d(grid, n1, n2, n3, -1);
    for (int ig = 0; ig < ng; ++ig) {
        int i = ((kp->g_idx[3 * ig] % n1) + n1) % n1;
        int j = ((kp->g_idx[3 * ig + 1] % n2) + n2) % n2;
        int k = ((kp->g_idx[3 * ig + 2] % n3) + n3) % n3;
        size_t idx = (size_t)i * n2 * n3 + (size_t)j * n3 + k;
        hpsi[2 * ig] += grid[2 * idx];
        hpsi[2 * ig + 1] += grid[2 * idx + 1];
    }

    /* nonlocal :200-304 */
    double* beta = (double*)malloc(sizeof(double) * ng);
    double* S = (double*)malloc(sizeof(double) * 2 * ng);
    int rc = HPSI_OK;
    for (int s = 0; s < sys->n_species && rc == HPSI_OK; ++s) {
        const hpsi_species* sp = &sys->species[s];
        for (int a = 0; a < sys->n_atoms && rc == HPSI_OK; ++a) {
            if (sys->atom_species[a] != s) continue;
            rc = oracle_structure_factor(ng, kp->g_idx, kp->k_frac, sys->atom_tau + 3 * a, n1, n2, n3, S);
            if (rc) break;
            for (int ip = 0; ip < sp->n_proj && rc == HPSI_OK; ++ip) {
                double lam = sp->lambda[ip];
                if (fabs(lam) < 1e-15) continue;
                int l = sp->proj_l[ip];
                const double* tab = sp->beta_q + (size_t)ip * sp->nq;
                for (int ig = 0; ig < ng; ++ig) {
                    rc = oracle_beta_interp(tab, sp->nq, sp->dq, sp->q_max, norm, P->q[ig], &beta[ig]);
                    if (rc) break;
                }
                if (rc) break;
                for (int m = -l; m <= l; ++m) {
                    const double* ylm = P->y + (size_t)(l * l + l + m) * ng;
                    double inr = 0.0, ini = 0.0;
                    for (int ig = 0; ig < ng; ++ig) {
                        double by = beta[ig] * ylm[ig];
                        double pr = by * S[2 * ig], pi_ = by * S[2 * ig + 1];
                        /* conj(p) * psi */
                        inr += pr * psi[2 * ig] + pi_ * psi[2 * ig + 1];
                        ini += pr * psi[2 * ig + 1] - pi_ * psi[2 * ig];
                    }
                    double cr = lam * inr, ci = lam * ini;
                    for (int ig = 0; ig < ng; ++ig) {
                        double by = beta[ig] * ylm[ig];
                        double pr = by * S[2 * ig], pi_ = by * S[2 * ig + 1];
                        hpsi[2 * ig] += cr * pr - ci * pi_;
                        hpsi[2 * ig + 1] += cr * pi_ + ci * pr;
                    }
                }
            }
        }
    }
    free(beta);
    free(S);
    return rc;
}

typedef struct {
    const hpsi_system* sys;
    const hpsi_kpoint* kp;
    const kprep* P;
    const double* psi;
    double* hpsi;
    int b0, b1, rc;
} hjob;

static void* hjob_run(void* arg)
{
    hjob* J = (hjob*)arg;
    size_t n123 = (size_t)J->sys->n1 * J->sys->n2 * J->sys->n3;
    double* grid = (double*)malloc(sizeof(double) * 2 * n123);
    size_t ng = (size_t)J->kp->npw;
    J->rc = HPSI_OK;
    for (int b = J->b0; b < J->b1 && J->rc == HPSI_OK; ++b)
        J->rc = hpsi_one(J->sys, J->kp, J->P, J->psi + 2 * ng * b, J->hpsi + 2 * ng * b, grid);
    free(grid);
    return NULL;
}

/* hpsi[b] += H psi[b], b < nb, on `nthreads` host threads (bands split evenly). */
int oracle_hpsi(const hpsi_system* sys, const hpsi_kpoint* kp, int nb, const double* psi, double* hpsi, int nthreads)
{
    if (!sys || !kp || nb < 0 || (nb > 0 && (!psi || !hpsi))) return HPSI_ERR_BAD_ARG;
    if (nb == 0 || kp->npw == 0) return HPSI_OK;
    kprep P;
    kprep_init(&P, sys, kp, 0);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > nb) nthreads = nb;
    hjob* jobs = (hjob*)calloc(nthreads, sizeof(hjob));
    pthread_t* th = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = (hjob){sys, kp, &P, psi, hpsi, nb * t / nthreads, nb * (t + 1) / nthreads, 0};
        if (nthreads == 1) hjob_run(&jobs[t]);
        else pthread_create(&th[t], NULL, hjob_run, &jobs[t]);
    }
    int rc = HPSI_OK;
    for (int t = 0; t < nthreads; ++t) {
        if (nthreads > 1) pthread_join(th[t], NULL);
        if (jobs[t].rc && !rc) rc = jobs[t].rc;
    }
    free(jobs);
    free(th);
    kprep_free(&P);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* dH/dk_alpha |psi> (src/H_psi/hamiltonian_gradient.cpp:116-294)            */
/* out[a] may be NULL (skip that direction).                                 */
/* ------------------------------------------------------------------------ */
static int grad_one(const hpsi_system* sys, const hpsi_kpoint* kp, const kprep* P, const double* psi, double* out[3])
{
    const int ng = kp->npw;
    const double norm = 1.0 / sqrt(sys->omega);
    for (int d = 0; d < 3; ++d) {
        if (!out[d]) continue;
        for (int ig = 0; ig < ng; ++ig) {
            out[d][2 * ig] += kp->kvec[3 * ig + d] * psi[2 * ig];
            out[d][2 * ig + 1] += kp->kvec[3 * ig + d] * psi[2 * ig + 1];
        }
    }
    double* beta = (double*)malloc(sizeof(double) * ng);
    double* dbeta = (double*)malloc(sizeof(double) * ng);
    double* S = (double*)malloc(sizeof(double) * 2 * ng);
    double* pv = (double*)malloc(sizeof(double) * 8 * ng); /* p, dp_x, dp_y, dp_z interleaved complex */
    int rc = HPSI_OK;
    for (int s = 0; s < sys->n_species && rc == HPSI_OK; ++s) {
        const hpsi_species* sp = &sys->species[s];
        if (!sp->dbeta_q) { rc = HPSI_ERR_STATE; break; }
        for (int a = 0; a < sys->n_atoms && rc == HPSI_OK; ++a) {
            if (sys->atom_species[a] != s) continue;
            rc = oracle_structure_factor(ng, kp->g_idx, kp->k_frac, sys->atom_tau + 3 * a, sys->n1, sys->n2, sys->n3, S);
            if (rc) break;
            for (int ip = 0; ip < sp->n_proj && rc == HPSI_OK; ++ip) {
                double lam = sp->lambda[ip];
                if (fabs(lam) < 1e-15) continue;
                int l = sp->proj_l[ip];
                const double* tab = sp->beta_q + (size_t)ip * sp->nq;
                const double* dtab = sp->dbeta_q + (size_t)ip * sp->nq;
                double db0;
                oracle_beta_interp(dtab, sp->nq, sp->dq, sp->q_max, norm, 0.0, &db0);
                for (int ig = 0; ig < ng && rc == HPSI_OK; ++ig) {
                    rc = oracle_beta_interp(tab, sp->nq, sp->dq, sp->q_max, norm, P->q[ig], &beta[ig]);
                    if (!rc) rc = oracle_beta_interp(dtab, sp->nq, sp->dq, sp->q_max, norm, P->q[ig], &dbeta[ig]);
                }
                if (rc) break;
                for (int m = -l; m <= l; ++m) {
                    size_t lm = (size_t)(l * l + l + m) * ng;
                    const double* y = P->y + lm;
                    const double* yt = P->yth + lm;
                    const double* yp = P->yph + lm;
                    double in[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
                    for (int ig = 0; ig < ng; ++ig) {
                        double q = P->q[ig];
                        double beta_ylm = beta[ig] * y[ig];
                        double boq = (q > 1e-12) ? beta[ig] / q : db0;
                        double gq = dbeta[ig] * y[ig];
                        double gt = boq * yt[ig];
                        double gp = boq * yp[ig];
                        double sth = P->st[ig], cth = P->ct[ig], sph = P->sp[ig], cph = P->cp[ig];
                        double f[4];
                        f[0] = beta_ylm;
                        f[1] = sth * cph * gq + cth * cph * gt - sph * gp;
                        f[2] = sth * sph * gq + cth * sph * gt + cph * gp;
                        f[3] = cth * gq - sth * gt;
                        double Sr = S[2 * ig], Si = S[2 * ig + 1];
                        for (int c = 0; c < 4; ++c) {
                            double pr = f[c] * Sr, pi_ = f[c] * Si;
                            pv[8 * ig + 2 * c] = pr;
                            pv[8 * ig + 2 * c + 1] = pi_;
                            in[c][0] += pr * psi[2 * ig] + pi_ * psi[2 * ig + 1];
                            in[c][1] += pr * psi[2 * ig + 1] - pi_ * psi[2 * ig];
                        }
                    }
                    for (int d = 0; d < 3; ++d) {
                        if (!out[d]) continue;
                        double* o = out[d];
                        for (int ig = 0; ig < ng; ++ig) {
                            double pr = pv[8 * ig], pi_ = pv[8 * ig + 1];
                            double dr = pv[8 * ig + 2 * (d + 1)], di = pv[8 * ig + 2 * (d + 1) + 1];
                            /* lambda * (<dp|psi> p + <p|psi> dp) */
                            double t1r = in[d + 1][0] * pr - in[d + 1][1] * pi_;
                            double t1i = in[d + 1][0] * pi_ + in[d + 1][1] * pr;
                            double t2r = in[0][0] * dr - in[0][1] * di;
                            double t2i = in[0][0] * di + in[0][1] * dr;
                            o[2 * ig] += lam * (t1r + t2r);
                            o[2 * ig + 1] += lam * (t1i + t2i);
                        }
                    }
                }
            }
        }
    }
    free(beta); free(dbeta); free(S); free(pv);
    return rc;
}

int oracle_grad(const hpsi_system* sys, const hpsi_kpoint* kp, int nb, const double* psi, double* dx, double* dy, double* dz)
{
    if (!sys || !kp || nb < 0) return HPSI_ERR_BAD_ARG;
    if (nb == 0 || kp->npw == 0) return HPSI_OK;
    kprep P;
    kprep_init(&P, sys, kp, 1);
    size_t ng = (size_t)kp->npw;
    int rc = HPSI_OK;
    for (int b = 0; b < nb && rc == HPSI_OK; ++b) {
        double* out[3] = {dx ? dx + 2 * ng * b : NULL, dy ? dy + 2 * ng * b : NULL, dz ? dz + 2 * ng * b : NULL};
        rc = grad_one(sys, kp, &P, psi + 2 * ng * b, out);
    }
    kprep_free(&P);
    return rc;
}

/* M[a][m][n] = sum_G conj(psi_m[G]) (dH/dk_a psi_n)[G]  (overwrites m_out) */
int oracle_velocity(const hpsi_system* sys, const hpsi_kpoint* kp, int nb, const double* psi, double* m_out)
{
    size_t ng = (size_t)kp->npw;
    double* g = (double*)calloc(3 * 2 * ng * (size_t)nb, sizeof(double));
    int rc = oracle_grad(sys, kp, nb, psi, g, g + 2 * ng * nb, g + 4 * ng * nb);
    if (rc == HPSI_OK) {
        for (int a = 0; a < 3; ++a)
            for (int m = 0; m < nb; ++m)
                for (int n = 0; n < nb; ++n) {
                    const double* pm = psi + 2 * ng * m;
                    const double* hn = g + 2 * ng * ((size_t)a * nb + n);
                    double sr = 0.0, si = 0.0;
                    for (size_t i = 0; i < ng; ++i) {
                        sr += pm[2 * i] * hn[2 * i] + pm[2 * i + 1] * hn[2 * i + 1];
                        si += pm[2 * i] * hn[2 * i + 1] - pm[2 * i + 1] * hn[2 * i];
                    }
                    m_out[2 * (((size_t)a * nb + m) * nb + n)] = sr;
                    m_out[2 * (((size_t)a * nb + m) * nb + n) + 1] = si;
                }
    }
    free(g);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Charge density (src/support/density.cppm:41-94): for every band with a      */
/* non-zero occupation, scatter psi onto a zeroed grid at (g mod n) (the last  */
/* write wins), G2R transform, rho[r] += occ * |psi(r)|^2.  rho accumulates.   */
/* ------------------------------------------------------------------------ */
int oracle_density(const hpsi_system* sys, const hpsi_kpoint* kp, int nb, const double* psi, const double* occ,
                   double* rho)
{
    const int n1 = sys->n1, n2 = sys->n2, n3 = sys->n3, ng = kp->npw;
    const size_t n123 = (size_t)n1 * n2 * n3;
    double* grid = (double*)malloc(sizeof(double) * 2 * n123);
    if (!grid) return HPSI_ERR_OOM;
    for (int b = 0; b < nb; ++b) {
        const double o = occ[b];
        if (o == 0.0) continue;  /* density.cppm:66 */
        const double* ps = psi + (size_t)2 * b * ng;
        memset(grid, 0, sizeof(double) * 2 * n123);
        for (int ig = 0; ig < ng; ++ig) {
            int i = ((kp->g_idx[3 * ig] % n1) + n1) % n1;
            int j = ((kp->g_idx[3 * ig + 1] % n2) + n2) % n2;
            int k = ((kp->g_idx[3 * ig + 2] % n3) + n3) % n3;
            size_t idx = (size_t)i * n2 * n3 + (size_t)j * n3 + k;
            grid[2 * idx] = ps[2 * ig];
            grid[2 * idx + 1] = ps[2 * ig + 1];
        }
        oracle_fft3d(grid, n1, n2, n3, +1);
        for (size_t r = 0; r < n123; ++r) {
            /* std::norm(z) = re^2 + im^2 */
            const double m = grid[2 * r] * grid[2 * r] + grid[2 * r + 1] * grid[2 * r + 1];
            rho[r] += o * m;
        }
    }
    free(grid);
    return HPSI_OK;
}

/* ------------------------------------------------------------------------ */
/* beta(q) and dbeta/dq tables (src/pseudo/ncpp_advance.cppm:524-641, 718-835) */
/* ------------------------------------------------------------------------ */
/* j_l(x) as SphericalBesselJ produces it (src/math/sph_bessel.cppm:15-50,     */
/* 184-210, 295-325): 0 -> delta_l0; x < 0.5 the power series; else j_0, j_1   */
/* in closed form and the upward recurrence.                                  */
static double ref_jl(int l, double x)
{
    if (x < 1e-15) return l == 0 ? 1.0 : 0.0;
    if (x < 0.5) {
        const double x2h = x * x / 2.0;
        double term = 1.0, sum = 1.0;
        for (int k = 1; k <= 50; ++k) {
            term *= -x2h / ((double)k * (2.0 * l + 2.0 * k + 1.0));
            sum += term;
            if (fabs(term) < 1e-16 * fabs(sum)) break;
        }
        double df = 1.0;
        for (int i = 3; i <= 2 * l + 1; i += 2) df *= i;
        return sum * pow(x, l) / df;
    }
    const double j0 = sin(x) / x;
    if (l == 0) return j0;
    const double j1 = j0 / x - cos(x) / x;
    double jp = j0, jc = j1;
    for (int n = 1; n < l; ++n) {
        const double jn = (2.0 * n + 1.0) / x * jc - jp;
        jp = jc;
        jc = jn;
    }
    return jc;
}

/* simpson (src/math/numerical.cppm:33-90): 3/8 rule on the first four points */
/* and 1/3 on the rest for an even count                                    */
static double ref_simpson(const double* f, const double* rab, int n, int uniform)
{
    if (n == 0) return 0.0;
    if (n == 1) return f[0] * rab[0];
    if (uniform) {
        const double dr = rab[0];
        if (n % 2 == 1) {
            double sum = f[0] + f[n - 1];
            for (int i = 1; i < n - 1; ++i) sum += (i % 2 == 0 ? 2.0 : 4.0) * f[i];
            return dr * sum / 3.0;
        }
        if (n == 2) return dr * 0.5 * (f[0] + f[1]);
        const double s38 = f[0] + 3.0 * f[1] + 3.0 * f[2] + f[3];
        double s13 = f[3] + f[n - 1];
        for (int i = 4; i < n - 1; ++i) s13 += (i % 2 == 0 ? 4.0 : 2.0) * f[i];
        return dr * (3.0 / 8.0 * s38 + s13 / 3.0);
    }
    if (n % 2 == 1) {
        double sum = f[0] * rab[0] + f[n - 1] * rab[n - 1];
        for (int i = 1; i < n - 1; ++i) sum += (i % 2 == 0 ? 2.0 : 4.0) * f[i] * rab[i];
        return sum / 3.0;
    }
    if (n == 2) return 0.5 * (f[0] * rab[0] + f[1] * rab[1]);
    const double s38 = f[0] * rab[0] + 3.0 * f[1] * rab[1] + 3.0 * f[2] * rab[2] + f[3] * rab[3];
    double s13 = f[3] * rab[3] + f[n - 1] * rab[n - 1];
    for (int i = 4; i < n - 1; ++i) s13 += (i % 2 == 0 ? 4.0 : 2.0) * f[i] * rab[i];
    return 3.0 / 8.0 * s38 + s13 / 3.0;
}

/* Tables on q_i = i dq, i < ceil(q_max/dq) + 4: beta_q = 4 pi S[beta r j_l(q r)], */
/* dbeta_q = 4 pi S[beta r^2 j_l'(q r)] with j_l' = (l/x) j_l - j_{l+1}          */
/* (j_1'(0) = 1/3, else 0 at x = 0); each projector's trailing zeros trimmed.     */
int oracle_beta_tables(int nr, const double* r, const double* rab, int uniform, int np, const int* l,
                       const double* beta, double dq, double q_max, double* bq, double* dbq)
{
    const int nq = (int)ceil(q_max / dq) + 1 + 3;
    double* f = (double*)malloc(sizeof(double) * (nr > 0 ? nr : 1));
    if (!f) return HPSI_ERR_OOM;
    const double FOUR_PI = 4.0 * 3.14159265358979323846;
    for (int p = 0; p < np; ++p) {
        const double* b = beta + (size_t)p * nr;
        int n = nr;
        while (n > 0 && b[n - 1] == 0.0) --n;
        for (int iq = 0; iq < nq; ++iq) {
            const double q = iq * dq;
            for (int i = 0; i < n; ++i) f[i] = b[i] * r[i] * ref_jl(l[p], q * r[i]);
            bq[(size_t)p * nq + iq] = n ? FOUR_PI * ref_simpson(f, rab, n, uniform) : 0.0;
            if (dbq) {
                for (int i = 0; i < n; ++i) {
                    const double x = q * r[i];
                    double d;
                    if (x < 1e-15) d = l[p] == 1 ? 1.0 / 3.0 : 0.0;
                    else d = (double)l[p] / x * ref_jl(l[p], x) - ref_jl(l[p] + 1, x);
                    f[i] = b[i] * r[i] * r[i] * d;
                }
                dbq[(size_t)p * nq + iq] = n ? FOUR_PI * ref_simpson(f, rab, n, uniform) : 0.0;
            }
        }
    }
    free(f);
    return HPSI_OK;
}

/* d2beta/dq2 tables as D2BetaqTables builds them (src/pseudo/ncpp_advance.cppm: */
/* 908-1085): 4 pi S[beta r^3 j_l''(q r)] with j_l'' from SphericalBesselJ::      */
/* secondDerivValue (src/math/sph_bessel.cppm:242-268):                          */
/*   j_l''(x) = (l(l-1)/x^2 - 1) j_l(x) + (2/x) j_{l+1}(x),  x >= 1e-15,          */
/*   j_0''(0) = -1/3, j_2''(0) = 2/15, else 0;                                    */
/* a q below 1e-15 gives 0 for l other than 0 and 2 (:1019-1023).  Same grid and  */
/* trimming as oracle_beta_tables.                                                */
int oracle_d2beta_tables(int nr, const double* r, const double* rab, int uniform, int np, const int* l,
                         const double* beta, double dq, double q_max, double* d2bq)
{
    const int nq = (int)ceil(q_max / dq) + 1 + 3;
    double* f = (double*)malloc(sizeof(double) * (nr > 0 ? nr : 1));
    if (!f) return HPSI_ERR_OOM;
    const double FOUR_PI = 4.0 * 3.14159265358979323846;
    for (int p = 0; p < np; ++p) {
        const double* b = beta + (size_t)p * nr;
        const int lp = l[p];
        int n = nr;
        while (n > 0 && b[n - 1] == 0.0) --n;
        for (int iq = 0; iq < nq; ++iq) {
            const double q = iq * dq;
            double* out = d2bq + (size_t)p * nq + iq;
            if (q < 1e-15 && lp != 0 && lp != 2) { *out = 0.0; continue; }
            for (int i = 0; i < n; ++i) {
                const double x = q * r[i];
                double d;
                if (fabs(x) < 1e-15) d = lp == 0 ? -1.0 / 3.0 : (lp == 2 ? 2.0 / 15.0 : 0.0);
                else {
                    const double inv_x = 1.0 / x;
                    d = ((double)(lp * (lp - 1)) * inv_x * inv_x - 1.0) * ref_jl(lp, x) + 2.0 * inv_x * ref_jl(lp + 1, x);
                }
                f[i] = b[i] * r[i] * r[i] * r[i] * d;
            }
            *out = n ? FOUR_PI * ref_simpson(f, rab, n, uniform) : 0.0;
        }
    }
    free(f);
    return HPSI_OK;
}

/* g_n(x) = j_n(x) / x^n: power series below x = n + 2, else ref_jl(n, x)/x^n */
static double oracle_gn(int n, double x)
{
    if (x < n + 2.0) {
        const double x2h = x * x / 2.0;
        double term = 1.0, sum = 1.0;
        for (int k = 1; k <= 80; ++k) {
            term *= -x2h / ((double)k * (2.0 * n + 2.0 * k + 1.0));
            sum += term;
            if (fabs(term) < 1e-17 * fabs(sum)) break;
        }
        double df = 1.0;
        for (int i = 3; i <= 2 * n + 1; i += 2) df *= i;
        return sum / df;
    }
    return ref_jl(n, x) / pow(x, n);
}

/* Radial tables of the Hessian's projector second derivatives on q_i = i dq, */
/* i < ceil(q_max/dq) + 4, out [3][np][nq] (F0, F1, F3, raw):                  */
/*   F0 =  4 pi S[beta r^(l+1) g_l(q r)]     = beta(q) / q^l                    */
/*   F1 = -4 pi S[beta r^(l+3) g_(l+1)(q r)] = F0'(q) / q                       */
/*   F3 =  4 pi S[beta r^(l+5) g_(l+2)(q r)] = (F0'' - F0'/q) / q^2             */
/* with the reference's Simpson rule and per-projector trimming.               */
int oracle_hess_tables(int nr, const double* r, const double* rab, int uniform, int np, const int* l,
                       const double* beta, double dq, double q_max, double* out)
{
    const int nq = (int)ceil(q_max / dq) + 1 + 3;
    double* f = (double*)malloc(sizeof(double) * (nr > 0 ? nr : 1));
    if (!f) return HPSI_ERR_OOM;
    const double FOUR_PI = 4.0 * 3.14159265358979323846;
    for (int p = 0; p < np; ++p) {
        const double* b = beta + (size_t)p * nr;
        const int lp = l[p];
        int n = nr;
        while (n > 0 && b[n - 1] == 0.0) --n;
        for (int iq = 0; iq < nq; ++iq) {
            const double q = iq * dq;
            for (int t = 0; t < 3; ++t) {
                const int e = lp + 1 + 2 * t, ord = lp + t;
                for (int i = 0; i < n; ++i) f[i] = b[i] * pow(r[i], e) * oracle_gn(ord, q * r[i]);
                const double v = n ? FOUR_PI * ref_simpson(f, rab, n, uniform) : 0.0;
                out[((size_t)t * np + p) * nq + iq] = t == 1 ? -v : v;
            }
        }
    }
    free(f);
    return HPSI_OK;
}

/* ------------------------------------------------------------------------ */
/* d2H/dk_a dk_b |psi>: the operator the reference declares with its six     */
/* outputs xx yy zz xy xz yz (src/H_psi/hamiltonian.cppm:84-91) and leaves    */
/* empty (src/H_psi/hamiltonian_hessian.cpp:48-50).                           */
/*   out_ab += delta_ab psi + sum_p lambda (|d_ab p><p| + |d_a p><d_b p|      */
/*                                          + |d_b p><d_a p| + |p><d_ab p|) psi */
/* p and d_a p exactly as oracle_grad (the reference's gradient); d_ab p of   */
/* u = beta(q) Y_lm = F0(q) R(K) with the radial tables F0 = beta/q^l,         */
/* F1 = F0'/q, F3 = (F0'' - F0'/q)/q^2 (ftab[species] = [3][n_proj][nq], raw;  */
/* the reference's Lagrange stencil, times 1/sqrt(omega), range q <=          */
/* dq (nq - 3)):                                                              */
/*   d_ab u = F3 K_a K_b R + F1 (delta_ab R + K_a d_b R + K_b d_a R) + F0 d_ab R */
/* where R = q^l Y_lm is the solid harmonic of the reference's Y_lm          */
/* (oracle_ylm) and its gradient and Hessian are central differences of step  */
/* 1 bohr^-1 — exact for these polynomials of degree l <= 2 (l > 2 refused).   */
/* out: [6][nb][npw] interleaved complex.                                     */
/* ------------------------------------------------------------------------ */
int oracle_hess(const hpsi_system* sys, const hpsi_kpoint* kp, int nb, const double* psi, const double* const* ftab,
                int nq, double dq, double* out)
{
    if (!sys || !kp || nb < 0 || !ftab) return HPSI_ERR_BAD_ARG;
    const int ng = kp->npw;
    if (nb == 0 || ng == 0) return HPSI_OK;
    const int lmax = species_lmax(sys);
    if (lmax > 2) return HPSI_ERR_BAD_ARG;
    const int nlm = (lmax + 1) * (lmax + 1);
    const double norm = 1.0 / sqrt(sys->omega);
    const double qtop = dq * (nq - 3);
    static const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
    const size_t nel = (size_t)nb * ng;
    /* kinetic: delta_ab */
    for (int k = 0; k < 3; ++k)
        for (size_t i = 0; i < 2 * nel; ++i) out[(size_t)k * 2 * nel + i] += psi[i];
    /* solid harmonics on the 19-point stencil of every G: K, K +- e_a, K +- e_a +- e_b */
    enum { NS = 19 };
    int off[NS][3];
    {
        int n = 0;
        off[n][0] = off[n][1] = off[n][2] = 0; ++n;
        for (int a = 0; a < 3; ++a)
            for (int sg = -1; sg <= 1; sg += 2) { off[n][0] = off[n][1] = off[n][2] = 0; off[n][a] = sg; ++n; }
        for (int a = 0; a < 3; ++a)
            for (int b = a + 1; b < 3; ++b)
                for (int sa = -1; sa <= 1; sa += 2)
                    for (int sb = -1; sb <= 1; sb += 2) {
                        off[n][0] = off[n][1] = off[n][2] = 0;
                        off[n][a] = sa; off[n][b] = sb; ++n;
                    }
    }
    const size_t npts = (size_t)NS * ng;
    double* Kp = (double*)malloc(sizeof(double) * 3 * npts);
    double* sq = (double*)malloc(sizeof(double) * 3 * npts);
    double* yv = (double*)malloc(sizeof(double) * (size_t)nlm * npts);
    double* R = (double*)malloc(sizeof(double) * (size_t)nlm * npts);
    if (!Kp || !sq || !yv || !R) { free(Kp); free(sq); free(yv); free(R); return HPSI_ERR_OOM; }
    for (int ig = 0; ig < ng; ++ig)
        for (int t = 0; t < NS; ++t)
            for (int d = 0; d < 3; ++d) Kp[3 * ((size_t)t * ng + ig) + d] = kp->kvec[3 * ig + d] + off[t][d];
    oracle_spherical((int)npts, Kp, sq, sq + npts, sq + 2 * npts);
    oracle_ylm(lmax, (int)npts, sq + npts, sq + 2 * npts, yv, NULL, NULL);
    for (int l = 0; l <= lmax; ++l)
        for (int m = -l; m <= l; ++m) {
            const size_t lm = (size_t)(l * l + l + m) * npts;
            for (size_t i = 0; i < npts; ++i) {
                double ql = 1.0;
                for (int e = 0; e < l; ++e) ql *= sq[i];
                R[lm + i] = ql * yv[lm + i];
            }
        }
    /* stencil index of K + s_a e_a (s = -1 -> 0, +1 -> 1) and of K + s_a e_a + s_b e_b */
#define ST1(a, s) (1 + 2 * (a) + ((s) > 0))
    int st2[3][3][2][2];
    {
        int n = 7;
        for (int a = 0; a < 3; ++a)
            for (int b = a + 1; b < 3; ++b)
                for (int sa = 0; sa < 2; ++sa)
                    for (int sb = 0; sb < 2; ++sb) st2[a][b][sa][sb] = n++;
    }
    double* beta = (double*)malloc(sizeof(double) * ng);
    double* dbeta = (double*)malloc(sizeof(double) * ng);
    double* F = (double*)malloc(sizeof(double) * 3 * ng);
    double* S = (double*)malloc(sizeof(double) * 2 * ng);
    double* pv = (double*)malloc(sizeof(double) * 20 * ng); /* p, d_x p, d_y p, d_z p, d_ab p (6): complex */
    double* cf = (double*)malloc(sizeof(double) * 20 * nb);
    int rc = (beta && dbeta && F && S && pv && cf) ? HPSI_OK : HPSI_ERR_OOM;
    kprep P;
    kprep_init(&P, sys, kp, 1);
    for (int s = 0; s < sys->n_species && rc == HPSI_OK; ++s) {
        const hpsi_species* sp = &sys->species[s];
        if (!sp->dbeta_q || !ftab[s]) { rc = HPSI_ERR_STATE; break; }
        for (int a = 0; a < sys->n_atoms && rc == HPSI_OK; ++a) {
            if (sys->atom_species[a] != s) continue;
            rc = oracle_structure_factor(ng, kp->g_idx, kp->k_frac, sys->atom_tau + 3 * a, sys->n1, sys->n2, sys->n3, S);
            if (rc) break;
            for (int ip = 0; ip < sp->n_proj && rc == HPSI_OK; ++ip) {
                const double lam = sp->lambda[ip];
                if (fabs(lam) < 1e-15) continue;
                const int l = sp->proj_l[ip];
                const double* tab = sp->beta_q + (size_t)ip * sp->nq;
                const double* dtab = sp->dbeta_q + (size_t)ip * sp->nq;
                double db0;
                oracle_beta_interp(dtab, sp->nq, sp->dq, sp->q_max, norm, 0.0, &db0);
                for (int ig = 0; ig < ng && rc == HPSI_OK; ++ig) {
                    rc = oracle_beta_interp(tab, sp->nq, sp->dq, sp->q_max, norm, P.q[ig], &beta[ig]);
                    if (!rc) rc = oracle_beta_interp(dtab, sp->nq, sp->dq, sp->q_max, norm, P.q[ig], &dbeta[ig]);
                    for (int t = 0; t < 3 && !rc; ++t)
                        rc = oracle_beta_interp(ftab[s] + ((size_t)t * sp->n_proj + ip) * nq, nq, dq, qtop, norm,
                                                P.q[ig], &F[3 * ig + t]);
                }
                if (rc) break;
                for (int m = -l; m <= l; ++m) {
                    const size_t lmk = (size_t)(l * l + l + m) * ng, lmR = (size_t)(l * l + l + m) * npts;
                    const double* y = P.y + lmk;
                    const double* yt = P.yth + lmk;
                    const double* yp = P.yph + lmk;
                    for (int ig = 0; ig < ng; ++ig) {
                        /* p and d_a p: oracle_grad's formulas */
                        const double q = P.q[ig];
                        const double boq = (q > 1e-12) ? beta[ig] / q : db0;
                        const double gq = dbeta[ig] * y[ig], gt = boq * yt[ig], gp = boq * yp[ig];
                        const double sth = P.st[ig], cth = P.ct[ig], sph = P.sp[ig], cph = P.cp[ig];
                        double f[10];
                        f[0] = beta[ig] * y[ig];
                        f[1] = sth * cph * gq + cth * cph * gt - sph * gp;
                        f[2] = sth * sph * gq + cth * sph * gt + cph * gp;
                        f[3] = cth * gq - sth * gt;
                        /* d_ab u from F0, F1, F3 and the solid harmonic's differences */
                        const double* Rl = R + lmR;
                        const double R0 = Rl[ig];
                        double dR[3], HR[6];
                        for (int d = 0; d < 3; ++d)
                            dR[d] = (Rl[(size_t)ST1(d, 1) * ng + ig] - Rl[(size_t)ST1(d, -1) * ng + ig]) / 2.0;
                        for (int c = 0; c < 6; ++c) {
                            const int ca = pa[c], cb = pb[c];
                            if (ca == cb)
                                HR[c] = Rl[(size_t)ST1(ca, 1) * ng + ig] - 2.0 * R0 + Rl[(size_t)ST1(ca, -1) * ng + ig];
                            else
                                HR[c] = (Rl[(size_t)st2[ca][cb][1][1] * ng + ig] - Rl[(size_t)st2[ca][cb][1][0] * ng + ig] -
                                         Rl[(size_t)st2[ca][cb][0][1] * ng + ig] + Rl[(size_t)st2[ca][cb][0][0] * ng + ig]) / 4.0;
                        }
                        const double* K = kp->kvec + 3 * ig;
                        const double F0 = F[3 * ig], F1 = F[3 * ig + 1], F3 = F[3 * ig + 2];
                        for (int c = 0; c < 6; ++c) {
                            const int ca = pa[c], cb = pb[c];
                            f[4 + c] = F3 * K[ca] * K[cb] * R0 + F1 * ((ca == cb ? R0 : 0.0) + K[ca] * dR[cb] + K[cb] * dR[ca]) +
                                       F0 * HR[c];
                        }
                        const double Sr = S[2 * ig], Si = S[2 * ig + 1];
                        for (int c = 0; c < 10; ++c) {
                            pv[20 * ig + 2 * c] = f[c] * Sr;
                            pv[20 * ig + 2 * c + 1] = f[c] * Si;
                        }
                    }
                    /* coefficients <f_c|psi_b> */
                    for (int b = 0; b < nb; ++b) {
                        const double* ps = psi + 2 * (size_t)ng * b;
                        for (int c = 0; c < 10; ++c) {
                            double cr = 0.0, ci = 0.0;
                            for (int ig = 0; ig < ng; ++ig) {
                                const double pr = pv[20 * ig + 2 * c], pi_ = pv[20 * ig + 2 * c + 1];
                                cr += pr * ps[2 * ig] + pi_ * ps[2 * ig + 1];
                                ci += pr * ps[2 * ig + 1] - pi_ * ps[2 * ig];
                            }
                            cf[20 * b + 2 * c] = cr;
                            cf[20 * b + 2 * c + 1] = ci;
                        }
                    }
                    for (int k = 0; k < 6; ++k) {
                        const int ka = pa[k], kb = pb[k];
                        /* (ket row, coefficient row): d_ab p <p|, d_a p <d_b p|, d_b p <d_a p|, p <d_ab p| */
                        const int ket[4] = {4 + k, 1 + ka, 1 + kb, 0}, bra[4] = {0, 1 + kb, 1 + ka, 4 + k};
                        for (int b = 0; b < nb; ++b) {
                            double* o = out + ((size_t)k * nb + b) * 2 * ng;
                            for (int ig = 0; ig < ng; ++ig) {
                                double sr = 0.0, si = 0.0;
                                for (int t = 0; t < 4; ++t) {
                                    const double vr = pv[20 * ig + 2 * ket[t]], vi = pv[20 * ig + 2 * ket[t] + 1];
                                    const double cr = cf[20 * b + 2 * bra[t]], ci = cf[20 * b + 2 * bra[t] + 1];
                                    sr += cr * vr - ci * vi;
                                    si += cr * vi + ci * vr;
                                }
                                o[2 * ig] += lam * sr;
                                o[2 * ig + 1] += lam * si;
                            }
                        }
                    }
                }
            }
        }
    }
#undef ST1
    kprep_free(&P);
    free(Kp); free(sq); free(yv); free(R);
    free(beta); free(dbeta); free(F); free(S); free(pv); free(cf);
    return rc;
}

/* 1-D transform with the pocketfft convention (test hook for the FFT KATs). */
int oracle_fft1d(double* c, int n, int sign, double fct)
{
    mrfft_plan_s* p = mrfft_make(n);
    if (!p) return HPSI_ERR_BAD_ARG;
    mrfft_exec(p, c, sign, fct);
    mrfft_free(p);
    return HPSI_OK;
}
