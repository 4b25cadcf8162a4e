// projectors.cu — the nonlocal projector build, fused from the three pieces
// the reference evaluates per k-point / per call:
//
//   Y_lm and angular gradients   src/math/sph_harmonics.cppm:120-170 (Q_l^m
//                                recurrence), :188-243 (R = Q/sin theta),
//                                :268-335 (dQ/dtheta), assembled as in
//                                get() :702-735, get_ang_grad_phi :737-787,
//                                get_ang_grad_theta :830-875; spherical
//                                coordinates from src/io/GKK.cppm:431-449
//   beta(q), dbeta/dq            BetaqTables/DBetaqTables::interpolate,
//                                src/pseudo/ncpp_advance.cppm:644-674,838-868
//                                (4-point Lagrange, src/math/numerical.cppm:93-104)
//   S(g,k)                       src/H_psi/structure_factor.cppm:92-123,136-159
//
// and the per-G projector value p = beta*Y*S
// (src/H_psi/hamiltonian_callable.cpp:264-267) and its k-derivative
// dp_alpha = grad_alpha[beta*Y]*S (src/H_psi/hamiltonian_gradient.cpp:242-269).
// All of this is FP64; only the final projector matrix is rounded to the
// compute precision of the GEMMs that consume it.
#include "kernels.cuh"

#define PI_D 3.141592653589793238462643383279502884

__device__ __forceinline__ double seed_coeff_d(int m)
{
    double coeff = 0.5 / sqrt(PI_D);
    if (m % 2 != 0) coeff = -coeff;
    for (int k = 1; k <= m; ++k) coeff *= sqrt((double)(2 * k + 1) / (2 * k));
    return coeff;
}

__device__ __forceinline__ void rec_coeffs_d(int l, int m, double& r1, double& r2, double& dn)
{
    r1 = (2.0 * l - 1.0) * sqrt(((2.0 * l + 1.0) * (l - m)) / ((2.0 * l - 1.0) * (l + m)));
    r2 = (l + m - 1.0) * sqrt(((2.0 * l + 1.0) * (l - m) * (l - m - 1)) / ((2.0 * l - 3.0) * (l + m) * (l + m - 1)));
    dn = 1.0 / (l - m);
}

#define TRI(l, m) ((l) * ((l) + 1) / 2 + (m))
#define NTRI ((HPSI_LMAX + 1) * (HPSI_LMAX + 2) / 2)

__global__ void gtab_kernel(GTabArgs a)
{
    const int ig = blockIdx.x * blockDim.x + threadIdx.x;
    if (ig >= a.npw) return;
    const int L = a.lmax;
    const double kx = a.kvec[3 * ig], ky = a.kvec[3 * ig + 1], kz = a.kvec[3 * ig + 2];
    const double q = sqrt(kx * kx + ky * ky + kz * kz);
    const double th = (q > 0.0) ? acos(kz / q) : 0.0;
    const double ph = atan2(ky, kx);
    const double ct = cos(th), st = sin(th), cp = cos(ph), sp = sin(ph);
    const int npw = a.npw;
    a.q[ig] = q;
    a.trig[ig] = st;
    a.trig[npw + ig] = ct;
    a.trig[2 * npw + ig] = sp;
    a.trig[3 * npw + ig] = cp;

    double Q[NTRI], R[NTRI], dQ[NTRI], cm[HPSI_LMAX + 1], sm[HPSI_LMAX + 1];
    double c = 1.0, s = 0.0;
    for (int m = 0; m <= L; ++m) {
        cm[m] = c;
        sm[m] = s;
        double oc = c;
        c = c * cp - s * sp;
        s = s * cp + oc * sp;
    }
    // Q_l^m columns
    for (int m = 0; m <= L; ++m) {
        double cur = (m == 0) ? 0.5 / sqrt(PI_D) : seed_coeff_d(m) * pow(st, (double)m);
        double prev = 0.0;
        Q[TRI(m, m)] = cur;
        if (m < L) {
            prev = cur;
            cur = sqrt(2.0 * m + 3.0) * ct * cur;
            Q[TRI(m + 1, m)] = cur;
            for (int l = m + 2; l <= L; ++l) {
                double r1, r2, dn;
                rec_coeffs_d(l, m, r1, r2, dn);
                double nx = (ct * r1 * cur - r2 * prev) * dn;
                prev = cur;
                cur = nx;
                Q[TRI(l, m)] = cur;
            }
        }
    }
    const bool grads = (a.yth != nullptr);
    if (grads) {
        // R_l^m = Q_l^m / sin(theta), m >= 1
        for (int l = 0; l <= L; ++l) R[TRI(l, 0)] = 0.0;
        for (int m = 1; m <= L; ++m) {
            double cur = (m == 1) ? seed_coeff_d(1) : seed_coeff_d(m) * pow(st, (double)(m - 1));
            double prev = 0.0;
            R[TRI(m, m)] = cur;
            if (m < L) {
                prev = cur;
                cur = sqrt(2.0 * m + 3.0) * ct * cur;
                R[TRI(m + 1, m)] = cur;
                for (int l = m + 2; l <= L; ++l) {
                    double r1, r2, dn;
                    rec_coeffs_d(l, m, r1, r2, dn);
                    double nx = (ct * r1 * cur - r2 * prev) * dn;
                    prev = cur;
                    cur = nx;
                    R[TRI(l, m)] = cur;
                }
            }
        }
        // dQ_l^m / dtheta
        for (int m = 0; m <= L; ++m) {
            double cur;
            if (m == 0) cur = 0.0;
            else if (m == 1) cur = seed_coeff_d(1) * ct;
            else cur = ((double)m * seed_coeff_d(m)) * pow(st, (double)(m - 1)) * ct;
            double prev = 0.0;
            dQ[TRI(m, m)] = cur;
            if (m < L) {
                prev = cur;
                cur = sqrt(2.0 * m + 3.0) * (-st * Q[TRI(m, m)] + ct * cur);
                dQ[TRI(m + 1, m)] = cur;
                for (int l = m + 2; l <= L; ++l) {
                    double r1, r2, dn;
                    rec_coeffs_d(l, m, r1, r2, dn);
                    double nx = (ct * r1 * cur - st * r1 * Q[TRI(l - 1, m)] - r2 * prev) * dn;
                    prev = cur;
                    cur = nx;
                    dQ[TRI(l, m)] = cur;
                }
            }
        }
    }
    const double sf = sqrt(2.0);
    for (int l = 0; l <= L; ++l) {
        for (int m = -l; m <= l; ++m) {
            const int ma = m < 0 ? -m : m;
            const size_t o = (size_t)(l * l + l + m) * npw + ig;
            double qv = Q[TRI(l, ma)];
            a.ylm[o] = (m == 0) ? qv : (m > 0 ? (sf * qv) * cm[ma] : (sf * qv) * sm[ma]);
            if (grads) {
                double rv = R[TRI(l, ma)];
                double dv = dQ[TRI(l, ma)];
                a.yph[o] = (m == 0) ? 0.0 : (m > 0 ? (-(double)m * sf) * rv * sm[ma] : ((double)ma * sf) * rv * cm[ma]);
                a.yth[o] = (m == 0) ? dv : (m > 0 ? sf * dv * cm[ma] : sf * dv * sm[ma]);
            }
        }
    }
}

cudaError_t launch_gtab(const GTabArgs& a, cudaStream_t st)
{
    if (a.npw == 0) return cudaSuccess;
    gtab_kernel<<<ceil_div(a.npw, 128), 128, 0, st>>>(a);
    return cudaGetLastError();
}

__device__ __forceinline__ double lagrange_cubic_d(double f0, double f1, double f2, double f3, double px)
{
    double ux = 1.0 - px, vx = 2.0 - px, wx = 3.0 - px;
    return f0 * ux * vx * wx / 6.0 + f1 * px * vx * wx / 2.0 - f2 * px * ux * wx / 2.0 + f3 * px * ux * vx / 6.0;
}

__device__ __forceinline__ double interp_d(const double* t, int nq, double dq, double q, double norm)
{
    if (q == 0.0) return t[0] * norm;
    double s = q / dq;
    int i0 = (int)floor(s) - 1;
    double px = s - (double)i0;
    if (i0 < 0) { i0 = 0; px = s; }
    if (i0 > nq - 4) i0 = nq - 4;  // unreachable for inputs that passed the host range check
    return lagrange_cubic_d(t[i0], t[i0 + 1], t[i0 + 2], t[i0 + 3], px) * norm;
}

__global__ void beta_kernel(BetaArgs a)
{
    const int ig = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (r >= a.nrad) return;
    const int nq = a.rad_nq[r];
    const double dq = a.rad_dq[r];
    if (ig == 0 && a.dbeta0) a.dbeta0[r] = a.dtables[(size_t)r * a.nq_max] * a.norm;
    if (ig >= a.npw) return;
    const double q = a.q[ig];
    a.beta[(size_t)r * a.npw + ig] = interp_d(a.tables + (size_t)r * a.nq_max, nq, dq, q, a.norm);
    if (a.dbeta) a.dbeta[(size_t)r * a.npw + ig] = interp_d(a.dtables + (size_t)r * a.nq_max, nq, dq, q, a.norm);
}

cudaError_t launch_beta(const BetaArgs& a, cudaStream_t st)
{
    if (a.nrad == 0 || a.npw == 0) return cudaSuccess;
    dim3 g(ceil_div(a.npw, 256), a.nrad);
    beta_kernel<<<g, 256, 0, st>>>(a);
    return cudaGetLastError();
}

__global__ void sf_kernel(SfArgs a)
{
    const int ig = blockIdx.x * blockDim.x + threadIdx.x;
    const int at = blockIdx.y;
    if (ig >= a.npw) return;
    const double tx = a.tau[3 * at], ty = a.tau[3 * at + 1], tz = a.tau[3 * at + 2];
    const double kd = -2.0 * PI_D * (a.kf0 * tx + a.kf1 * ty + a.kf2 * tz);
    double sr, si;
    sincos(kd, &si, &sr);
    double2 s = make_double2(sr, si);
    const double tau3[3] = {tx, ty, tz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double ang = -2.0 * PI_D * (double)a.g[3 * ig + d] * tau3[d];
        double c, sn;
        sincos(ang, &sn, &c);
        s = cmul(s, make_double2(c, sn));
    }
    a.sf[(size_t)at * a.npw + ig] = s;
}

cudaError_t launch_sf(const SfArgs& a, cudaStream_t st)
{
    if (a.natom == 0 || a.npw == 0) return cudaSuccess;
    dim3 g(ceil_div(a.npw, 256), a.natom);
    sf_kernel<<<g, 256, 0, st>>>(a);
    return cudaGetLastError();
}

template <typename C>
__global__ void assemble_kernel(int P, int npw, const ProjRow* __restrict__ rows, const double* __restrict__ beta,
                                const double* __restrict__ dbeta, const double* __restrict__ dbeta0,
                                const double* __restrict__ q, const double* __restrict__ trig,
                                const double* __restrict__ ylm, const double* __restrict__ yth,
                                const double* __restrict__ yph, const double2* __restrict__ sf, bool grad,
                                C* __restrict__ out, size_t ld)
{
    const int ig = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = blockIdx.y;
    if (ig >= npw) return;
    const ProjRow r = rows[row];
    const size_t lm = (size_t)(r.l * r.l + r.l + r.m) * npw + ig;
    const double b = beta[(size_t)r.rad * npw + ig];
    const double y = ylm[lm];
    const double2 S = sf[(size_t)r.atom * npw + ig];
    const double by = b * y;
    out[(size_t)row * ld + ig] = from_c128<C>(make_double2(by * S.x, by * S.y));
    if (grad) {
        const double qq = q[ig];
        const double boq = (qq > 1e-12) ? b / qq : dbeta0[r.rad];
        const double gq = dbeta[(size_t)r.rad * npw + ig] * y;
        const double gt = boq * yth[lm];
        const double gp = boq * yph[lm];
        const double s_th = trig[ig], c_th = trig[npw + ig], s_ph = trig[2 * npw + ig], c_ph = trig[3 * npw + ig];
        const double f[3] = {s_th * c_ph * gq + c_th * c_ph * gt - s_ph * gp,
                             s_th * s_ph * gq + c_th * s_ph * gt + c_ph * gp, c_th * gq - s_th * gt};
#pragma unroll
        for (int d = 0; d < 3; ++d)
            out[((size_t)(d + 1) * P + row) * ld + ig] = from_c128<C>(make_double2(f[d] * S.x, f[d] * S.y));
    }
}

template <typename C>
cudaError_t launch_assemble(int P, int npw, const ProjRow* rows, const double* beta, const double* dbeta,
                            const double* dbeta0, const double* q, const double* trig, const double* ylm,
                            const double* yth, const double* yph, const double2* sf, bool grad, C* out, size_t ld,
                            cudaStream_t st)
{
    if (P == 0 || npw == 0) return cudaSuccess;
    dim3 g(ceil_div(npw, 256), P);
    assemble_kernel<C><<<g, 256, 0, st>>>(P, npw, rows, beta, dbeta, dbeta0, q, trig, ylm, yth, yph, sf, grad, out, ld);
    return cudaGetLastError();
}

template cudaError_t launch_assemble<double2>(int, int, const ProjRow*, const double*, const double*, const double*,
                                              const double*, const double*, const double*, const double*,
                                              const double*, const double2*, bool, double2*, size_t, cudaStream_t);
template cudaError_t launch_assemble<float2>(int, int, const ProjRow*, const double*, const double*, const double*,
                                             const double*, const double*, const double*, const double*,
                                             const double*, const double2*, bool, float2*, size_t, cudaStream_t);
