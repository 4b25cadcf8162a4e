// hpsi_api.cu — the C ABI (include/hpsi_gb300.h): context, k-point binding,
// device memory and the launch sequence of H|psi>, dH/dk|psi> and the
// band-pair velocity matrix.
//
// Device-resident state (kept in HBM for the life of the context):
//   V_loc(r) in FP64 and FP32 ([i][j][k] layout), the raw beta / dbeta tables,
//   atom positions, FFT twiddles; per bound k-point: kinetic, K, q, trig,
//   Y_lm (+ angular gradients), beta(q) per radial function, S(G) per atom,
//   the plane decomposition of the G-sphere, and the projector matrices
//   Pr[P][npw] (+ dPr_alpha for the gradient) in the precisions requested.
// Per call, a grow-only workspace holds host staging, the FFT intermediate and
// the projection partial sums.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "ctx.cuh"

thread_local std::string g_last_error;

extern "C" int hpsi_abi_version(void) { return HPSI_ABI_VERSION; }

extern "C" const char* hpsi_last_error(const hpsi_ctx* ctx)
{
    if (!ctx) return g_last_error.c_str();
    return ctx->err.c_str();
}

extern "C" int hpsi_ctx_destroy(hpsi_ctx* c)
{
    if (!c) return HPSI_ERR_BAD_ARG;
    cudaSetDevice(c->dev);
    for (auto& kv : c->slots) slot_free(kv.second);
    dfree(c->d_tables); dfree(c->d_rad_nq); dfree(c->d_rad_dq); dfree(c->d_tau); dfree(c->d_v64); dfree(c->d_v32); dfree(c->d_dv32);
    dfree(c->d_tw64); dfree(c->d_tw32); dfree(c->d_err); dfree(c->d_hess);
    if (c->ws) cudaFree(c->ws);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->ev_copy_after) cudaEventDestroy(c->ev_copy_after);
    if (c->ev_copy_done) cudaEventDestroy(c->ev_copy_done);
    for (cudaEvent_t e : {c->ev_half_in[0], c->ev_half_in[1], c->ev_half_exp, c->ev_half_out, c->ev_psi_in[0],
                          c->ev_psi_in[1]})
        if (e) cudaEventDestroy(e);
    for (auto& r : c->prof.recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : c->prof.pool) cudaEventDestroy(e);
    delete c;
    return HPSI_OK;
}

extern "C" int hpsi_profile(hpsi_ctx* c, int enable)
{
    if (!c) return HPSI_ERR_BAD_ARG;
    CUDA_TRY(c, cudaSetDevice(c->dev));
    for (auto& r : c->prof.recs) { c->prof.pool.push_back(r.a); c->prof.pool.push_back(r.b); }
    c->prof.recs.clear();
    c->prof.on = enable != 0;
    return HPSI_OK;
}

extern "C" int hpsi_profile_read(hpsi_ctx* c, double* ms, long long* launches)
{
    if (!c || !ms || !launches) return HPSI_ERR_BAD_ARG;
    CUDA_TRY(c, cudaSetDevice(c->dev));
    for (int i = 0; i < HPSI_PROFILE_PHASES; ++i) { ms[i] = 0.0; launches[i] = 0; }
    for (auto& r : c->prof.recs) {
        CUDA_TRY(c, cudaEventSynchronize(r.b));
        float t = 0.f;
        CUDA_TRY(c, cudaEventElapsedTime(&t, r.a, r.b));
        ms[r.phase] += t;
        launches[r.phase] += r.kernels;
    }
    return HPSI_OK;
}

static int ctx_init(hpsi_ctx* c, const hpsi_system* s)
{
    if (s->n1 < 1 || s->n2 < 1 || s->n3 < 1) return fail(c, HPSI_ERR_BAD_ARG, "FFT grid must be positive");
    if (!(s->omega > 0)) return fail(c, HPSI_ERR_BAD_ARG, "omega must be positive");
    if (!s->v_loc) return fail(c, HPSI_ERR_BAD_ARG, "v_loc is NULL");
    if (s->n_atoms < 0 || s->n_species < 0) return fail(c, HPSI_ERR_BAD_ARG, "negative counts");
    if (s->n_atoms > 0 && (!s->atom_species || !s->atom_tau)) return fail(c, HPSI_ERR_BAD_ARG, "atoms NULL");
    if (s->n_species > 0 && !s->species) return fail(c, HPSI_ERR_BAD_ARG, "species NULL");
    c->n1 = s->n1; c->n2 = s->n2; c->n3 = s->n3;
    const int ns[3] = {s->n1, s->n2, s->n3};
    for (int d = 0; d < 3; ++d)
        if (!fft_factor(ns[d], &c->L[d]))
            return fail(c, HPSI_ERR_BAD_ARG, "FFT length %d not supported (primes <= 13, n <= %d)", ns[d], HPSI_FFT_MAXN);
    c->omega = s->omega;
    c->natom = s->n_atoms;
    for (int a = 0; a < s->n_atoms; ++a) {
        int sp = s->atom_species[a];
        if (sp < 0 || sp >= s->n_species) return fail(c, HPSI_ERR_BAD_ARG, "atom %d: species index %d out of range", a, sp);
        c->atom_species.push_back(sp);
        for (int d = 0; d < 3; ++d) c->tau.push_back(s->atom_tau[3 * a + d]);
    }
    for (int sp = 0; sp < s->n_species; ++sp) {
        const hpsi_species& S = s->species[sp];
        c->rad_off.push_back(c->nrad);
        if (S.n_proj < 0) return fail(c, HPSI_ERR_BAD_ARG, "species %d: n_proj < 0", sp);
        if (S.n_proj > 0 && (!S.proj_l || !S.lambda || !S.beta_q))
            return fail(c, HPSI_ERR_BAD_ARG, "species %d: NULL table", sp);
        if (S.n_proj > 0 && (S.nq < 4 || !(S.dq > 0) || S.q_max < 0))
            return fail(c, HPSI_ERR_BAD_ARG, "species %d: table needs nq >= 4, dq > 0, q_max >= 0", sp);
        if (!S.dbeta_q) c->have_dbeta = false;
        for (int i = 0; i < S.n_proj; ++i) {
            if (S.proj_l[i] < 0 || S.proj_l[i] > HPSI_LMAX)
                return fail(c, HPSI_ERR_BAD_ARG, "species %d projector %d: l=%d outside [0,%d]", sp, i, S.proj_l[i], HPSI_LMAX);
            c->rad_l.push_back(S.proj_l[i]);
            c->rad_lam.push_back(S.lambda[i]);
            c->rad_nq.push_back(S.nq);
            c->rad_dq.push_back(S.dq);
            c->rad_qmax.push_back(S.q_max);
            c->nq_max = std::max(c->nq_max, S.nq);
            c->lmax = std::max(c->lmax, S.proj_l[i]);
            c->nrad++;
        }
    }
    // plane FFT kernels keep two n2*n3 planes in shared memory
    LocalArgs la{};
    la.n1 = c->n1; la.n2 = c->n2; la.n3 = c->n3;
    if (local_smem_bytes(la, true) > 227 * 1024)
        return fail(c, HPSI_ERR_BAD_ARG, "FFT grid %dx%dx%d: two complex128 n2*n3 planes exceed shared memory", c->n1, c->n2, c->n3);

    CUDA_TRY(c, cudaGetDevice(&c->dev));
    CUDA_TRY(c, cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    CUDA_TRY(c, cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking));
    CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_copy_after, cudaEventDisableTiming));
    CUDA_TRY(c, cudaEventCreateWithFlags(&c->ev_copy_done, cudaEventDisableTiming));
    for (cudaEvent_t* e : {&c->ev_half_in[0], &c->ev_half_in[1], &c->ev_half_exp, &c->ev_half_out, &c->ev_psi_in[0],
                           &c->ev_psi_in[1]})
        CUDA_TRY(c, cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    CUDA_TRY(c, dalloc(&c->d_err, (size_t)1));
    CUDA_TRY(c, cudaMemset(c->d_err, 0, sizeof(int)));
    const size_t N = (size_t)c->n1 * c->n2 * c->n3;
    CUDA_TRY(c, dalloc(&c->d_v64, N));
    CUDA_TRY(c, dalloc(&c->d_v32, N));
    CUDA_TRY(c, dalloc(&c->d_dv32, N));
    CUDA_TRY(c, cudaMemcpy(c->d_v64, s->v_loc, N * sizeof(double), cudaMemcpyHostToDevice));
    {
        std::vector<float> v32(N), dv32(N);
        for (size_t i = 0; i < N; ++i) {
            v32[i] = (float)s->v_loc[i];
            dv32[i] = (float)(s->v_loc[i] - (double)v32[i]);
        }
        CUDA_TRY(c, cudaMemcpy(c->d_v32, v32.data(), N * sizeof(float), cudaMemcpyHostToDevice));
        CUDA_TRY(c, cudaMemcpy(c->d_dv32, dv32.data(), N * sizeof(float), cudaMemcpyHostToDevice));
    }
    const int ntw = c->n1 + c->n2 + c->n3;
    std::vector<double2> tw64(ntw);
    std::vector<float2> tw32(ntw);
    int o = 0;
    for (int d = 0; d < 3; ++d)
        for (int j = 0; j < ns[d]; ++j, ++o) {
            double a = 6.283185307179586476925286766559 * (double)j / (double)ns[d];
            tw64[o] = make_double2(std::cos(a), std::sin(a));
            tw32[o] = make_float2((float)tw64[o].x, (float)tw64[o].y);
        }
    CUDA_TRY(c, dalloc(&c->d_tw64, ntw));
    CUDA_TRY(c, dalloc(&c->d_tw32, ntw));
    CUDA_TRY(c, cudaMemcpy(c->d_tw64, tw64.data(), ntw * sizeof(double2), cudaMemcpyHostToDevice));
    CUDA_TRY(c, cudaMemcpy(c->d_tw32, tw32.data(), ntw * sizeof(float2), cudaMemcpyHostToDevice));
    if (c->natom > 0) {
        CUDA_TRY(c, dalloc(&c->d_tau, (size_t)3 * c->natom));
        CUDA_TRY(c, cudaMemcpy(c->d_tau, c->tau.data(), 3 * c->natom * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (c->nrad > 0) {
        std::vector<double> tab((size_t)2 * c->nrad * c->nq_max, 0.0);
        int r = 0;
        for (int sp = 0; sp < s->n_species; ++sp) {
            const hpsi_species& S = s->species[sp];
            for (int i = 0; i < S.n_proj; ++i, ++r) {
                std::memcpy(&tab[(size_t)r * c->nq_max], S.beta_q + (size_t)i * S.nq, S.nq * sizeof(double));
                if (S.dbeta_q)
                    std::memcpy(&tab[((size_t)c->nrad + r) * c->nq_max], S.dbeta_q + (size_t)i * S.nq,
                                S.nq * sizeof(double));
            }
        }
        CUDA_TRY(c, dalloc(&c->d_tables, tab.size()));
        CUDA_TRY(c, cudaMemcpy(c->d_tables, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice));
        CUDA_TRY(c, dalloc(&c->d_rad_nq, (size_t)c->nrad));
        CUDA_TRY(c, dalloc(&c->d_rad_dq, (size_t)c->nrad));
        CUDA_TRY(c, cudaMemcpy(c->d_rad_nq, c->rad_nq.data(), c->nrad * sizeof(int), cudaMemcpyHostToDevice));
        CUDA_TRY(c, cudaMemcpy(c->d_rad_dq, c->rad_dq.data(), c->nrad * sizeof(double), cudaMemcpyHostToDevice));
    }
    return HPSI_OK;
}

extern "C" int hpsi_ctx_create(const hpsi_system* sys, hpsi_ctx** out)
{
    if (!out) return HPSI_ERR_BAD_ARG;
    *out = nullptr;
    if (!sys) return HPSI_ERR_BAD_ARG;
    hpsi_ctx* c = new hpsi_ctx();
    int rc = ctx_init(c, sys);
    if (rc != HPSI_OK) {
        g_last_error = c->err;  // readable through hpsi_last_error(NULL)
        hpsi_ctx_destroy(c);
        return rc;
    }
    *out = c;
    return HPSI_OK;
}

static KSlot* get_slot(hpsi_ctx* c, int kid)
{
    auto it = c->slots.find(kid);
    if (it == c->slots.end() || !it->second.valid) return nullptr;
    return &it->second;
}

extern "C" int hpsi_dim(const hpsi_ctx* ctx, int kid)
{
    if (!ctx) return HPSI_ERR_BAD_ARG;
    auto it = ctx->slots.find(kid);
    if (it == ctx->slots.end() || !it->second.valid) return HPSI_ERR_STATE;
    return it->second.npw;
}

extern "C" int hpsi_set_kpoint(hpsi_ctx* c, int kid, const hpsi_kpoint* kp)
{
    if (!c) return HPSI_ERR_BAD_ARG;
    if (!kp) return fail(c, HPSI_ERR_BAD_ARG, "kpoint is NULL");
    if (kid < 0 || kid >= 4096) return fail(c, HPSI_ERR_BAD_ARG, "kid %d outside [0, 4096)", kid);
    const int npw = kp->npw;
    if (npw < 0) return fail(c, HPSI_ERR_BAD_ARG, "npw < 0");
    if (npw > 0 && (!kp->g_idx || !kp->kvec || !kp->kinetic)) return fail(c, HPSI_ERR_BAD_ARG, "kpoint arrays NULL");
    CUDA_TRY(c, cudaSetDevice(c->dev));
    const int n[3] = {c->n1, c->n2, c->n3};

    // --- host-side validation: the reference's domain_error / assert cases
    for (int ig = 0; ig < npw; ++ig) {
        for (int d = 0; d < 3; ++d) {
            int gd = kp->g_idx[3 * ig + d];
            int idx = gd + n[d] / 2 + 4;  // structure-factor cache index, src/H_psi/structure_factor.cppm:68-72
            if (idx < 0 || idx >= n[d] + 8)
                return fail(c, HPSI_ERR_RANGE, "G %d: g[%d]=%d outside [-n/2-4, n/2+3] for n=%d", ig, d, gd, n[d]);
        }
        const double kx = kp->kvec[3 * ig], ky = kp->kvec[3 * ig + 1], kz = kp->kvec[3 * ig + 2];
        const double q = std::sqrt(kx * kx + ky * ky + kz * kz);
        for (int r = 0; r < c->nrad; ++r) {
            if (std::fabs(c->rad_lam[r]) < 1e-15) continue;
            if (q > c->rad_qmax[r])
                return fail(c, HPSI_ERR_RANGE, "G %d: q=%.17g exceeds q_max=%.17g", ig, q, c->rad_qmax[r]);
            if (q > 0 && (int)std::floor(q / c->rad_dq[r]) + 2 >= c->rad_nq[r])
                return fail(c, HPSI_ERR_RANGE, "G %d: q=%.17g beyond the table (nq=%d)", ig, q, c->rad_nq[r]);
        }
    }

    // --- plane decomposition of the sphere on the FFT grid
    std::vector<int> gi(npw), jk(npw);
    std::vector<int> plane_of_x(c->n1, -1);
    std::map<long, int> last;
    for (int ig = 0; ig < npw; ++ig) {
        int i = ((kp->g_idx[3 * ig] % n[0]) + n[0]) % n[0];
        int j = ((kp->g_idx[3 * ig + 1] % n[1]) + n[1]) % n[1];
        int k = ((kp->g_idx[3 * ig + 2] % n[2]) + n[2]) % n[2];
        gi[ig] = i;
        jk[ig] = j * n[2] + k;
        last[(long)i * n[1] * n[2] + jk[ig]] = ig;  // the reference's scatter: the last write wins
        plane_of_x[i] = 1;
    }
    std::vector<int> plane_x;
    for (int i = 0; i < c->n1; ++i)
        if (plane_of_x[i] > 0) { plane_of_x[i] = (int)plane_x.size(); plane_x.push_back(i); }
    const int nxs = (int)plane_x.size();
    std::vector<int> plane_off(nxs + 1, 0);
    for (int ig = 0; ig < npw; ++ig) plane_off[plane_of_x[gi[ig]] + 1]++;
    for (int p = 0; p < nxs; ++p) plane_off[p + 1] += plane_off[p];
    std::vector<int> fill(plane_off.begin(), plane_off.end() - 1);
    std::vector<int> ent_ig(npw), ent_jk(npw);
    bool aliased = false;
    for (int ig = 0; ig < npw; ++ig) {
        int p = plane_of_x[gi[ig]];
        int e = fill[p]++;
        bool scatter = last[(long)gi[ig] * n[1] * n[2] + jk[ig]] == ig;
        ent_ig[e] = scatter ? ig : (int)((unsigned)ig | 0x80000000u);
        ent_jk[e] = jk[ig];
        aliased = aliased || !scatter;
    }
    // rows in use per plane: |G_y| <= plane_jr[p], i.e. j <= jr or j >= n2 - jr
    std::vector<int> plane_jr(nxs, 0);
    for (int p = 0; p < nxs; ++p)
        for (int e = plane_off[p]; e < plane_off[p + 1]; ++e) {
            const int j = ent_jk[e] / n[2];
            plane_jr[p] = std::max(plane_jr[p], std::min(j, n[1] - j));
        }

    // --- projector rows
    std::vector<ProjRow> rows;
    std::vector<double> lam;
    for (int a = 0; a < c->natom; ++a) {
        int sp = c->atom_species[a];
        int r0 = c->rad_off[sp];
        int r1 = (sp + 1 < (int)c->rad_off.size()) ? c->rad_off[sp + 1] : c->nrad;
        for (int r = r0; r < r1; ++r) {
            if (std::fabs(c->rad_lam[r]) < 1e-15) continue;  // src/H_psi/hamiltonian_callable.cpp:226-227
            int l = c->rad_l[r];
            for (int m = -l; m <= l; ++m) {
                rows.push_back(ProjRow{a, r, l, m});
                lam.push_back(c->rad_lam[r]);
            }
        }
    }

    KSlot& s = c->slots[kid];
    slot_free(s);
    s.gen = ++c->gen_counter;
    s.npw = npw;
    for (int d = 0; d < 3; ++d) s.kf[d] = kp->k_frac[d];
    s.nxs = nxs;
    s.aliased = aliased;
    s.P = (int)rows.size();
    if (npw > 0) {
        const int nlm = (c->lmax + 1) * (c->lmax + 1);
        const bool grads = c->have_dbeta;
        CUDA_TRY(c, dalloc(&s.d_kin, (size_t)npw));
        CUDA_TRY(c, dalloc(&s.d_kvec, (size_t)3 * npw));
        CUDA_TRY(c, dalloc(&s.d_g, (size_t)3 * npw));
        CUDA_TRY(c, dalloc(&s.d_q, (size_t)npw));
        CUDA_TRY(c, dalloc(&s.d_trig, (size_t)4 * npw));
        CUDA_TRY(c, dalloc(&s.d_ylm, (size_t)(grads ? 3 : 1) * nlm * npw));
        CUDA_TRY(c, dalloc(&s.d_plane, (size_t)3 * nxs + 1 + 2 * (size_t)npw));
        CUDA_TRY(c, cudaMemcpy(s.d_kin, kp->kinetic, npw * sizeof(double), cudaMemcpyHostToDevice));
        CUDA_TRY(c, cudaMemcpy(s.d_kvec, kp->kvec, 3 * npw * sizeof(double), cudaMemcpyHostToDevice));
        CUDA_TRY(c, cudaMemcpy(s.d_g, kp->g_idx, 3 * npw * sizeof(int), cudaMemcpyHostToDevice));
        std::vector<int> pl;
        pl.insert(pl.end(), plane_x.begin(), plane_x.end());
        pl.insert(pl.end(), plane_off.begin(), plane_off.end());
        pl.insert(pl.end(), ent_ig.begin(), ent_ig.end());
        pl.insert(pl.end(), ent_jk.begin(), ent_jk.end());
        pl.insert(pl.end(), plane_jr.begin(), plane_jr.end());
        CUDA_TRY(c, cudaMemcpy(s.d_plane, pl.data(), pl.size() * sizeof(int), cudaMemcpyHostToDevice));

        GTabArgs ga{npw, c->lmax, s.d_kvec, s.d_q, s.d_trig, s.d_ylm, grads ? s.d_ylm + (size_t)nlm * npw : nullptr,
                    grads ? s.d_ylm + (size_t)2 * nlm * npw : nullptr};
        CUDA_TRY(c, launch_gtab(ga, 0));
        if (c->nrad > 0) {
            CUDA_TRY(c, dalloc(&s.d_beta, (size_t)(grads ? 2 : 1) * c->nrad * npw));
            CUDA_TRY(c, dalloc(&s.d_dbeta0, (size_t)c->nrad));
            BetaArgs ba{npw, c->nrad, s.d_q, c->d_tables, grads ? c->d_tables + (size_t)c->nrad * c->nq_max : nullptr,
                        c->d_rad_nq, c->d_rad_dq, c->nq_max, 1.0 / std::sqrt(c->omega), s.d_beta,
                        grads ? s.d_beta + (size_t)c->nrad * npw : nullptr, grads ? s.d_dbeta0 : nullptr};
            CUDA_TRY(c, launch_beta(ba, 0));
        }
        if (c->natom > 0) {
            CUDA_TRY(c, dalloc(&s.d_sf, (size_t)c->natom * npw));
            SfArgs sa{npw, c->natom, s.d_g, c->d_tau, s.kf[0], s.kf[1], s.kf[2], s.d_sf};
            CUDA_TRY(c, launch_sf(sa, 0));
        }
        if (s.P > 0) {
            CUDA_TRY(c, dalloc(&s.d_rows, (size_t)s.P));
            CUDA_TRY(c, dalloc(&s.d_lam, (size_t)s.P));
            CUDA_TRY(c, cudaMemcpy(s.d_rows, rows.data(), s.P * sizeof(ProjRow), cudaMemcpyHostToDevice));
            s.rows.assign(rows.begin(), rows.begin() + s.P);
            CUDA_TRY(c, cudaMemcpy(s.d_lam, lam.data(), s.P * sizeof(double), cudaMemcpyHostToDevice));
        }
        CUDA_TRY(c, cudaDeviceSynchronize());
    }
    s.valid = true;
    return HPSI_OK;
}

// The slot's projector matrix and projector second derivatives in complex type C
template <typename C> static C*& slot_pr(KSlot& s);
template <> double2*& slot_pr<double2>(KSlot& s) { return s.pr64; }
template <> float2*& slot_pr<float2>(KSlot& s) { return s.pr32; }
template <typename C> static C*& slot_hess(KSlot& s);
template <> double2*& slot_hess<double2>(KSlot& s) { return s.hess64; }
template <> float2*& slot_hess<float2>(KSlot& s) { return s.hess32; }

// Build (once) the projector matrices of slot s in complex type C.
template <typename C>
static int ensure_proj(hpsi_ctx* c, KSlot& s, bool grad, cudaStream_t st)
{
    C*& pr = slot_pr<C>(s);
    bool& has_grad = std::is_same<C, double2>::value ? s.pr64_grad : s.pr32_grad;
    if (s.P == 0 || s.npw == 0) return HPSI_OK;
    if (pr && (has_grad || !grad)) return HPSI_OK;
    if (grad && !c->have_dbeta) return fail(c, HPSI_ERR_STATE, "gradient needs dbeta tables for every species");
    dfree(pr);
    const bool g = grad || c->have_dbeta;  // build the derivative rows together when tables allow
    CUDA_TRY(c, dalloc(&pr, (size_t)(g ? 4 : 1) * s.P * s.npw));
    const int nlm = (c->lmax + 1) * (c->lmax + 1);
    const double* yth = c->have_dbeta ? s.d_ylm + (size_t)nlm * s.npw : nullptr;
    const double* yph = c->have_dbeta ? s.d_ylm + (size_t)2 * nlm * s.npw : nullptr;
    const double* dbeta = c->have_dbeta ? s.d_beta + (size_t)c->nrad * s.npw : nullptr;
    int h = c->prof.open(PH_BUILD, st);
    CUDA_TRY(c, launch_assemble<C>(s.P, s.npw, s.d_rows, s.d_beta, dbeta, s.d_dbeta0, s.d_q, s.d_trig, s.d_ylm, yth,
                                   yph, s.d_sf, g, pr, (size_t)s.npw, st));
    c->prof.close(h, st);
    has_grad = g;
    return HPSI_OK;
}

static int split_for(int M, int N, int K) { return proj_gemm_splits(M, N, K); }

// hpsi_out[nb][npw] += nonlocal(psi) using projector matrix pr (complex C)
template <typename C, typename Acc>
static int nonlocal_apply(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* hpsi, const C* pr,
                          unsigned char* ws, cudaStream_t st, double* e_nl = nullptr)
{
    if (s.P == 0 || nb == 0) return HPSI_OK;
    const int ns = split_for(s.P, nb, s.npw);
    Carver cv;
    size_t o_part = cv.take<Acc>((size_t)ns * s.P * nb);
    size_t o_w = cv.take<C>((size_t)s.P * nb);
    Acc* part = reinterpret_cast<Acc*>(ws + o_part);
    C* W = reinterpret_cast<C*>(ws + o_w);
    int h = c->prof.open(PH_PROJ, st);
    CUDA_TRY(c, (launch_proj_gemm<C, double2, Acc>(s.P, nb, s.npw, pr, (size_t)s.npw, psi, (size_t)s.npw, part, ns, st)));
    c->prof.close(h, st);
    if (e_nl) CUDA_TRY(c, launch_nl_energy<Acc>(s.P, nb, ns, part, s.d_lam, e_nl, st));
    h = c->prof.open(PH_REDUCE, st);
    CUDA_TRY(c, (launch_reduce_splits<Acc, C>(s.P, nb, ns, part, s.d_lam, s.P, W, (size_t)nb, st)));
    c->prof.close(h, st);
    h = c->prof.open(PH_EXPAND, st);
    CUDA_TRY(c, launch_expand_gemm<C>(s.P, nb, s.npw, W, (size_t)nb, pr, (size_t)s.npw, hpsi, (size_t)s.npw, st));
    c->prof.close(h, st);
    return HPSI_OK;
}

template <typename C, typename Acc>
static size_t nonlocal_ws(const KSlot& s, int nb, int rows_mult)
{
    const int M = rows_mult * s.P;
    const int ns = split_for(M, nb, s.npw);
    Carver cv;
    cv.take<Acc>((size_t)ns * M * nb);
    cv.take<C>((size_t)M * nb);
    return cv.off;
}

static int chunk_bands(const KSlot& s, const hpsi_ctx* c, int nb, size_t csize)
{
    size_t per = (size_t)s.nxs * c->n2 * c->n3 * csize;
    if (per == 0) return nb;
    long ch = (long)((512ull << 20) / per);
    return (int)std::max(1L, std::min((long)nb, ch));
}

template <typename C, typename V>
static int local_apply(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* hpsi, unsigned char* ws,
                       const V* vloc, const C* tw, cudaStream_t st, double* epart = nullptr,
                       float2* out32 = nullptr, unsigned* rowmax = nullptr, cudaEvent_t after_g2r = nullptr,
                       const cudaEvent_t* psi_in = nullptr, int psi_mid = 0)
{
    if (nb == 0 || s.npw == 0) return HPSI_OK;
    const int* pl = s.d_plane;
    LocalArgs a{};
    a.n1 = c->n1; a.n2 = c->n2; a.n3 = c->n3;
    a.npw = s.npw;
    a.nxs = s.nxs;
    local_xpass_shape(&a, sizeof(C));
    a.inv_n = 1.0 / ((double)c->n1 * c->n2 * c->n3);
    a.plane_x = pl;
    a.plane_off = pl + s.nxs;
    a.ent_ig = pl + 2 * s.nxs + 1;
    a.ent_jk = pl + 2 * s.nxs + 1 + s.npw;
    a.plane_jr = pl + 2 * s.nxs + 1 + 2 * s.npw;
    a.Lx = c->L[0]; a.Ly = c->L[1]; a.Lz = c->L[2];
    const int ch = chunk_bands(s, c, nb, sizeof(C));
    C* T = reinterpret_cast<C*>(ws);
    if (psi_in && ch < nb) {
        // several band chunks: no split, every launch after all of psi
        for (int i = 0; i < 2; ++i) CUDA_TRY(c, cudaStreamWaitEvent(st, psi_in[i], 0));
        psi_in = nullptr;
    }
    for (int b0 = 0; b0 < nb; b0 += ch) {
        int nbc = std::min(ch, nb - b0);
        a.epart = epart;
        a.e_band0 = b0;
        a.out32 = out32 ? out32 + (size_t)b0 * s.npw : nullptr;
        a.rowmax = rowmax ? rowmax + b0 : nullptr;
        a.after_g2r = b0 == 0 ? after_g2r : nullptr;
        a.dv32 = (epart && sizeof(V) == sizeof(float)) ? c->d_dv32 : nullptr;
        // psi in two band halves (one chunk only; the plans that run the lane-pair G->r pass)
        const bool split = psi_in && b0 == 0 && nbc == nb;
        a.psi_in[0] = split ? psi_in[0] : nullptr;
        a.psi_in[1] = split ? psi_in[1] : nullptr;
        a.psi_mid = split ? psi_mid : 0;
        CUDA_TRY(c, (launch_local<C, V>(a, nbc, psi + (size_t)b0 * s.npw, hpsi + (size_t)b0 * s.npw, s.d_kin, T, vloc,
                                        tw, tw + c->n1, tw + c->n1 + c->n2, st, &c->prof)));
    }
    return HPSI_OK;
}

static size_t local_ws(const hpsi_ctx* c, const KSlot& s, int nb, size_t csize);

// rho += sum_b occ_b |psi_b(r)|^2 on device pointers (T chunks in ws)
template <typename C>
static int density_apply(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, const double* occ, double* rho,
                         unsigned char* ws, const C* tw, cudaStream_t st)
{
    if (nb == 0 || s.npw == 0) return HPSI_OK;
    const int* pl = s.d_plane;
    LocalArgs a{};
    a.n1 = c->n1; a.n2 = c->n2; a.n3 = c->n3;
    a.npw = s.npw;
    a.nxs = s.nxs;
    local_xpass_shape(&a, sizeof(C));
    a.inv_n = 1.0 / ((double)c->n1 * c->n2 * c->n3);
    a.plane_x = pl;
    a.plane_off = pl + s.nxs;
    a.ent_ig = pl + 2 * s.nxs + 1;
    a.ent_jk = pl + 2 * s.nxs + 1 + s.npw;
    a.plane_jr = pl + 2 * s.nxs + 1 + 2 * s.npw;
    a.Lx = c->L[0]; a.Ly = c->L[1]; a.Lz = c->L[2];
    const int ch = chunk_bands(s, c, nb, sizeof(C));
    C* T = reinterpret_cast<C*>(ws);
    // the register density pass's group partials, after T
    double* part = density_part_bytes(a, ch, sizeof(C))
                       ? reinterpret_cast<double*>(ws + (local_ws(c, s, nb, sizeof(C)) + 255) / 256 * 256)
                       : nullptr;
    for (int b0 = 0; b0 < nb; b0 += ch) {
        const int nbc = std::min(ch, nb - b0);
        CUDA_TRY(c, launch_density<C>(a, nbc, psi + (size_t)b0 * s.npw, occ + b0, rho, T, tw, tw + c->n1,
                                      tw + c->n1 + c->n2, st, part));
    }
    return HPSI_OK;
}

static size_t local_ws(const hpsi_ctx* c, const KSlot& s, int nb, size_t csize)
{
    int ch = chunk_bands(s, c, nb, csize);
    Carver cv;
    cv.take<unsigned char>((size_t)ch * s.nxs * c->n2 * c->n3 * csize);
    return cv.off;
}

static int check_call(hpsi_ctx* c, int kid, int nb, KSlot** sp, int flags)
{
    if (!c) return HPSI_ERR_BAD_ARG;
    if (nb < 0) return fail(c, HPSI_ERR_BAD_ARG, "nb < 0");
    int prec = flags & HPSI_PREC_MASK;
    if (prec != HPSI_PREC_FP64 && prec != HPSI_PREC_FP32 && prec != HPSI_PREC_TC && prec != HPSI_PREC_TC_BF16)
        return fail(c, HPSI_ERR_BAD_ARG, "unknown precision %d", prec);
    KSlot* s = get_slot(c, kid);
    if (!s) return fail(c, HPSI_ERR_STATE, "k-point slot %d is not bound", kid);
    *sp = s;
    cudaError_t e = cudaSetDevice(c->dev);
    if (e) return fail(c, HPSI_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    return HPSI_OK;
}

// ---- tensor-core nonlocal term ----------------------------------------------
static int ensure_tc(hpsi_ctx* c, KSlot& s, int fmt, cudaStream_t st)
{
    if (s.P == 0 || s.npw == 0) return HPSI_OK;
    s.tc_fmt = -1;
    if (s.tc_mem[fmt]) {
        s.tc_fmt = fmt;
        return HPSI_OK;
    }
    // by rows: the distinct (radial function, lm) pairs of the projectors
    std::vector<int2> prow((size_t)s.P), byinfo;
    std::map<std::pair<int, int>, int> at;
    for (int p = 0; p < s.P; ++p) {
        const ProjRow& r = s.rows[(size_t)p];
        const std::pair<int, int> key(r.rad, r.l * r.l + r.l + r.m);
        auto it = at.find(key);
        if (it == at.end()) {
            it = at.emplace(key, (int)byinfo.size()).first;
            byinfo.push_back(make_int2(key.first, key.second));
        }
        prow[(size_t)p] = make_int2(r.atom, it->second);
    }
    const int nby = (int)byinfo.size();
    CUDA_TRY(c, dalloc(&s.tc_mem[fmt], tc_gen_bytes(s.P, s.npw, nby, c->natom)));
    int h = c->prof.open(PH_BUILD, st);
    CUDA_TRY(c, tc_build_gen(s.tc_mem[fmt], s.P, s.npw, prow.data(), byinfo.data(), nby, c->natom, s.d_beta,
                             s.d_ylm, s.d_sf, fmt == 0, &s.tcgen[fmt], st));
    c->prof.close(h, st, 4);
    s.tc_proj[fmt] = TcOperand{nullptr, nullptr, const_cast<float*>(s.tcgen[fmt].p_inv), tc_round_k(2 * (size_t)s.npw)};
    s.tc_expand[fmt] = TcOperand{nullptr, nullptr, const_cast<float*>(s.tcgen[fmt].g_inv), tc_round_k(2 * (size_t)s.P)};
    s.tc_fmt = fmt;
    return HPSI_OK;
}

// Split count of the tensor-core projection.  With band energies the FP32
// accumulation chains in TMEM are kept to kEnergyChainK of K per split (the
// partials are summed in FP64): the tensor cores' FP32 accumulation drifts
// over long chains, which the band energies would show at the 1e-8 Ha level.
constexpr int kEnergyChainK = 1024;
// the band-pair velocity GEMMs (K = 2 npw deep, results compared element-wise)
// need shorter chains still: 256 of K keeps them within 1e-6 of FP64
constexpr int kVelocityChainK = 256;
static int tc_splits(const KSlot& s, int nb, bool energy)
{
    const size_t k1 = tc_round_k(2 * (size_t)s.npw);
    const int ns = tc_proj_splits(s.P, nb, k1);
    if (!energy) return ns;
    return std::max(ns, tc_chain_splits(k1, kEnergyChainK));
}

// Workspace of the tensor-core nonlocal term: split band operand, partials,
// W and its split operand, per-band maxima, nonlocal energy terms
struct TcNlOffsets {
    size_t b1h, b1l, b1s, part, w, b2h, b2l, b2s, rowmax, eterm, bytes;
    size_t k1, k2;
    int ns;
};

static TcNlOffsets tc_offsets(const KSlot& s, int nb, bool energy)
{
    const int NB = tc_band_rows(nb);
    TcNlOffsets o;
    o.k1 = tc_round_k(2 * (size_t)s.npw);
    o.k2 = tc_round_k(2 * (size_t)s.P);
    o.ns = tc_splits(s, nb, energy);
    Carver cv;
    o.b1h = cv.take<uint16_t>((size_t)NB * o.k1);
    o.b1l = cv.take<uint16_t>((size_t)NB * o.k1);
    o.b1s = cv.take<float>((size_t)NB);
    o.part = cv.take<float>((size_t)o.ns * s.P * NB);
    o.w = cv.take<float2>((size_t)s.P * nb);
    o.b2h = cv.take<uint16_t>((size_t)NB * o.k2);
    o.b2l = cv.take<uint16_t>((size_t)NB * o.k2);
    o.b2s = cv.take<float>((size_t)NB);
    o.rowmax = cv.take<unsigned>((size_t)nb);
    o.eterm = energy ? cv.take<double>((size_t)s.P * nb) : 0;
    o.bytes = cv.off;
    return o;
}

static size_t tc_ws(const KSlot& s, int nb, bool energy = false) { return tc_offsets(s, nb, energy).bytes; }

struct TcNl {
    TcOperand B1, B2;
    float* part;
    float2* W;
    unsigned* rowmax;
    double* eterm;
    int ns;
};

static TcNl tc_layout(const KSlot& s, int nb, unsigned char* ws, bool energy)
{
    const TcNlOffsets o = tc_offsets(s, nb, energy);
    TcNl t;
    t.ns = o.ns;
    t.B1 = TcOperand{ws + o.b1h, ws + o.b1l, reinterpret_cast<float*>(ws + o.b1s), o.k1};
    t.B2 = TcOperand{ws + o.b2h, ws + o.b2l, reinterpret_cast<float*>(ws + o.b2s), o.k2};
    t.part = reinterpret_cast<float*>(ws + o.part);
    t.W = reinterpret_cast<float2*>(ws + o.w);
    t.rowmax = reinterpret_cast<unsigned*>(ws + o.rowmax);
    t.eterm = energy ? reinterpret_cast<double*>(ws + o.eterm) : nullptr;
    return t;
}

// Projection half: split psi, W = lambda <p|psi> (+ nonlocal energies), split W
static int tc_nonlocal_project(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, unsigned char* ws,
                               cudaStream_t st, double* e_nl, bool have_max = false)
{
    const bool fp16 = s.tc_fmt == 0;
    TcNl t = tc_layout(s, nb, ws, e_nl != nullptr);
    // kernels of the operand builders: band maxima (unless taken), split rows,
    // and zero rows when the last 128-band block is partial
    const int zero_rows = tc_band_rows(nb) / 2 > nb ? 1 : 0;
    int h = c->prof.open(PH_OTHER, st);
    CUDA_TRY(c, tc_band_operand(psi, nb, s.npw, fp16, &t.B1, t.rowmax, st, have_max));
    c->prof.close(h, st, (have_max ? 1 : 2) + zero_rows);
    const int f = s.tc_fmt;
    CUDA_TRY(c, tc_projection(s.tc_proj[f], s.P, t.B1, nb, t.ns, fp16, t.part, s.d_lam, s.P, t.W, c->d_err, st,
                              &c->prof, t.eterm, e_nl, &s.tcgen[f]));
    h = c->prof.open(PH_OTHER, st);
    CUDA_TRY(c, tc_w_operand(t.W, s.P, nb, fp16, &t.B2, t.rowmax, st));
    c->prof.close(h, st, 2 + zero_rows);
    return HPSI_OK;
}

// Expansion half: hpsi += P^T W (+ add32, the local term in complex64)
static int tc_nonlocal_expand(hpsi_ctx* c, KSlot& s, int nb, double2* hpsi, unsigned char* ws, cudaStream_t st,
                              bool energy, const float2* add32, int row0 = 0, int row1 = -1)
{
    TcNl t = tc_layout(s, nb, ws, energy);
    const int f = s.tc_fmt;
    CUDA_TRY(c, tc_expansion(s.tc_expand[f], s.npw, t.B2, nb, f == 0, hpsi, c->d_err, st, &c->prof, add32,
                             &s.tcgen[f], row0, row1));
    return HPSI_OK;
}

static int ensure_tc_grad(hpsi_ctx* c, KSlot& s, int fmt, cudaStream_t st)
{
    if (s.P == 0 || s.npw == 0) return HPSI_OK;
    if (s.tcg_fmt == fmt && s.tcg_mem) return HPSI_OK;
    int rc;
    if ((rc = ensure_proj<float2>(c, s, true, st))) return rc;
    dfree(s.tcg_mem);
    s.tcg_fmt = -1;
    const size_t k1 = tc_round_k(2 * (size_t)s.npw), k2 = tc_round_k(4 * (size_t)s.P);
    Carver cv;
    const size_t rp = tc_rows_pad(4 * (size_t)s.P), rg = tc_rows_pad(s.npw);
    const size_t o1h = cv.take<uint16_t>(rp * k1), o1l = cv.take<uint16_t>(rp * k1);
    const size_t o1s = cv.take<float>((size_t)4 * s.P);
    size_t oh[3], ol[3], os[3];
    for (int a = 0; a < 3; ++a) {
        oh[a] = cv.take<uint16_t>(rg * k2);
        ol[a] = cv.take<uint16_t>(rg * k2);
        os[a] = cv.take<float>((size_t)s.npw);
    }
    const size_t ocm = cv.take<float>((size_t)s.npw);
    CUDA_TRY(c, dalloc(&s.tcg_mem, cv.off));
    CUDA_TRY(c, cudaMemsetAsync(s.tcg_mem, 0, cv.off, st));  // padding rows and K padding read as zero
    s.tcg_proj = TcOperand{s.tcg_mem + o1h, s.tcg_mem + o1l, reinterpret_cast<float*>(s.tcg_mem + o1s), k1};
    for (int a = 0; a < 3; ++a)
        s.tcg_exp[a] = TcOperand{s.tcg_mem + oh[a], s.tcg_mem + ol[a], reinterpret_cast<float*>(s.tcg_mem + os[a]), k2};
    int h = c->prof.open(PH_BUILD, st);
    CUDA_TRY(c, tc_build_grad_operands(s.pr32, s.P, s.npw, fmt == 0, &s.tcg_proj, s.tcg_exp,
                                       reinterpret_cast<float*>(s.tcg_mem + ocm), st));
    c->prof.close(h, st);
    s.tcg_fmt = fmt;
    return HPSI_OK;
}

static size_t tc_grad_ws(const KSlot& s, int nb)
{
    const int NB = tc_band_rows(nb);
    const size_t k1 = tc_round_k(2 * (size_t)s.npw), k2 = tc_round_k(4 * (size_t)s.P);
    const int ns = tc_proj_splits(4 * s.P, nb, k1);
    Carver cv;
    cv.take<uint16_t>((size_t)NB * k1);
    cv.take<uint16_t>((size_t)NB * k1);
    cv.take<float>((size_t)NB);
    cv.take<float>((size_t)ns * 4 * s.P * NB);
    cv.take<float2>((size_t)4 * s.P * nb);
    cv.take<float2>((size_t)2 * s.P * nb);
    cv.take<uint16_t>((size_t)NB * k2);
    cv.take<uint16_t>((size_t)NB * k2);
    cv.take<float>((size_t)NB);
    cv.take<unsigned>((size_t)nb);
    return cv.off;
}

// d_alpha += nonlocal part of dH/dk_alpha psi on the tensor cores (device pointers)
static int tc_grad_nonlocal(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* d[3], unsigned char* ws,
                            cudaStream_t st)
{
    if (s.P == 0 || nb == 0) return HPSI_OK;
    const bool fp16 = s.tcg_fmt == 0;
    const int NB = tc_band_rows(nb), P = s.P, P4 = 4 * s.P;
    const size_t k1 = s.tcg_proj.ldk, k2 = s.tcg_exp[0].ldk;
    const int ns = tc_proj_splits(P4, nb, k1);
    Carver cv;
    const size_t ob1h = cv.take<uint16_t>((size_t)NB * k1), ob1l = cv.take<uint16_t>((size_t)NB * k1);
    const size_t ob1s = cv.take<float>((size_t)NB);
    const size_t opart = cv.take<float>((size_t)ns * P4 * NB);
    const size_t ow = cv.take<float2>((size_t)P4 * nb);
    const size_t ow2 = cv.take<float2>((size_t)2 * P * nb);
    const size_t ob2h = cv.take<uint16_t>((size_t)NB * k2), ob2l = cv.take<uint16_t>((size_t)NB * k2);
    const size_t ob2s = cv.take<float>((size_t)NB);
    unsigned* rowmax = reinterpret_cast<unsigned*>(ws + cv.take<unsigned>((size_t)nb));
    TcOperand B1{ws + ob1h, ws + ob1l, reinterpret_cast<float*>(ws + ob1s), k1};
    TcOperand B2{ws + ob2h, ws + ob2l, reinterpret_cast<float*>(ws + ob2s), k2};
    float2* W = reinterpret_cast<float2*>(ws + ow);    // [4P][nb]: <p|psi>, <dp_x|psi>, <dp_y|psi>, <dp_z|psi> (x lambda)
    float2* W2 = reinterpret_cast<float2*>(ws + ow2);  // [2P][nb]: (<dp_a|psi>, <p|psi>) for one direction
    int h = c->prof.open(PH_OTHER, st);
    CUDA_TRY(c, tc_band_operand(psi, nb, s.npw, fp16, &B1, rowmax, st));
    c->prof.close(h, st);
    CUDA_TRY(c, tc_projection(s.tcg_proj, P4, B1, nb, ns, fp16, reinterpret_cast<float*>(ws + opart), s.d_lam, P, W,
                              c->d_err, st, &c->prof));
    const size_t blk = (size_t)P * nb * sizeof(float2);
    for (int a = 0; a < 3; ++a) {
        if (!d[a]) continue;
        // out_a += sum_p lambda <dp_a|psi> p + lambda <p|psi> dp_a: K = (p block, dp_a block)
        CUDA_TRY(c, cudaMemcpyAsync(W2, W + (size_t)(1 + a) * P * nb, blk, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(c, cudaMemcpyAsync(W2 + (size_t)P * nb, W, blk, cudaMemcpyDeviceToDevice, st));
        h = c->prof.open(PH_OTHER, st);
        CUDA_TRY(c, tc_w_operand(W2, 2 * P, nb, fp16, &B2, rowmax, st));
        c->prof.close(h, st);
        CUDA_TRY(c, tc_expansion(s.tcg_exp[a], s.npw, B2, nb, fp16, d[a], c->d_err, st, &c->prof));
    }
    return HPSI_OK;
}

// After a synchronising call: report a bounded-wait timeout of the tensor-core kernels.
static int check_device_flag(hpsi_ctx* c)
{
    int v = 0;
    CUDA_TRY(c, cudaMemcpy(&v, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (v) {
        cudaMemset(c->d_err, 0, sizeof(int));
        return fail(c, HPSI_ERR_TIMEOUT, "tensor-core GEMM: a bounded pipeline wait gave up (site %d)", v);
    }
    return HPSI_OK;
}

__global__ void grad_kinetic_kernel(int npw, int nb, const double* __restrict__ kvec, const double2* __restrict__ psi,
                                    double2* dx, double2* dy, double2* dz)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)npw * nb) return;
    int g = (int)(i % npw);
    double2 p = psi[i];
    double2* out[3] = {dx, dy, dz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (!out[d]) continue;
        double k = kvec[3 * g + d];
        double2 o = out[d][i];
        o.x += k * p.x;
        o.y += k * p.y;
        out[d][i] = o;
    }
}

// d_alpha += dH/dk_alpha psi, all pointers on the device
template <typename C, typename Acc>
static int grad_device(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* d[3], unsigned char* work,
                       cudaStream_t st)
{
    const size_t nel = (size_t)nb * s.npw;
    int h = c->prof.open(PH_OTHER, st);
    grad_kinetic_kernel<<<ceil_div((long)nel, 256), 256, 0, st>>>(s.npw, nb, s.d_kvec, psi, d[0], d[1], d[2]);
    c->prof.close(h, st);
    CUDA_TRY(c, cudaGetLastError());
    if (s.P == 0) return HPSI_OK;
    int rc;
    if ((rc = ensure_proj<C>(c, s, true, st))) return rc;
    const C* pr = std::is_same<C, double2>::value ? (const C*)s.pr64 : (const C*)s.pr32;
    const int M = 4 * s.P;
    const int ns = split_for(M, nb, s.npw);
    Carver cv;
    size_t o_part = cv.take<Acc>((size_t)ns * M * nb);
    size_t o_w = cv.take<C>((size_t)M * nb);
    Acc* part = reinterpret_cast<Acc*>(work + o_part);
    C* W = reinterpret_cast<C*>(work + o_w);
    h = c->prof.open(PH_PROJ, st);
    CUDA_TRY(c, (launch_proj_gemm<C, double2, Acc>(M, nb, s.npw, pr, (size_t)s.npw, psi, (size_t)s.npw, part, ns, st)));
    c->prof.close(h, st);
    h = c->prof.open(PH_REDUCE, st);
    CUDA_TRY(c, (launch_reduce_splits<Acc, C>(M, nb, ns, part, s.d_lam, s.P, W, (size_t)nb, st)));
    c->prof.close(h, st);
    const size_t PN = (size_t)s.P * s.npw;
    for (int a = 0; a < 3; ++a) {
        if (!d[a]) continue;
        h = c->prof.open(PH_EXPAND, st);
        // lambda <dp_a|psi> p
        CUDA_TRY(c, launch_expand_gemm<C>(s.P, nb, s.npw, W + (size_t)(a + 1) * s.P * nb, (size_t)nb, pr, (size_t)s.npw,
                                          d[a], (size_t)s.npw, st));
        // lambda <p|psi> dp_a
        CUDA_TRY(c, launch_expand_gemm<C>(s.P, nb, s.npw, W, (size_t)nb, pr + (size_t)(a + 1) * PN, (size_t)s.npw, d[a],
                                          (size_t)s.npw, st));
        c->prof.close(h, st);
    }
    return HPSI_OK;
}

template <typename C, typename Acc>
static size_t grad_ws(const KSlot& s, int nb)
{
    return nonlocal_ws<C, Acc>(s, nb, 4);
}

static int grad_tc(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* d[3], unsigned char* work, int fmt,
                   cudaStream_t st)
{
    const size_t nel = (size_t)nb * s.npw;
    int h = c->prof.open(PH_OTHER, st);
    grad_kinetic_kernel<<<ceil_div((long)nel, 256), 256, 0, st>>>(s.npw, nb, s.d_kvec, psi, d[0], d[1], d[2]);
    c->prof.close(h, st);
    CUDA_TRY(c, cudaGetLastError());
    int rc;
    if ((rc = ensure_tc_grad(c, s, fmt, st))) return rc;
    return tc_grad_nonlocal(c, s, nb, psi, d, work, st);
}


static bool is_tc(int prec) { return prec == HPSI_PREC_TC || prec == HPSI_PREC_TC_BF16; }

int prepare_slot(hpsi_ctx* c, KSlot& s, int prec, bool grad, cudaStream_t st)
{
    int rc;
    if (prec == HPSI_PREC_FP64) return ensure_proj<double2>(c, s, grad, st);
    if (is_tc(prec)) {
        if ((rc = ensure_tc(c, s, prec == HPSI_PREC_TC ? 0 : 1, st))) return rc;
        if (grad && (rc = ensure_tc_grad(c, s, prec == HPSI_PREC_TC ? 0 : 1, st))) return rc;
        return HPSI_OK;
    }
    return ensure_proj<float2>(c, s, grad, st);
}

// workspace of one H|psi> on device pointers
static size_t apply_ws_bytes(const hpsi_ctx* c, const KSlot& s, int nb, int prec, bool energy = false)
{
    const bool fp64 = prec == HPSI_PREC_FP64;
    size_t wl = local_ws(c, s, nb, fp64 ? sizeof(double2) : sizeof(float2));
    // disjoint: the two halves run concurrently; then the complex64 local term
    if (is_tc(prec)) {
        Carver cv;
        cv.take<float2>((size_t)nb * s.npw);
        return wl + tc_ws(s, nb, energy) + (s.P > 0 ? cv.off : 0);
    }
    size_t wn = fp64 ? nonlocal_ws<double2, double2>(s, nb, 1) : nonlocal_ws<float2, float2>(s, nb, 1);
    return std::max(wl, wn);
}

// hpsi += H psi on device pointers with an explicit workspace (prepare_slot first)
// hpsi_ready: an event after which hpsi holds its input (an H2D copy on
// another stream); only the tensor-core expansion reads hpsi, so only it waits
// hpsi_apply with host buffers: hpsi arrives in two G halves [0, mid) and
// [mid, npw) (events in[0], in[1]); the expansion runs per half, and the first
// half goes back to host_out on the side stream while the second half is
// expanded (out: recorded after that copy).
struct HostHalves {
    int mid;
    cudaEvent_t in[2];
    double* host_out;
    cudaEvent_t out;
    cudaEvent_t psi_in[2];  // psi's band halves [0, psi_mid), [psi_mid, nb) (null: psi is on st already)
    int psi_mid;
};

static int apply_dev(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* hpsi, int prec, unsigned char* work,
                     cudaStream_t st, double* epart = nullptr, double* e_nl = nullptr, bool fork = true,
                     cudaEvent_t hpsi_ready = nullptr, const HostHalves* halves = nullptr)
{
    int rc;
    if ((rc = prepare_slot(c, s, prec, false, st))) return rc;
    if (prec == HPSI_PREC_FP64) {
        if ((rc = local_apply<double2, double>(c, s, nb, psi, hpsi, work, c->d_v64, c->d_tw64, st, epart))) return rc;
        return nonlocal_apply<double2, double2>(c, s, nb, psi, hpsi, s.pr64, work, st, e_nl);
    }
    if (hpsi_ready && !(is_tc(prec) && s.P > 0 && nb > 0 && fork))
        CUDA_TRY(c, cudaStreamWaitEvent(st, hpsi_ready, 0));  // the other paths read hpsi from the start
    if (is_tc(prec) && s.P > 0 && nb > 0) {
        // the projection chain on the side stream, beside the FFT passes; the
        // expansion joins back after the r->G pass (both add into hpsi).  With
        // fork false (the server's lanes already overlap) all runs on st.
        // The local term goes to a complex64 buffer (loc32) that the expansion
        // adds with its own product: one FP64 read-modify-write of hpsi.
        const size_t wl = local_ws(c, s, nb, sizeof(float2));
        unsigned char* wnl = work + wl;
        float2* loc32 = reinterpret_cast<float2*>(work + wl + tc_ws(s, nb, e_nl != nullptr));
        // The G->r pass takes the per-band maxima of psi that scale the band
        // operand when it covers all bands in one launch
        unsigned* rowmax = tc_layout(s, nb, wnl, e_nl != nullptr).rowmax;
        const bool g2r_max = chunk_bands(s, c, nb, sizeof(float2)) >= nb;
        if (g2r_max) CUDA_TRY(c, cudaMemsetAsync(rowmax, 0, sizeof(unsigned) * nb, st));
        unsigned* rm = g2r_max ? rowmax : nullptr;
        if (!fork) {
            if ((rc = local_apply<float2, float>(c, s, nb, psi, hpsi, work, c->d_v32, c->d_tw32, st, epart, loc32,
                                                 rm)))
                return rc;
            if ((rc = tc_nonlocal_project(c, s, nb, psi, wnl, st, e_nl, g2r_max))) return rc;
            return tc_nonlocal_expand(c, s, nb, hpsi, wnl, st, e_nl != nullptr, loc32);
        }
        // fork after the G->r pass when it takes the maxima, else right away
        if (!g2r_max) CUDA_TRY(c, cudaEventRecord(c->ev_fork, st));
        rc = local_apply<float2, float>(c, s, nb, psi, hpsi, work, c->d_v32, c->d_tw32, st, epart, loc32, rm,
                                        g2r_max ? c->ev_fork : nullptr, halves ? halves->psi_in : nullptr,
                                        halves ? halves->psi_mid : 0);
        if (rc) return rc;
        CUDA_TRY(c, cudaStreamWaitEvent(c->side, c->ev_fork, 0));
        if (halves && halves->psi_in[1]) CUDA_TRY(c, cudaStreamWaitEvent(c->side, halves->psi_in[1], 0));
        if ((rc = tc_nonlocal_project(c, s, nb, psi, wnl, c->side, e_nl, g2r_max))) {
            cudaEventRecord(c->ev_join, c->side);  // still join, so that no work is left unordered
            cudaStreamWaitEvent(st, c->ev_join, 0);
            return rc;
        }
        CUDA_TRY(c, cudaEventRecord(c->ev_join, c->side));
        CUDA_TRY(c, cudaStreamWaitEvent(st, c->ev_join, 0));
        if (halves) {
            const size_t pitch = (size_t)s.npw * sizeof(double2);
            CUDA_TRY(c, cudaStreamWaitEvent(st, halves->in[0], 0));
            if ((rc = tc_nonlocal_expand(c, s, nb, hpsi, wnl, st, e_nl != nullptr, loc32, 0, halves->mid))) {
                cudaStreamWaitEvent(st, halves->in[1], 0);  // leave no copy unordered behind st
                return rc;
            }
            CUDA_TRY(c, cudaEventRecord(c->ev_half_exp, st));
            CUDA_TRY(c, cudaStreamWaitEvent(c->side, c->ev_half_exp, 0));
            CUDA_TRY(c, cudaMemcpy2DAsync(halves->host_out, pitch, hpsi, pitch, (size_t)halves->mid * sizeof(double2),
                                          nb, cudaMemcpyDeviceToHost, c->side));
            CUDA_TRY(c, cudaEventRecord(halves->out, c->side));
            CUDA_TRY(c, cudaStreamWaitEvent(st, halves->in[1], 0));
            return tc_nonlocal_expand(c, s, nb, hpsi, wnl, st, e_nl != nullptr, loc32, halves->mid, s.npw);
        }
        if (hpsi_ready) CUDA_TRY(c, cudaStreamWaitEvent(st, hpsi_ready, 0));
        return tc_nonlocal_expand(c, s, nb, hpsi, wnl, st, e_nl != nullptr, loc32);
    }
    if ((rc = local_apply<float2, float>(c, s, nb, psi, hpsi, work, c->d_v32, c->d_tw32, st, epart))) return rc;
    return nonlocal_apply<float2, float2>(c, s, nb, psi, hpsi, s.pr32, work, st, e_nl);
}

// Band energies beside H|psi>: scratch layout in front of the apply workspace
struct EnergyWs {
    size_t kn, loc, enl, epart, dots, work;
    int nslots;
};

static EnergyWs energy_layout(const hpsi_ctx* c, int nb, int prec)
{
    LocalArgs a{};
    a.n1 = c->n1; a.n2 = c->n2; a.n3 = c->n3;
    a.Lx = c->L[0]; a.Ly = c->L[1]; a.Lz = c->L[2];
    const size_t csize = prec == HPSI_PREC_FP64 ? sizeof(double2) : sizeof(float2);
    local_xpass_shape(&a, csize);
    EnergyWs w;
    w.nslots = local_energy_slots(a, csize);
    Carver cv;
    w.kn = cv.take<double>((size_t)kin_norm_words(nb));
    w.loc = cv.take<double>(2 * (size_t)nb);
    w.enl = cv.take<double>((size_t)nb);
    w.epart = cv.take<double>((size_t)nb * w.nslots * 2);
    w.dots = cv.take<double>(2 * (size_t)nb);
    w.work = cv.off;
    return w;
}

// hpsi += H psi and e[b] = <psi_b|H|psi_b> with FP64 reductions, device pointers
static int energies_dev(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* hpsi, double* e, int prec,
                        unsigned char* ws, cudaStream_t st, bool fork = true)
{
    int rc;
    if ((rc = prepare_slot(c, s, prec, false, st))) return rc;
    const EnergyWs w = energy_layout(c, nb, prec);
    double* kn = reinterpret_cast<double*>(ws + w.kn);
    double* loc = reinterpret_cast<double*>(ws + w.loc);
    double* enl = reinterpret_cast<double*>(ws + w.enl);
    double* epart = reinterpret_cast<double*>(ws + w.epart);
    double* dots = reinterpret_cast<double*>(ws + w.dots);
    if (s.aliased) {
        // two G-vectors share a grid point: the Parseval identity does not hold,
        // so the energy is the Rayleigh quotient of the computed H|psi>
        CUDA_TRY(c, launch_band_dot(s.npw, nb, psi, hpsi, dots, st));
        if ((rc = apply_dev(c, s, nb, psi, hpsi, prec, ws + w.work, st))) return rc;
        CUDA_TRY(c, launch_band_dot(s.npw, nb, psi, hpsi, dots + nb, st));
        CUDA_TRY(c, launch_band_sub(nb, dots + nb, dots, e, st));
        return HPSI_OK;
    }
    int h = c->prof.open(PH_OTHER, st);
    CUDA_TRY(c, launch_kin_norm(s.npw, nb, psi, s.d_kin, kn, st));
    c->prof.close(h, st);
    if ((rc = apply_dev(c, s, nb, psi, hpsi, prec, ws + w.work, st, epart, enl, fork))) return rc;
    h = c->prof.open(PH_OTHER, st);
    CUDA_TRY(c, launch_local_sums(nb, w.nslots, epart, loc, st));
    CUDA_TRY(c, launch_energy_combine(nb, kn, loc, s.P > 0 ? enl : nullptr, e, st));
    c->prof.close(h, st);
    return HPSI_OK;
}

static size_t grad_ws_bytes(const KSlot& s, int nb, int prec)
{
    if (prec == HPSI_PREC_FP64) return grad_ws<double2, double2>(s, nb);
    return is_tc(prec) ? tc_grad_ws(s, nb) : grad_ws<float2, float2>(s, nb);
}

// d_a += dH/dk_a psi on device pointers (NULL d_a skipped)
static int grad_dev(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* d[3], int prec, unsigned char* work,
                    cudaStream_t st)
{
    int rc;
    if ((rc = prepare_slot(c, s, prec, true, st))) return rc;
    if (is_tc(prec)) return grad_tc(c, s, nb, psi, d, work, prec == HPSI_PREC_TC ? 0 : 1, st);
    return prec == HPSI_PREC_FP64 ? grad_device<double2, double2>(c, s, nb, psi, d, work, st)
                                  : grad_device<float2, float2>(c, s, nb, psi, d, work, st);
}

// velocity workspace: G_a (3 nb npw complex128), then either the gradient's
// workspace or (after the gradient) the psi^H G GEMM's: SIMT split partials, or
// the tensor-core operands (psi rows, G_a band rows) and partials
struct VelWs {
    size_t g, rest;           // G_a; start of the shared region
    size_t vp;                // SIMT partials (relative to rest)
    size_t ah, al, as, bh, bl, bs, part, rowmax;  // tensor-core pieces (relative to rest)
    size_t gemm_bytes;        // bytes of the GEMM region
    int nsv;                  // SIMT split count
    int ns_tc;                // tensor-core split count
    size_t k1;
};

static VelWs vel_layout(const KSlot& s, int nb, int prec)
{
    VelWs w{};
    Carver cv;
    w.g = cv.take<double2>((size_t)3 * nb * s.npw);
    w.rest = cv.off;
    w.nsv = split_for(nb, nb, s.npw);
    Carver g;
    if (is_tc(prec)) {
        const int NB = tc_band_rows(nb);
        w.k1 = tc_round_k(2 * (size_t)s.npw);
        // short FP32 accumulation chains in TMEM (FP64 sums of the splits)
        w.ns_tc = std::max(tc_proj_splits(nb, nb, w.k1), tc_chain_splits(w.k1, kVelocityChainK));
        w.ah = g.take<uint16_t>(tc_rows_pad(nb) * w.k1);
        w.al = g.take<uint16_t>(tc_rows_pad(nb) * w.k1);
        w.as = g.take<float>((size_t)nb);
        w.bh = g.take<uint16_t>((size_t)NB * w.k1);
        w.bl = g.take<uint16_t>((size_t)NB * w.k1);
        w.bs = g.take<float>((size_t)NB);
        w.part = g.take<float>((size_t)w.ns_tc * nb * NB);
        w.rowmax = g.take<unsigned>((size_t)nb);
    } else {
        w.vp = g.take<double2>((size_t)w.nsv * nb * nb);
    }
    w.gemm_bytes = g.off;
    return w;
}

static size_t vel_ws_bytes(const KSlot& s, int nb, int prec)
{
    const VelWs w = vel_layout(s, nb, prec);
    return w.rest + std::max(w.gemm_bytes, grad_ws_bytes(s, nb, prec));
}

// m[a][i][j] = sum_G conj(psi_i) (dH_a psi_j), overwritten, device pointers
static int velocity_dev(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* m, int prec, unsigned char* ws,
                        cudaStream_t st)
{
    const size_t nel = (size_t)nb * s.npw;
    const VelWs w = vel_layout(s, nb, prec);
    double2* g = reinterpret_cast<double2*>(ws + w.g);
    unsigned char* rest = ws + w.rest;
    CUDA_TRY(c, cudaMemsetAsync(g, 0, 3 * nel * sizeof(double2), st));
    double2* d[3] = {g, g + nel, g + 2 * nel};
    int rc = grad_dev(c, s, nb, psi, d, prec, rest, st);
    if (rc) return rc;
    if (is_tc(prec)) {
        // tensor cores: psi rows split once, each G_a as the band operand.  Both
        // tensor-core precisions use the scaled FP16 split here: a BF16 hi + lo
        // pair holds a value to ~2^-17, which leaves ~7e-6 in these K = 2 npw
        // band-pair sums, while the FP16 pair (per-row power-of-two scale) holds ~2^-22
        const bool fp16 = true;
        TcOperand A{rest + w.ah, rest + w.al, reinterpret_cast<float*>(rest + w.as), w.k1};
        TcOperand B{rest + w.bh, rest + w.bl, reinterpret_cast<float*>(rest + w.bs), w.k1};
        unsigned* rowmax = reinterpret_cast<unsigned*>(rest + w.rowmax);
        float* part = reinterpret_cast<float*>(rest + w.part);
        int h = c->prof.open(PH_OTHER, st);
        CUDA_TRY(c, tc_rows_operand(psi, nb, s.npw, fp16, &A, st));
        for (int a = 0; a < 3; ++a) {
            CUDA_TRY(c, tc_band_operand(d[a], nb, s.npw, fp16, &B, rowmax, st));
            CUDA_TRY(c, tc_gemm_c128(A, nb, B, nb, w.ns_tc, fp16, part, m + (size_t)a * nb * nb, c->d_err, st));
        }
        c->prof.close(h, st);
        return HPSI_OK;
    }
    for (int a = 0; a < 3; ++a) {
        int h = c->prof.open(PH_OTHER, st);
        if (prec == HPSI_PREC_FP64) {
            double2* vp = reinterpret_cast<double2*>(rest + w.vp);
            CUDA_TRY(c, (launch_proj_gemm<double2, double2, double2>(nb, nb, s.npw, psi, (size_t)s.npw, d[a],
                                                                     (size_t)s.npw, vp, w.nsv, st)));
            CUDA_TRY(c, (launch_reduce_splits<double2, double2>(nb, nb, w.nsv, vp, nullptr, 0, m + (size_t)a * nb * nb,
                                                                (size_t)nb, st)));
        } else {
            // FP32 products of the FP64 inputs, FP64 split-K reduction
            float2* vp = reinterpret_cast<float2*>(rest + w.vp);
            CUDA_TRY(c, (launch_proj_gemm<double2, double2, float2>(nb, nb, s.npw, psi, (size_t)s.npw, d[a],
                                                                    (size_t)s.npw, vp, w.nsv, st)));
            CUDA_TRY(c, (launch_reduce_splits<float2, double2>(nb, nb, w.nsv, vp, nullptr, 0, m + (size_t)a * nb * nb,
                                                               (size_t)nb, st)));
        }
        c->prof.close(h, st);
    }
    return HPSI_OK;
}

extern "C" int hpsi_apply(hpsi_ctx* c, int kid, int nb, const double* psi_, double* hpsi_, int flags, void* stream)
{
    KSlot* s = nullptr;
    int rc = check_call(c, kid, nb, &s, flags);
    if (rc) return rc;
    if (nb > 0 && (!psi_ || !hpsi_)) return fail(c, HPSI_ERR_BAD_ARG, "psi/hpsi NULL");
    if (nb == 0 || s->npw == 0) return HPSI_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int prec = flags & HPSI_PREC_MASK;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    const size_t nel = (size_t)nb * s->npw;
    Carver cv;
    size_t o_psi = dev ? 0 : cv.take<double2>(nel);
    size_t o_hpsi = dev ? 0 : cv.take<double2>(nel);
    size_t o_work = cv.off;
    if ((rc = ws_reserve(c, o_work + apply_ws_bytes(c, *s, nb, prec)))) return rc;
    const double2* psi = (const double2*)psi_;
    double2* hpsi = (double2*)hpsi_;
    const bool fork = !(flags & HPSI_ONE_STREAM);
    cudaEvent_t hpsi_ready = nullptr;
    // host buffers on the forked tensor-core path: hpsi in two G halves
    const int mid = (s->npw / 2 + 127) / 128 * 128;
    const bool halves = !dev && fork && is_tc(prec) && s->P > 0 && mid > 0 && mid < s->npw;
    const int pmid = nb / 2;  // psi's band halves
    HostHalves hh{mid, {c->ev_half_in[0], c->ev_half_in[1]}, hpsi_, c->ev_half_out,
                  {c->ev_psi_in[0], c->ev_psi_in[1]}, pmid};
    const size_t pitch = (size_t)s->npw * sizeof(double2);
    if (!dev) {
        psi = reinterpret_cast<const double2*>(c->ws + o_psi);
        hpsi = reinterpret_cast<double2*>(c->ws + o_hpsi);
        if (halves) {
            // every upload on the copy stream, after the work already queued on
            // st (which may still use the staging area): psi in two band halves,
            // each half of the G->r pass waiting for its own; then hpsi in two G
            // halves, one per expansion launch
            CUDA_TRY(c, cudaEventRecord(c->ev_copy_after, st));
            CUDA_TRY(c, cudaStreamWaitEvent(c->copy, c->ev_copy_after, 0));
            const size_t pb = (size_t)pmid * s->npw;
            if (pb)
                CUDA_TRY(c, cudaMemcpyAsync((void*)psi, psi_, pb * sizeof(double2), cudaMemcpyHostToDevice, c->copy));
            CUDA_TRY(c, cudaEventRecord(c->ev_psi_in[0], c->copy));
            CUDA_TRY(c, cudaMemcpyAsync((void*)(psi + pb), psi_ + 2 * pb, (nel - pb) * sizeof(double2),
                                        cudaMemcpyHostToDevice, c->copy));
            CUDA_TRY(c, cudaEventRecord(c->ev_psi_in[1], c->copy));
            CUDA_TRY(c, cudaMemcpy2DAsync(hpsi, pitch, hpsi_, pitch, (size_t)mid * sizeof(double2), nb,
                                          cudaMemcpyHostToDevice, c->copy));
            CUDA_TRY(c, cudaEventRecord(c->ev_half_in[0], c->copy));
            CUDA_TRY(c, cudaMemcpy2DAsync(hpsi + mid, pitch, hpsi_ + 2 * (size_t)mid, pitch,
                                          (size_t)(s->npw - mid) * sizeof(double2), nb, cudaMemcpyHostToDevice,
                                          c->copy));
            CUDA_TRY(c, cudaEventRecord(c->ev_half_in[1], c->copy));
        } else {
            CUDA_TRY(c, cudaMemcpyAsync((void*)psi, psi_, nel * sizeof(double2), cudaMemcpyHostToDevice, st));
            if (fork && is_tc(prec) && s->P > 0) {
                // hpsi is read only by the expansion at the end: copy it on the
                // copy stream, after the work already queued on st (which may
                // still use the staging area), beside the FFT passes
                CUDA_TRY(c, cudaEventRecord(c->ev_copy_after, st));
                CUDA_TRY(c, cudaStreamWaitEvent(c->copy, c->ev_copy_after, 0));
                CUDA_TRY(c, cudaMemcpyAsync(hpsi, hpsi_, nel * sizeof(double2), cudaMemcpyHostToDevice, c->copy));
                CUDA_TRY(c, cudaEventRecord(c->ev_copy_done, c->copy));
                hpsi_ready = c->ev_copy_done;
            } else {
                CUDA_TRY(c, cudaMemcpyAsync(hpsi, hpsi_, nel * sizeof(double2), cudaMemcpyHostToDevice, st));
            }
        }
    }
    rc = apply_dev(c, *s, nb, psi, hpsi, prec, c->ws + o_work, st, nullptr, nullptr, fork, hpsi_ready,
                   halves ? &hh : nullptr);
    if (rc) {
        // leave no copy unordered behind st
        if (hpsi_ready) cudaStreamWaitEvent(st, hpsi_ready, 0);
        if (halves) {
            cudaStreamWaitEvent(st, c->ev_half_in[1], 0);  // the last upload on the copy stream
            cudaStreamSynchronize(c->side);
        }
        return rc;
    }
    if (halves) {
        // the second half; the first one is on its way on the side stream
        CUDA_TRY(c, cudaMemcpy2DAsync(hpsi_ + 2 * (size_t)mid, pitch, hpsi + mid, pitch,
                                      (size_t)(s->npw - mid) * sizeof(double2), nb, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(c, cudaStreamWaitEvent(st, c->ev_half_out, 0));
    } else if (!dev) {
        CUDA_TRY(c, cudaMemcpyAsync(hpsi_, hpsi, nel * sizeof(double2), cudaMemcpyDeviceToHost, st));
    }
    if (!dev || (flags & HPSI_SYNC)) {
        CUDA_TRY(c, cudaStreamSynchronize(st));
        if (is_tc(prec) && (rc = check_device_flag(c))) return rc;
    }
    return HPSI_OK;
}

extern "C" int hpsi_apply_energies(hpsi_ctx* c, int kid, int nb, const double* psi_, double* hpsi_, double* eout,
                                   int flags, void* stream)
{
    KSlot* s = nullptr;
    int rc = check_call(c, kid, nb, &s, flags);
    if (rc) return rc;
    if (nb > 0 && (!psi_ || !hpsi_ || !eout)) return fail(c, HPSI_ERR_BAD_ARG, "psi/hpsi/e NULL");
    if (nb == 0) return HPSI_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int prec = flags & HPSI_PREC_MASK;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    if (s->npw == 0) {
        if (dev) CUDA_TRY(c, cudaMemsetAsync(eout, 0, nb * sizeof(double), st));
        else memset(eout, 0, nb * sizeof(double));
        return HPSI_OK;
    }
    const size_t nel = (size_t)nb * s->npw;
    Carver cv;
    size_t o_psi = dev ? 0 : cv.take<double2>(nel);
    size_t o_hpsi = dev ? 0 : cv.take<double2>(nel);
    size_t o_e = dev ? 0 : cv.take<double>((size_t)nb);
    size_t o_work = cv.off;
    const EnergyWs w = energy_layout(c, nb, prec);
    if ((rc = ws_reserve(c, o_work + w.work + apply_ws_bytes(c, *s, nb, prec, true)))) return rc;
    const double2* psi = (const double2*)psi_;
    double2* hpsi = (double2*)hpsi_;
    double* e = eout;
    if (!dev) {
        psi = reinterpret_cast<const double2*>(c->ws + o_psi);
        hpsi = reinterpret_cast<double2*>(c->ws + o_hpsi);
        e = reinterpret_cast<double*>(c->ws + o_e);
        CUDA_TRY(c, cudaMemcpyAsync((void*)psi, psi_, nel * sizeof(double2), cudaMemcpyHostToDevice, st));
        CUDA_TRY(c, cudaMemcpyAsync(hpsi, hpsi_, nel * sizeof(double2), cudaMemcpyHostToDevice, st));
    }
    if ((rc = energies_dev(c, *s, nb, psi, hpsi, e, prec, c->ws + o_work, st, !(flags & HPSI_ONE_STREAM))))
        return rc;
    if (!dev) {
        CUDA_TRY(c, cudaMemcpyAsync(hpsi_, hpsi, nel * sizeof(double2), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(c, cudaMemcpyAsync(eout, e, nb * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    if (!dev || (flags & HPSI_SYNC)) {
        CUDA_TRY(c, cudaStreamSynchronize(st));
        if (is_tc(prec) && (rc = check_device_flag(c))) return rc;
    }
    return HPSI_OK;
}

// ---------------------------------------------------------------- Sternheimer
// v <- P_c v = v - psi (psi^H v) for nb vectors against the nv occupied bands
// psi (FP64 SIMT GEMMs: the nv x nb overlap, split over G, then the update).
struct ProjWs {
    double2* part;   // [ns][nv][nb]
    double2* W;      // [nv][nb]
    double* minus;   // nv x (-1)
    int ns;
};

static int project_out(hpsi_ctx* c, KSlot& s, int nv, const double2* psi, int nb, double2* v, const ProjWs& w,
                       cudaStream_t st)
{
    CUDA_TRY(c, (launch_proj_gemm<double2, double2, double2>(nv, nb, s.npw, psi, (size_t)s.npw, v, (size_t)s.npw, w.part,
                                                             w.ns, st)));
    CUDA_TRY(c, (launch_reduce_splits<double2, double2>(nv, nb, w.ns, w.part, w.minus, nv, w.W, (size_t)nb, st)));
    CUDA_TRY(c, launch_expand_gemm<double2>(nv, nb, s.npw, w.W, (size_t)nb, psi, (size_t)s.npw, v, (size_t)s.npw, st));
    return HPSI_OK;
}

extern "C" int hpsi_sternheimer(hpsi_ctx* c, int kid, int nv, const double* psi_, const double* eps_, int direction,
                                double tol, int max_iter, double* x_, int* iterations, double* residual, int flags,
                                void* stream)
{
    KSlot* s = nullptr;
    int rc = check_call(c, kid, nv, &s, flags);
    if (rc) return rc;
    if (direction < 0 || direction > 2) return fail(c, HPSI_ERR_BAD_ARG, "direction must be 0, 1 or 2");
    if (!(tol > 0.0) || max_iter < 1) return fail(c, HPSI_ERR_BAD_ARG, "need tol > 0 and max_iter >= 1");
    if (nv > 0 && (!psi_ || !eps_ || !x_)) return fail(c, HPSI_ERR_BAD_ARG, "psi/eps/x NULL");
    if (nv == 0 || s->npw == 0) return HPSI_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int prec = flags & HPSI_PREC_MASK;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    const int npw = s->npw;
    const size_t nel = (size_t)nv * npw;
    const int ns = split_for(nv, nv, npw);
    // workspace: inputs (host case), x, r, z, p, q, projection and scalars, then H / gradient workspace
    Carver cv;
    const size_t o_psi = dev ? 0 : cv.take<double2>(nel);
    const size_t o_eps = dev ? 0 : cv.take<double>((size_t)nv);
    const size_t o_x = dev ? 0 : cv.take<double2>(nel);
    const size_t o_r = cv.take<double2>(nel), o_z = cv.take<double2>(nel), o_p = cv.take<double2>(nel);
    const size_t o_q = cv.take<double2>(nel);
    const size_t o_part = cv.take<double2>((size_t)ns * nv * nv), o_W = cv.take<double2>((size_t)nv * nv);
    const size_t o_min = cv.take<double>((size_t)nv);
    const size_t o_sc = cv.take<double>((size_t)8 * nv);
    const size_t o_act = cv.take<int>((size_t)nv);
    const size_t o_work = cv.off;
    const size_t work = std::max(apply_ws_bytes(c, *s, nv, prec), grad_ws_bytes(*s, nv, prec));
    if ((rc = ws_reserve(c, o_work + work))) return rc;
    unsigned char* ws = c->ws;
    const double2* psi = dev ? (const double2*)psi_ : reinterpret_cast<const double2*>(ws + o_psi);
    const double* eps = dev ? eps_ : reinterpret_cast<const double*>(ws + o_eps);
    double2* x = dev ? (double2*)x_ : reinterpret_cast<double2*>(ws + o_x);
    double2 *r = reinterpret_cast<double2*>(ws + o_r), *z = reinterpret_cast<double2*>(ws + o_z);
    double2 *p = reinterpret_cast<double2*>(ws + o_p), *q = reinterpret_cast<double2*>(ws + o_q);
    double* sc = reinterpret_cast<double*>(ws + o_sc);
    double *rz = sc, *rz_new = sc + nv, *pq = sc + 2 * nv, *alpha = sc + 3 * nv, *beta = sc + 4 * nv;
    double *rr = sc + 5 * nv, *bb = sc + 6 * nv;
    int* active = reinterpret_cast<int*>(ws + o_act);
    ProjWs pw{reinterpret_cast<double2*>(ws + o_part), reinterpret_cast<double2*>(ws + o_W),
              reinterpret_cast<double*>(ws + o_min), ns};
    unsigned char* wk = ws + o_work;
    if (!dev) {
        CUDA_TRY(c, cudaMemcpyAsync((void*)psi, psi_, nel * sizeof(double2), cudaMemcpyHostToDevice, st));
        CUDA_TRY(c, cudaMemcpyAsync((void*)eps, eps_, nv * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    {
        std::vector<double> m1(nv, -1.0);
        std::vector<int> one(nv, 1);
        CUDA_TRY(c, cudaMemcpyAsync(pw.minus, m1.data(), nv * sizeof(double), cudaMemcpyHostToDevice, st));
        CUDA_TRY(c, cudaMemcpyAsync(active, one.data(), nv * sizeof(int), cudaMemcpyHostToDevice, st));
        CUDA_TRY(c, cudaStreamSynchronize(st));  // the host vectors go out of scope
    }
    // b = -P_c dH/dk_a psi  (in r), x = 0
    CUDA_TRY(c, cudaMemsetAsync(q, 0, nel * sizeof(double2), st));
    double2* d3[3] = {nullptr, nullptr, nullptr};
    d3[direction] = q;
    if ((rc = grad_dev(c, *s, nv, psi, d3, prec, wk, st))) return rc;
    if ((rc = project_out(c, *s, nv, psi, nv, q, pw, st))) return rc;
    CUDA_TRY(c, cudaMemsetAsync(r, 0, nel * sizeof(double2), st));
    CUDA_TRY(c, launch_baxpy(npw, nv, nullptr, -1.0, q, r, st));
    CUDA_TRY(c, cudaMemsetAsync(x, 0, nel * sizeof(double2), st));
    CUDA_TRY(c, launch_bdot(npw, nv, r, r, bb, st));
    // z = P_c M^-1 r, p = z, rz = <r, z>
    const double tau = 1.0;  // Ha: keeps the diagonal preconditioner positive
    CUDA_TRY(c, launch_bprec(npw, nv, s->d_kin, eps, tau, r, z, st));
    if ((rc = project_out(c, *s, nv, psi, nv, z, pw, st))) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(p, z, nel * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    CUDA_TRY(c, launch_bdot(npw, nv, r, z, rz, st));
    std::vector<double> hb(nv), hr(nv);
    std::vector<int> hact(nv, 1);
    CUDA_TRY(c, cudaMemcpyAsync(hb.data(), bb, nv * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaStreamSynchronize(st));
    int it = 0, n_active = 0;
    for (int b = 0; b < nv; ++b) {
        hact[b] = hb[b] > 0.0;
        n_active += hact[b];
    }
    CUDA_TRY(c, cudaMemcpyAsync(active, hact.data(), nv * sizeof(int), cudaMemcpyHostToDevice, st));
    for (; it < max_iter && n_active > 0; ++it) {
        // q = A p = P_c (H p - e p)
        CUDA_TRY(c, cudaMemsetAsync(q, 0, nel * sizeof(double2), st));
        if ((rc = apply_dev(c, *s, nv, p, q, prec, wk, st))) return rc;
        CUDA_TRY(c, launch_bscale_add(npw, nv, eps, -1.0, p, q, st));
        if ((rc = project_out(c, *s, nv, psi, nv, q, pw, st))) return rc;
        // alpha = rz / <p, q>;  x += alpha p;  r -= alpha q
        CUDA_TRY(c, launch_bdot(npw, nv, p, q, pq, st));
        CUDA_TRY(c, launch_bratio(nv, rz, pq, active, alpha, st));
        CUDA_TRY(c, launch_baxpy(npw, nv, alpha, 1.0, p, x, st));
        CUDA_TRY(c, launch_baxpy(npw, nv, alpha, -1.0, q, r, st));
        // convergence: |r| <= tol |b| per band
        CUDA_TRY(c, launch_bdot(npw, nv, r, r, rr, st));
        CUDA_TRY(c, cudaMemcpyAsync(hr.data(), rr, nv * sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(c, cudaStreamSynchronize(st));
        n_active = 0;
        for (int b = 0; b < nv; ++b) {
            if (hact[b] && hr[b] <= tol * tol * hb[b]) hact[b] = 0;
            n_active += hact[b];
        }
        CUDA_TRY(c, cudaMemcpyAsync(active, hact.data(), nv * sizeof(int), cudaMemcpyHostToDevice, st));
        if (n_active == 0) { ++it; break; }
        // z = P_c M^-1 r;  beta = <r, z>_new / <r, z>;  p = z + beta p
        CUDA_TRY(c, launch_bprec(npw, nv, s->d_kin, eps, tau, r, z, st));
        if ((rc = project_out(c, *s, nv, psi, nv, z, pw, st))) return rc;
        CUDA_TRY(c, launch_bdot(npw, nv, r, z, rz_new, st));
        CUDA_TRY(c, launch_bratio(nv, rz_new, rz, active, beta, st));
        CUDA_TRY(c, launch_baxpby(npw, nv, nullptr, 1.0, z, beta, p, st));
        CUDA_TRY(c, cudaMemcpyAsync(rz, rz_new, nv * sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    if (iterations) *iterations = it;
    if (residual)
        for (int b = 0; b < nv; ++b) residual[b] = hb[b] > 0.0 ? std::sqrt(hr[b] / hb[b]) : 0.0;
    if (!dev) CUDA_TRY(c, cudaMemcpyAsync(x_, x, nel * sizeof(double2), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(c, cudaStreamSynchronize(st));
    if (is_tc(prec) && (rc = check_device_flag(c))) return rc;
    if (n_active > 0)
        return fail(c, HPSI_ERR_TIMEOUT, "Sternheimer CG: %d of %d bands above tol after %d iterations", n_active, nv,
                    it);
    return HPSI_OK;
}

extern "C" int hpsi_beta_table_length(double dq, double q_max)
{
    if (!(dq > 0.0) || !(q_max >= 0.0)) return fail(nullptr, HPSI_ERR_BAD_ARG, "need dq > 0 and q_max >= 0");
    return beta_table_nq(dq, q_max);
}

extern "C" int hpsi_beta_tables(int nr, const double* r_, const double* rab_, int uniform_mesh, int n_proj,
                                const int* l_, const double* beta_, double dq, double q_max, double* beta_q,
                                double* dbeta_q, int flags, void* stream)
{
    if (nr < 0 || n_proj < 0) return fail(nullptr, HPSI_ERR_BAD_ARG, "nr and n_proj must be >= 0");
    if (!(dq > 0.0) || !(q_max >= 0.0)) return fail(nullptr, HPSI_ERR_BAD_ARG, "need dq > 0 and q_max >= 0");
    if (n_proj == 0) return HPSI_OK;
    if (!r_ || !rab_ || !l_ || !beta_ || !beta_q || nr == 0)
        return fail(nullptr, HPSI_ERR_BAD_ARG, "r/rab/l/beta/beta_q NULL or nr == 0");
    const int nq = beta_table_nq(dq, q_max);
    cudaStream_t st = (cudaStream_t)stream;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    const size_t tb = (size_t)n_proj * nq * sizeof(double);
    Carver cv;
    const size_t o_r = dev ? 0 : cv.take<double>((size_t)nr), o_rab = dev ? 0 : cv.take<double>((size_t)nr);
    const size_t o_l = dev ? 0 : cv.take<int>((size_t)n_proj);
    const size_t o_b = dev ? 0 : cv.take<double>((size_t)n_proj * nr);
    const size_t o_bq = dev ? 0 : cv.take<double>((size_t)n_proj * nq);
    const size_t o_dq = (dev || !dbeta_q) ? 0 : cv.take<double>((size_t)n_proj * nq);
    const size_t o_nm = cv.take<int>((size_t)n_proj);
    unsigned char* buf = nullptr;
    cudaError_t e;
#define TB_TRY(expr)                                                                                           \
    do {                                                                                                        \
        if ((e = (expr)) != cudaSuccess) {                                                                      \
            if (buf) cudaFree(buf);                                                                             \
            return fail(nullptr, e == cudaErrorMemoryAllocation ? HPSI_ERR_OOM : HPSI_ERR_CUDA, "%s: %s", #expr, \
                        cudaGetErrorString(e));                                                                 \
        }                                                                                                       \
    } while (0)
    TB_TRY(cudaMalloc(&buf, cv.off));
    const double* r = dev ? r_ : reinterpret_cast<const double*>(buf + o_r);
    const double* rab = dev ? rab_ : reinterpret_cast<const double*>(buf + o_rab);
    const int* l = dev ? l_ : reinterpret_cast<const int*>(buf + o_l);
    const double* beta = dev ? beta_ : reinterpret_cast<const double*>(buf + o_b);
    double* bq = dev ? beta_q : reinterpret_cast<double*>(buf + o_bq);
    double* dbq = dev ? dbeta_q : (dbeta_q ? reinterpret_cast<double*>(buf + o_dq) : nullptr);
    int* nmax = reinterpret_cast<int*>(buf + o_nm);
    if (!dev) {
        TB_TRY(cudaMemcpyAsync((void*)r, r_, nr * sizeof(double), cudaMemcpyHostToDevice, st));
        TB_TRY(cudaMemcpyAsync((void*)rab, rab_, nr * sizeof(double), cudaMemcpyHostToDevice, st));
        TB_TRY(cudaMemcpyAsync((void*)l, l_, n_proj * sizeof(int), cudaMemcpyHostToDevice, st));
        TB_TRY(cudaMemcpyAsync((void*)beta, beta_, (size_t)n_proj * nr * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    TB_TRY(launch_trim(nr, n_proj, beta, nmax, st));
    TB_TRY(launch_beta_tables(nr, r, rab, uniform_mesh, n_proj, l, nmax, beta, dq, nq, bq, dbq, st));
    if (!dev) {
        TB_TRY(cudaMemcpyAsync(beta_q, bq, tb, cudaMemcpyDeviceToHost, st));
        if (dbeta_q) TB_TRY(cudaMemcpyAsync(dbeta_q, dbq, tb, cudaMemcpyDeviceToHost, st));
    }
    TB_TRY(cudaStreamSynchronize(st));
    cudaFree(buf);
#undef TB_TRY
    return HPSI_OK;
}

extern "C" int hpsi_gsphere(const double* lattice, const double* k_frac, double ecut, int max_npw, int* g_idx,
                            double* kvec, double* kinetic, int* npw_out, int flags, void* stream)
{
    if (!lattice || !k_frac || !npw_out) return fail(nullptr, HPSI_ERR_BAD_ARG, "lattice/k_frac/npw_out NULL");
    if (!(ecut > 0.0)) return fail(nullptr, HPSI_ERR_BAD_ARG, "ecut must be > 0");
    // B = 2 pi A^-T (rows = reciprocal vectors), by the adjugate
    const double* A = lattice;
    const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                       A[2] * (A[3] * A[7] - A[4] * A[6]);
    if (!(std::fabs(det) > 0.0)) return fail(nullptr, HPSI_ERR_BAD_ARG, "singular lattice");
    const double tp = 2.0 * 3.14159265358979323846 / det;
    double B[9];
    B[0] = tp * (A[4] * A[8] - A[5] * A[7]); B[1] = tp * (A[5] * A[6] - A[3] * A[8]); B[2] = tp * (A[3] * A[7] - A[4] * A[6]);
    B[3] = tp * (A[2] * A[7] - A[1] * A[8]); B[4] = tp * (A[0] * A[8] - A[2] * A[6]); B[5] = tp * (A[1] * A[6] - A[0] * A[7]);
    B[6] = tp * (A[1] * A[5] - A[2] * A[4]); B[7] = tp * (A[2] * A[3] - A[0] * A[5]); B[8] = tp * (A[0] * A[4] - A[1] * A[3]);
    // box half-width: sqrt(2 ecut) over the shortest reciprocal vector, twice, plus margin
    double bmin = 1e300;
    for (int d = 0; d < 3; ++d)
        bmin = std::min(bmin, std::sqrt(B[3 * d] * B[3 * d] + B[3 * d + 1] * B[3 * d + 1] + B[3 * d + 2] * B[3 * d + 2]));
    const int gmax = (int)std::ceil(std::sqrt(2.0 * ecut) / bmin * 2.0) + 2;
    if (gmax > 512) return fail(nullptr, HPSI_ERR_BAD_ARG, "ecut too large for the G box (gmax %d)", gmax);
    const int L = 2 * gmax + 1;
    cudaStream_t st = (cudaStream_t)stream;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    int* cnt = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&cnt, 2 * L * sizeof(int))))
        return fail(nullptr, HPSI_ERR_OOM, "cudaMalloc: %s", cudaGetErrorString(e));
    std::vector<int> h(L), off(L);
    auto done = [&](int code) { cudaFree(cnt); return code; };
    if ((e = launch_gs_count(B, k_frac, ecut, gmax, cnt, st)) ||
        (e = cudaMemcpyAsync(h.data(), cnt, L * sizeof(int), cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st)))
        return done(fail(nullptr, HPSI_ERR_CUDA, "G-sphere count: %s", cudaGetErrorString(e)));
    long npw = 0;
    for (int i = 0; i < L; ++i) { off[i] = (int)npw; npw += h[i]; }
    *npw_out = (int)npw;
    if (!g_idx || !kvec || !kinetic) return done(HPSI_OK);  // size query
    if (npw > max_npw) return done(fail(nullptr, HPSI_ERR_RANGE, "G-sphere holds %ld vectors, room for %d", npw, max_npw));
    int *dg = g_idx;
    double *dk = kvec, *dkin = kinetic;
    unsigned char* buf = nullptr;
    if (!dev) {
        if ((e = cudaMalloc(&buf, (size_t)npw * (3 * sizeof(int) + 4 * sizeof(double)) + 64)))
            return done(fail(nullptr, HPSI_ERR_OOM, "cudaMalloc: %s", cudaGetErrorString(e)));
        dk = reinterpret_cast<double*>(buf);
        dkin = dk + 3 * npw;
        dg = reinterpret_cast<int*>(dkin + npw);
    }
    if ((e = cudaMemcpyAsync(cnt + L, off.data(), L * sizeof(int), cudaMemcpyHostToDevice, st)) ||
        (e = launch_gs_write(B, k_frac, ecut, gmax, cnt + L, dg, dk, dkin, st)))
        goto cuda_fail;
    if (!dev) {
        if ((e = cudaMemcpyAsync(g_idx, dg, npw * 3 * sizeof(int), cudaMemcpyDeviceToHost, st)) ||
            (e = cudaMemcpyAsync(kvec, dk, npw * 3 * sizeof(double), cudaMemcpyDeviceToHost, st)) ||
            (e = cudaMemcpyAsync(kinetic, dkin, npw * sizeof(double), cudaMemcpyDeviceToHost, st)))
            goto cuda_fail;
    }
    if ((e = cudaStreamSynchronize(st))) goto cuda_fail;
    if (buf) cudaFree(buf);
    return done(HPSI_OK);
cuda_fail:
    if (buf) cudaFree(buf);
    return done(fail(nullptr, HPSI_ERR_CUDA, "G-sphere write: %s", cudaGetErrorString(e)));
}

// ------------------------------------------------------------------- Hessian
extern "C" int hpsi_hessian_tables(int nr, const double* r_, const double* rab_, int uniform_mesh, int n_proj,
                                   const int* l_, const double* beta_, double dq, double q_max, double* f_out,
                                   int flags, void* stream)
{
    if (nr <= 0 || n_proj < 0) return fail(nullptr, HPSI_ERR_BAD_ARG, "need nr > 0 and n_proj >= 0");
    if (!(dq > 0.0) || !(q_max >= 0.0)) return fail(nullptr, HPSI_ERR_BAD_ARG, "need dq > 0 and q_max >= 0");
    if (n_proj == 0) return HPSI_OK;
    if (!r_ || !rab_ || !l_ || !beta_ || !f_out) return fail(nullptr, HPSI_ERR_BAD_ARG, "NULL argument");
    for (int p = 0; p < n_proj && !(flags & HPSI_DEVICE_PTRS); ++p)
        if (l_[p] < 0 || l_[p] > HPSI_LMAX) return fail(nullptr, HPSI_ERR_BAD_ARG, "l outside [0, %d]", HPSI_LMAX);
    const int nq = beta_table_nq(dq, q_max);
    cudaStream_t st = (cudaStream_t)stream;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    Carver cv;
    const size_t o_r = dev ? 0 : cv.take<double>((size_t)nr), o_rab = dev ? 0 : cv.take<double>((size_t)nr);
    const size_t o_l = dev ? 0 : cv.take<int>((size_t)n_proj);
    const size_t o_b = dev ? 0 : cv.take<double>((size_t)n_proj * nr);
    const size_t o_f = dev ? 0 : cv.take<double>((size_t)3 * n_proj * nq);
    const size_t o_nm = cv.take<int>((size_t)n_proj);
    unsigned char* buf = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&buf, cv.off))) return fail(nullptr, HPSI_ERR_OOM, "cudaMalloc: %s", cudaGetErrorString(e));
    const double* r = dev ? r_ : reinterpret_cast<const double*>(buf + o_r);
    const double* rab = dev ? rab_ : reinterpret_cast<const double*>(buf + o_rab);
    const int* l = dev ? l_ : reinterpret_cast<const int*>(buf + o_l);
    const double* beta = dev ? beta_ : reinterpret_cast<const double*>(buf + o_b);
    double* f = dev ? f_out : reinterpret_cast<double*>(buf + o_f);
    int* nmax = reinterpret_cast<int*>(buf + o_nm);
    if (!dev) {
        if ((e = cudaMemcpyAsync((void*)r, r_, nr * sizeof(double), cudaMemcpyHostToDevice, st)) ||
            (e = cudaMemcpyAsync((void*)rab, rab_, nr * sizeof(double), cudaMemcpyHostToDevice, st)) ||
            (e = cudaMemcpyAsync((void*)l, l_, n_proj * sizeof(int), cudaMemcpyHostToDevice, st)) ||
            (e = cudaMemcpyAsync((void*)beta, beta_, (size_t)n_proj * nr * sizeof(double), cudaMemcpyHostToDevice, st)))
            goto fail_cuda;
    }
    if ((e = launch_trim(nr, n_proj, beta, nmax, st)) ||
        (e = launch_hess_tables(nr, r, rab, uniform_mesh, n_proj, l, nmax, beta, dq, nq, f, st)))
        goto fail_cuda;
    if (!dev && (e = cudaMemcpyAsync(f_out, f, (size_t)3 * n_proj * nq * sizeof(double), cudaMemcpyDeviceToHost, st)))
        goto fail_cuda;
    if ((e = cudaStreamSynchronize(st))) goto fail_cuda;
    cudaFree(buf);
    return HPSI_OK;
fail_cuda:
    cudaFree(buf);
    return fail(nullptr, HPSI_ERR_CUDA, "Hessian tables: %s", cudaGetErrorString(e));
}

extern "C" int hpsi_set_hessian_tables(hpsi_ctx* c, int species, int nq, double dq, const double* f)
{
    if (!c) return HPSI_ERR_BAD_ARG;
    const int nsp = (int)c->rad_off.size();
    if (species < 0 || species >= nsp) return fail(c, HPSI_ERR_BAD_ARG, "species %d outside [0, %d)", species, nsp);
    if (nq < 4 || !(dq > 0.0) || !f) return fail(c, HPSI_ERR_BAD_ARG, "need nq >= 4, dq > 0 and tables");
    if (c->d_hess && (nq != c->hess_nq || dq != c->hess_dq))
        return fail(c, HPSI_ERR_BAD_ARG, "all species need the same table grid (nq %d, dq %g)", c->hess_nq, c->hess_dq);
    CUDA_TRY(c, cudaSetDevice(c->dev));
    if (!c->d_hess) {
        CUDA_TRY(c, dalloc(&c->d_hess, (size_t)std::max(c->nrad, 1) * 3 * nq));
        CUDA_TRY(c, cudaMemset(c->d_hess, 0, (size_t)std::max(c->nrad, 1) * 3 * nq * sizeof(double)));
        c->hess_nq = nq;
        c->hess_dq = dq;
        c->hess_set.assign(c->nrad, 0);
    }
    const int r0 = c->rad_off[species];
    const int r1 = species + 1 < nsp ? c->rad_off[species + 1] : c->nrad;
    const int np = r1 - r0;
    // input [3][np][nq] -> stored [rad][3][nq]
    std::vector<double> rows((size_t)np * 3 * nq);
    for (int p = 0; p < np; ++p)
        for (int t = 0; t < 3; ++t)
            std::memcpy(&rows[((size_t)p * 3 + t) * nq], f + ((size_t)t * np + p) * nq, nq * sizeof(double));
    CUDA_TRY(c, cudaMemcpy(c->d_hess + (size_t)r0 * 3 * nq, rows.data(), rows.size() * sizeof(double),
                           cudaMemcpyHostToDevice));
    for (int r = r0; r < r1; ++r) c->hess_set[r] = 1;
    // slots bound before: their second-derivative rows are rebuilt on next use
    for (auto& kv : c->slots) { dfree(kv.second.hess64); dfree(kv.second.hess32); }
    return HPSI_OK;
}

template <typename C>
static int ensure_hess(hpsi_ctx* c, KSlot& s, cudaStream_t st)
{
    C*& d2 = slot_hess<C>(s);
    if (d2 || s.P == 0 || s.npw == 0) return HPSI_OK;
    for (int r = 0; r < c->nrad; ++r)
        if (std::fabs(c->rad_lam[r]) >= 1e-15 && (c->hess_set.empty() || !c->hess_set[r]))
            return fail(c, HPSI_ERR_STATE, "Hessian tables missing for radial function %d (hpsi_set_hessian_tables)", r);
    // q range of the tables
    const double qtop = c->hess_dq * (c->hess_nq - 3);
    std::vector<double> q(s.npw);
    CUDA_TRY(c, cudaMemcpy(q.data(), s.d_q, s.npw * sizeof(double), cudaMemcpyDeviceToHost));
    for (double v : q)
        if (v > qtop) return fail(c, HPSI_ERR_RANGE, "q=%.17g beyond the Hessian tables (%.17g)", v, qtop);
    CUDA_TRY(c, dalloc(&d2, (size_t)6 * s.P * s.npw));
    CUDA_TRY(c, launch_hess_assemble<C>(s.P, s.npw, s.d_rows, c->d_hess, c->hess_nq, c->hess_dq,
                                        1.0 / std::sqrt(c->omega), s.d_kvec, s.d_sf, d2, st));
    return HPSI_OK;
}

// out_c += d2H/dk_a dk_b psi for the requested components c (device pointers)
template <typename C, typename Acc>
static int hess_device(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* out[6], unsigned char* ws,
                       const C* pr, const C* d2, cudaStream_t st)
{
    static const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
    const size_t nel = (size_t)nb * s.npw;
    for (int k = 0; k < 6; ++k)
        if (out[k] && pa[k] == pb[k]) CUDA_TRY(c, launch_add(nel, psi, out[k], st));  // kinetic: delta_ab
    if (s.P == 0 || nb == 0) return HPSI_OK;
    const int P = s.P, ns = split_for(6 * P, nb, s.npw), ns4 = split_for(4 * P, nb, s.npw);
    Carver cv;
    Acc* part = reinterpret_cast<Acc*>(ws + cv.take<Acc>(std::max((size_t)ns * 6, (size_t)ns4 * 4) * P * nb));
    C* W4 = reinterpret_cast<C*>(ws + cv.take<C>((size_t)4 * P * nb));   // lambda <p|psi>, lambda <d_a p|psi>
    C* W6 = reinterpret_cast<C*>(ws + cv.take<C>((size_t)6 * P * nb));   // lambda <d_ab p|psi>
    CUDA_TRY(c, (launch_proj_gemm<C, double2, Acc>(4 * P, nb, s.npw, pr, (size_t)s.npw, psi, (size_t)s.npw, part, ns4,
                                                   st)));
    CUDA_TRY(c, (launch_reduce_splits<Acc, C>(4 * P, nb, ns4, part, s.d_lam, P, W4, (size_t)nb, st)));
    CUDA_TRY(c, (launch_proj_gemm<C, double2, Acc>(6 * P, nb, s.npw, d2, (size_t)s.npw, psi, (size_t)s.npw, part, ns,
                                                   st)));
    CUDA_TRY(c, (launch_reduce_splits<Acc, C>(6 * P, nb, ns, part, s.d_lam, P, W6, (size_t)nb, st)));
    const size_t PN = (size_t)P * s.npw, PB = (size_t)P * nb;
    for (int k = 0; k < 6; ++k) {
        if (!out[k]) continue;
        const int a = pa[k], b = pb[k];
        // |d_ab p> lambda <p|psi> + |d_a p> lambda <d_b p|psi> + |d_b p> lambda <d_a p|psi> + |p> lambda <d_ab p|psi>
        CUDA_TRY(c, launch_expand_gemm<C>(P, nb, s.npw, W4, (size_t)nb, d2 + k * PN, (size_t)s.npw, out[k],
                                          (size_t)s.npw, st));
        CUDA_TRY(c, launch_expand_gemm<C>(P, nb, s.npw, W4 + (1 + b) * PB, (size_t)nb, pr + (1 + a) * PN,
                                          (size_t)s.npw, out[k], (size_t)s.npw, st));
        CUDA_TRY(c, launch_expand_gemm<C>(P, nb, s.npw, W4 + (1 + a) * PB, (size_t)nb, pr + (1 + b) * PN,
                                          (size_t)s.npw, out[k], (size_t)s.npw, st));
        CUDA_TRY(c, launch_expand_gemm<C>(P, nb, s.npw, W6 + k * PB, (size_t)nb, pr, (size_t)s.npw, out[k],
                                          (size_t)s.npw, st));
    }
    return HPSI_OK;
}

extern "C" int hpsi_hess_apply(hpsi_ctx* c, int kid, int nb, const double* psi_, double* xx, double* yy, double* zz,
                               double* xy, double* xz, double* yz, int flags, void* stream)
{
    KSlot* s = nullptr;
    int rc = check_call(c, kid, nb, &s, flags);
    if (rc) return rc;
    double* o_[6] = {xx, yy, zz, xy, xz, yz};
    if (nb > 0 && !psi_) return fail(c, HPSI_ERR_BAD_ARG, "psi NULL");
    if (nb == 0 || s->npw == 0) return HPSI_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int prec = flags & HPSI_PREC_MASK;
    const bool fp64 = prec == HPSI_PREC_FP64;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    const size_t nel = (size_t)nb * s->npw;
    int nout = 0;
    for (double* o : o_) nout += o != nullptr;
    if (nout == 0) return HPSI_OK;
    // projector matrices with their first-derivative rows, and the second-derivative rows
    if ((rc = prepare_slot(c, *s, fp64 ? HPSI_PREC_FP64 : HPSI_PREC_FP32, true, st))) return rc;
    if ((rc = fp64 ? ensure_hess<double2>(c, *s, st) : ensure_hess<float2>(c, *s, st))) return rc;
    Carver cv;
    const size_t o_psi = dev ? 0 : cv.take<double2>(nel);
    size_t o_out[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 6; ++k)
        if (o_[k] && !dev) o_out[k] = cv.take<double2>(nel);
    const size_t o_work = cv.off;
    const int P = s->P;
    const size_t nsp = std::max((size_t)split_for(6 * P, nb, s->npw) * 6, (size_t)split_for(4 * P, nb, s->npw) * 4);
    const size_t work = (nsp * P * nb + (size_t)10 * P * nb) * sizeof(double2) + 4096;
    if ((rc = ws_reserve(c, o_work + work))) return rc;
    const double2* psi = dev ? (const double2*)psi_ : reinterpret_cast<const double2*>(c->ws + o_psi);
    double2* out[6];
    for (int k = 0; k < 6; ++k)
        out[k] = !o_[k] ? nullptr : (dev ? (double2*)o_[k] : reinterpret_cast<double2*>(c->ws + o_out[k]));
    if (!dev) {
        CUDA_TRY(c, cudaMemcpyAsync((void*)psi, psi_, nel * sizeof(double2), cudaMemcpyHostToDevice, st));
        for (int k = 0; k < 6; ++k)
            if (out[k]) CUDA_TRY(c, cudaMemcpyAsync(out[k], o_[k], nel * sizeof(double2), cudaMemcpyHostToDevice, st));
    }
    rc = fp64 ? hess_device<double2, double2>(c, *s, nb, psi, out, c->ws + o_work, s->pr64, s->hess64, st)
              : hess_device<float2, float2>(c, *s, nb, psi, out, c->ws + o_work, s->pr32, s->hess32, st);
    if (rc) return rc;
    if (!dev)
        for (int k = 0; k < 6; ++k)
            if (out[k]) CUDA_TRY(c, cudaMemcpyAsync(o_[k], out[k], nel * sizeof(double2), cudaMemcpyDeviceToHost, st));
    if (!dev || (flags & HPSI_SYNC)) CUDA_TRY(c, cudaStreamSynchronize(st));
    return HPSI_OK;
}

extern "C" int hpsi_density(hpsi_ctx* c, int kid, int nb, const double* psi_, const double* occ_, double* rho_,
                            int flags, void* stream)
{
    KSlot* s = nullptr;
    int rc = check_call(c, kid, nb, &s, flags);
    if (rc) return rc;
    if (nb > 0 && (!psi_ || !occ_ || !rho_)) return fail(c, HPSI_ERR_BAD_ARG, "psi/occ/rho NULL");
    if (nb == 0 || s->npw == 0) return HPSI_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int prec = flags & HPSI_PREC_MASK;
    const bool fp64 = prec == HPSI_PREC_FP64;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    const size_t nel = (size_t)nb * s->npw, N = (size_t)c->n1 * c->n2 * c->n3;
    Carver cv;
    const size_t o_psi = dev ? 0 : cv.take<double2>(nel);
    const size_t o_occ = dev ? 0 : cv.take<double>((size_t)nb);
    const size_t o_rho = dev ? 0 : cv.take<double>(N);
    const size_t o_work = cv.off;
    const size_t csz = fp64 ? sizeof(double2) : sizeof(float2);
    LocalArgs la{};
    la.n1 = c->n1; la.n2 = c->n2; la.n3 = c->n3;
    la.Lx = c->L[0]; la.Ly = c->L[1]; la.Lz = c->L[2];
    const size_t part = density_part_bytes(la, chunk_bands(*s, c, nb, csz), csz);
    if ((rc = ws_reserve(c, o_work + (local_ws(c, *s, nb, csz) + 255) / 256 * 256 + part))) return rc;
    const double2* psi = (const double2*)psi_;
    const double* occ = occ_;
    double* rho = rho_;
    if (!dev) {
        psi = reinterpret_cast<const double2*>(c->ws + o_psi);
        occ = reinterpret_cast<const double*>(c->ws + o_occ);
        rho = reinterpret_cast<double*>(c->ws + o_rho);
        CUDA_TRY(c, cudaMemcpyAsync((void*)psi, psi_, nel * sizeof(double2), cudaMemcpyHostToDevice, st));
        CUDA_TRY(c, cudaMemcpyAsync((void*)occ, occ_, nb * sizeof(double), cudaMemcpyHostToDevice, st));
        CUDA_TRY(c, cudaMemcpyAsync(rho, rho_, N * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    rc = fp64 ? density_apply<double2>(c, *s, nb, psi, occ, rho, c->ws + o_work, c->d_tw64, st)
              : density_apply<float2>(c, *s, nb, psi, occ, rho, c->ws + o_work, c->d_tw32, st);
    if (rc) return rc;
    if (!dev) CUDA_TRY(c, cudaMemcpyAsync(rho_, rho, N * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (!dev || (flags & HPSI_SYNC)) CUDA_TRY(c, cudaStreamSynchronize(st));
    return HPSI_OK;
}

extern "C" int hpsi_kp_sums(int nb, int n_low, const double* m_, const double* e_in, double deg_tol, double* s_out,
                            int* n_skipped, int flags, void* stream)
{
    if (nb < 0 || n_low < 0 || n_low > nb) return fail(nullptr, HPSI_ERR_BAD_ARG, "need 0 <= n_low <= nb");
    if (n_low == 0) return HPSI_OK;
    if (!m_ || !e_in || !s_out) return fail(nullptr, HPSI_ERR_BAD_ARG, "m/e/s NULL");
    if (!(deg_tol >= 0.0)) return fail(nullptr, HPSI_ERR_BAD_ARG, "deg_tol must be >= 0");
    cudaStream_t st = (cudaStream_t)stream;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    const size_t mb = (size_t)3 * nb * nb * sizeof(double2), eb = (size_t)nb * sizeof(double);
    const size_t sb = (size_t)n_low * 9 * sizeof(double), kb = (size_t)n_low * sizeof(int);
    const double2* M = (const double2*)m_;
    const double* E = e_in;
    double* S = s_out;
    int* K = n_skipped;
    unsigned char* buf = nullptr;
    cudaError_t e;
#define KP_TRY(expr)                                                                                          \
    do {                                                                                                       \
        if ((e = (expr)) != cudaSuccess) {                                                                     \
            if (buf) cudaFree(buf);                                                                            \
            return fail(nullptr, e == cudaErrorMemoryAllocation ? HPSI_ERR_OOM : HPSI_ERR_CUDA, "%s: %s", #expr, \
                        cudaGetErrorString(e));                                                                \
        }                                                                                                      \
    } while (0)
    if (!dev) {
        KP_TRY(cudaMalloc(&buf, mb + eb + sb + kb));
        M = reinterpret_cast<const double2*>(buf);
        E = reinterpret_cast<const double*>(buf + mb);
        S = reinterpret_cast<double*>(buf + mb + eb);
        K = reinterpret_cast<int*>(buf + mb + eb + sb);
        KP_TRY(cudaMemcpyAsync((void*)M, m_, mb, cudaMemcpyHostToDevice, st));
        KP_TRY(cudaMemcpyAsync((void*)E, e_in, eb, cudaMemcpyHostToDevice, st));
    }
    KP_TRY(launch_kp_sums(nb, n_low, M, E, deg_tol, S, K, st));
    if (!dev) {
        KP_TRY(cudaMemcpyAsync(s_out, S, sb, cudaMemcpyDeviceToHost, st));
        if (n_skipped) KP_TRY(cudaMemcpyAsync(n_skipped, K, kb, cudaMemcpyDeviceToHost, st));
        KP_TRY(cudaStreamSynchronize(st));
        cudaFree(buf);
    } else if (flags & HPSI_SYNC) {
        KP_TRY(cudaStreamSynchronize(st));
    }
#undef KP_TRY
    return HPSI_OK;
}

extern "C" int hpsi_grad_apply(hpsi_ctx* c, int kid, int nb, const double* psi_, double* dx, double* dy, double* dz,
                               int flags, void* stream)
{
    KSlot* s = nullptr;
    int rc = check_call(c, kid, nb, &s, flags);
    if (rc) return rc;
    if (nb > 0 && !psi_) return fail(c, HPSI_ERR_BAD_ARG, "psi NULL");
    if (nb == 0 || s->npw == 0 || (!dx && !dy && !dz)) return HPSI_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int prec = flags & HPSI_PREC_MASK;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    const size_t nel = (size_t)nb * s->npw;
    double* outs[3] = {dx, dy, dz};
    Carver cv;
    size_t o_psi = dev ? 0 : cv.take<double2>(nel);
    size_t o_out[3] = {0, 0, 0};
    for (int a = 0; a < 3; ++a)
        if (!dev && outs[a]) o_out[a] = cv.take<double2>(nel);
    size_t o_work = cv.off;
    if ((rc = ws_reserve(c, o_work + grad_ws_bytes(*s, nb, prec)))) return rc;
    const double2* psi = (const double2*)psi_;
    double2* d[3] = {(double2*)dx, (double2*)dy, (double2*)dz};
    if (!dev) {
        psi = reinterpret_cast<const double2*>(c->ws + o_psi);
        CUDA_TRY(c, cudaMemcpyAsync((void*)psi, psi_, nel * sizeof(double2), cudaMemcpyHostToDevice, st));
        for (int a = 0; a < 3; ++a) {
            if (!outs[a]) continue;
            d[a] = reinterpret_cast<double2*>(c->ws + o_out[a]);
            CUDA_TRY(c, cudaMemcpyAsync(d[a], outs[a], nel * sizeof(double2), cudaMemcpyHostToDevice, st));
        }
    }
    if ((rc = grad_dev(c, *s, nb, psi, d, prec, c->ws + o_work, st))) return rc;
    if (!dev)
        for (int a = 0; a < 3; ++a)
            if (outs[a]) CUDA_TRY(c, cudaMemcpyAsync(outs[a], d[a], nel * sizeof(double2), cudaMemcpyDeviceToHost, st));
    if (!dev || (flags & HPSI_SYNC)) {
        CUDA_TRY(c, cudaStreamSynchronize(st));
        if (is_tc(prec) && (rc = check_device_flag(c))) return rc;
    }
    return HPSI_OK;
}

extern "C" int hpsi_velocity_matrix(hpsi_ctx* c, int kid, int nb, const double* psi_, double* m_, int flags,
                                    void* stream)
{
    KSlot* s = nullptr;
    int rc = check_call(c, kid, nb, &s, flags);
    if (rc) return rc;
    if (nb > 0 && (!psi_ || !m_)) return fail(c, HPSI_ERR_BAD_ARG, "psi/m NULL");
    if (nb == 0) return HPSI_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int prec = flags & HPSI_PREC_MASK;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    const size_t nel = (size_t)nb * s->npw;
    const size_t nm = (size_t)3 * nb * nb;
    if (s->npw == 0) {
        if (dev) CUDA_TRY(c, cudaMemsetAsync(m_, 0, nm * sizeof(double2), st));
        else std::memset(m_, 0, nm * sizeof(double2));
        return HPSI_OK;
    }
    Carver cv;
    size_t o_psi = dev ? 0 : cv.take<double2>(nel);
    size_t o_m = dev ? 0 : cv.take<double2>(nm);
    size_t o_work = cv.off;
    if ((rc = ws_reserve(c, o_work + vel_ws_bytes(*s, nb, prec)))) return rc;
    const double2* psi = (const double2*)psi_;
    double2* m = (double2*)m_;
    if (!dev) {
        psi = reinterpret_cast<const double2*>(c->ws + o_psi);
        m = reinterpret_cast<double2*>(c->ws + o_m);
        CUDA_TRY(c, cudaMemcpyAsync((void*)psi, psi_, nel * sizeof(double2), cudaMemcpyHostToDevice, st));
    }
    if ((rc = velocity_dev(c, *s, nb, psi, m, prec, c->ws + o_work, st))) return rc;
    if (!dev) CUDA_TRY(c, cudaMemcpyAsync(m_, m, nm * sizeof(double2), cudaMemcpyDeviceToHost, st));
    if (!dev || (flags & HPSI_SYNC)) {
        CUDA_TRY(c, cudaStreamSynchronize(st));
        if (is_tc(prec) && (rc = check_device_flag(c))) return rc;
    }
    return HPSI_OK;
}

// Self-test: the device tables of a bound k-point as the projector build
// reads them — Y_lm, dY_lm/dtheta and (1/sin theta) dY_lm/dphi for
// l <= l_max ([3][(l_max+1)^2][npw], the last two only with dbeta tables) and
// the structure factors S_a(G) ([n_atoms][npw] complex) — copied to host
// buffers (either may be NULL), for known-answer tests of the kernels that
// build them.
extern "C" int hpsi_selftest_kpoint_tables(hpsi_ctx* c, int kid, double* ylm, double* sf)
{
    KSlot* s = nullptr;
    int rc = check_call(c, kid, 0, &s, 0);
    if (rc) return rc;
    if (s->npw == 0) return HPSI_OK;
    const size_t nlm = (size_t)(c->lmax + 1) * (c->lmax + 1);
    if (ylm) CUDA_TRY(c, cudaMemcpy(ylm, s->d_ylm, (c->have_dbeta ? 3 : 1) * nlm * s->npw * sizeof(double),
                                    cudaMemcpyDeviceToHost));
    if (sf && c->natom > 0)
        CUDA_TRY(c, cudaMemcpy(sf, s->d_sf, (size_t)c->natom * s->npw * sizeof(double2), cudaMemcpyDeviceToHost));
    return HPSI_OK;
}

// ---------------------------------------------------------------------------
// hpsi_apply_noalloc — H|psi> for callers that cannot allocate device memory.
//
// Some callers of this library may not call cudaMalloc once they are running:
// a k.p or eigensolver loop that runs under a fixed device-memory budget set
// at start-up, a host runtime whose own allocator owns all device memory and
// forbids other allocations, or code that must not add the implicit device
// synchronisation an allocation can cause between its kernels.  For them this
// entry point computes what hpsi_apply computes at FP64 or FP32, but all
// per-call scratch (the FFT planes of the local term, the split-K partial sums
// and the projected coefficients of the nonlocal term) lives in one
// file-scope device array of HPSI_NOALLOC_SCRATCH_BYTES (32 MiB).  Every GPU
// that loads this library holds that array until the process exits.
//
// Rules:
//  * psi and hpsi are device pointers (HPSI_DEVICE_PTRS is required);
//  * precision HPSI_PREC_FP64 or HPSI_PREC_FP32; the tensor-core precisions
//    need operand buffers per call and are refused with HPSI_ERR_BAD_ARG;
//  * the projector matrices of the requested precision must already exist:
//    the first hpsi_apply / hpsi_grad_apply at that precision on the k-point
//    builds them (that call allocates); otherwise HPSI_ERR_STATE;
//  * the whole chunk plan (bands per local-term chunk, bands per nonlocal
//    chunk and its last, shorter chunk) is checked against the scratch before
//    the first launch: a call that does not fit is refused with
//    HPSI_ERR_BAD_ARG and leaves hpsi untouched;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (which may load the module) and keeps it for the
//    process; make that first call before any stream capture.  The kept
//    address is not valid after cudaDeviceReset;
//  * every call shares the one array and leaves its contents behind (each
//    call writes all scratch it reads, so nothing needs clearing); calls that
//    overlap on the GPU — on two streams, or from two threads — race.
// ---------------------------------------------------------------------------
#include <mutex>

static __device__ __align__(256) unsigned char g_noalloc_scratch[HPSI_NOALLOC_SCRATCH_BYTES];

static int noalloc_scratch(hpsi_ctx* c, unsigned char** out)
{
    static std::mutex mu;
    static void* ptrs[256] = {nullptr};
    if (c->dev < 0 || c->dev >= 256) return fail(c, HPSI_ERR_BAD_ARG, "device ordinal %d out of range", c->dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!ptrs[c->dev]) {
        // host-side name of the array is a stand-in; its device address comes from the runtime
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(c, HPSI_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        ptrs[c->dev] = p;
    }
    *out = static_cast<unsigned char*>(ptrs[c->dev]);
    return HPSI_OK;
}

// Scratch bytes of one nonlocal chunk of nbc bands (split-K partials, then the
// projected coefficients), and its split count.
template <typename C, typename Acc>
static size_t noalloc_nl_bytes(const KSlot& s, int nbc, int* ns)
{
    *ns = split_for(s.P, nbc, s.npw);
    Carver cv;
    cv.take<Acc>((size_t)*ns * s.P * nbc);
    cv.take<C>((size_t)s.P * nbc);
    return cv.off;
}

// Bands per nonlocal chunk such that every chunk, the last (shorter) one
// included, fits the scratch: the split count, and with it the bytes, is not
// monotone in the band count, so both chunk sizes are checked.  0: none fits.
template <typename C, typename Acc>
static int noalloc_nl_chunk(const KSlot& s, int nb, size_t cap)
{
    int ns = 0;
    for (int nbc = nb; nbc >= 1; nbc = (nbc == 1) ? 0 : (nbc + 1) / 2) {
        if (noalloc_nl_bytes<C, Acc>(s, nbc, &ns) > cap) continue;
        const int rem = nb % nbc;
        if (rem && noalloc_nl_bytes<C, Acc>(s, rem, &ns) > cap) continue;
        return nbc;
    }
    return 0;
}

template <typename C, typename Acc, typename V>
static int apply_noalloc_impl(hpsi_ctx* c, KSlot& s, int nb, const double2* psi, double2* hpsi, const C* pr,
                              const V* vloc, const C* tw, unsigned char* scratch, cudaStream_t st)
{
    const size_t cap = HPSI_NOALLOC_SCRATCH_BYTES;
    Prof off;  // never records: creating events is not allowed here
    // the whole plan first: no launch before every chunk is known to fit
    const size_t plane_bytes = (size_t)s.nxs * c->n2 * c->n3 * sizeof(C);
    if (plane_bytes > cap)
        return fail(c, HPSI_ERR_BAD_ARG,
                    "hpsi_apply_noalloc: one band's FFT planes need %zu bytes, above the %zu-byte scratch", plane_bytes,
                    cap);
    int nbc = 0;
    if (s.P > 0) {
        nbc = noalloc_nl_chunk<C, Acc>(s, nb, cap);
        int ns = 0;
        if (nbc == 0)
            return fail(c, HPSI_ERR_BAD_ARG,
                        "hpsi_apply_noalloc: %d projectors need %zu bytes of partial sums per band, above the %zu-byte "
                        "scratch", s.P, noalloc_nl_bytes<C, Acc>(s, 1, &ns), cap);
    }
    // local term: bands in chunks whose FFT planes fit the scratch
    if (plane_bytes > 0) {
        LocalArgs a{};
        a.n1 = c->n1; a.n2 = c->n2; a.n3 = c->n3;
        a.npw = s.npw;
        a.nxs = s.nxs;
        local_xpass_shape(&a, sizeof(C));
        a.inv_n = 1.0 / ((double)c->n1 * c->n2 * c->n3);
        a.plane_x = s.d_plane;
        a.plane_off = s.d_plane + s.nxs;
        a.ent_ig = s.d_plane + 2 * s.nxs + 1;
        a.ent_jk = s.d_plane + 2 * s.nxs + 1 + s.npw;
        a.plane_jr = s.d_plane + 2 * s.nxs + 1 + 2 * s.npw;
        a.Lx = c->L[0]; a.Ly = c->L[1]; a.Lz = c->L[2];
        const int ch = (int)std::min<size_t>((size_t)nb, cap / plane_bytes);
        for (int b0 = 0; b0 < nb; b0 += ch) {
            const int n = std::min(ch, nb - b0);
            CUDA_TRY(c, (launch_local<C, V>(a, n, psi + (size_t)b0 * s.npw, hpsi + (size_t)b0 * s.npw, s.d_kin,
                                            reinterpret_cast<C*>(scratch), vloc, tw, tw + c->n1, tw + c->n1 + c->n2,
                                            st, &off)));
        }
    }
    // nonlocal term: bands in chunks of nbc (checked above)
    if (s.P == 0) return HPSI_OK;
    for (int b0 = 0; b0 < nb; b0 += nbc) {
        const int n = std::min(nbc, nb - b0);
        int ns = 0;
        noalloc_nl_bytes<C, Acc>(s, n, &ns);
        Carver cv;
        const size_t o_part = cv.take<Acc>((size_t)ns * s.P * n);
        const size_t o_w = cv.take<C>((size_t)s.P * n);
        Acc* part = reinterpret_cast<Acc*>(scratch + o_part);
        C* W = reinterpret_cast<C*>(scratch + o_w);
        CUDA_TRY(c, (launch_proj_gemm<C, double2, Acc>(s.P, n, s.npw, pr, (size_t)s.npw, psi + (size_t)b0 * s.npw,
                                                       (size_t)s.npw, part, ns, st)));
        CUDA_TRY(c, (launch_reduce_splits<Acc, C>(s.P, n, ns, part, s.d_lam, s.P, W, (size_t)n, st)));
        CUDA_TRY(c, launch_expand_gemm<C>(s.P, n, s.npw, W, (size_t)n, pr, (size_t)s.npw, hpsi + (size_t)b0 * s.npw,
                                          (size_t)s.npw, st));
    }
    return HPSI_OK;
}

extern "C" int hpsi_apply_noalloc(hpsi_ctx* c, int kid, int nb, const double* psi_, double* hpsi_, int flags,
                                  void* stream)
{
    KSlot* s = nullptr;
    int rc = check_call(c, kid, nb, &s, flags);
    if (rc) return rc;
    const int prec = flags & HPSI_PREC_MASK;
    if (prec != HPSI_PREC_FP64 && prec != HPSI_PREC_FP32)
        return fail(c, HPSI_ERR_BAD_ARG,
                    "hpsi_apply_noalloc: precision %d is not offered; HPSI_PREC_FP64 or HPSI_PREC_FP32 only (the "
                    "tensor-core path needs per-call operand buffers)", prec);
    if (!(flags & HPSI_DEVICE_PTRS))
        return fail(c, HPSI_ERR_BAD_ARG, "hpsi_apply_noalloc: psi/hpsi must be device pointers (HPSI_DEVICE_PTRS)");
    if (nb > 0 && (!psi_ || !hpsi_)) return fail(c, HPSI_ERR_BAD_ARG, "psi/hpsi NULL");
    if (nb == 0 || s->npw == 0) return HPSI_OK;
    const bool fp64 = prec == HPSI_PREC_FP64;
    if (s->P > 0 && !(fp64 ? (void*)s->pr64 : (void*)s->pr32))
        return fail(c, HPSI_ERR_STATE,
                    "hpsi_apply_noalloc: projector matrices of this precision are not built yet; one hpsi_apply or "
                    "hpsi_grad_apply at this precision on k-point %d builds them", kid);
    unsigned char* scratch = nullptr;
    if ((rc = noalloc_scratch(c, &scratch))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const double2* psi = (const double2*)psi_;
    double2* hpsi = (double2*)hpsi_;
    rc = fp64 ? apply_noalloc_impl<double2, double2, double>(c, *s, nb, psi, hpsi, s->pr64, c->d_v64, c->d_tw64,
                                                              scratch, st)
              : apply_noalloc_impl<float2, float2, float>(c, *s, nb, psi, hpsi, s->pr32, c->d_v32, c->d_tw32, scratch,
                                                           st);
    if (rc) return rc;
    if (flags & HPSI_SYNC) CUDA_TRY(c, cudaStreamSynchronize(st));
    return HPSI_OK;
}

// ===========================================================================
// Serving: a device-resident request loop with continuous batching.
//
// The systems (contexts) keep V_loc, the projector tables and the projector
// matrices of their bound k-points resident in HBM.  Clients submit requests
// (each a list of k-point jobs: psi in, hpsi accumulated, optional velocity
// matrix) from any thread.  The scheduler works on jobs, not requests: every
// job of a request enters one pending queue in arrival order, and one
// scheduler thread admits jobs whenever a lane (CUDA stream) is free and the
// job's buffers fit in the device arena (the HBM budget).  A request is
// retired when its last job's lane event fires.
//   * Arrival order, with bounded overtaking: a later job that fits may start
//     before an older one that does not, while the oldest pending job has
//     waited less than bypass_ms; after that only the oldest may start.
//   * Merging: jobs of a cell with few projectors (P <= 256) — the small cells
//     whose work is a handful of short launches — are gathered from the
//     pending queue (up to merge_max_bands bands of one cell) into one unit:
//     one ragged local-term launch set over all their bands (the batched
//     plans' item tables) and one ragged projection / expansion pair, instead
//     of a launch sequence per job.
// So requests that arrive while others run are admitted as lanes and memory
// free up, and the work of different requests overlaps on the device.  All
// CUDA calls are issued from the scheduler thread.
// ===========================================================================
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>

namespace {

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// first-fit allocator over [0, size) in 256-byte units
struct Arena {
    size_t size = 0;
    std::map<size_t, size_t> free_;  // offset -> length
    void init(size_t n) { size = n; free_.clear(); free_[0] = n; }
    bool alloc(size_t n, size_t* off)
    {
        n = (n + 255) / 256 * 256;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                *off = it->first;
                size_t rest = it->second - n, o = it->first + n;
                free_.erase(it);
                if (rest) free_[o] = rest;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t n)
    {
        n = (n + 255) / 256 * 256;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
        }
    }
    size_t in_use() const
    {
        size_t f = 0;
        for (auto& kv : free_) f += kv.second;
        return size - f;
    }
};

struct SrvReq {
    long long ticket = 0;
    std::vector<hpsi_job> jobs;
    int remaining = 0;  // jobs not yet retired
    int status = HPSI_OK;
    double t_submit = 0, t_admit = -1, t_done = 0;
    bool done = false;
    std::string err;
};

// one k-point job of a request
struct SrvTask {
    SrvReq* req = nullptr;
    int job = 0;
    size_t bytes = 0;  // arena bytes when it runs on its own
};

// what one lane runs: one job, or several merged jobs of one cell
struct SrvUnit {
    std::vector<SrvTask> tasks;
    bool merged = false;
    size_t bytes = 0, off = 0;
};

// Ragged work of a merged unit: offsets in its arena block and launch choices
struct MergePlan {
    size_t o_psi = 0, o_hpsi = 0, o_m = 0, o_T = 0, o_part = 0, o_W = 0, o_li = 0, o_bi = 0, o_xb = 0, o_gi = 0,
           o_ws = 0, bytes = 0;
    int nbands = 0, nb_max = 0, npw_max = 0, max_nxs = 0, nsplit = 1, P = 0, nxblk = 0;
};

}  // namespace

struct hpsi_server {
    std::vector<hpsi_ctx*> sys;
    int prec = HPSI_PREC_TC;
    int dev = 0;
    int merge_max_bands = 0;
    double bypass_ms = 0.0;
    unsigned char* arena_mem = nullptr;
    Arena arena;
    std::vector<cudaStream_t> lanes;
    std::vector<cudaEvent_t> lane_ev;
    std::vector<SrvUnit*> lane_unit;
    std::mutex mu;
    std::condition_variable cv_done, cv_work;
    std::deque<SrvTask> pending;
    std::map<long long, SrvReq*> reqs;
    long long next_ticket = 1;
    bool stop = false;
    std::thread th;
    size_t peak_in_use = 0;
    long long completed = 0, units = 0, merged_units = 0, merged_jobs = 0;
    std::string err;
};

static int srv_fail(hpsi_server* s, int code, const std::string& m)
{
    if (s) s->err = m;
    else g_last_error = m;
    return code;
}

static constexpr int kMergeMaxP = 256;  // cells with at most this many projectors merge

static bool srv_mergeable(const hpsi_server* S, const hpsi_job& j)
{
    if (S->merge_max_bands <= 0) return false;
    const hpsi_ctx* c = S->sys[j.system];
    auto it = c->slots.find(j.kid);
    return it != c->slots.end() && it->second.P <= kMergeMaxP && it->second.npw > 0 && j.nb > 0 &&
           j.nb <= S->merge_max_bands;
}

// device bytes of one job run on its own
static int srv_job_bytes(hpsi_server* S, const hpsi_job& j, size_t* bytes, std::string* why)
{
    if (j.system < 0 || j.system >= (int)S->sys.size()) { *why = "job system index out of range"; return HPSI_ERR_BAD_ARG; }
    hpsi_ctx* c = S->sys[j.system];
    auto it = c->slots.find(j.kid);
    if (it == c->slots.end() || !it->second.valid) { *why = "job k-point slot not bound"; return HPSI_ERR_STATE; }
    if (j.nb < 0 || (j.nb > 0 && (!j.psi || !j.hpsi))) { *why = "job psi/hpsi NULL or nb < 0"; return HPSI_ERR_BAD_ARG; }
    const KSlot& s = it->second;
    const size_t nel = (size_t)j.nb * s.npw;
    size_t ws = apply_ws_bytes(c, s, j.nb, S->prec), m = 0;
    if (j.vel) {
        m = (size_t)3 * j.nb * j.nb * sizeof(double2);
        ws = std::max(ws, vel_ws_bytes(s, j.nb, S->prec));
    }
    Carver cv;
    cv.take<double2>(nel);
    cv.take<double2>(nel);
    cv.take<unsigned char>(m);
    cv.take<unsigned char>(ws);
    *bytes = cv.off;
    return HPSI_OK;
}

static size_t srv_csize(const hpsi_server* S) { return S->prec == HPSI_PREC_FP64 ? sizeof(double2) : sizeof(float2); }

// layout of a merged unit of jobs of one cell
static MergePlan srv_merge_plan(const hpsi_server* S, const std::vector<SrvTask>& tasks)
{
    MergePlan m;
    const hpsi_ctx* c = S->sys[tasks[0].req->jobs[tasks[0].job].system];
    const size_t cs = srv_csize(S);
    size_t nel = 0, t_el = 0, vel_m = 0, vel_ws = 0;
    for (const SrvTask& t : tasks) {
        const hpsi_job& j = t.req->jobs[t.job];
        const KSlot& s = c->slots.at(j.kid);
        nel += (size_t)j.nb * s.npw;
        t_el += (size_t)j.nb * s.nxs * c->n2 * c->n3;
        m.nbands += j.nb;
        m.nb_max = std::max(m.nb_max, j.nb);
        m.npw_max = std::max(m.npw_max, s.npw);
        m.max_nxs = std::max(m.max_nxs, s.nxs);
        m.P = s.P;
        if (j.vel) {
            vel_m = std::max(vel_m, (size_t)3 * j.nb * j.nb * sizeof(double2));
            vel_ws = std::max(vel_ws, vel_ws_bytes(s, j.nb, S->prec));
        }
    }
    // split count of the ragged projection: enough blocks for the SMs, K >= 128 per split
    const long blocks = (long)tasks.size() * ceil_div(std::max(m.P, 1), 32) * ceil_div(std::max(m.nb_max, 1), 64);
    while (m.nsplit < 32 && blocks * m.nsplit < 2 * 152 && m.npw_max / (2 * m.nsplit) >= 64) m.nsplit *= 2;
    m.nxblk = m.nbands;  // upper bound: one x-pass band block per band
    Carver cv;
    m.o_psi = cv.take<double2>(nel);
    m.o_hpsi = cv.take<double2>(nel);
    m.o_m = cv.take<unsigned char>(vel_m);
    m.o_T = cv.take<unsigned char>(t_el * cs);
    m.o_part = cv.take<unsigned char>((size_t)m.nsplit * m.P * m.nbands * cs);
    m.o_W = cv.take<unsigned char>((size_t)m.P * m.nbands * cs);
    m.o_li = cv.take<LocalItem>(tasks.size());
    m.o_bi = cv.take<int>((size_t)m.nbands);
    m.o_xb = cv.take<int2>((size_t)m.nbands);
    m.o_gi = cv.take<BGemmItem>(tasks.size());
    m.o_ws = cv.take<unsigned char>(vel_ws);
    m.bytes = cv.off;
    return m;
}

// copy a job's outputs back to the host (hpsi, and the velocity matrix)
static int srv_copy_back(SrvReq* r, const hpsi_job& j, size_t nel, const double2* hpsi, const double2* m,
                         cudaStream_t st)
{
    cudaError_t e;
    if ((e = cudaMemcpyAsync(j.hpsi, hpsi, nel * sizeof(double2), cudaMemcpyDeviceToHost, st))) {
        r->err = cudaGetErrorString(e);
        return HPSI_ERR_CUDA;
    }
    if (j.vel && (e = cudaMemcpyAsync(j.vel, m, (size_t)3 * j.nb * j.nb * sizeof(double2), cudaMemcpyDeviceToHost, st))) {
        r->err = cudaGetErrorString(e);
        return HPSI_ERR_CUDA;
    }
    return HPSI_OK;
}

// one job on its lane (scheduler thread)
static int srv_issue_one(hpsi_server* S, SrvUnit* u, cudaStream_t st)
{
    SrvReq* r = u->tasks[0].req;
    const hpsi_job& j = r->jobs[u->tasks[0].job];
    if (j.nb == 0) return HPSI_OK;
    hpsi_ctx* c = S->sys[j.system];
    KSlot& s = c->slots[j.kid];
    const size_t nel = (size_t)j.nb * s.npw;
    if (s.npw == 0) return HPSI_OK;
    Carver cv;
    unsigned char* base = S->arena_mem + u->off;
    double2* psi = reinterpret_cast<double2*>(base + cv.take<double2>(nel));
    double2* hpsi = reinterpret_cast<double2*>(base + cv.take<double2>(nel));
    double2* m = reinterpret_cast<double2*>(base + cv.take<unsigned char>(j.vel ? (size_t)3 * j.nb * j.nb * sizeof(double2) : 0));
    unsigned char* ws = base + cv.take<unsigned char>(0);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(psi, j.psi, nel * sizeof(double2), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(hpsi, j.hpsi, nel * sizeof(double2), cudaMemcpyHostToDevice, st))) {
        r->err = cudaGetErrorString(e);
        return HPSI_ERR_CUDA;
    }
    int rc = apply_dev(c, s, j.nb, psi, hpsi, S->prec, ws, st, nullptr, nullptr, false);
    if (!rc && j.vel) rc = velocity_dev(c, s, j.nb, psi, m, S->prec, ws, st);
    if (rc) { r->err = c->err; return rc; }
    return srv_copy_back(r, j, nel, hpsi, m, st);
}

template <typename C, typename V>
static cudaError_t srv_merged_launches(hpsi_ctx* c, const LocalArgs& la, const MergePlan& m, unsigned char* base,
                                       const BGemmItem* d_gi, int n_items, const V* vloc, const C* tw, cudaStream_t st)
{
    cudaError_t e = launch_local_batch<C, V>(la, m.nbands, m.max_nxs, m.nxblk, reinterpret_cast<C*>(base + m.o_T), vloc,
                                             tw, tw + c->n1, tw + c->n1 + c->n2, st);
    if (e || m.P == 0) return e;
    if ((e = launch_bproj<C, C>(m.P, d_gi, n_items, m.nb_max, m.nsplit, m.P <= 16 ? 0 : 3,
                                reinterpret_cast<C*>(base + m.o_part), st)))
        return e;
    return launch_bexp<C, C>(m.P, d_gi, n_items, m.nb_max, m.npw_max, m.nsplit, 3,
                             reinterpret_cast<const C*>(base + m.o_part), reinterpret_cast<C*>(base + m.o_W), st);
}

// several jobs of one cell on a lane: one ragged launch set over all their bands
static int srv_issue_merged(hpsi_server* S, SrvUnit* u, cudaStream_t st)
{
    const hpsi_job& j0 = u->tasks[0].req->jobs[u->tasks[0].job];
    hpsi_ctx* c = S->sys[j0.system];
    const bool f64 = S->prec == HPSI_PREC_FP64;
    const MergePlan m = srv_merge_plan(S, u->tasks);
    unsigned char* base = S->arena_mem + u->off;
    double2* psi = reinterpret_cast<double2*>(base + m.o_psi);
    double2* hpsi = reinterpret_cast<double2*>(base + m.o_hpsi);
    std::vector<LocalItem> li;
    std::vector<BGemmItem> gi;
    std::vector<int> band_item;
    std::vector<size_t> off;
    size_t el = 0, t_off = 0;
    int band0 = 0;
    cudaError_t e;
    for (const SrvTask& t : u->tasks) {
        const hpsi_job& j = t.req->jobs[t.job];
        KSlot& s = c->slots[j.kid];
        const size_t nel = (size_t)j.nb * s.npw;
        off.push_back(el);
        if ((e = cudaMemcpyAsync(psi + el, j.psi, nel * sizeof(double2), cudaMemcpyHostToDevice, st)) ||
            (e = cudaMemcpyAsync(hpsi + el, j.hpsi, nel * sizeof(double2), cudaMemcpyHostToDevice, st))) {
            t.req->err = cudaGetErrorString(e);
            return HPSI_ERR_CUDA;
        }
        const int* pl = s.d_plane;
        LocalItem L{};
        L.plane_x = pl;
        L.plane_off = pl + s.nxs;
        L.ent_ig = pl + 2 * s.nxs + 1;
        L.ent_jk = pl + 2 * s.nxs + 1 + s.npw;
        L.plane_jr = pl + 2 * s.nxs + 1 + 2 * s.npw;
        L.kinetic = s.d_kin;
        L.psi = psi + el;
        L.hpsi = hpsi + el;
        L.t_off = t_off;
        L.npw = s.npw;
        L.nxs = s.nxs;
        L.nb = j.nb;
        L.band0 = band0;
        for (int k = 0; k < j.nb; ++k) band_item.push_back((int)li.size());
        li.push_back(L);
        BGemmItem G{};
        G.pr = f64 ? (const void*)s.pr64 : (const void*)s.pr32;
        G.psi = L.psi;
        G.hpsi = L.hpsi;
        G.lam = s.d_lam;
        G.part_off = (size_t)m.nsplit * m.P * band0;
        G.w_off = (size_t)m.P * band0;
        G.nb = j.nb;
        G.npw = s.npw;
        gi.push_back(G);
        el += nel;
        t_off += (size_t)j.nb * s.nxs * c->n2 * c->n3;
        band0 += j.nb;
    }
    LocalArgs la{};
    la.n1 = c->n1; la.n2 = c->n2; la.n3 = c->n3;
    la.inv_n = 1.0 / ((double)c->n1 * c->n2 * c->n3);
    la.Lx = c->L[0]; la.Ly = c->L[1]; la.Lz = c->L[2];
    local_xpass_shape(&la, srv_csize(S));
    std::vector<int2> xb;
    for (size_t i = 0; i < li.size(); ++i)
        for (int b0 = 0; b0 < li[i].nb; b0 += la.bb) xb.push_back(make_int2((int)i, b0));
    MergePlan mp = m;
    mp.nxblk = (int)xb.size();
    la.items = reinterpret_cast<const LocalItem*>(base + m.o_li);
    la.band_item = reinterpret_cast<const int*>(base + m.o_bi);
    la.xblk = reinterpret_cast<const int2*>(base + m.o_xb);
    // item tables: pageable host vectors, staged by the copy call itself
    SrvReq* r0 = u->tasks[0].req;
    if ((e = cudaMemcpyAsync(base + m.o_li, li.data(), li.size() * sizeof(LocalItem), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(base + m.o_bi, band_item.data(), band_item.size() * sizeof(int), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(base + m.o_xb, xb.data(), xb.size() * sizeof(int2), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(base + m.o_gi, gi.data(), gi.size() * sizeof(BGemmItem), cudaMemcpyHostToDevice, st))) {
        r0->err = cudaGetErrorString(e);
        return HPSI_ERR_CUDA;
    }
    const BGemmItem* d_gi = reinterpret_cast<const BGemmItem*>(base + m.o_gi);
    e = f64 ? srv_merged_launches<double2, double>(c, la, mp, base, d_gi, (int)gi.size(), c->d_v64, c->d_tw64, st)
            : srv_merged_launches<float2, float>(c, la, mp, base, d_gi, (int)gi.size(), c->d_v32, c->d_tw32, st);
    if (e) { r0->err = cudaGetErrorString(e); return HPSI_ERR_CUDA; }
    double2* mv = reinterpret_cast<double2*>(base + m.o_m);
    for (size_t i = 0; i < u->tasks.size(); ++i) {
        const SrvTask& t = u->tasks[i];
        const hpsi_job& j = t.req->jobs[t.job];
        KSlot& s = c->slots[j.kid];
        if (j.vel) {
            const int rc = velocity_dev(c, s, j.nb, psi + off[i], mv, S->prec, base + m.o_ws, st);
            if (rc) { t.req->err = c->err; return rc; }
        }
        const int rc = srv_copy_back(t.req, j, (size_t)j.nb * s.npw, hpsi + off[i], mv, st);
        if (rc) return rc;
    }
    return HPSI_OK;
}

// Take the next unit from the pending queue that fits the arena (lock held):
// the oldest job, or — while the oldest has waited less than bypass_ms — the
// first later one that fits; with merging, further pending jobs of the same
// cell join it up to merge_max_bands bands while the unit still fits.
static SrvUnit* srv_take_unit(hpsi_server* S, double now)
{
    if (S->pending.empty()) return nullptr;
    const bool may_bypass = now - S->pending.front().req->t_submit < S->bypass_ms;
    const size_t scan = may_bypass ? std::min<size_t>(S->pending.size(), 256) : 1;
    for (size_t i = 0; i < scan; ++i) {
        const SrvTask& t = S->pending[i];
        const hpsi_job& j = t.req->jobs[t.job];
        SrvUnit* u = new SrvUnit();
        u->tasks.push_back(t);
        u->bytes = t.bytes;
        std::vector<size_t> taken{i};
        if (srv_mergeable(S, j)) {
            int bands = j.nb;
            for (size_t k = i + 1; k < S->pending.size() && k < i + 512; ++k) {
                const SrvTask& t2 = S->pending[k];
                const hpsi_job& j2 = t2.req->jobs[t2.job];
                if (j2.system != j.system || !srv_mergeable(S, j2) || bands + j2.nb > S->merge_max_bands) continue;
                u->tasks.push_back(t2);
                const MergePlan mp = srv_merge_plan(S, u->tasks);
                if (mp.bytes > S->arena.size) { u->tasks.pop_back(); continue; }
                taken.push_back(k);
                bands += j2.nb;
            }
            if (u->tasks.size() > 1) {
                u->merged = true;
                u->bytes = srv_merge_plan(S, u->tasks).bytes;
            }
        }
        size_t off = 0;
        bool ok = S->arena.alloc(u->bytes, &off);
        while (!ok && u->tasks.size() > 1) {
            // does not fit now: fewer merged jobs, else the next candidate
            u->tasks.pop_back();
            taken.pop_back();
            u->merged = u->tasks.size() > 1;
            u->bytes = u->merged ? srv_merge_plan(S, u->tasks).bytes : u->tasks[0].bytes;
            ok = S->arena.alloc(u->bytes, &off);
        }
        if (!ok) { delete u; continue; }
        u->off = off;
        for (size_t k = taken.size(); k-- > 0;) S->pending.erase(S->pending.begin() + (long)taken[k]);
        return u;
    }
    return nullptr;
}

static void srv_loop(hpsi_server* S)
{
    cudaSetDevice(S->dev);
    std::unique_lock<std::mutex> lk(S->mu);
    while (!S->stop) {
        bool progress = false;
        // admit jobs while a lane is free and a unit fits
        for (;;) {
            int lane = -1;
            for (int i = 0; i < (int)S->lanes.size(); ++i)
                if (!S->lane_unit[i]) { lane = i; break; }
            if (lane < 0) break;
            const double t = now_ms();
            SrvUnit* u = srv_take_unit(S, t);
            if (!u) break;
            for (const SrvTask& tk : u->tasks)
                if (tk.req->t_admit < 0) tk.req->t_admit = t;
            S->lane_unit[lane] = u;
            S->units++;
            if (u->merged) { S->merged_units++; S->merged_jobs += (long long)u->tasks.size(); }
            S->peak_in_use = std::max(S->peak_in_use, S->arena.in_use());
            lk.unlock();
            const int rc = u->merged ? srv_issue_merged(S, u, S->lanes[lane]) : srv_issue_one(S, u, S->lanes[lane]);
            cudaEventRecord(S->lane_ev[lane], S->lanes[lane]);
            lk.lock();
            if (rc)
                for (const SrvTask& tk : u->tasks)
                    if (tk.req->status == HPSI_OK) tk.req->status = rc;
            progress = true;
        }
        // retire finished lanes
        for (int i = 0; i < (int)S->lanes.size(); ++i) {
            SrvUnit* u = S->lane_unit[i];
            if (!u) continue;
            cudaError_t q = cudaEventQuery(S->lane_ev[i]);
            if (q == cudaErrorNotReady) continue;
            const double t = now_ms();
            for (const SrvTask& tk : u->tasks) {
                SrvReq* r = tk.req;
                if (q != cudaSuccess && r->status == HPSI_OK) { r->status = HPSI_ERR_CUDA; r->err = cudaGetErrorString(q); }
                if (--r->remaining == 0) {
                    r->t_done = t;
                    r->done = true;
                    S->completed++;
                }
            }
            S->arena.release(u->off, u->bytes);
            S->lane_unit[i] = nullptr;
            delete u;
            progress = true;
        }
        if (progress) S->cv_done.notify_all();
        else S->cv_work.wait_for(lk, std::chrono::microseconds(50));
    }
}

extern "C" int hpsi_server_create(hpsi_ctx* const* systems, int n_systems, const hpsi_server_config* cfg,
                                  hpsi_server** out)
{
    if (!out) return HPSI_ERR_BAD_ARG;
    *out = nullptr;
    if (!systems || n_systems <= 0 || !cfg) return srv_fail(nullptr, HPSI_ERR_BAD_ARG, "server: no systems / config");
    const int prec = cfg->precision & HPSI_PREC_MASK;
    if (prec < HPSI_PREC_FP64 || prec > HPSI_PREC_TC_BF16) return srv_fail(nullptr, HPSI_ERR_BAD_ARG, "server: precision");
    if (cfg->lanes < 1 || cfg->lanes > 64) return srv_fail(nullptr, HPSI_ERR_BAD_ARG, "server: lanes must be 1..64");
    if (!(cfg->device_budget_bytes > 0)) return srv_fail(nullptr, HPSI_ERR_BAD_ARG, "server: device budget");
    if (cfg->merge_max_bands < 0 || cfg->merge_max_bands > 65535 || !(cfg->bypass_ms >= 0.0))
        return srv_fail(nullptr, HPSI_ERR_BAD_ARG, "server: merge_max_bands must be 0..65535 and bypass_ms >= 0");
    hpsi_server* S = new hpsi_server();
    S->prec = prec;
    S->dev = systems[0]->dev;
    S->merge_max_bands = cfg->merge_max_bands;
    S->bypass_ms = cfg->bypass_ms;
    for (int i = 0; i < n_systems; ++i) {
        if (!systems[i] || systems[i]->dev != S->dev) {
            delete S;
            return srv_fail(nullptr, HPSI_ERR_BAD_ARG, "server: systems must live on one device");
        }
        S->sys.push_back(systems[i]);
    }
    cudaSetDevice(S->dev);
    // make every bound k-point resident in this precision (projector matrices and
    // operands, with the gradient ones where the tables allow)
    for (hpsi_ctx* c : S->sys)
        for (auto& kv : c->slots) {
            if (!kv.second.valid) continue;
            int rc = prepare_slot(c, kv.second, prec, c->have_dbeta, 0);
            // merged units run the small cells' nonlocal term on the SIMT matrices
            if (!rc && S->merge_max_bands > 0 && kv.second.P <= kMergeMaxP && prec != HPSI_PREC_FP64)
                rc = ensure_proj<float2>(c, kv.second, false, 0);
            if (rc) {
                std::string m = "server: preparing k-point slot: " + c->err;
                delete S;
                return srv_fail(nullptr, rc, m);
            }
        }
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMalloc((void**)&S->arena_mem, cfg->device_budget_bytes) != cudaSuccess) {
        delete S;
        return srv_fail(nullptr, HPSI_ERR_OOM, "server: cannot allocate the device budget");
    }
    S->arena.init(cfg->device_budget_bytes);
    for (int i = 0; i < cfg->lanes; ++i) {
        cudaStream_t st;
        cudaEvent_t ev;
        cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        S->lanes.push_back(st);
        S->lane_ev.push_back(ev);
        S->lane_unit.push_back(nullptr);
    }
    S->th = std::thread(srv_loop, S);
    *out = S;
    return HPSI_OK;
}

extern "C" int hpsi_server_submit(hpsi_server* S, const hpsi_job* jobs, int n_jobs, long long* ticket)
{
    if (!S || !ticket || n_jobs < 0 || (n_jobs > 0 && !jobs)) return HPSI_ERR_BAD_ARG;
    SrvReq* r = new SrvReq();
    r->jobs.assign(jobs, jobs + n_jobs);
    std::lock_guard<std::mutex> lk(S->mu);
    std::vector<SrvTask> tasks;
    for (int i = 0; i < n_jobs; ++i) {
        std::string why;
        SrvTask t;
        t.req = r;
        t.job = i;
        const int rc = srv_job_bytes(S, r->jobs[i], &t.bytes, &why);
        if (rc) { delete r; return srv_fail(S, rc, "server submit: " + why); }
        if (t.bytes > S->arena.size) {
            delete r;
            return srv_fail(S, HPSI_ERR_OOM, "server submit: a job needs more than the whole device budget");
        }
        tasks.push_back(t);
    }
    r->ticket = S->next_ticket++;
    r->t_submit = now_ms();
    r->remaining = n_jobs;
    S->reqs[r->ticket] = r;
    *ticket = r->ticket;
    if (n_jobs == 0) {
        r->t_admit = r->t_done = r->t_submit;
        r->done = true;
        S->completed++;
        S->cv_done.notify_all();
        return HPSI_OK;
    }
    for (const SrvTask& t : tasks) S->pending.push_back(t);
    S->cv_work.notify_one();
    return HPSI_OK;
}

extern "C" int hpsi_server_wait(hpsi_server* S, long long ticket, double timeout_s, hpsi_request_times* times)
{
    if (!S) return HPSI_ERR_BAD_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return srv_fail(S, HPSI_ERR_BAD_ARG, "server wait: unknown ticket");
    SrvReq* r = it->second;
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (!r->done) {
        if (S->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !r->done)
            return srv_fail(S, HPSI_ERR_TIMEOUT, "server wait: timed out");
    }
    if (times) {
        times->queue_ms = r->t_admit - r->t_submit;
        times->run_ms = r->t_done - r->t_admit;
        times->total_ms = r->t_done - r->t_submit;
    }
    int rc = r->status;
    if (rc) S->err = "server request: " + r->err;
    S->reqs.erase(it);
    delete r;
    return rc;
}

extern "C" int hpsi_server_stats(hpsi_server* S, hpsi_server_statistics* out)
{
    if (!S || !out) return HPSI_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    out->completed = S->completed;
    out->queued = (long long)S->pending.size();
    long long run = 0;
    for (auto* u : S->lane_unit) run += u ? (long long)u->tasks.size() : 0;
    out->running = run;
    out->budget_bytes = (double)S->arena.size;
    out->peak_bytes = (double)S->peak_in_use;
    out->units = S->units;
    out->merged_units = S->merged_units;
    out->merged_jobs = S->merged_jobs;
    return HPSI_OK;
}

extern "C" const char* hpsi_server_last_error(const hpsi_server* S)
{
    if (!S) return g_last_error.c_str();
    return S->err.c_str();
}

extern "C" int hpsi_server_destroy(hpsi_server* S)
{
    if (!S) return HPSI_ERR_BAD_ARG;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        S->cv_work.notify_all();
    }
    if (S->th.joinable()) S->th.join();
    cudaSetDevice(S->dev);
    for (auto st : S->lanes) cudaStreamSynchronize(st);
    for (auto st : S->lanes) cudaStreamDestroy(st);
    for (auto ev : S->lane_ev) cudaEventDestroy(ev);
    for (auto* u : S->lane_unit) delete u;
    for (auto& kv : S->reqs) delete kv.second;
    if (S->arena_mem) cudaFree(S->arena_mem);
    delete S;
    return HPSI_OK;
}
