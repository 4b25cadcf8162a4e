// ctx.cuh — internal state of a context (hpsi_ctx) and of its bound
// k-points, shared by the C-ABI translation units (hpsi_api.cu, batch.cu).
#pragma once

#include <cstdarg>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/hpsi_gb300.h"
#include "kernels.cuh"
#include "tc_gemm.cuh"

struct KSlot {
    bool valid = false;
    int npw = 0;
    double kf[3] = {0, 0, 0};
    double* d_kin = nullptr;
    double* d_kvec = nullptr;
    int* d_g = nullptr;
    double* d_q = nullptr;
    double* d_trig = nullptr;
    double* d_ylm = nullptr;   // ylm, yth, yph consecutive
    double* d_beta = nullptr;  // beta, dbeta consecutive
    double* d_dbeta0 = nullptr;
    double2* d_sf = nullptr;
    int nxs = 0;
    bool aliased = false;          // two G-vectors map to one grid point (the scatter keeps the last)
    int* d_plane = nullptr;    // plane_x[nxs], plane_off[nxs+1], ent_ig[npw], ent_jk[npw]
    int P = 0;
    std::vector<ProjRow> rows;     // host copy of d_rows
    ProjRow* d_rows = nullptr;
    double* d_lam = nullptr;
    double2* pr64 = nullptr;
    bool pr64_grad = false;
    float2* pr32 = nullptr;
    bool pr32_grad = false;
    // tensor-core H|psi>: generator tables of the projector operands, one set
    // per split format (0 FP16, 1 BF16), built from the FP64 tables on first
    // use and kept until the slot is rebound (batch plans hold pointers into
    // them); tc_proj and tc_expand carry only their K depth and row factors.
    // tc_fmt: the format of the last preparation, which the call that follows
    // it uses.
    int tc_fmt = -1;
    unsigned char* tc_mem[2] = {nullptr, nullptr};
    TcGen tcgen[2];
    TcOperand tc_proj[2], tc_expand[2];
    int tcg_fmt = -1;              // gradient operands (4P-row projection, per-direction expansion)
    unsigned char* tcg_mem = nullptr;
    TcOperand tcg_proj, tcg_exp[3];
    long gen = 0;                  // binding generation: changes when the slot is rebound
    double2* hess64 = nullptr;     // projector second derivatives [6][P][npw] (Hessian), per precision
    float2* hess32 = nullptr;
};

template <typename T>
inline cudaError_t dalloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void**)p, count * sizeof(T));
}

template <typename T>
inline void dfree(T*& p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

inline void slot_free(KSlot& s)
{
    dfree(s.d_kin); dfree(s.d_kvec); dfree(s.d_g); dfree(s.d_q); dfree(s.d_trig); dfree(s.d_ylm);
    dfree(s.d_beta); dfree(s.d_dbeta0); dfree(s.d_sf); dfree(s.d_plane); dfree(s.d_rows); dfree(s.d_lam);
    dfree(s.pr64); dfree(s.pr32); dfree(s.tc_mem[0]); dfree(s.tc_mem[1]); dfree(s.tcg_mem); dfree(s.hess64);
    dfree(s.hess32);
    s = KSlot();
}

struct hpsi_ctx {
    int dev = 0;
    int n1 = 0, n2 = 0, n3 = 0;
    double omega = 0;
    int natom = 0, nrad = 0, nq_max = 0, lmax = 0;
    bool have_dbeta = true;
    std::vector<int> atom_species, rad_off, rad_l, rad_nq;
    std::vector<double> tau, rad_lam, rad_dq, rad_qmax;
    double* d_tables = nullptr;   // beta then dbeta, [2][nrad][nq_max]
    int* d_rad_nq = nullptr;
    double* d_rad_dq = nullptr;
    double* d_tau = nullptr;
    double* d_v64 = nullptr;
    float* d_v32 = nullptr;
    float* d_dv32 = nullptr;      // V64 - V32 per grid point (the energy sums' FP64 correction)
    double2* d_tw64 = nullptr;    // twiddles x, y, z consecutive
    float2* d_tw32 = nullptr;
    FftLen L[3];
    std::map<int, KSlot> slots;
    unsigned char* ws = nullptr;
    size_t ws_size = 0;
    Prof prof;
    int* d_err = nullptr;         // device-side error flag of the bounded waits (tcgen05 GEMMs)
    // side stream of the tensor-core H|psi>: the projection chain runs there
    // beside the FFT passes (fork/join by events on the caller's stream)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // copy stream of hpsi_apply with host buffers: the H2D copy of hpsi, which
    // only the tensor-core expansion reads, runs beside the FFT passes
    cudaStream_t copy = nullptr;
    cudaEvent_t ev_copy_after = nullptr, ev_copy_done = nullptr;
    // hpsi_apply with host buffers on the tensor-core path: hpsi moves in and
    // out in two G halves (uploads on the copy stream, the first half's
    // download on the side stream beside the second half's expansion)
    cudaEvent_t ev_half_in[2] = {nullptr, nullptr}, ev_half_exp = nullptr, ev_half_out = nullptr;
    cudaEvent_t ev_psi_in[2] = {nullptr, nullptr};  // psi's two band halves on the copy stream
    long gen_counter = 0;         // source of KSlot::gen
    double* d_hess = nullptr;     // Hessian radial tables [nrad][3][hess_nq] (F0, F1, F3), raw
    int hess_nq = 0;
    double hess_dq = 0.0;
    std::vector<char> hess_set;   // per radial function: tables given
    std::string err;
};

// Message of the last failure that had no context to hold it (hpsi_ctx_create,
// batch plans).
extern thread_local std::string g_last_error;

inline int fail(hpsi_ctx* c, int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    else g_last_error = buf;
    return code;
}

#define CUDA_TRY(ctx, expr)                                                                             \
    do {                                                                                                \
        cudaError_t e_ = (expr);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? HPSI_ERR_OOM : HPSI_ERR_CUDA, "%s: %s (%s:%d)", \
                        #expr, cudaGetErrorString(e_), __FILE__, __LINE__);                             \
    } while (0)

// Workspace carving: each piece 256-byte aligned.
struct Carver {
    size_t off = 0;
    template <typename T>
    size_t take(size_t count)
    {
        size_t o = off;
        off += ((count * sizeof(T)) + 255) / 256 * 256;
        return o;
    }
};

inline int ws_reserve(hpsi_ctx* c, size_t bytes)
{
    if (bytes <= c->ws_size) return HPSI_OK;
    if (c->ws) cudaFree(c->ws);
    c->ws = nullptr;
    c->ws_size = 0;
    size_t want = bytes + bytes / 8;
    CUDA_TRY(c, cudaMalloc((void**)&c->ws, want));
    c->ws_size = want;
    return HPSI_OK;
}


// Build, once, what a precision needs on slot s (projector matrices, tensor-core
// operands; with grad also the derivative operands).  Allocates.
int prepare_slot(hpsi_ctx* c, KSlot& s, int prec, bool grad, cudaStream_t st);
