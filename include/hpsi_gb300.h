/*
 * hpsi_gb300.h — C ABI of the GB300 (sm_103a) H|psi> library, libhpsi_gb300.so.
 *
 * It replaces the reference's C++23-module operator API of src/H_psi:
 *
 *   reference                                            here
 *   ---------------------------------------------------  ----------------------------------
 *   Hamiltonian::finalize (src/H_psi/hamiltonian.cpp:267-392;
 *     tables, lambda, FFT plan)                           hpsi_ctx_create
 *   Hamiltonian::at_k / Callable::set_ikpt
 *     (src/H_psi/hamiltonian.cppm:186-188,205;
 *      src/H_psi/hamiltonian_callable.cpp:62-85)          hpsi_set_kpoint
 *   Callable::operator()(psi, hpsi)
 *     (src/H_psi/hamiltonian.cppm:177-178;
 *      src/H_psi/hamiltonian_callable.cpp:94-356)         hpsi_apply (nb = 1)
 *   Callable::operator()(n_bands, psi, hpsi)
 *     (src/H_psi/hamiltonian.cppm:180-182; declared there,
 *      never defined in the reference)                    hpsi_apply (nb > 1)
 *   Callable::dim() (src/H_psi/hamiltonian.cppm:184)      hpsi_dim
 *   Gradient::Callable::operator()(psi, GradHPsi)
 *     (src/H_psi/hamiltonian.cppm:228-229;
 *      src/H_psi/hamiltonian_gradient.cpp:116-294)        hpsi_grad_apply
 *   Hessian::Callable::operator()(psi, HessHPsi)
 *     (declared, src/H_psi/hamiltonian.cppm:84-91; empty
 *      body, src/H_psi/hamiltonian_hessian.cpp:48-50)      hpsi_hess_apply
 *   (no counterpart; band-pair <psi_m|dH/dk_a|psi_n>)     hpsi_velocity_matrix
 *   C++ exceptions (runtime_error, out_of_range,
 *     domain_error)                                       negative status + hpsi_last_error
 *
 * Semantics kept from the reference:
 *   - outputs ACCUMULATE (hpsi += H psi); the caller zeroes them first
 *     (src/H_psi/hamiltonian_callable.cpp:90-92);
 *   - psi/hpsi of one band are npw contiguous complex<double> values (re, im)
 *     in the G-vector order of the k-point (the GKK/WG order); a block of nb
 *     bands is band-major: psi[b*npw + g];
 *   - a NULL gradient output skips that Cartesian direction (the reference's
 *     empty GradHPsi span, src/H_psi/hamiltonian.cppm:53-70);
 *   - projectors with |lambda| < 1e-15 are skipped
 *     (src/H_psi/hamiltonian_callable.cpp:226-227);
 *   - q > q_max is an error, like BetaqTables::interpolate's domain_error
 *     (src/pseudo/ncpp_advance.cppm:656-661).
 *
 * Threading: one context per host thread; calls on one context are serialised
 * by the caller.  All device work of a call is queued on `stream` (NULL = the
 * legacy default stream); with HPSI_SYNC the call returns after it finished.
 */
#ifndef HPSI_GB300_H
#define HPSI_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define HPSI_ABI_VERSION 1

/* status codes */
#define HPSI_OK            0
#define HPSI_ERR_BAD_ARG  -1   /* std::invalid_argument / out_of_range in the reference */
#define HPSI_ERR_OOM      -2   /* device allocation failed */
#define HPSI_ERR_RANGE    -3   /* q > q_max, or a G index outside the FFT grid (domain_error) */
#define HPSI_ERR_TIMEOUT  -4   /* a bounded device-side wait gave up */
#define HPSI_ERR_CUDA     -5   /* CUDA runtime error */
#define HPSI_ERR_STATE    -6   /* k-point not set, missing table (runtime_error) */

/* flags: precision in bits 0-3 */
#define HPSI_PREC_FP64      0  /* complex128 FFTs, FP64 projector sums: parity path */
#define HPSI_PREC_FP32      1  /* complex64 FFTs, FP32 projector GEMMs, FP64 phases */
#define HPSI_PREC_TC        2  /* complex64 FFTs, tcgen05 tensor-core projector GEMMs on split FP16
                                  (x*2^s = hi + lo per row, 3 products, FP32 accumulation) */
#define HPSI_PREC_TC_BF16   3  /* as HPSI_PREC_TC with split BF16 (hi + lo, 3 products, no scaling) */
#define HPSI_PREC_MASK    0xF
#define HPSI_DEVICE_PTRS  0x10 /* psi/outputs are device pointers (else host memory) */
#define HPSI_SYNC         0x20 /* synchronise `stream` before returning */
#define HPSI_ONE_STREAM   0x40 /* tensor-core hpsi_apply / hpsi_apply_energies: run the
                                * projection chain on `stream` too instead of on the
                                * context's side stream beside the FFT passes */

/* One pseudopotential species after the per-l diagonalisation of D
 * (src/pseudo/ncpp_advance.cppm:65-153): projector i has angular momentum
 * proj_l[i], KB strength lambda[i] (Ha) and a radial table on q_j = j*dq. */
typedef struct hpsi_species {
    int n_proj;
    const int* proj_l;        /* [n_proj] */
    const double* lambda;     /* [n_proj], Ha */
    int nq;                   /* table length; interpolation needs floor(q/dq)+2 < nq */
    double dq;                /* bohr^-1 */
    double q_max;             /* interpolation domain; q > q_max -> HPSI_ERR_RANGE */
    const double* beta_q;     /* [n_proj][nq] raw beta(q_j), without 1/sqrt(omega) */
    const double* dbeta_q;    /* [n_proj][nq] raw dbeta/dq(q_j); NULL: no gradient */
} hpsi_species;

typedef struct hpsi_system {
    int n1, n2, n3;           /* FFT grid */
    double lattice[9];        /* row n = lattice vector a_n, bohr */
    double omega;             /* cell volume (bohr^3): projector norm 1/sqrt(omega) */
    const double* v_loc;      /* [n1*n2*n3] Ha, index (i*n2 + j)*n3 + k */
    int n_species;
    const hpsi_species* species;
    int n_atoms;
    const int* atom_species;  /* [n_atoms] index into species */
    const double* atom_tau;   /* [n_atoms][3] fractional coordinates */
} hpsi_system;

/* G-sphere of one k-point: what GKK::loadKPoint provides (src/io/GKK.cppm:60-72). */
typedef struct hpsi_kpoint {
    int npw;
    double k_frac[3];         /* k in reciprocal-lattice coordinates */
    const int* g_idx;         /* [npw][3] integer G, centred convention */
    const double* kvec;       /* [npw][3] K = k+G, Cartesian bohr^-1 */
    const double* kinetic;    /* [npw] |k+G|^2/2, Ha, as provided (not recomputed) */
} hpsi_kpoint;

typedef struct hpsi_ctx hpsi_ctx;

int hpsi_abi_version(void);

/* Build a context on the current CUDA device: uploads V_loc, tables, atoms.
 * On failure *out is NULL and hpsi_last_error(NULL) gives the reason. */
int hpsi_ctx_create(const hpsi_system* sys, hpsi_ctx** out);
int hpsi_ctx_destroy(hpsi_ctx* ctx);

/* Bind G-sphere data to slot `kid` (0 <= kid < 4096): derives q, theta, phi,
 * Y_lm, beta(q) and the structure factors on the device.  The first call at a
 * precision builds what it needs from them: the projector matrices for
 * HPSI_PREC_FP64 / HPSI_PREC_FP32; for the tensor-core precisions the
 * beta*Y_lm rows, structure-factor rows and split scales from which the GEMMs
 * generate their projector tiles in shared memory.  Rebinding a slot
 * replaces it. */
int hpsi_set_kpoint(hpsi_ctx* ctx, int kid, const hpsi_kpoint* kp);

/* Number of plane waves of slot kid (Callable::dim), or a negative status. */
int hpsi_dim(const hpsi_ctx* ctx, int kid);

/* hpsi[b] += H psi[b] for nb bands (kinetic + local + nonlocal). */
int hpsi_apply(hpsi_ctx* ctx, int kid, int nb, const double* psi, double* hpsi,
               int flags, void* stream);

/* Radial beta(q) and dbeta/dq tables on the device: what the reference's
 * BetaqTables / DBetaqTables compute in Hamiltonian::finalize
 * (src/pseudo/ncpp_advance.cppm:524-641, 718-835) from the radial mesh and the
 * projectors after its sortByL / diagonalizeNonlocal, as the input tables of
 * hpsi_species (raw, without 1/sqrt(omega)):
 *   beta_q[p][i]  = 4 pi Simpson[beta_p(r) r j_l(q_i r)],
 *   dbeta_q[p][i] = 4 pi Simpson[beta_p(r) r^2 j_l'(q_i r)],   q_i = i dq,
 * i < hpsi_beta_table_length(dq, q_max) = ceil(q_max/dq) + 4.  r, rab: nr
 * mesh points and dr/di (uniform_mesh != 0: rab[0] is the constant step);
 * beta: [n_proj][nr], trailing zeros trimmed per projector; l: [n_proj].
 * dbeta_q may be NULL.  Host or device pointers per HPSI_DEVICE_PTRS; the call
 * allocates its scratch and synchronises stream. */
int hpsi_beta_table_length(double dq, double q_max);
int hpsi_beta_tables(int nr, const double* r, const double* rab, int uniform_mesh, int n_proj, const int* l,
                     const double* beta, double dq, double q_max, double* beta_q, double* dbeta_q, int flags,
                     void* stream);

/* G-sphere of a k-point generated on the device: every integer G with
 * |k+G|^2/2 < ecut (Ha), K = (k_frac + g) B with B = 2 pi A^-T (A rows =
 * lattice vectors, bohr), in lexicographic (g1, g2, g3) order, as the
 * hpsi_kpoint arrays g_idx [npw][3], kvec [npw][3], kinetic [npw].  The
 * reference reads these from OUT.GKK (src/io/GKK.cppm:511-593); here they
 * need no host enumeration.  With g_idx/kvec/kinetic NULL the call only
 * stores the count in *npw_out; a count above max_npw is HPSI_ERR_RANGE.
 * Output arrays host or device per HPSI_DEVICE_PTRS; synchronises stream. */
int hpsi_gsphere(const double* lattice, const double* k_frac, double ecut, int max_npw, int* g_idx,
                 double* kvec, double* kinetic, int* npw_out, int flags, void* stream);

/* Hessian d2H/dk_a dk_b |psi> (the reference declares it with six outputs,
 * src/H_psi/hamiltonian.cppm:84-91, and leaves the operator empty,
 * src/H_psi/hamiltonian_hessian.cpp:48-50):
 *   out_ab += delta_ab psi + sum_p lambda_p (|d_ab p><p| + |d_a p><d_b p|
 *                                            + |d_b p><d_a p| + |p><d_ab p|) psi
 * for ab = xx, yy, zz, xy, xz, yz (NULL outputs are skipped).  The projector
 * second derivatives come from radial tables, smooth at q = 0 (g_n(x) =
 * j_n(x)/x^n):  F0 = 4 pi Int beta r^(l+1) g_l(qr) dr  (= beta/q^l),
 * F1 = -4 pi Int beta r^(l+3) g_(l+1)(qr) dr  (= F0'/q),
 * F3 = 4 pi Int beta r^(l+5) g_(l+2)(qr) dr  (= (F0'' - F0'/q)/q^2), times
 * the solid harmonics R_lm = |K|^l Y_lm:
 *   d_ab(beta Y) = F3 K_a K_b R + F1 (delta_ab R + K_a d_b R + K_b d_a R) + F0 d_ab R.
 * hpsi_hessian_tables builds f = [3][n_proj][nq] (F0, F1, F3 on q_i = i dq,
 * nq = hpsi_beta_table_length(dq, q_max)) from radial projectors as in
 * hpsi_beta_tables; hpsi_set_hessian_tables attaches them to a species of ctx
 * (the same dq and nq for all species).  hpsi_hess_apply runs FP64 for
 * HPSI_PREC_FP64 and FP32 otherwise; HPSI_ERR_STATE without tables. */
int hpsi_hessian_tables(int nr, const double* r, const double* rab, int uniform_mesh, int n_proj, const int* l,
                        const double* beta, double dq, double q_max, double* f, int flags, void* stream);
int hpsi_set_hessian_tables(hpsi_ctx* ctx, int species, int nq, double dq, const double* f);
int hpsi_hess_apply(hpsi_ctx* ctx, int kid, int nb, const double* psi, double* xx, double* yy, double* zz,
                    double* xy, double* xz, double* yz, int flags, void* stream);

/* Sternheimer equations for the k-derivative of the occupied bands (the
 * reference's roadmap item: conjugate-gradient solution of the linear
 * equations, docs/roadmap.md): for each of the nv occupied bands psi_n with
 * eigenvalue eps_n (orthonormal eigenstates of this k-point's H, lowest first)
 *   P_c (H - eps_n) P_c x_n = -P_c dH/dk_a psi_n,   P_c = 1 - sum_m |psi_m><psi_m|,
 * x_n = P_c dpsi_n/dk_a.  One preconditioned CG per band, all bands batched
 * (each iteration applies H to nv vectors through the hpsi_apply path of the
 * flags' precision; dots, updates and the projections are FP64), stopping
 * when |r_n| <= tol |b_n| for every band.  x: nv x npw output (overwritten);
 * iterations (may be NULL): CG iterations taken; residual (may be NULL, host):
 * nv final relative residuals.  HPSI_ERR_TIMEOUT when max_iter is reached
 * first (x then holds the last iterate).  psi, eps, x: host or device per
 * HPSI_DEVICE_PTRS.  The reference has no implementation of this step. */
int hpsi_sternheimer(hpsi_ctx* ctx, int kid, int nv, const double* psi, const double* eps, int direction,
                     double tol, int max_iter, double* x, int* iterations, double* residual, int flags,
                     void* stream);

/* Charge density of one k-point: rho[i][j][k] += sum_b occ[b] |psi_b(r)|^2,
 * psi_b(r) the unnormalised G->r transform of the band scattered onto the grid
 * (the last of several aliasing G wins), as the reference's buildDensity
 * (src/support/density.cppm:41-94) accumulates it per k-point and band; call
 * once per k-point to sum a Monkhorst-Pack grid.  rho: n1*n2*n3 doubles in
 * [i][j][k] order (the RHO file order), accumulated; occ: nb doubles.  The
 * transform runs in complex128 for HPSI_PREC_FP64 and complex64 otherwise;
 * the band sums are FP64 in band order.  Host or device pointers as in
 * hpsi_apply. */
int hpsi_density(hpsi_ctx* ctx, int kid, int nb, const double* psi, const double* occ, double* rho,
                 int flags, void* stream);

/* k·p sums of second-order perturbation theory, FP64, for the lowest n_low bands:
 *   s[n][a][b] = sum_{m != n, |e_n - e_m| > deg_tol} Re(m_a[n][m] m_b[m][n]) / (e_n - e_m)
 * from a velocity matrix m ([3][nb][nb] complex, hpsi_velocity_matrix's layout)
 * and band energies e[nb] (Ha).  Without a nonlocal second derivative the
 * inverse effective-mass tensor of band n is delta_ab + 2 s[n][a][b].  Pairs
 * within deg_tol are left out and counted in n_skipped[n] (may be NULL).
 * s: [n_low][3][3] doubles.  m, e, s, n_skipped: device memory with
 * HPSI_DEVICE_PTRS, else host memory (the call then allocates a staging
 * buffer and synchronises).  No counterpart in the reference. */
int hpsi_kp_sums(int nb, int n_low, const double* m, const double* e, double deg_tol, double* s,
                 int* n_skipped, int flags, void* stream);

/* hpsi += H psi (as hpsi_apply) and e[b] = <psi_b|H|psi_b> (Ha) with FP64
 * reductions on the device: kinetic energy summed in FP64; local energy
 * (1/N) sum_r V|psi_b(r)|^2 from the G->r transform of the call, divided by
 * that transform's own Parseval norm sum_r |psi_b(r)|^2 / (N sum_G |psi_b|^2),
 * which cancels the gain error of the complex64 FFTs; nonlocal energy
 * sum_p lambda_p |<p|psi_b>|^2 from the projection's split sums in FP64 (the
 * tensor-core projection then keeps its FP32 accumulation chains in TMEM to
 * 1024 of K, so hpsi differs from hpsi_apply's within the path's
 * tolerance; FP64 and FP32 hpsi are bit-identical to hpsi_apply's).  When two
 * G-vectors of the k-point share a grid point the Rayleigh quotient of the
 * computed hpsi is returned instead.  e: nb doubles (device memory with
 * HPSI_DEVICE_PTRS).  The reference forms these Rayleigh quotients on the host
 * (test/H_psi/test_hpsi_eigen.cpp:92-106); it has no such call. */
int hpsi_apply_energies(hpsi_ctx* ctx, int kid, int nb, const double* psi, double* hpsi, double* e,
                        int flags, void* stream);

/* d{x,y,z}[b] += dH/dk_{x,y,z} psi[b]; NULL outputs are skipped.
 * (The tensor-core precisions use the FP32 GEMMs here.) */
int hpsi_grad_apply(hpsi_ctx* ctx, int kid, int nb, const double* psi,
                    double* dx, double* dy, double* dz, int flags, void* stream);

/* m[a][m][n] = <psi_m| dH/dk_a |psi_n>, a = x,y,z, complex, overwritten (not accumulated).
 * Output layout [3][nb][nb] complex<double>; psi as in hpsi_apply.  With the
 * tensor-core precisions the band-pair GEMMs psi^H (dH_a psi) also run on the
 * tensor cores, for both in the scaled split-FP16 form (FP32 accumulation in
 * short chains, FP64 split-K sums). */
int hpsi_velocity_matrix(hpsi_ctx* ctx, int kid, int nb, const double* psi, double* m,
                         int flags, void* stream);

/* hpsi_apply for callers that cannot allocate device memory during the call
 * (a fixed device-memory budget, a host runtime whose allocator owns all
 * device memory, or code that must not add an allocation's implicit device
 * synchronisation).  No counterpart in the reference.  Same result as
 * hpsi_apply at HPSI_PREC_FP64 or HPSI_PREC_FP32; the tensor-core precisions
 * are refused with HPSI_ERR_BAD_ARG.  psi/hpsi must be device pointers
 * (HPSI_DEVICE_PTRS).  All scratch lives in one static device array of
 * HPSI_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit; a call whose chunks do not fit is rejected with HPSI_ERR_BAD_ARG
 * before any launch, leaving hpsi untouched.  The projector matrices of the
 * precision must exist (built by a first hpsi_apply/hpsi_grad_apply at that
 * precision), else HPSI_ERR_STATE.  The first call on a device looks up the
 * array's address and keeps it (make it before any stream capture; the kept
 * address is not valid after cudaDeviceReset).  Calls share the array:
 * calls that overlap on the GPU race. */
#define HPSI_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int hpsi_apply_noalloc(hpsi_ctx* ctx, int kid, int nb, const double* psi, double* hpsi,
                       int flags, void* stream);

/* Per-phase CUDA-event profile of the device work queued by later calls
 * (instrumentation for benchmarks; off by default).  hpsi_profile(ctx, on)
 * resets the record and switches it on or off; hpsi_profile_read waits for
 * the recorded work and fills, per phase, the summed milliseconds and the
 * number of kernel launches.  Phases: 0 projector build, 1 G->r planes
 * (scatter + z/y FFT), 2 x pass (x FFT, V, x FFT), 3 r->G planes (y/z FFT +
 * gather + kinetic), 4 projection GEMM, 5 split-K reduction, 6 expansion GEMM,
 * 7 other (gradient kinetic term, velocity GEMMs). */
#define HPSI_PROFILE_PHASES 8
int hpsi_profile(hpsi_ctx* ctx, int enable);
int hpsi_profile_read(hpsi_ctx* ctx, double* ms, long long* launches);

/* ---- Serving: a device-resident request loop with continuous batching ------
 * Systems (contexts with their bound k-points) stay resident in HBM; requests
 * are lists of k-point jobs submitted from any host thread.  One scheduler
 * thread admits jobs in arrival order when a lane (CUDA stream) is free and
 * the job's buffers fit in the device budget (a later job that fits may
 * overtake an older one while the oldest has waited less than bypass_ms), runs
 * them concurrently on the lanes, and retires a request when its last job
 * finishes.  With merge_max_bands > 0, pending jobs of a cell with at most 256
 * projectors are merged (up to that many bands) into one ragged launch set
 * whose nonlocal term runs on the FP32 (FP64 for HPSI_PREC_FP64) SIMT GEMMs.
 * psi/hpsi/vel of a job are host
 * memory (pinned memory gives asynchronous copies) and must stay valid until
 * hpsi_server_wait returns; hpsi accumulates (+=) as in hpsi_apply, vel (if not
 * NULL) receives the [3][nb][nb] velocity matrix.  While a server runs, its
 * contexts must not be used directly.  No counterpart in the reference. */
typedef struct hpsi_server hpsi_server;
typedef struct hpsi_job {
    int system;               /* index into the server's systems */
    int kid;                  /* bound k-point slot of that system */
    int nb;
    const double* psi;        /* [nb][npw] complex */
    double* hpsi;             /* [nb][npw] complex, accumulated */
    double* vel;              /* [3][nb][nb] complex or NULL */
} hpsi_job;
typedef struct hpsi_server_config {
    int lanes;                /* concurrent work units (CUDA streams), 1..64 */
    double device_budget_bytes; /* arena for in-flight request buffers and workspaces */
    int precision;            /* HPSI_PREC_* for every request */
    int merge_max_bands;      /* 0: no merging; else bands of one cell per merged unit (<= 65535) */
    double bypass_ms;         /* 0: strict arrival order; else how long the oldest pending
                               * job may be overtaken by later jobs that fit */
} hpsi_server_config;
typedef struct hpsi_request_times {
    double queue_ms, run_ms, total_ms;  /* submit->admit, admit->done, submit->done */
} hpsi_request_times;
typedef struct hpsi_server_statistics {
    long long completed;      /* requests retired */
    long long queued, running; /* jobs pending, jobs on the lanes */
    double budget_bytes, peak_bytes;
    long long units, merged_units, merged_jobs; /* units admitted; merged ones and their jobs */
} hpsi_server_statistics;
int hpsi_server_create(hpsi_ctx* const* systems, int n_systems, const hpsi_server_config* cfg, hpsi_server** out);
int hpsi_server_submit(hpsi_server* srv, const hpsi_job* jobs, int n_jobs, long long* ticket);
int hpsi_server_wait(hpsi_server* srv, long long ticket, double timeout_s, hpsi_request_times* times);
int hpsi_server_stats(hpsi_server* srv, hpsi_server_statistics* out);
int hpsi_server_destroy(hpsi_server* srv);
const char* hpsi_server_last_error(const hpsi_server* srv);

/* ---- Batched k-points: many (context, k-point, bands) items in one plan ----
 * A plan fixes a list of items (different k-points with ragged npw and band
 * counts, possibly of several contexts/cells) and keeps their psi and hpsi
 * resident on the device, packed item after item, each [nb][npw] band-major.
 * Per cell, each phase is one launch over all of the cell's items (scatter +
 * z/y FFT planes, x FFT/V/x FFT, y/z FFT planes + gather + kinetic, the ragged
 * projection GEMM, the split-K reduction with lambda, the expansion GEMM); the
 * cells run as parallel branches, the projections beside the FFTs, and the
 * whole sequence is captured in one CUDA graph.  At creation a tuner times the
 * candidate FFT block shapes, GEMM tiles and split-K counts on the plan's own
 * buffers and keeps the fastest (results are cached per shape for the
 * process).  Precisions: HPSI_PREC_FP64, HPSI_PREC_FP32, or HPSI_PREC_TC /
 * HPSI_PREC_TC_BF16 (the complex64 local term of FP32 and the nonlocal term as
 * ragged tensor-core GEMMs over the items, in blocks of up to 128 bands; a
 * bounded wait of those GEMMs that gives up is reported as HPSI_ERR_TIMEOUT by
 * a synchronising hpsi_batch_apply).  The items' slots
 * must stay bound: rebinding one makes later runs fail with HPSI_ERR_STATE;
 * destroy plans before their contexts.  The reference has no batched call: it
 * applies Callable::operator() per k-point and band
 * (src/H_psi/hamiltonian_callable.cpp:94-356). */
#define HPSI_BATCH_NO_GRAPH 0x100  /* run the launches eagerly instead of a graph */
#define HPSI_BATCH_NO_TUNE  0x200  /* built-in tile choices, no timing at creation */
typedef struct hpsi_batch hpsi_batch;
typedef struct hpsi_batch_item {
    hpsi_ctx* ctx;
    int kid;                  /* bound k-point slot of ctx */
    int nb;                   /* bands (0 allowed) */
} hpsi_batch_item;
int hpsi_batch_create(const hpsi_batch_item* items, int n_items, int flags, hpsi_batch** out);
/* Device buffers of the plan: psi and hpsi, n_complex complex<double> each. */
int hpsi_batch_buffers(hpsi_batch* b, double** psi, double** hpsi, size_t* n_complex);
/* Offset (in complex values) of item i in the packed buffers. */
int hpsi_batch_offset(const hpsi_batch* b, int item, size_t* offset);
/* hpsi_buffer += H psi_buffer for every item, queued on stream. */
int hpsi_batch_run(hpsi_batch* b, void* stream);
/* Copies psi and hpsi (packed, host or device per HPSI_DEVICE_PTRS) into the
 * plan's buffers, runs, and copies hpsi back (hpsi += H psi, as hpsi_apply). */
int hpsi_batch_apply(hpsi_batch* b, const double* psi, double* hpsi, int flags, void* stream);
/* The tuned choices as a JSON text; returns the length it needs (buf may be
 * NULL). */
int hpsi_batch_info(const hpsi_batch* b, char* buf, size_t len);
int hpsi_batch_destroy(hpsi_batch* b);
const char* hpsi_batch_last_error(const hpsi_batch* b);

/* Self-test of the integer-pipe FP64 <-> FP32 conversions the complex64
 * kernels use: for n doubles x (host memory) returns the conversion to float
 * by bit arithmetic (f_bits) and by the hardware (f_hw), and the conversion of
 * f_hw back to double both ways (d_bits, d_hw).  No reference counterpart. */
int hpsi_selftest_convert(const double* x, long n, float* f_bits, float* f_hw, double* d_bits, double* d_hw);

/* Self-test of the device line transforms (no reference counterpart): the
 * reference's FFT3D (src/math/fft.cppm:60-85) on an n1 x n2 x n3 grid of
 * complex<double> in host memory, transformed in place: dir = +1 G->r
 * (unnormalised, exp(+i..)), -1 r->G (exp(-i..), 1/n per axis), lines along z,
 * then y, then x.  HPSI_PREC_FP64: the complex128 runtime-plan stages;
 * HPSI_PREC_FP32: complex64, with the compile-time plans and the x pass's
 * register transform when n1 = n2 = n3 is 24, 36, 64 or 72. */
int hpsi_selftest_fft3d(int n1, int n2, int n3, double* grid, int dir, int flags);

/* Self-test of the k-point tables (no reference counterpart): copies the
 * device Y_lm, dY_lm/dtheta, (1/sin theta) dY_lm/dphi ([3][(l_max+1)^2][npw];
 * the derivatives only with dbeta tables) and S_a(G) ([n_atoms][npw]
 * complex) of slot kid to host buffers (either may be NULL). */
int hpsi_selftest_kpoint_tables(hpsi_ctx* ctx, int kid, double* ylm, double* sf);

/* Test hook of the bounded pipeline waits (no reference counterpart): sets
 * the poll limit of the tensor-core GEMMs' MMA issuer for the current device
 * (0: its wait for a loaded stage gives up at once; polls < 0: back to the
 * default of about a second).  With a lowered limit the GEMM takes its error
 * path (error flag, abort, bounded drain of the copies in flight, TMEM freed)
 * and the next synchronising call returns HPSI_ERR_TIMEOUT. */
int hpsi_selftest_wait_limit(long polls);

/* Message of the last failed call on ctx (never NULL); with ctx == NULL the
 * message of the calling thread's last failed hpsi_ctx_create. */
const char* hpsi_last_error(const hpsi_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif
