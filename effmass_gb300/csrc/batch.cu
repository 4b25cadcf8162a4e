// batch.cu — batched k-point plans (hpsi_batch_*): many (cell, k-point,
// bands) items applied by one CUDA graph, with tile shapes chosen by timing.
//
// The reference applies H one k-point and one band at a time
// (Callable::operator(), src/H_psi/hamiltonian_callable.cpp:94-356); a k·p
// or band-structure run loops that over a Monkhorst-Pack grid.  Here the
// items of one cell (one hpsi_ctx) share every launch:
//   side stream : ragged projection GEMM over all items (split-K partials)
//   main stream : g2r planes -> x pass -> r2g planes over all items' bands,
//                 then (after the projection) the split-K reduction with
//                 lambda and the ragged expansion GEMM.
// Cells are independent branches.  The sequence is captured once into a CUDA
// graph, so a run is one graph launch whatever the number of k-points.
// Tensor-core plans (HPSI_PREC_TC / TC_BF16) run the nonlocal term as ragged
// tcgen05 GEMMs over an item table instead (tc_rag_project / tc_rag_expand:
// generated projector tiles per k-point, band operands of up to 128 bands per
// item), with the complex64 local term of the FP32 plans.
//
// Tuning: for each cell the plan times, on its own buffers, the x-pass line
// shapes (z-values x bands per block), the plane-kernel block size, the
// projection tile and split count, and the expansion tile; the fastest of
// each is kept and cached per shape for the life of the process.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>

#include "ctx.cuh"

namespace {

struct BItem {
    hpsi_ctx* ctx;
    int kid, nb, npw;
    long gen;
    size_t off;  // complex offset in the packed buffers
};

struct Tune {
    int kt = 0, bb = 0, plane_threads = 0;
    int proj_tile = 3, exp_tile = 3, nsplit = 1;
    double local_ms = 0, proj_ms = 0, exp_ms = 0;
    int candidates = 0;
};

struct Group {
    hpsi_ctx* ctx = nullptr;
    std::vector<int> items;  // batch item indices with nb > 0 and npw > 0
    int P = 0, nbands = 0, max_nxs = 0, nb_max = 0, npw_max = 0;
    size_t t_elems = 0;
    std::vector<LocalItem> litems;
    std::vector<BGemmItem> gitems;
    LocalItem* d_litems = nullptr;
    int* d_band_item = nullptr;
    int2* d_xblk = nullptr;  // room for nbands entries (bb = 1)
    int nxblk = 0;
    BGemmItem* d_gitems = nullptr;
    void* T = nullptr;
    void* part = nullptr;
    void* W = nullptr;       // reduced projections [P][nbands] (complex of the precision)
    int max_split = 1;
    LocalArgs la{};
    Tune tune;
    bool tuned = false, cached = false;
    cudaStream_t s_main = nullptr, s_side = nullptr;
    cudaEvent_t ev_proj = nullptr, ev_done = nullptr;
    // tensor-core plans: ragged items (<= 128 bands each) and their tables
    std::vector<TcRagItem> rag;
    TcRagItem* d_rag = nullptr;
    int2* d_rag_bands = nullptr;   // (item, band)
    int2* d_rag_rows = nullptr;    // (item, j < nbp)
    int2* d_rag_tiles = nullptr;   // (item, 128-row G tile)
    int rag_bands = 0, rag_rows = 0, rag_tiles = 0, rag_k1t_max = 0, rag_nz_max = 0;
    unsigned char* rag_mem = nullptr;
    unsigned* rag_rowmax = nullptr;
    size_t rag_nrowmax = 0;
};

constexpr int kSplits[] = {1, 2, 4, 8, 16, 32};
constexpr size_t kPartBudget = 256ull << 20;  // bytes of split-K partials a cell may use
constexpr int kGridYZ = 65535;

std::mutex g_tune_mu;
std::map<std::string, Tune> g_tune_cache;

}  // namespace

struct hpsi_batch {
    int dev = 0;
    int prec = HPSI_PREC_FP32;
    bool use_graph = true, tuned = false;
    std::vector<BItem> items;
    size_t n_complex = 0;
    double2* psi = nullptr;
    double2* hpsi = nullptr;
    std::vector<Group> groups;
    cudaStream_t s_cap = nullptr;
    cudaEvent_t ev_start = nullptr, t0 = nullptr, t1 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    double tune_ms = 0;
    std::string err;
};

static int bfail(hpsi_batch* b, int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (b) b->err = buf;
    g_last_error = buf;
    return code;
}

#define BCUDA(b, expr)                                                                                  \
    do {                                                                                                \
        cudaError_t e_ = (expr);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? HPSI_ERR_OOM : HPSI_ERR_CUDA, "%s: %s (%s:%d)", \
                         #expr, cudaGetErrorString(e_), __FILE__, __LINE__);                            \
    } while (0)

static void batch_free(hpsi_batch* b)
{
    if (!b) return;
    cudaSetDevice(b->dev);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (Group& g : b->groups) {
        if (g.s_main) cudaStreamSynchronize(g.s_main);
        if (g.s_side) cudaStreamSynchronize(g.s_side);
        dfree(g.d_litems); dfree(g.d_band_item); dfree(g.d_xblk); dfree(g.d_gitems);
        dfree(g.d_rag); dfree(g.d_rag_bands); dfree(g.d_rag_rows); dfree(g.d_rag_tiles); dfree(g.rag_mem);
        if (g.T) cudaFree(g.T);
        if (g.part) cudaFree(g.part);
        if (g.W) cudaFree(g.W);
        if (g.s_main) cudaStreamDestroy(g.s_main);
        if (g.s_side) cudaStreamDestroy(g.s_side);
        if (g.ev_proj) cudaEventDestroy(g.ev_proj);
        if (g.ev_done) cudaEventDestroy(g.ev_done);
    }
    if (b->s_cap) cudaStreamDestroy(b->s_cap);
    for (cudaEvent_t e : {b->ev_start, b->t0, b->t1})
        if (e) cudaEventDestroy(e);
    dfree(b->psi);
    dfree(b->hpsi);
    delete b;
}

static bool fp64(const hpsi_batch* b) { return b->prec == HPSI_PREC_FP64; }
static bool tc(const hpsi_batch* b) { return b->prec == HPSI_PREC_TC || b->prec == HPSI_PREC_TC_BF16; }
static size_t csize(const hpsi_batch* b) { return fp64(b) ? sizeof(double2) : sizeof(float2); }

// x-pass band blocks of the current la.bb, uploaded to g.d_xblk
static int upload_xblk(hpsi_batch* b, Group& g)
{
    std::vector<int2> xb;
    for (size_t i = 0; i < g.litems.size(); ++i)
        for (int b0 = 0; b0 < g.litems[i].nb; b0 += g.la.bb) xb.push_back(make_int2((int)i, b0));
    g.nxblk = (int)xb.size();
    BCUDA(b, cudaMemcpy(g.d_xblk, xb.data(), xb.size() * sizeof(int2), cudaMemcpyHostToDevice));
    return HPSI_OK;
}

// GEMM items with the partial offsets of a split count, uploaded to g.d_gitems
static int upload_gitems(hpsi_batch* b, Group& g, int nsplit)
{
    size_t band0 = 0;
    for (BGemmItem& it : g.gitems) {
        it.part_off = (size_t)nsplit * g.P * band0;
        band0 += it.nb;
    }
    BCUDA(b, cudaMemcpy(g.d_gitems, g.gitems.data(), g.gitems.size() * sizeof(BGemmItem), cudaMemcpyHostToDevice));
    return HPSI_OK;
}

static cudaError_t launch_group_local(const hpsi_batch* b, const Group& g, cudaStream_t st)
{
    const hpsi_ctx* c = g.ctx;
    if (fp64(b))
        return launch_local_batch<double2, double>(g.la, g.nbands, g.max_nxs, g.nxblk, (double2*)g.T, c->d_v64,
                                                   c->d_tw64, c->d_tw64 + c->n1, c->d_tw64 + c->n1 + c->n2, st);
    return launch_local_batch<float2, float>(g.la, g.nbands, g.max_nxs, g.nxblk, (float2*)g.T, c->d_v32, c->d_tw32,
                                             c->d_tw32 + c->n1, c->d_tw32 + c->n1 + c->n2, st);
}

static cudaError_t launch_group_rag_proj(const hpsi_batch* b, const Group& g, cudaStream_t st)
{
    return tc_rag_project(g.d_rag, (int)g.rag.size(), g.d_rag_bands, g.rag_bands, g.d_rag_rows, g.rag_rows, g.P,
                          g.rag_k1t_max, g.rag_nz_max, b->prec == HPSI_PREC_TC, g.rag_rowmax, g.rag_nrowmax,
                          g.ctx->d_err, st);
}

static cudaError_t launch_group_rag_exp(const hpsi_batch* b, const Group& g, cudaStream_t st)
{
    return tc_rag_expand(g.d_rag, g.d_rag_tiles, g.rag_tiles, g.P, b->prec == HPSI_PREC_TC, g.ctx->d_err, st);
}

static cudaError_t launch_group_proj(const hpsi_batch* b, const Group& g, int tile, int nsplit, cudaStream_t st)
{
    if (fp64(b))
        return launch_bproj<double2, double2>(g.P, g.d_gitems, (int)g.gitems.size(), g.nb_max, nsplit, tile,
                                              (double2*)g.part, st);
    return launch_bproj<float2, float2>(g.P, g.d_gitems, (int)g.gitems.size(), g.nb_max, nsplit, tile,
                                        (float2*)g.part, st);
}

static cudaError_t launch_group_exp(const hpsi_batch* b, const Group& g, int tile, int nsplit, cudaStream_t st)
{
    if (fp64(b))
        return launch_bexp<double2, double2>(g.P, g.d_gitems, (int)g.gitems.size(), g.nb_max, g.npw_max, nsplit,
                                             tile, (const double2*)g.part, (double2*)g.W, st);
    return launch_bexp<float2, float2>(g.P, g.d_gitems, (int)g.gitems.size(), g.nb_max, g.npw_max, nsplit, tile,
                                       (const float2*)g.part, (float2*)g.W, st);
}

// mean milliseconds of fn over reps launches on st (after one untimed launch)
template <typename F>
static int time_ms(hpsi_batch* b, cudaStream_t st, int reps, F&& fn, double* ms)
{
    BCUDA(b, fn());
    BCUDA(b, cudaEventRecord(b->t0, st));
    for (int r = 0; r < reps; ++r) BCUDA(b, fn());
    BCUDA(b, cudaEventRecord(b->t1, st));
    BCUDA(b, cudaEventSynchronize(b->t1));
    float f = 0;
    BCUDA(b, cudaEventElapsedTime(&f, b->t0, b->t1));
    *ms = f / reps;
    return HPSI_OK;
}

static std::string tune_key(const hpsi_batch* b, const Group& g)
{
    const hpsi_ctx* c = g.ctx;
    long sum_npw = 0;
    for (const LocalItem& it : g.litems) sum_npw += (long)it.npw * it.nb;
    char buf[256];
    snprintf(buf, sizeof buf, "%d|%dx%dx%d|P%d|i%zu|b%d|nb%d|npw%d|s%ld|x%d", b->prec, c->n1, c->n2, c->n3, g.P,
             g.litems.size(), g.nbands, g.nb_max, g.npw_max, sum_npw, g.max_nxs);
    return buf;
}

static bool xshape_ok(const hpsi_batch* b, const Group& g, int kt, int bb)
{
    LocalArgs a = g.la;
    a.kt = kt;
    a.bb = bb;
    const size_t limit = fp64(b) ? 160 * 1024 : 96 * 1024;
    if (local_xpass_smem(a, fp64(b)) > limit) return false;
    long nxblk = 0;
    for (const LocalItem& it : g.litems) nxblk += ceil_div(it.nb, bb);
    return nxblk <= kGridYZ;
}

static void set_xshape(Group& g, int kt, int bb)
{
    g.la.kt = kt;
    g.la.bb = bb;
    g.la.nl_x = make_fastdiv((uint32_t)(kt * bb));
    g.la.kt_f = make_fastdiv((uint32_t)kt);
}

static int tune_group(hpsi_batch* b, Group& g)
{
    cudaStream_t st = g.s_main;
    int rc;
    const int reps = 3;
    Tune t;
    // local term: x-pass shapes at the default plane block, then plane blocks
    double best = 1e30;
    int bk = g.la.kt, bbb = g.la.bb;
    for (int nl : {4, 8, 16, 32, 64, 128}) {
        for (int kt : {1, 2, 4, 8}) {
            if (kt > nl || kt > g.ctx->n3) continue;
            const int bb = nl / kt;
            if (!xshape_ok(b, g, kt, bb)) continue;
            set_xshape(g, kt, bb);
            if ((rc = upload_xblk(b, g))) return rc;
            double ms = 0.0;
            if ((rc = time_ms(b, st, reps, [&] { return launch_group_local(b, g, st); }, &ms))) return rc;
            ++t.candidates;
            if (ms < best) { best = ms; bk = kt; bbb = bb; }
        }
    }
    set_xshape(g, bk, bbb);
    if ((rc = upload_xblk(b, g))) return rc;
    // plane blocks: a candidate replaces the default block size (timed in the
    // x-pass search above, bpt = 0) only when it is faster
    int bpt = 0;
    static const int kPlaneThreads64[] = {64, 128, 256, 0}, kPlaneThreads32[] = {128, 256, 512, 768};
    const int* cand = fp64(b) ? kPlaneThreads64 : kPlaneThreads32;
    for (int ci = 0; ci < 4 && cand[ci] > 0; ++ci) {
        const int pt = cand[ci];
        g.la.plane_threads = pt;
        double ms = 0.0;
        if ((rc = time_ms(b, st, reps, [&] { return launch_group_local(b, g, st); }, &ms))) return rc;
        ++t.candidates;
        if (ms < best) { best = ms; bpt = pt; }
    }
    g.la.plane_threads = bpt;
    t.kt = bk; t.bb = bbb; t.plane_threads = bpt; t.local_ms = best;
    if (tc(b)) {
        // the ragged tensor-core GEMMs have no shape to choose: timed for the report
        if (g.P > 0) {
            if ((rc = time_ms(b, st, reps, [&] { return launch_group_rag_proj(b, g, st); }, &t.proj_ms))) return rc;
            if ((rc = time_ms(b, st, reps, [&] { return launch_group_rag_exp(b, g, st); }, &t.exp_ms))) return rc;
        }
        g.tune = t;
        g.tuned = true;
        return HPSI_OK;
    }
    // projection: tile x split
    best = 1e30;
    for (int ns : kSplits) {
        if (ns > g.max_split || (ns > 1 && g.npw_max / ns < 64)) continue;
        if ((long)g.gitems.size() * ns > kGridYZ) continue;
        if ((rc = upload_gitems(b, g, ns))) return rc;
        for (int tile = 0; tile < bgemm_tile_count(); ++tile) {
            double ms = 0.0;
            if ((rc = time_ms(b, st, reps, [&] { return launch_group_proj(b, g, tile, ns, st); }, &ms))) return rc;
            ++t.candidates;
            if (ms < best) { best = ms; t.proj_tile = tile; t.nsplit = ns; }
        }
    }
    t.proj_ms = best;
    if ((rc = upload_gitems(b, g, t.nsplit))) return rc;
    // expansion tile (with the split reduction) at the chosen split, on the partials of the chosen projection
    BCUDA(b, launch_group_proj(b, g, t.proj_tile, t.nsplit, st));
    best = 1e30;
    for (int tile = 0; tile < bgemm_tile_count(); ++tile) {
        double ms = 0.0;
        if ((rc = time_ms(b, st, reps, [&] { return launch_group_exp(b, g, tile, t.nsplit, st); }, &ms))) return rc;
        ++t.candidates;
        if (ms < best) { best = ms; t.exp_tile = tile; }
    }
    t.exp_ms = best;
    g.tune = t;
    g.tuned = true;
    return HPSI_OK;
}

// default choices without timing
static void default_tune(Group& g)
{
    Tune t;
    t.kt = g.la.kt;
    t.bb = g.la.bb;
    t.plane_threads = 0;
    t.proj_tile = g.P <= 16 ? 0 : 3;
    t.exp_tile = 3;
    int ns = 1;
    const long blocks = (long)g.gitems.size() * ceil_div(g.P, 32) * ceil_div(g.nb_max, 64);
    while (ns < g.max_split && blocks * ns < 2 * 152 && g.npw_max / (2 * ns) >= 64) ns *= 2;
    t.nsplit = ns;
    g.tune = t;
}

static int apply_tune(hpsi_batch* b, Group& g)
{
    int rc;
    set_xshape(g, g.tune.kt, g.tune.bb);
    g.la.plane_threads = g.tune.plane_threads;
    if ((rc = upload_xblk(b, g))) return rc;
    if (tc(b)) return HPSI_OK;
    return upload_gitems(b, g, g.tune.nsplit);
}

// Queue one application of the whole batch, forking from and joining into origin.
static int enqueue(hpsi_batch* b, cudaStream_t origin)
{
    BCUDA(b, cudaEventRecord(b->ev_start, origin));
    for (Group& g : b->groups) {
        BCUDA(b, cudaStreamWaitEvent(g.s_side, b->ev_start, 0));
        BCUDA(b, cudaStreamWaitEvent(g.s_main, b->ev_start, 0));
        if (tc(b)) BCUDA(b, launch_group_rag_proj(b, g, g.s_side));
        else BCUDA(b, launch_group_proj(b, g, g.tune.proj_tile, g.tune.nsplit, g.s_side));
        BCUDA(b, cudaEventRecord(g.ev_proj, g.s_side));
        BCUDA(b, launch_group_local(b, g, g.s_main));
        BCUDA(b, cudaStreamWaitEvent(g.s_main, g.ev_proj, 0));
        if (tc(b)) BCUDA(b, launch_group_rag_exp(b, g, g.s_main));
        else BCUDA(b, launch_group_exp(b, g, g.tune.exp_tile, g.tune.nsplit, g.s_main));
        BCUDA(b, cudaEventRecord(g.ev_done, g.s_main));
        BCUDA(b, cudaStreamWaitEvent(origin, g.ev_done, 0));
    }
    return HPSI_OK;
}

// Ragged tensor-core items of a cell: one per (k-point, block of <= 128
// bands), their operand workspace carved from one allocation, and the band,
// row and tile tables of the launches.  Splits: K per split chosen so that
// the projection fills about two waves of the SMs, at most 96 k-tiles (3072
// of K) per FP32 accumulation chain.
static int build_rag(hpsi_batch* b, Group& g)
{
    hpsi_ctx* c = g.ctx;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t k2 = tc_round_k(2 * (size_t)g.P);
    long kt_sum = 0;
    for (size_t i = 0; i < g.items.size(); ++i) {
        const KSlot& s = c->slots[b->items[g.items[i]].kid];
        const int nbk = ceil_div(b->items[g.items[i]].nb, 128);
        kt_sum += (long)nbk * (long)(tc_round_k(2 * (size_t)s.npw) / 32);
    }
    int per = (int)std::max(1L, (kt_sum + 2L * sms - 1) / (2L * sms));
    per = std::min(per, 96);
    Carver cv;
    struct Off { size_t b1h, b1l, b1s, part, w, b2h, b2l, b2s, rm; };
    std::vector<Off> offs;
    std::vector<int2> bands, rows, tiles;
    g.rag.clear();
    for (size_t i = 0; i < g.items.size(); ++i) {
        const BItem& it = b->items[g.items[i]];
        KSlot& s = c->slots[it.kid];
        for (int b0 = 0; b0 < it.nb; b0 += 128) {
            TcRagItem r{};
            r.gen = s.tcgen[b->prec == HPSI_PREC_TC ? 0 : 1];
            r.psi = b->psi + it.off + (size_t)b0 * s.npw;
            r.hpsi = b->hpsi + it.off + (size_t)b0 * s.npw;
            r.lam = s.d_lam;
            r.nb = std::min(128, it.nb - b0);
            r.nbp = tc_rag_nbp(r.nb);
            r.npw = s.npw;
            r.k1t = (int)(tc_round_k(2 * (size_t)s.npw) / 32);
            r.per = per;
            r.nz = ceil_div(r.k1t, per);
            const size_t rp = tc_rows_pad(2 * (size_t)r.nbp), k1 = (size_t)r.k1t * 32;
            Off o;
            o.b1h = cv.take<uint16_t>(rp * k1);
            o.b1l = cv.take<uint16_t>(rp * k1);
            o.b1s = cv.take<float>(2 * (size_t)r.nbp);
            o.part = cv.take<float>((size_t)r.nz * g.P * 2 * r.nbp);
            o.w = cv.take<float2>((size_t)g.P * r.nb);
            o.b2h = cv.take<uint16_t>(rp * k2);
            o.b2l = cv.take<uint16_t>(rp * k2);
            o.b2s = cv.take<float>(2 * (size_t)r.nbp);
            offs.push_back(o);
            const int ri = (int)g.rag.size();
            for (int j = 0; j < r.nb; ++j) bands.push_back(make_int2(ri, j));
            for (int j = 0; j < r.nbp; ++j) rows.push_back(make_int2(ri, j));
            for (int t = 0; t < ceil_div(s.npw, 128); ++t) tiles.push_back(make_int2(ri, t));
            g.rag_k1t_max = std::max(g.rag_k1t_max, r.k1t);
            g.rag_nz_max = std::max(g.rag_nz_max, r.nz);
            g.rag.push_back(r);
        }
    }
    // band maxima of every item, contiguous (one memset per operand build)
    const size_t rm0 = cv.off;
    size_t nrm = 0;
    for (TcRagItem& r : g.rag) nrm += (size_t)r.nbp;
    cv.take<unsigned>(nrm);
    if (g.rag.size() > 65535 || rows.size() > 65535 || bands.size() > 65535)
        return bfail(b, HPSI_ERR_BAD_ARG, "a tensor-core plan holds at most 65535 bands of one cell");
    BCUDA(b, dalloc(&g.rag_mem, cv.off));
    BCUDA(b, cudaMemset(g.rag_mem, 0, cv.off));
    g.rag_rowmax = reinterpret_cast<unsigned*>(g.rag_mem + rm0);
    g.rag_nrowmax = nrm;
    size_t rmo = 0;
    for (size_t i = 0; i < g.rag.size(); ++i) {
        TcRagItem& r = g.rag[i];
        const Off& o = offs[i];
        r.b1h = g.rag_mem + o.b1h;
        r.b1l = g.rag_mem + o.b1l;
        r.b1s = reinterpret_cast<float*>(g.rag_mem + o.b1s);
        r.part = reinterpret_cast<float*>(g.rag_mem + o.part);
        r.W = reinterpret_cast<float2*>(g.rag_mem + o.w);
        r.b2h = g.rag_mem + o.b2h;
        r.b2l = g.rag_mem + o.b2l;
        r.b2s = reinterpret_cast<float*>(g.rag_mem + o.b2s);
        r.rowmax = g.rag_rowmax + rmo;
        rmo += (size_t)r.nbp;
    }
    g.rag_bands = (int)bands.size();
    g.rag_rows = (int)rows.size();
    g.rag_tiles = (int)tiles.size();
    BCUDA(b, dalloc(&g.d_rag, g.rag.size()));
    BCUDA(b, dalloc(&g.d_rag_bands, bands.size()));
    BCUDA(b, dalloc(&g.d_rag_rows, rows.size()));
    BCUDA(b, dalloc(&g.d_rag_tiles, tiles.size()));
    BCUDA(b, cudaMemcpy(g.d_rag, g.rag.data(), g.rag.size() * sizeof(TcRagItem), cudaMemcpyHostToDevice));
    BCUDA(b, cudaMemcpy(g.d_rag_bands, bands.data(), bands.size() * sizeof(int2), cudaMemcpyHostToDevice));
    BCUDA(b, cudaMemcpy(g.d_rag_rows, rows.data(), rows.size() * sizeof(int2), cudaMemcpyHostToDevice));
    BCUDA(b, cudaMemcpy(g.d_rag_tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice));
    return HPSI_OK;
}

static int build_group(hpsi_batch* b, Group& g)
{
    hpsi_ctx* c = g.ctx;
    const size_t cs = csize(b);
    g.litems.clear();
    g.gitems.clear();
    std::vector<int> band_item;
    size_t t_off = 0;
    for (int idx : g.items) {
        const BItem& it = b->items[idx];
        KSlot& s = c->slots[it.kid];
        // the batched nonlocal term reads the complex64 (or complex128) projector
        // matrix, or, on the tensor cores, the k-point's generator tables
        int rc = prepare_slot(c, s, tc(b) ? b->prec : (fp64(b) ? HPSI_PREC_FP64 : HPSI_PREC_FP32), false, 0);
        if (rc) return bfail(b, rc, "item %d: %s", idx, c->err.c_str());
        if (g.litems.empty()) g.P = s.P;
        if (s.P != g.P) return bfail(b, HPSI_ERR_STATE, "item %d: projector count differs within a cell", idx);
        const int* pl = s.d_plane;
        LocalItem li{};
        li.plane_x = pl;
        li.plane_off = pl + s.nxs;
        li.ent_ig = pl + 2 * s.nxs + 1;
        li.ent_jk = pl + 2 * s.nxs + 1 + s.npw;
        li.plane_jr = pl + 2 * s.nxs + 1 + 2 * s.npw;
        li.kinetic = s.d_kin;
        li.psi = b->psi + it.off;
        li.hpsi = b->hpsi + it.off;
        li.t_off = t_off;
        li.npw = s.npw;
        li.nxs = s.nxs;
        li.nb = it.nb;
        li.band0 = g.nbands;
        for (int k = 0; k < it.nb; ++k) band_item.push_back((int)g.litems.size());
        t_off += (size_t)it.nb * s.nxs * c->n2 * c->n3;
        g.litems.push_back(li);
        BGemmItem gi{};
        gi.pr = fp64(b) ? (const void*)s.pr64 : (const void*)s.pr32;
        gi.psi = li.psi;
        gi.hpsi = li.hpsi;
        gi.lam = s.d_lam;
        gi.w_off = (size_t)g.P * g.nbands;
        gi.nb = it.nb;
        gi.npw = s.npw;
        g.gitems.push_back(gi);
        g.nbands += it.nb;
        g.max_nxs = std::max(g.max_nxs, s.nxs);
        g.nb_max = std::max(g.nb_max, it.nb);
        g.npw_max = std::max(g.npw_max, s.npw);
    }
    if (g.nbands > kGridYZ)
        return bfail(b, HPSI_ERR_BAD_ARG, "a cell holds %d bands in one plan (at most %d)", g.nbands, kGridYZ);
    if (g.P > 0 && (long)g.gitems.size() > kGridYZ)
        return bfail(b, HPSI_ERR_BAD_ARG, "too many k-points of one cell in one plan (at most %d)", kGridYZ);
    g.t_elems = t_off;
    BCUDA(b, cudaDeviceSynchronize());
    // device tables and buffers
    BCUDA(b, dalloc(&g.d_litems, g.litems.size()));
    BCUDA(b, dalloc(&g.d_band_item, band_item.size()));
    BCUDA(b, dalloc(&g.d_xblk, (size_t)g.nbands));
    BCUDA(b, dalloc(&g.d_gitems, g.gitems.size()));
    BCUDA(b, cudaMemcpy(g.d_litems, g.litems.data(), g.litems.size() * sizeof(LocalItem), cudaMemcpyHostToDevice));
    BCUDA(b, cudaMemcpy(g.d_band_item, band_item.data(), band_item.size() * sizeof(int), cudaMemcpyHostToDevice));
    BCUDA(b, cudaMalloc(&g.T, std::max<size_t>(g.t_elems, 1) * cs));
    g.max_split = 1;
    if (g.P > 0 && tc(b)) {
        int rc = build_rag(b, g);
        if (rc) return rc;
    } else if (g.P > 0) {
        for (int ns : kSplits)
            if ((size_t)ns * g.P * g.nbands * cs <= kPartBudget) g.max_split = ns;
        BCUDA(b, cudaMalloc(&g.part, (size_t)g.max_split * g.P * g.nbands * cs));
        BCUDA(b, cudaMalloc(&g.W, (size_t)g.P * g.nbands * cs));
    }
    // local arguments shared by every launch of the cell
    LocalArgs& a = g.la;
    a = LocalArgs{};
    a.n1 = c->n1; a.n2 = c->n2; a.n3 = c->n3;
    a.inv_n = 1.0 / ((double)c->n1 * c->n2 * c->n3);
    a.Lx = c->L[0]; a.Ly = c->L[1]; a.Lz = c->L[2];
    local_xpass_shape(&a, cs);
    a.items = g.d_litems;
    a.band_item = g.d_band_item;
    a.xblk = g.d_xblk;
    BCUDA(b, cudaStreamCreateWithFlags(&g.s_main, cudaStreamNonBlocking));
    BCUDA(b, cudaStreamCreateWithFlags(&g.s_side, cudaStreamNonBlocking));
    BCUDA(b, cudaEventCreateWithFlags(&g.ev_proj, cudaEventDisableTiming));
    BCUDA(b, cudaEventCreateWithFlags(&g.ev_done, cudaEventDisableTiming));
    return HPSI_OK;
}

static int batch_init(hpsi_batch* b, const hpsi_batch_item* items, int n_items, bool tune)
{
    // items, offsets, cells
    std::map<hpsi_ctx*, int> group_of;
    for (int i = 0; i < n_items; ++i) {
        hpsi_ctx* c = items[i].ctx;
        if (!c) return bfail(b, HPSI_ERR_BAD_ARG, "item %d: ctx is NULL", i);
        if (items[i].nb < 0) return bfail(b, HPSI_ERR_BAD_ARG, "item %d: nb < 0", i);
        if (i == 0) b->dev = c->dev;
        if (c->dev != b->dev) return bfail(b, HPSI_ERR_BAD_ARG, "item %d: contexts on different devices", i);
        auto it = c->slots.find(items[i].kid);
        if (it == c->slots.end() || !it->second.valid)
            return bfail(b, HPSI_ERR_STATE, "item %d: k-point slot %d is not bound", i, items[i].kid);
        BItem bi{c, items[i].kid, items[i].nb, it->second.npw, it->second.gen, b->n_complex};
        b->n_complex += (size_t)bi.nb * bi.npw;
        b->items.push_back(bi);
        if (bi.nb > 0 && bi.npw > 0) {
            auto g = group_of.find(c);
            if (g == group_of.end()) {
                group_of[c] = (int)b->groups.size();
                b->groups.emplace_back();
                b->groups.back().ctx = c;
                b->groups.back().items.push_back(i);
            } else {
                b->groups[g->second].items.push_back(i);
            }
        }
    }
    BCUDA(b, cudaSetDevice(b->dev));
    BCUDA(b, dalloc(&b->psi, std::max<size_t>(b->n_complex, 1)));
    BCUDA(b, dalloc(&b->hpsi, std::max<size_t>(b->n_complex, 1)));
    BCUDA(b, cudaMemset(b->psi, 0, std::max<size_t>(b->n_complex, 1) * sizeof(double2)));
    BCUDA(b, cudaStreamCreateWithFlags(&b->s_cap, cudaStreamNonBlocking));
    BCUDA(b, cudaEventCreateWithFlags(&b->ev_start, cudaEventDisableTiming));
    BCUDA(b, cudaEventCreate(&b->t0));
    BCUDA(b, cudaEventCreate(&b->t1));
    int rc = HPSI_OK;
    for (Group& g : b->groups)
        if ((rc = build_group(b, g))) return rc;
    // tile choices: cached, timed, or built in
    b->tuned = tune;
    const auto t_start = std::chrono::steady_clock::now();
    for (Group& g : b->groups) {
        if (!tune) { default_tune(g); continue; }
        const std::string key = tune_key(b, g);
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end()) { g.tune = it->second; g.tuned = g.cached = true; continue; }
        }
        if ((rc = tune_group(b, g))) break;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = g.tune;
    }
    if (rc) return rc;
    b->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    for (Group& g : b->groups)
        if ((rc = apply_tune(b, g))) return rc;
    BCUDA(b, cudaDeviceSynchronize());
    // the tuning runs wrote into hpsi and T
    BCUDA(b, cudaMemset(b->hpsi, 0, std::max<size_t>(b->n_complex, 1) * sizeof(double2)));
    if (b->use_graph) {
        BCUDA(b, cudaStreamBeginCapture(b->s_cap, cudaStreamCaptureModeThreadLocal));
        rc = enqueue(b, b->s_cap);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->s_cap, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        BCUDA(b, e);
        b->graph = graph;
        BCUDA(b, cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    return HPSI_OK;
}

static int batch_check(hpsi_batch* b)
{
    for (size_t i = 0; i < b->items.size(); ++i) {
        const BItem& it = b->items[i];
        auto s = it.ctx->slots.find(it.kid);
        if (s == it.ctx->slots.end() || !s->second.valid || s->second.gen != it.gen)
            return bfail(b, HPSI_ERR_STATE, "item %zu: k-point slot %d was rebound after the plan was made", i, it.kid);
    }
    return HPSI_OK;
}

extern "C" int hpsi_batch_create(const hpsi_batch_item* items, int n_items, int flags, hpsi_batch** out)
{
    if (!out) return bfail(nullptr, HPSI_ERR_BAD_ARG, "out is NULL");
    *out = nullptr;
    if (n_items <= 0 || !items) return bfail(nullptr, HPSI_ERR_BAD_ARG, "a batch needs at least one item");
    const int prec = flags & HPSI_PREC_MASK;
    if (prec != HPSI_PREC_FP64 && prec != HPSI_PREC_FP32 && prec != HPSI_PREC_TC && prec != HPSI_PREC_TC_BF16)
        return bfail(nullptr, HPSI_ERR_BAD_ARG,
                     "batched plans run HPSI_PREC_FP64, HPSI_PREC_FP32, HPSI_PREC_TC or HPSI_PREC_TC_BF16 (got %d)", prec);
    hpsi_batch* b = new hpsi_batch();
    b->prec = prec;
    b->use_graph = !(flags & HPSI_BATCH_NO_GRAPH);
    int rc = batch_init(b, items, n_items, !(flags & HPSI_BATCH_NO_TUNE));
    if (rc) {
        g_last_error = b->err;
        batch_free(b);
        return rc;
    }
    *out = b;
    return HPSI_OK;
}

extern "C" int hpsi_batch_buffers(hpsi_batch* b, double** psi, double** hpsi, size_t* n_complex)
{
    if (!b) return HPSI_ERR_BAD_ARG;
    if (psi) *psi = (double*)b->psi;
    if (hpsi) *hpsi = (double*)b->hpsi;
    if (n_complex) *n_complex = b->n_complex;
    return HPSI_OK;
}

extern "C" int hpsi_batch_offset(const hpsi_batch* b, int item, size_t* offset)
{
    if (!b || !offset || item < 0 || item >= (int)b->items.size()) return HPSI_ERR_BAD_ARG;
    *offset = b->items[item].off;
    return HPSI_OK;
}

extern "C" int hpsi_batch_run(hpsi_batch* b, void* stream)
{
    if (!b) return HPSI_ERR_BAD_ARG;
    int rc = batch_check(b);
    if (rc) return rc;
    BCUDA(b, cudaSetDevice(b->dev));
    cudaStream_t st = (cudaStream_t)stream;
    if (b->exec) {
        BCUDA(b, cudaGraphLaunch(b->exec, st));
        return HPSI_OK;
    }
    return enqueue(b, st);
}

extern "C" int hpsi_batch_apply(hpsi_batch* b, const double* psi, double* hpsi, int flags, void* stream)
{
    if (!b) return HPSI_ERR_BAD_ARG;
    if (b->n_complex && (!psi || !hpsi)) return bfail(b, HPSI_ERR_BAD_ARG, "psi/hpsi NULL");
    int rc = batch_check(b);
    if (rc) return rc;
    BCUDA(b, cudaSetDevice(b->dev));
    cudaStream_t st = (cudaStream_t)stream;
    const bool dev = flags & HPSI_DEVICE_PTRS;
    const cudaMemcpyKind in = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const cudaMemcpyKind out = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t bytes = b->n_complex * sizeof(double2);
    if (bytes) {
        BCUDA(b, cudaMemcpyAsync(b->psi, psi, bytes, in, st));
        BCUDA(b, cudaMemcpyAsync(b->hpsi, hpsi, bytes, in, st));
    }
    if ((rc = hpsi_batch_run(b, stream))) return rc;
    if (bytes) BCUDA(b, cudaMemcpyAsync(hpsi, b->hpsi, bytes, out, st));
    if (!dev || (flags & HPSI_SYNC)) {
        BCUDA(b, cudaStreamSynchronize(st));
        if (tc(b)) {
            // a bounded wait of the tensor-core GEMMs that gave up (any cell)
            for (const Group& g : b->groups) {
                int v = 0;
                BCUDA(b, cudaMemcpy(&v, g.ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
                if (v) {
                    cudaMemset(g.ctx->d_err, 0, sizeof(int));
                    return bfail(b, HPSI_ERR_TIMEOUT, "tensor-core GEMM: a bounded pipeline wait gave up (site %d)", v);
                }
            }
        }
    }
    return HPSI_OK;
}

extern "C" int hpsi_batch_info(const hpsi_batch* b, char* buf, size_t len)
{
    if (!b) return HPSI_ERR_BAD_ARG;
    std::string s;
    char t[768];
    snprintf(t, sizeof t, "{\"precision\": \"%s\", \"graph\": %s, \"tuned\": %s, \"tune_ms\": %.3f, \"items\": %zu, "
             "\"cells\": [", fp64(b) ? "fp64" : (b->prec == HPSI_PREC_TC ? "tc" : (tc(b) ? "tc_bf16" : "fp32")), b->exec ? "true" : "false", b->tuned ? "true" : "false",
             b->tune_ms, b->items.size());
    s += t;
    for (size_t i = 0; i < b->groups.size(); ++i) {
        const Group& g = b->groups[i];
        int ptm, ptn, etm, etn;
        bgemm_tile_shape(g.tune.proj_tile, &ptm, &ptn);
        bgemm_tile_shape(g.tune.exp_tile, &etm, &etn);
        snprintf(t, sizeof t,
                 "%s{\"grid\": [%d, %d, %d], \"kpoints\": %zu, \"bands\": %d, \"projectors\": %d, \"npw_max\": %d, "
                 "\"x_pass\": {\"z_per_block\": %d, \"bands_per_block\": %d}, \"plane_threads\": %d, "
                 "\"proj_tile\": [%d, %d], \"nsplit\": %d, \"exp_tile\": [%d, %d], \"timed\": {\"local_ms\": %.4f, "
                 "\"proj_ms\": %.4f, \"exp_ms\": %.4f}, \"candidates\": %d, \"cached\": %s}",
                 i ? ", " : "", g.ctx->n1, g.ctx->n2, g.ctx->n3, g.litems.size(), g.nbands, g.P, g.npw_max, g.la.kt,
                 g.la.bb, g.la.plane_threads, 16 * ptm, 16 * ptn, g.tune.nsplit, 16 * etm, 16 * etn, g.tune.local_ms,
                 g.tune.proj_ms, g.tune.exp_ms, g.tune.candidates, g.cached ? "true" : "false");
        s += t;
    }
    s += "]}";
    if (buf && len) {
        size_t n = std::min(len - 1, s.size());
        memcpy(buf, s.data(), n);
        buf[n] = 0;
    }
    return (int)s.size() + 1;
}

extern "C" int hpsi_batch_destroy(hpsi_batch* b)
{
    if (!b) return HPSI_ERR_BAD_ARG;
    batch_free(b);
    return HPSI_OK;
}

extern "C" const char* hpsi_batch_last_error(const hpsi_batch* b)
{
    if (!b) return g_last_error.c_str();
    return b->err.c_str();
}
