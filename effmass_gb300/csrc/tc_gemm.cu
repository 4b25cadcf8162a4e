// tc_gemm.cu — tensor-core (tcgen05) projector GEMMs for the nonlocal term.
//
// Both nonlocal GEMMs are cast as real "TN" GEMMs C[m][n] = sum_k A[m][k] B[n][k]
// with K-major operands:
//   projection  A = Pr      [P][2*npw]  (interleaved re/im of each projector row)
//               B = Psi'    [NB][2*npw] rows (psi_r, psi_i) and (psi_i, -psi_r)
//               C[p][.]     -> W[p][b] = lambda_p (C[p][re b] + i C[p][im b])
//   expansion   A = Pr^T    [npw][2*P]   (row g: (Pr_r, Pr_i)[p] interleaved)
//               B = W'      [NB][2*P]    rows (W_r, -W_i) and (W_i, W_r)
//               C[g][.]     -> hpsi[b][g] += C[g][re b] + i C[g][im b]
// Band rows are blocked by 128: row (t*256 + c*128 + j) holds band 128t+j, part c
// (0 = re, 1 = im), so an N tile of 256 holds both parts of 128 bands.
//
// Precision: every operand x is split as x*2^s = hi + lo in FP16 (s a per-row
// power of two that puts the row maximum at ~2^14) or in BF16 (s = 0); the
// product uses three MMAs hi*hi + hi*lo + lo*hi with FP32 accumulation in
// TMEM, and the epilogue removes 2^-(s_a + s_b).  FP16 pieces carry 11
// significand bits each, so hi+lo represents x to ~2^-22; BF16 pieces to ~2^-18.
//
// Kernels (cta_group::1, UMMA M=128, N=256, K=16; 32-deep K stages of A_hi,
// A_lo, B_hi, B_lo in four pipeline stages): warp 0 issues the bulk copies of
// the pre-tiled operands (see tile_off), warp 1 owns TMEM and issues the MMAs
// from one thread, the other warps drain TMEM.  With generator tables (TcGen)
// the A pieces are written in shared memory by eight generator warps instead
// of copied (H|psi> and band energies).
//   tc_gemm_kernel    one 128 x 256 tile per CTA, split over K (projection,
//                     complex128 band-pair GEMMs); partials per split
//   tc_expand_kernel  persistent over the tiles of the expansion, TMEM
//                     accumulators alternating by tile so that the hpsi
//                     read-modify-write of one tile overlaps the next's MMAs
//   rag_*             the batch plans' ragged GEMMs over an item table
// Every mbarrier wait is bounded; on timeout the CTA sets an error flag,
// drains its copies and frees TMEM.
#include <type_traits>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

#include "kernels.cuh"
#include "tc_gemm.cuh"

namespace {

constexpr int BM = 128, BN = 256, BK = 32, STAGES = 4;
constexpr int A_TILE = BM * BK * 2;   // bytes of one A piece per stage (8 KB)
constexpr int B_TILE = BN * BK * 2;   // 16 KB
constexpr int MAX_CHAIN_K = 3072;     // K depth of one split (FP32 accumulation chain length)
constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
constexpr uint32_t TMEM_COLS = 512;  // two 256-column FP32 accumulators, alternating by k-tile
constexpr uint32_t WAIT_LIMIT = 1u << 24;
static_assert(BK == 32 && BM == 128 && BN == 2 * BM, "tile_off assumes 128-row x 32-deep tiles");

// Tiled operand layout.  The K-major operands are stored as 128-row x BK
// tiles of 8 KB, each in the byte order that a TMA SWIZZLE_64B load would
// leave in shared memory (row r at 64 r bytes, its 16-byte chunk c at chunk
// c ^ ((r >> 1) & 3)), tiles ordered (row block, k block) with k fastest.  A
// pipeline stage then fills with six 8 KB bulk copies of contiguous HBM
// instead of tensor-map boxes of 64-byte rows a whole row stride apart.
__host__ __device__ __forceinline__ size_t tile_off(size_t row, size_t k, size_t ldk)
{
    const size_t r = row & 127, kk = k & 31;
    const size_t c = (kk >> 3) ^ ((r >> 1) & 3);
    return (((row >> 7) * (ldk >> 5) + (k >> 5)) << 12) + (r << 5) + (c << 3) + (kk & 7);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: false after WAIT_LIMIT polls (about a second)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
    for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if (i > 32) __nanosleep(40);
    }
    return false;
}

// bounded wait with a given poll limit (0: give up at once, without polling)
__device__ __forceinline__ bool mbar_wait_n(uint64_t* bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if (i > 32) __nanosleep(40);
    }
    return false;
}

// bounded wait that also gives up as soon as another thread of the CTA has
// set *abort (the producer's wait for a stage the MMA issuer will not free)
__device__ __forceinline__ bool mbar_wait_abort(uint64_t* bar, uint32_t parity, const uint32_t* abort)
{
    for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*(const volatile uint32_t*)abort) return false;
        if (i > 32) __nanosleep(40);
    }
    return false;
}

// Poll limit of the MMA issuer's wait for a loaded stage.  WAIT_LIMIT unless a
// test lowers it (tc_set_issue_wait_limit) to make that wait run out: the
// kernel then takes its error path (flag, abort, bounded drain of the copies
// in flight, TMEM freed), which no fault or trap is needed to reach.
__device__ uint32_t g_tc_issue_wait_limit = WAIT_LIMIT;

// bulk copy of bytes (multiple of 16, both addresses 16-byte aligned) from
// global to shared memory, completing on an mbarrier transaction count
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// SMEM matrix descriptor for a K-major tile in the SWIZZLE_64B layout:
// 8-row x 64-byte swizzle atoms stacked along M/N every 512 bytes (SBO);
// LBO is not used by swizzled K-major layouts (encoded as 1).
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(512 >> 4) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of sm_100-class tensor cores
    d |= (uint64_t)4 << 61;  // SWIZZLE_64B
    return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = F16 (fmt 0) or BF16
// (fmt 1), both K-major, no negation, shape M x N.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N, uint32_t fmt)
{
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcSmem {
    uint64_t full[STAGES];   // the stage's bulk copies have landed
    uint64_t gfull[STAGES];  // generated A: the generator threads have written the stage's A pieces
    uint64_t empty[STAGES];
    uint64_t done;
    uint64_t tfull[2];       // persistent expansion: accumulator a final
    uint64_t tempty[2];      // persistent expansion: accumulator a read out by the epilogue warps
    uint64_t tlast;          // persistent expansion: the CTA's last tile final (one phase)
    uint32_t tmem_base;
    uint32_t abort_flag;
};

// ---- generated projector tiles (GEN) ---------------------------------------
// The A operand of the projection (Pr [P][2 npw]) or of the expansion
// (Pr^T [npw][2 P]) is written into each stage's shared memory by the eight
// epilogue warps, which are otherwise idle during the main loop: Pr[p][G] =
// by[j(p)][G] * sf[a(p)][G] (TcGen), times the row's power-of-two split
// scale, split into hi + lo in the swizzled K-major layout of the copied
// tiles (16 complex values of a row per 32-deep stage).  The table loads of
// two stages ahead are in flight while a stage is split and stored.
constexpr int GEN_THREADS = 256;
constexpr int TC_THREADS = 64 + GEN_THREADS;  // producer warp, MMA warp, 8 epilogue / generator warps

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// make this thread's generic-proxy shared-memory writes visible to the tensor cores
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// hi + lo pieces of two consecutive K elements (a at the lower address)
template <typename T>
__device__ __forceinline__ void split_pair(float a, float b, uint32_t& hi, uint32_t& lo);
template <>
__device__ __forceinline__ void split_pair<__half>(float a, float b, uint32_t& hi, uint32_t& lo)
{
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}
template <>
__device__ __forceinline__ void split_pair<__nv_bfloat16>(float a, float b, uint32_t& hi, uint32_t& lo)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// Wait until stage s may be overwritten (phase ph of its empty barrier).  The
// decision to go on is taken by the whole warp (shuffles follow).
__device__ __forceinline__ bool gen_wait_empty(TcSmem* sh, int s, uint32_t ph, int* err)
{
    bool ok = mbar_wait_abort(&sh->empty[s], ph ^ 1, &sh->abort_flag);
    if (!ok && !*(volatile uint32_t*)&sh->abort_flag) { atomicExch(err, 4); sh->abort_flag = 1; }
    ok = ok && !*(volatile uint32_t*)&sh->abort_flag;
    return __all_sync(0xffffffffu, ok);
}

// every lane fences its own stores for the tensor cores; after the warp
// barrier (which orders the lanes' stores before lane 0) one arrival per warp
__device__ __forceinline__ void gen_publish(TcSmem* sh, int s)
{
    fence_proxy_async_smem();
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(&sh->gfull[s]);
}

// Projection operand (rows = projectors, K pairs = G).  Lane l of generator
// warp w (0..7) writes the 16-byte chunk c = l & 3 (G 4c .. 4c+3 of the
// stage) of tile rows 8 w + (l >> 2) and 64 + 8 w + (l >> 2): float4 table
// loads of 64- and 128-byte row pieces, and stores of which each group of 8
// lanes fills two whole 64-byte rows (all 32 banks).
template <typename T>
struct GenRows {
    int bo[2], fo[2], so[2];
    float sc[2];
    float4 b[3][2], f[3][4];
    __device__ __forceinline__ void load(const TcGen& gen, int buf, int g)
    {
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            b[buf][i] = __ldg(reinterpret_cast<const float4*>(gen.by + bo[i] + g));
            const float4* f4 = reinterpret_cast<const float4*>(gen.sf + fo[i] + g);
            f[buf][2 * i] = __ldg(f4);
            f[buf][2 * i + 1] = __ldg(f4 + 1);
        }
    }
    __device__ __forceinline__ bool emit(TcSmem* sh, unsigned char* tiles, int it, int buf, int* err)
    {
        uint4 hi[2], lo[2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const float4 bv = b[buf][i];
            const float4 f0 = f[buf][2 * i], f1 = f[buf][2 * i + 1];
            const float s = sc[i];  // a power of two (or 0 past the last row): exact
            const float b0 = bv.x * s, b1 = bv.y * s, b2 = bv.z * s, b3 = bv.w * s;
            split_pair<T>(b0 * f0.x, b0 * f0.y, hi[i].x, lo[i].x);
            split_pair<T>(b1 * f0.z, b1 * f0.w, hi[i].y, lo[i].y);
            split_pair<T>(b2 * f1.x, b2 * f1.y, hi[i].z, lo[i].z);
            split_pair<T>(b3 * f1.z, b3 * f1.w, hi[i].w, lo[i].w);
        }
        const int s = it % STAGES;
        if (!gen_wait_empty(sh, s, (it / STAGES) & 1, err)) return false;
        unsigned char* st = tiles + s * STAGE_BYTES;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            *reinterpret_cast<uint4*>(st + so[i]) = hi[i];
            *reinterpret_cast<uint4*>(st + A_TILE + so[i]) = lo[i];
        }
        gen_publish(sh, s);
        return true;
    }
};

template <typename T>
__device__ void gen_loop_rows(const TcGen& gen, TcSmem* sh, unsigned char* tiles, int m0, int kt0, int nk, int t,
                              int* err)
{
    const int lane = t & 31, w = t >> 5, c = lane & 3;
    GenRows<T> R;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int r = 64 * i + 8 * w + (lane >> 2);
        const int p = m0 + r;
        const int2 o = p < gen.P ? __ldg(gen.rows + p) : make_int2(0, gen.zero_off);
        R.fo[i] = o.x;
        R.bo[i] = o.y;
        R.sc[i] = p < gen.P ? __ldg(gen.p_scale + p) : 0.f;
        R.so[i] = 64 * r + 16 * (c ^ ((r >> 1) & 3));
    }
    const int g0 = 16 * kt0 + 4 * c;
    if (nk > 0) R.load(gen, 0, g0);
    if (nk > 1) R.load(gen, 1, g0 + 16);
    for (int it = 0; it < nk; it += 3) {
        if (it + 2 < nk) R.load(gen, 2, g0 + 16 * (it + 2));
        if (!R.emit(sh, tiles, it, 0, err) || it + 1 >= nk) break;
        if (it + 3 < nk) R.load(gen, 0, g0 + 16 * (it + 3));
        if (!R.emit(sh, tiles, it + 1, 1, err) || it + 2 >= nk) break;
        if (it + 4 < nk) R.load(gen, 1, g0 + 16 * (it + 4));
        if (!R.emit(sh, tiles, it + 2, 2, err)) break;
    }
}

// Expansion operand (rows = G, K pairs = projectors).  Thread t writes rows
// G = m0 + 2 (t & 63) and the next, projectors 4 (t >> 6) .. +3 of each stage
// (the 16-byte chunk t >> 6 of both rows): float2 / float4 table loads of
// two consecutive G, coalesced over the warp, and warp-uniform 32-byte loads
// of the projectors' table offsets.  Lanes store their two rows in an order
// chosen so that each group of 8 lanes writes 8 distinct bank quads.
template <typename T>
struct GenCols {
    int4 o[3][2];    // offsets (sf, by) of the 4 projectors, two per int4
    float2 b[2][4];  // by of each projector at the two rows
    float4 f[2][4];  // sf of each projector at the two rows
    bool e[2][3];    // projector i + 1 has projector i's structure-factor row (f not loaded)
    __device__ __forceinline__ void load_offsets(const TcGen& gen, int buf, int p0)
    {
        const int4* src = reinterpret_cast<const int4*>(gen.rows + p0);
        o[buf][0] = __ldg(src);
        o[buf][1] = __ldg(src + 1);
    }
    __device__ __forceinline__ void load(const TcGen& gen, int buf, int obuf, int g)
    {
        const int4 v0 = o[obuf][0], v1 = o[obuf][1];
        b[buf][0] = __ldg(reinterpret_cast<const float2*>(gen.by + v0.y + g));
        b[buf][1] = __ldg(reinterpret_cast<const float2*>(gen.by + v0.w + g));
        b[buf][2] = __ldg(reinterpret_cast<const float2*>(gen.by + v1.y + g));
        b[buf][3] = __ldg(reinterpret_cast<const float2*>(gen.by + v1.w + g));
        // consecutive projectors of one atom share its structure-factor row: a
        // row equal to the previous projector's is not loaded again, and emit
        // takes it from that projector once the loads have arrived (the
        // offsets are the same in all lanes of a warp, so is the choice; the
        // values, and so the tiles, are unchanged)
        const int s0 = v0.x, s1 = v0.z, s2 = v1.x, s3 = v1.z;
        e[buf][0] = s1 == s0;
        e[buf][1] = s2 == s1;
        e[buf][2] = s3 == s2;
        f[buf][0] = __ldg(reinterpret_cast<const float4*>(gen.sf + s0 + g));
        if (!e[buf][0]) f[buf][1] = __ldg(reinterpret_cast<const float4*>(gen.sf + s1 + g));
        if (!e[buf][1]) f[buf][2] = __ldg(reinterpret_cast<const float4*>(gen.sf + s2 + g));
        if (!e[buf][2]) f[buf][3] = __ldg(reinterpret_cast<const float4*>(gen.sf + s3 + g));
    }
    __device__ __forceinline__ bool emit(TcSmem* sh, unsigned char* tiles, int it, int buf, float sc0, float sc1,
                                         int r0, int c, int first, int* err)
    {
        uint4 h0, l0, h1, l1;  // rows r0, r0 + 1
        uint32_t* hp0 = reinterpret_cast<uint32_t*>(&h0);
        uint32_t* lp0 = reinterpret_cast<uint32_t*>(&l0);
        uint32_t* hp1 = reinterpret_cast<uint32_t*>(&h1);
        uint32_t* lp1 = reinterpret_cast<uint32_t*>(&l1);
        float4 fv = f[buf][0];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 bv = b[buf][i];
            if (i > 0 && !e[buf][i - 1]) fv = f[buf][i];
            const float b0 = bv.x * sc0, b1 = bv.y * sc1;  // power-of-two scales: exact
            split_pair<T>(b0 * fv.x, b0 * fv.y, hp0[i], lp0[i]);
            split_pair<T>(b1 * fv.z, b1 * fv.w, hp1[i], lp1[i]);
        }
        const int s = it % STAGES;
        if (!gen_wait_empty(sh, s, (it / STAGES) & 1, err)) return false;
        unsigned char* st = tiles + s * STAGE_BYTES;
        const int ra = r0 + first, rb = r0 + 1 - first;
        const int oa = 64 * ra + 16 * (c ^ ((ra >> 1) & 3)), ob = 64 * rb + 16 * (c ^ ((rb >> 1) & 3));
        *reinterpret_cast<uint4*>(st + oa) = first ? h1 : h0;
        *reinterpret_cast<uint4*>(st + A_TILE + oa) = first ? l1 : l0;
        *reinterpret_cast<uint4*>(st + ob) = first ? h0 : h1;
        *reinterpret_cast<uint4*>(st + A_TILE + ob) = first ? l0 : l1;
        gen_publish(sh, s);
        return true;
    }
};

// it0: the stage counter of the ring at this tile's first k-tile (tiles of a
// persistent CTA share the ring); false when the kernel aborted
template <typename T>
__device__ bool gen_loop_cols(const TcGen& gen, TcSmem* sh, unsigned char* tiles, int m0, int kt0, int nk, int t,
                              int* err, int it0 = 0)
{
    const int rp = t & 63, c = t >> 6;
    const int r0 = 2 * rp;
    const int g = m0 + r0;  // g + 1 < ldg (a multiple of 128)
    // 1 past npw, where the tables are zero
    const float sc0 = __ldg(gen.g_scale + g), sc1 = __ldg(gen.g_scale + g + 1);
    const int first = (rp >> 2) & 1;
    const int p0 = 16 * kt0 + 4 * c;
    GenCols<T> C;
    // offsets run two stages ahead of the stores, the values one
    if (nk > 0) C.load_offsets(gen, 0, p0);
    if (nk > 1) C.load_offsets(gen, 1, p0 + 16);
    if (nk > 0) C.load(gen, 0, 0, g);
    for (int it = 0; it < nk; it += 6) {
#pragma unroll
        for (int u = 0; u < 6; ++u) {
            // stage it + u: values in buffer u & 1, offsets of it + u in buffer u % 3
            if (it + u >= nk) return true;
            if (it + u + 2 < nk) C.load_offsets(gen, (u + 2) % 3, p0 + 16 * (it + u + 2));
            if (it + u + 1 < nk) C.load(gen, (u + 1) & 1, (u + 1) % 3, g);
            if (!C.emit(sh, tiles, it0 + it + u, u & 1, sc0, sc1, r0, c, first, err)) return false;
        }
    }
    return true;
}

// Split-K GEMM with partials (the projection and the complex128 GEMMs):
//   part[z][m][n] = C[m][n] * sa[m] * sb[n]   (row-major per split)
// over K range z of A [M][K] and B [N][K].  GEN: the A operand is generated in
// shared memory from gen (GEN_FP16 selects the FP16 split, else BF16)
// instead of bulk-copied from Ah / Al.
template <bool GEN = false, bool GEN_FP16 = true>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const unsigned char* __restrict__ Ah, const unsigned char* __restrict__ Al,
                   const unsigned char* __restrict__ Bh, const unsigned char* __restrict__ Bl, TcEpilogue ep, int M,
                   int N, int ktiles_total, int ktiles_per_split, uint32_t idesc, int* err, TcGen gen = TcGen{})
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned tile area
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* tiles = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    TcSmem* sh = reinterpret_cast<TcSmem*>(tiles + STAGES * STAGE_BYTES);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kt0 = blockIdx.z * ktiles_per_split;
    const int kt1 = min(ktiles_total, kt0 + ktiles_per_split);
    const int nk = max(0, kt1 - kt0);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&sh->full[s], 1);
            mbar_init(&sh->gfull[s], GEN ? GEN_THREADS / 32 : 1);
            mbar_init(&sh->empty[s], 1);
        }
        mbar_init(&sh->done, 1);
        sh->abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;

    if (warp == 0 && lane == 0) {
        // ---- bulk-copy producer: tiles (row block, k block) of the tiled operands
        const size_t KT = (size_t)ktiles_total;
        const unsigned char* ah = GEN ? nullptr : Ah + (size_t)blockIdx.x * KT * A_TILE;
        const unsigned char* al = GEN ? nullptr : Al + (size_t)blockIdx.x * KT * A_TILE;
        const unsigned char* bh = Bh + (size_t)(2 * blockIdx.y) * KT * A_TILE;  // 128-row blocks n0/128, +1
        const unsigned char* bl = Bl + (size_t)(2 * blockIdx.y) * KT * A_TILE;
        int issued = 0;
        for (int it = 0; it < nk; ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (it / STAGES) & 1;
            if (!mbar_wait_abort(&sh->empty[s], ph ^ 1, &sh->abort_flag)) {
                if (!*(volatile uint32_t*)&sh->abort_flag) { atomicExch(err, 1); sh->abort_flag = 1; }
                break;
            }
            if (*(volatile uint32_t*)&sh->abort_flag) break;
            unsigned char* st = tiles + s * STAGE_BYTES;
            mbar_arrive_expect_tx(&sh->full[s], GEN ? 2 * B_TILE : STAGE_BYTES);
            const size_t kt = (size_t)(kt0 + it);
            if (!GEN) {
                bulk_load(st, ah + kt * A_TILE, A_TILE, &sh->full[s]);
                bulk_load(st + A_TILE, al + kt * A_TILE, A_TILE, &sh->full[s]);
            }
            bulk_load(st + 2 * A_TILE, bh + kt * A_TILE, A_TILE, &sh->full[s]);
            bulk_load(st + 3 * A_TILE, bh + (KT + kt) * A_TILE, A_TILE, &sh->full[s]);
            bulk_load(st + 2 * A_TILE + B_TILE, bl + kt * A_TILE, A_TILE, &sh->full[s]);
            bulk_load(st + 3 * A_TILE + B_TILE, bl + (KT + kt) * A_TILE, A_TILE, &sh->full[s]);
            issued = it + 1;
        }
        // drain: copies in flight must land before the CTA exits (bounded)
        for (int it = max(0, issued - STAGES); it < issued; ++it)
            mbar_wait(&sh->full[it % STAGES], (it / STAGES) & 1);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer
        bool ok = true;
        const uint32_t lim = g_tc_issue_wait_limit;
        for (int it = 0; it < nk; ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (it / STAGES) & 1;
            if (!mbar_wait_n(&sh->full[s], ph, lim) || (GEN && !mbar_wait_n(&sh->gfull[s], ph, lim))) {
                atomicExch(err, 2);
                sh->abort_flag = 1;
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t st = smem_u32(tiles + s * STAGE_BYTES);
            const uint64_t ah = sdesc_sw64(st), al = sdesc_sw64(st + A_TILE);
            const uint64_t bh = sdesc_sw64(st + 2 * A_TILE), bl = sdesc_sw64(st + 2 * A_TILE + B_TILE);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
                const uint64_t adv = (uint64_t)((kk * 32) >> 4);  // 16 elements = 32 bytes along K
                // even k-tiles accumulate into columns [0,256), odd ones into [256,512):
                // two half-length FP32 accumulation chains, summed by the epilogue
                const uint32_t acc = tmem + (uint32_t)((it & 1) * BN);
                const uint32_t first = (it < 2 && kk == 0) ? 0u : 1u;
                tc_mma(acc, ah + adv, bh + adv, idesc, first);
                tc_mma(acc, ah + adv, bl + adv, idesc, 1u);
                tc_mma(acc, al + adv, bh + adv, idesc, 1u);
            }
            tc_commit(&sh->empty[s]);  // stage reusable once these MMAs have read it
        }
        (void)ok;
        tc_commit(&sh->done);  // accumulator final (arrives after all prior MMAs)
    } else if (warp >= 2) {
        // ---- generated A (GEN): these warps write each stage's A pieces first
        using GT = typename std::conditional<GEN_FP16, __half, __nv_bfloat16>::type;
        if constexpr (GEN) gen_loop_rows<GT>(gen, sh, tiles, m0, kt0, nk, threadIdx.x - 64, err);
        // ---- epilogue: warp w reads TMEM lanes 32*(w%4) .. +31; warps 2-5
        // take the first half of the columns, warps 6-9 the second
        const int q = warp & 3;
        const int half = (warp - 2) >> 2;
        const int row = m0 + q * 32 + lane;
        bool ok = mbar_wait(&sh->done, 0);
        tc_fence_after();
        if (!ok) atomicExch(err, 3);
        const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16);
        // warp-uniform decision: tcgen05.ld is a .sync.aligned warp instruction
        const bool go = __all_sync(0xffffffffu, ok && nk > 0 && !*(volatile uint32_t*)&sh->abort_flag);
        if (go) {
            const float sa = (row < M) ? ep.sa_scale[row] : 0.f;
            const bool two = nk > 1;  // the odd accumulator holds data only with two or more k-tiles
            {
                // row-major partials [z][M][N].  A lane holds one row; each
                // 32 x 32 block is transposed through the warp's own slice of
                // the stage buffers (free: every MMA has read them once `done`
                // completed), so that each store instruction writes one row's
                // 128 contiguous bytes.
                float* tr = reinterpret_cast<float*>(tiles) + (warp - 2) * 32 * 33;
                const int rbase = m0 + q * 32;
                float* out = ep.part + ((size_t)blockIdx.z * M + rbase) * (size_t)N + n0;
#pragma unroll 1
                for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 32) {
                    float v[32], w[32];
                    tmem_ld32(tbase + c0, v);
                    if (two) {
                        tmem_ld32(tbase + BN + c0, w);
#pragma unroll
                        for (int i = 0; i < 32; ++i) v[i] += w[i];
                    }
                    const float sbl = ep.sb_scale[n0 + c0 + lane];  // this lane's column after the transpose
                    __syncwarp();
#pragma unroll
                    for (int i = 0; i < 32; ++i) tr[lane * 33 + i] = v[i] * sa;
                    __syncwarp();
#pragma unroll 8
                    for (int i = 0; i < 32; ++i)
                        if (rbase + i < M) out[(size_t)i * N + c0 + lane] = tr[i * 33 + lane] * sbl;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// hpsi[b][row] += (re + i im) * sa * sb[col] + add32[b][row] for the 16 bands of
// one accumulator chunk (band b0 + i at scale column sb0 + i): read-modify-write
// in groups of 8 bands, all loads of a group issued before its stores, so that
// the HBM round trips overlap instead of following one another band by band.
__device__ __forceinline__ void expand_rmw(const TcEpilogue& ep, int row, float sa, int b0, int sb0,
                                           const float (&re)[16], const float (&im)[16])
{
    const bool add = ep.add32 != nullptr;
#pragma unroll
    for (int h0 = 0; h0 < 16; h0 += 8) {
        double2 o[8];
        float2 ad[8];
        float f[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int b = b0 + h0 + i;
            const size_t at = (size_t)b * ep.ldh + row;
            f[i] = sa * ep.sb_scale[sb0 + h0 + i];
            o[i] = b < ep.nb ? ep.hpsi[at] : make_double2(0.0, 0.0);
            ad[i] = (add && b < ep.nb) ? ep.add32[at] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int b = b0 + h0 + i;
            if (b < ep.nb) {
                o[i].x += f2d_bits(fmaf(re[h0 + i], f[i], ad[i].x));
                o[i].y += f2d_bits(fmaf(im[h0 + i], f[i], ad[i].y));
                ep.hpsi[(size_t)b * ep.ldh + row] = o[i];
            }
        }
    }
}

constexpr int TCP_THREADS = TC_THREADS + 128;  // + 4 epilogue warps (10..13)

// The expansion, hpsi[b][g] += (C[g][re b] + i C[g][im b]) * sa[g] * sb[b]
// (+ add32), as a persistent kernel: one CTA per SM walks the 128 x 256
// output tiles (tile, tile + gridDim.x, ...).  The stage ring runs on across
// tiles; the two 256-column TMEM accumulators alternate by tile, so that the
// four epilogue warps drain tile i (the hpsi read-modify-write, HBM-bound)
// while the tensor cores accumulate tile i + 1.  Warp 0 copies B (and A
// without GEN), warp 1 issues the MMAs, warps 2-9 generate A (GEN).
template <bool GEN, bool GEN_FP16>
__global__ void __launch_bounds__(TCP_THREADS, 1)
    tc_expand_kernel(const unsigned char* __restrict__ Ah, const unsigned char* __restrict__ Al,
                     const unsigned char* __restrict__ Bh, const unsigned char* __restrict__ Bl, TcEpilogue ep, int M,
                     int N, int ktiles, uint32_t idesc, int* err, TcGen gen, int row0)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* tiles = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    TcSmem* sh = reinterpret_cast<TcSmem*>(tiles + STAGES * STAGE_BYTES);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // output rows [row0, M) (row0 a multiple of BM)
    const int mt = (M - row0 + BM - 1) / BM, ntile = mt * (N / BN);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&sh->full[s], 1);
            mbar_init(&sh->gfull[s], GEN ? GEN_THREADS / 32 : 1);
            mbar_init(&sh->empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&sh->tfull[a], 1);
            mbar_init(&sh->tempty[a], 4);
        }
        mbar_init(&sh->tlast, 1);
        mbar_init(&sh->done, 1);
        sh->abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;
    volatile uint32_t* abort = &sh->abort_flag;

    if (warp == 0 && lane == 0) {
        // ---- bulk-copy producer
        const size_t KT = (size_t)ktiles;
        int git = 0;  // stage uses issued
        bool stop = false;
        for (int tile = blockIdx.x; tile < ntile && !stop; tile += gridDim.x) {
            const int mb = row0 / BM + tile % mt, nbk = tile / mt;
            const unsigned char* ah = GEN ? nullptr : Ah + (size_t)mb * KT * A_TILE;
            const unsigned char* al = GEN ? nullptr : Al + (size_t)mb * KT * A_TILE;
            const unsigned char* bh = Bh + (size_t)(2 * nbk) * KT * A_TILE;
            const unsigned char* bl = Bl + (size_t)(2 * nbk) * KT * A_TILE;
            for (int kt = 0; kt < ktiles; ++kt) {
                const int s = git % STAGES;
                const uint32_t ph = (git / STAGES) & 1;
                if (!mbar_wait_abort(&sh->empty[s], ph ^ 1, &sh->abort_flag)) {
                    if (!*abort) { atomicExch(err, 1); *abort = 1; }
                    stop = true;
                    break;
                }
                if (*abort) { stop = true; break; }
                unsigned char* st = tiles + s * STAGE_BYTES;
                mbar_arrive_expect_tx(&sh->full[s], GEN ? 2 * B_TILE : STAGE_BYTES);
                if (!GEN) {
                    bulk_load(st, ah + kt * A_TILE, A_TILE, &sh->full[s]);
                    bulk_load(st + A_TILE, al + kt * A_TILE, A_TILE, &sh->full[s]);
                }
                bulk_load(st + 2 * A_TILE, bh + kt * A_TILE, A_TILE, &sh->full[s]);
                bulk_load(st + 3 * A_TILE, bh + (KT + kt) * A_TILE, A_TILE, &sh->full[s]);
                bulk_load(st + 2 * A_TILE + B_TILE, bl + kt * A_TILE, A_TILE, &sh->full[s]);
                bulk_load(st + 3 * A_TILE + B_TILE, bl + (KT + kt) * A_TILE, A_TILE, &sh->full[s]);
                ++git;
            }
        }
        // drain: copies in flight must land before the CTA exits (bounded)
        for (int i = max(0, git - STAGES); i < git; ++i) mbar_wait(&sh->full[i % STAGES], (i / STAGES) & 1);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer
        const uint32_t lim = g_tc_issue_wait_limit;
        int git = 0, lt = 0;
        bool stop = false;
        for (int tile = blockIdx.x; tile < ntile && !stop; tile += gridDim.x, ++lt) {
            const int a = lt & 1;
            // accumulator a free: its previous tile read out by the epilogue warps
            if (!mbar_wait_abort(&sh->tempty[a], ((lt >> 1) & 1) ^ 1, &sh->abort_flag)) {
                if (!*abort) { atomicExch(err, 5); *abort = 1; }
                break;
            }
            tc_fence_after();
            const uint32_t acc = tmem + (uint32_t)(a * BN);
            for (int kt = 0; kt < ktiles; ++kt) {
                const int s = git % STAGES;
                const uint32_t ph = (git / STAGES) & 1;
                if (!mbar_wait_n(&sh->full[s], ph, lim) || (GEN && !mbar_wait_n(&sh->gfull[s], ph, lim))) {
                    atomicExch(err, 2);
                    *abort = 1;
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t st = smem_u32(tiles + s * STAGE_BYTES);
                const uint64_t adh = sdesc_sw64(st), adl = sdesc_sw64(st + A_TILE);
                const uint64_t bdh = sdesc_sw64(st + 2 * A_TILE), bdl = sdesc_sw64(st + 2 * A_TILE + B_TILE);
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
                    const uint64_t adv = (uint64_t)((kk * 32) >> 4);  // 16 elements = 32 bytes along K
                    const uint32_t first = (kt == 0 && kk == 0) ? 0u : 1u;
                    tc_mma(acc, adh + adv, bdh + adv, idesc, first);
                    tc_mma(acc, adh + adv, bdl + adv, idesc, 1u);
                    tc_mma(acc, adl + adv, bdh + adv, idesc, 1u);
                }
                tc_commit(&sh->empty[s]);
                ++git;
            }
            if (!stop) {
                tc_commit(&sh->tfull[a]);
                if (tile + (int)gridDim.x >= ntile) tc_commit(&sh->tlast);
            }
        }
        // every MMA issued has completed before the accumulators are freed (bounded)
        tc_commit(&sh->done);
        mbar_wait(&sh->done, 0);
    } else if (warp >= 2) {
        // The CTA's last tile: its epilogue is exposed (no next tile to overlap),
        // so warps 2-13 share it, three per TMEM lane quadrant (the epilogue
        // warp, then generator warps w < 6 and w >= 6 take the 16-band chunks
        // c with c % 3 = 0, 1, 2).  Earlier tiles: the epilogue warps alone.
        const int last_lt = (ntile - 1 - (int)blockIdx.x) / (int)gridDim.x;
        const int role = warp >= 10 ? 0 : (warp < 6 ? 1 : 2);
        const int q = warp & 3;
        int lt = 0;
        if (warp < 10) {
            // ---- generated A
            if constexpr (GEN) {
                using GT = typename std::conditional<GEN_FP16, __half, __nv_bfloat16>::type;
                int git = 0;
                for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
                    if (!gen_loop_cols<GT>(gen, sh, tiles, row0 + (tile % mt) * BM, 0, ktiles, threadIdx.x - 64, err,
                                           git))
                        break;
                    git += ktiles;
                }
            }
            lt = last_lt;
        }
        // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31
        for (int tile = blockIdx.x + lt * gridDim.x; tile < ntile; tile += gridDim.x, ++lt) {
            const int a = lt & 1, mb = row0 / BM + tile % mt, nbk = tile / mt;
            const bool last = lt == last_lt;
            // warps 2-9 join at the last tile only, at any point of the
            // accumulators' phases: they wait on the single-phase barrier
            bool ok = warp < 10 ? mbar_wait_abort(&sh->tlast, 0, &sh->abort_flag)
                                : mbar_wait_abort(&sh->tfull[a], (lt >> 1) & 1, &sh->abort_flag);
            if (!ok && !*abort) { atomicExch(err, 3); *abort = 1; }
            // warp-uniform: tcgen05.ld is a .sync.aligned warp instruction
            if (!__all_sync(0xffffffffu, ok && !*abort)) break;
            tc_fence_after();
            const int row = mb * BM + q * 32 + lane;
            const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * BN);
            const float sa = (row < M) ? ep.sa_scale[row] : 0.f;
            // columns [0,128): real parts of bands 128 nbk + j, [128,256): imaginary
#pragma unroll 1
            for (int c = 0; c < 8; ++c) {
                if (last && c % 3 != role) continue;
                const int c0 = 16 * c;
                float re[16], im[16];
                tmem_ld16(tbase + c0, re);
                tmem_ld16(tbase + 128 + c0, im);
                if (!last && c == 7) {
                    // accumulator read out (tcgen05.ld waited): hand it back to the MMA warp
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&sh->tempty[a]);
                }
                if (row < M) expand_rmw(ep, row, sa, nbk * 128 + c0, nbk * BN + c0, re, im);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ---------------------------------------------------------------- prep kernels
template <typename T>
__device__ __forceinline__ void split_store(float x, T* hi, T* lo);
template <>
__device__ __forceinline__ void split_store<__half>(float x, __half* hi, __half* lo)
{
    __half h = __float2half_rn(x);
    *hi = h;
    *lo = __float2half_rn(x - __half2float(h));
}
template <>
__device__ __forceinline__ void split_store<__nv_bfloat16>(float x, __nv_bfloat16* hi, __nv_bfloat16* lo)
{
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    *hi = h;
    *lo = __float2bfloat16_rn(x - __bfloat162float(h));
}

// power-of-two row scale 2^s with max*2^s in [2^13, 2^14] (FP16); 1 for BF16
__device__ __forceinline__ float row_scale(float mx, bool fp16)
{
    if (!fp16 || !(mx > 0.f)) return 1.f;
    int e;
    frexpf(mx, &e);  // mx = f * 2^e, f in [0.5, 1)
    return ldexpf(1.f, 14 - e);
}

__device__ __forceinline__ float block_max(float v, float* red)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        float w = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) w = fmaxf(w, __shfl_xor_sync(0xffffffffu, w, o));
        if (threadIdx.x == 0) red[0] = w;
    }
    __syncthreads();
    float r = red[0];
    __syncthreads();
    return r;
}

// split of an FP64 value: hi from its FP32 rounding, lo from the FP64 remainder
template <typename T>
__device__ __forceinline__ void split_store_d(double x, T* hi, T* lo);
template <>
__device__ __forceinline__ void split_store_d<__half>(double x, __half* hi, __half* lo)
{
    __half h = __float2half_rn((float)x);
    *hi = h;
    *lo = __float2half_rn((float)(x - (double)__half2float(h)));
}
template <>
__device__ __forceinline__ void split_store_d<__nv_bfloat16>(double x, __nv_bfloat16* hi, __nv_bfloat16* lo)
{
    __nv_bfloat16 h = __float2bfloat16_rn((float)x);
    *hi = h;
    *lo = __float2bfloat16_rn((float)(x - (double)__bfloat162float(h)));
}

__device__ __forceinline__ void split_any(float x, float sc, __half* h, __half* l) { split_store<__half>(x * sc, h, l); }
__device__ __forceinline__ void split_any(float x, float sc, __nv_bfloat16* h, __nv_bfloat16* l)
{
    split_store<__nv_bfloat16>(x * sc, h, l);
}
__device__ __forceinline__ void split_any(double x, float sc, __half* h, __half* l) { split_store_d<__half>(x * sc, h, l); }
__device__ __forceinline__ void split_any(double x, float sc, __nv_bfloat16* h, __nv_bfloat16* l)
{
    split_store_d<__nv_bfloat16>(x * sc, h, l);
}

// Projection A: row p of a complex matrix (complex64 Pr or complex128 psi,
// length npw) -> [hi|lo][p][kpad] interleaved re/im
template <typename T, typename S>
__global__ void split_rows_kernel(const S* __restrict__ pr, int npw, size_t ldk, T* hi, T* lo, float* inv_scale,
                                  bool fp16)
{
    using R = typename Real<S>::type;
    __shared__ float red[32];
    const int p = blockIdx.x;
    const S* row = pr + (size_t)p * npw;
    float mx = 0.f;
    for (int g = threadIdx.x; g < npw; g += blockDim.x)
        mx = fmaxf(mx, fmaxf(fabsf((float)row[g].x), fabsf((float)row[g].y)));
    mx = block_max(mx, red);
    const float sc = row_scale(mx, fp16);
    if (threadIdx.x == 0) inv_scale[p] = 1.f / sc;
    for (size_t k = threadIdx.x; k < ldk; k += blockDim.x) {
        R x = 0;
        if (k < 2 * (size_t)npw) {
            S v = row[k >> 1];
            x = (k & 1) ? v.y : v.x;
        }
        const size_t o = tile_off(p, k, ldk);
        split_any(x, sc, hi + o, lo + o);
    }
}

// Column maxima over projectors: cmax[g] = max_p max(|re|, |im|) of pr and,
// if given, of pr2 (the two row blocks that share one row of the transposed operand)
__global__ void col_max_kernel(const float2* __restrict__ pr, const float2* __restrict__ pr2, int P, int npw,
                               float* cmax)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= npw) return;
    float mx = 0.f;
    for (int p = 0; p < P; ++p) {
        float2 v = pr[(size_t)p * npw + g];
        mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
        if (pr2) {
            float2 w = pr2[(size_t)p * npw + g];
            mx = fmaxf(mx, fmaxf(fabsf(w.x), fabsf(w.y)));
        }
    }
    cmax[g] = mx;
}

// Expansion A: Pr^T rows g: [hi|lo][g][2p + c], scaled by the row scale of g
template <typename T>
__global__ void transpose_split_kernel(const float2* __restrict__ pr, int P, int npw, size_t ldk, size_t koff,
                                       const float* __restrict__ cmax, T* hi, T* lo, float* inv_scale, bool fp16)
{
    __shared__ float2 tile[32][33];
    const int g0 = blockIdx.x * 32, p0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
    for (int r = ty; r < 32; r += 8) {
        const int p = p0 + r, g = g0 + tx;
        tile[r][tx] = (p < P && g < npw) ? pr[(size_t)p * npw + g] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int g = g0 + r;
        if (g >= npw) continue;
        const float sc = row_scale(cmax[g], fp16);
        if (blockIdx.y == 0 && tx == 0) inv_scale[g] = 1.f / sc;
        const float2 v = tile[tx][r];
        const int p = p0 + tx;
        const size_t k = koff + 2 * (size_t)p;
        if (k + 1 < ldk) {
            const size_t o = tile_off(g, k, ldk);  // k even: k + 1 sits at o + 1
            split_store<T>(v.x * sc, hi + o, lo + o);
            split_store<T>(v.y * sc, hi + o + 1, lo + o + 1);
        }
    }
}

// B rows from band data.  src is complex [nb][len] (psi, FROM_W = false) or
// [len][nb] (W, FROM_W = true).  Row layout: t*256 + c*128 + j for band
// b = 128 t + j.  Projection: re row (x_r, x_i), im row (x_i, -x_r);
// expansion: re row (w_r, -w_i), im row (w_i, w_r).  Two passes: the band
// maxima (atomicMax on the float bits, non-negative) then the split writes.
template <typename S, bool FROM_W>
__device__ __forceinline__ double2 band_get(const S* src, int nb, int len, int b, int i)
{
    if (FROM_W) return as_c128(src[(size_t)i * nb + b]);
    return as_c128(src[(size_t)b * len + i]);
}

// |x| of a complex128 or complex64 component as a non-negative float whose
// binary exponent is that of |x| rounded to float: the row scale depends on
// the exponent alone, so a truncated mantissa is enough (no FP64 arithmetic)
__device__ __forceinline__ uint32_t abs_key(double x)
{
    const uint32_t hi = (uint32_t)__double2hiint(x) & 0x7fffffffu;
    return __float_as_uint(d2f_bits(__hiloint2double((int)hi, 0)));
}
__device__ __forceinline__ uint32_t abs_key(float x) { return __float_as_uint(x) & 0x7fffffffu; }

template <typename S, bool FROM_W>
__global__ void band_max_kernel(const S* __restrict__ src, int nb, int len, unsigned* rowmax)
{
    const int b = blockIdx.y;
    uint32_t mx = 0u;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        const S v = FROM_W ? src[(size_t)i * nb + b] : src[(size_t)b * len + i];
        mx = max(mx, max(abs_key(v.x), abs_key(v.y)));
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(rowmax + b, mx);
}

template <typename T>
__device__ __forceinline__ void split2(float x, T& h, T& l);
template <>
__device__ __forceinline__ void split2<__half>(float x, __half& h, __half& l)
{
    h = __float2half_rn(x);
    l = __float2half_rn(x - __half2float(h));
}
template <>
__device__ __forceinline__ void split2<__nv_bfloat16>(float x, __nv_bfloat16& h, __nv_bfloat16& l)
{
    h = __float2bfloat16_rn(x);
    l = __float2bfloat16_rn(x - __bfloat162float(h));
}

// Two complex elements per thread: k = 4t .. 4t+3 of both rows of band b,
// written as one 8-byte store per row and piece (ldk is a multiple of BK, so
// 4t < ldk implies 4t+3 < ldk).
template <typename T, typename S, bool FROM_W>
__global__ void band_write_kernel(const S* __restrict__ src, int nb, int len, size_t ldk, T* hi, T* lo,
                                  float* inv_scale, const unsigned* __restrict__ rowmax, bool fp16)
{
    const int b = blockIdx.y;
    const int t = b / 128, j = b % 128;
    const size_t rre = (size_t)t * 256 + j, rim = rre + 128;
    const float sc = row_scale(__uint_as_float(rowmax[b]), fp16);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        inv_scale[rre] = 1.f / sc;
        inv_scale[rim] = 1.f / sc;
    }
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t k = 4 * (size_t)q;
    if (k >= ldk) return;
    float a[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const int i = 2 * q + e;
        if (i < len) {
            const float2 v = to_c64(band_get<S, FROM_W>(src, nb, len, b, i));
            const float r = v.x * sc, m = v.y * sc;  // sc: a power of two
            if (!FROM_W) { a[2 * e] = r; a[2 * e + 1] = m; c[2 * e] = m; c[2 * e + 1] = -r; }
            else { a[2 * e] = r; a[2 * e + 1] = -m; c[2 * e] = m; c[2 * e + 1] = r; }
        }
    }
    __align__(8) T ah[4], al[4], ch[4], cl[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        split2<T>(a[e], ah[e], al[e]);
        split2<T>(c[e], ch[e], cl[e]);
    }
    // k = 4q .. 4q+3 lie in one 16-byte chunk of the tiled layout
    const size_t ore = tile_off(rre, k, ldk), oim = tile_off(rim, k, ldk);
    *reinterpret_cast<uint2*>(hi + ore) = *reinterpret_cast<const uint2*>(ah);
    *reinterpret_cast<uint2*>(lo + ore) = *reinterpret_cast<const uint2*>(al);
    *reinterpret_cast<uint2*>(hi + oim) = *reinterpret_cast<const uint2*>(ch);
    *reinterpret_cast<uint2*>(lo + oim) = *reinterpret_cast<const uint2*>(cl);
}

template <typename T, typename S, bool FROM_W>
static void band_rows(const S* src, int nb, int len, size_t ldk, T* hi, T* lo, float* inv_scale, unsigned* rowmax,
                      bool fp16, cudaStream_t st, bool have_max = false)
{
    if (!have_max) {
        cudaMemsetAsync(rowmax, 0, sizeof(unsigned) * nb, st);
        const int chunks = min(64, ceil_div(len, 256 * 4));
        band_max_kernel<S, FROM_W><<<dim3(chunks, nb), 256, 0, st>>>(src, nb, len, rowmax);
    }
    band_write_kernel<T, S, FROM_W><<<dim3(ceil_div((long)(ldk / 4), 256), nb), 256, 0, st>>>(
        src, nb, len, ldk, hi, lo, inv_scale, rowmax, fp16);
}

// rows of bands missing from the last 128-block: zero hi/lo, unit scale
template <typename T>
__global__ void zero_rows_kernel(int nb, int nbp, size_t ldk, T* hi, T* lo, float* inv_scale)
{
    const int b = nb + blockIdx.x;
    if (b >= nbp) return;
    const int t = b / 128, j = b % 128;
    for (int c = 0; c < 2; ++c) {
        const size_t r = (size_t)t * 256 + c * 128 + j;
        if (threadIdx.x == 0) inv_scale[r] = 1.f;
        for (size_t k = threadIdx.x; k < ldk; k += blockDim.x) {
            hi[tile_off(r, k, ldk)] = T(0.f);
            lo[tile_off(r, k, ldk)] = T(0.f);
        }
    }
}

// W[p][b] = lambda_p * sum_z (C[z][p][re b] + i C[z][p][im b]) (and, with eterm,
// lambda_p |sum|^2 in FP64); consecutive threads take consecutive bands, so the
// reads of a split's row are coalesced, as are the writes of W[p][.]
template <typename CW>
__global__ void proj_reduce_kernel(int P, int nb, int N, int nsplit, const float* __restrict__ part,
                                   const double* __restrict__ lam, int period, CW* W, double* eterm = nullptr)
{
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)P * nb) return;
    const int p = (int)(idx / nb), b = (int)(idx % nb);
    const int t = b / 128, j = b % 128;
    const size_t cre = (size_t)t * 256 + j, cim = cre + 128;
    const size_t zs = (size_t)P * N;
    const float* pre = part + (size_t)p * N + cre;
    const float* pim = part + (size_t)p * N + cim;
    if constexpr (std::is_same<CW, float2>::value) {
        Sum2f re, im;  // complex64 W: compensated FP32 sums, no FP64 pipe
#pragma unroll 4
        for (int z = 0; z < nsplit; ++z) {
            re.add(pre[z * zs]);
            im.add(pim[z * zs]);
        }
        const float f = lam ? d2f_bits(lam[p % period]) : 1.f;
        W[idx] = make_float2(f * re.value(), f * im.value());
        if (eterm) {
            // lambda_p |<p|psi_b>|^2 in FP64 from the two-float sums
            const double sr = f2d_bits(re.s) + f2d_bits(re.c), si = f2d_bits(im.s) + f2d_bits(im.c);
            eterm[idx] = (lam ? lam[p % period] : 1.0) * (sr * sr + si * si);
        }
        return;
    }
    double sr = 0.0, si = 0.0;
    for (int z = 0; z < nsplit; ++z) {
        sr += pre[z * zs];
        si += pim[z * zs];
    }
    const double f = lam ? lam[p % period] : 1.0;
    W[idx] = from_c128<CW>(make_double2(f * sr, f * si));
    if (eterm) eterm[idx] = f * (sr * sr + si * si);  // lambda_p |<p|psi_b>|^2, FP64
}

// out[b] = sum_p eterm[p][b], in p order
__global__ void __launch_bounds__(256) eterm_sum_kernel(int P, int nb, const double* __restrict__ eterm,
                                                        double* __restrict__ out)
{
    __shared__ double red[32];
    const int b = blockIdx.x;
    double e = 0.0;
    for (int p = threadIdx.x; p < P; p += blockDim.x) e += eterm[(size_t)p * nb + b];
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        out[b] = s;
    }
}

}  // namespace

size_t tc_round_k(size_t k) { return (k + BK - 1) / BK * BK; }
int tc_band_rows(int nb) { return (nb + 127) / 128 * 256; }
size_t tc_rows_pad(size_t rows) { return (rows + BM - 1) / BM * BM; }

size_t tc_gemm_smem_bytes() { return (size_t)STAGES * STAGE_BYTES + 1024 + sizeof(TcSmem) + 64; }

cudaError_t tc_build_grad_operands(const float2* pr4, int P, int npw, bool fp16, TcOperand* proj4, TcOperand* exp3,
                                   float* cmax_scratch, cudaStream_t st)
{
    if (P == 0 || npw == 0) return cudaSuccess;
    const int P4 = 4 * P;
    if (fp16)
        split_rows_kernel<__half, float2><<<P4, 256, 0, st>>>(pr4, npw, proj4->ldk, (__half*)proj4->hi, (__half*)proj4->lo,
                                                      proj4->inv_scale, true);
    else
        split_rows_kernel<__nv_bfloat16, float2><<<P4, 256, 0, st>>>(pr4, npw, proj4->ldk, (__nv_bfloat16*)proj4->hi,
                                                             (__nv_bfloat16*)proj4->lo, proj4->inv_scale, false);
    const size_t PN = (size_t)P * npw;
    dim3 g(ceil_div(npw, 32), ceil_div(P, 32));
    for (int a = 0; a < 3; ++a) {
        // row g of the alpha operand: (Pr[p][g], p < P) then (dPr_alpha[p][g], p < P), one row scale
        const float2* dpa = pr4 + (size_t)(1 + a) * PN;
        TcOperand* E = &exp3[a];
        col_max_kernel<<<ceil_div(npw, 256), 256, 0, st>>>(pr4, dpa, P, npw, cmax_scratch);
        for (int blk = 0; blk < 2; ++blk) {
            const float2* src = blk == 0 ? pr4 : dpa;
            const size_t koff = blk == 0 ? 0 : 2 * (size_t)P;
            if (fp16)
                transpose_split_kernel<__half><<<g, 256, 0, st>>>(src, P, npw, E->ldk, koff, cmax_scratch,
                                                                  (__half*)E->hi, (__half*)E->lo, E->inv_scale, true);
            else
                transpose_split_kernel<__nv_bfloat16><<<g, 256, 0, st>>>(src, P, npw, E->ldk, koff, cmax_scratch,
                                                                         (__nv_bfloat16*)E->hi, (__nv_bfloat16*)E->lo,
                                                                         E->inv_scale, false);
        }
    }
    return cudaGetLastError();
}

cudaError_t tc_band_operand(const double2* psi, int nb, int npw, bool fp16, TcOperand* B, unsigned* rowmax,
                            cudaStream_t st, bool have_max)
{
    const int nbp = tc_band_rows(nb) / 2;
    if (fp16)
        band_rows<__half, double2, false>(psi, nb, npw, B->ldk, (__half*)B->hi, (__half*)B->lo, B->inv_scale, rowmax,
                                          true, st, have_max);
    else
        band_rows<__nv_bfloat16, double2, false>(psi, nb, npw, B->ldk, (__nv_bfloat16*)B->hi,
                                                 (__nv_bfloat16*)B->lo, B->inv_scale, rowmax, false, st, have_max);
    if (nbp > nb) {
        if (fp16)
            zero_rows_kernel<__half><<<nbp - nb, 256, 0, st>>>(nb, nbp, B->ldk, (__half*)B->hi, (__half*)B->lo,
                                                              B->inv_scale);
        else
            zero_rows_kernel<__nv_bfloat16><<<nbp - nb, 256, 0, st>>>(nb, nbp, B->ldk, (__nv_bfloat16*)B->hi,
                                                                     (__nv_bfloat16*)B->lo, B->inv_scale);
    }
    return cudaGetLastError();
}

cudaError_t tc_w_operand(const float2* W, int P, int nb, bool fp16, TcOperand* B, unsigned* rowmax, cudaStream_t st)
{
    const int nbp = tc_band_rows(nb) / 2;
    if (fp16)
        band_rows<__half, float2, true>(W, nb, P, B->ldk, (__half*)B->hi, (__half*)B->lo, B->inv_scale, rowmax, true,
                                        st);
    else
        band_rows<__nv_bfloat16, float2, true>(W, nb, P, B->ldk, (__nv_bfloat16*)B->hi, (__nv_bfloat16*)B->lo,
                                               B->inv_scale, rowmax, false, st);
    if (nbp > nb) {
        if (fp16)
            zero_rows_kernel<__half><<<nbp - nb, 256, 0, st>>>(nb, nbp, B->ldk, (__half*)B->hi, (__half*)B->lo,
                                                              B->inv_scale);
        else
            zero_rows_kernel<__nv_bfloat16><<<nbp - nb, 256, 0, st>>>(nb, nbp, B->ldk, (__nv_bfloat16*)B->hi,
                                                                     (__nv_bfloat16*)B->lo, B->inv_scale);
    }
    return cudaGetLastError();
}

// SMs of the current device (one CTA of the GEMM per SM); 152 on GB300
static int sm_count()
{
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess || n <= 0)
        return 152;
    return n;
}

// Split-K of the projection: at most MAX_CHAIN_K of K per CTA (short FP32
// accumulation chains: with the two alternating accumulators at most half of
// that, 288 MMAs, add into one accumulator), rounded up so that the CTAs fill
// whole waves of the device's SMs.
int tc_proj_splits(int P, int nb, size_t ldk)
{
    const int sms = sm_count();
    const int tiles = ceil_div(P, BM) * (tc_band_rows(nb) / BN);
    const int ktiles = (int)(ldk / BK);
    int s = ceil_div(ktiles, MAX_CHAIN_K / BK);
    if (tiles * s < sms) s = ceil_div(sms, tiles);
    // cost model: waves x K per split (in 64-deep units), plus the partial-sum reduction
    int best = s;
    double best_cost = 1e300;
    for (int c = s; c <= 2 * s && c <= ktiles; ++c) {
        const double cost = (double)ceil_div(tiles * c, sms) * ceil_div(ktiles, c) * (BK / 64.0) + c / 8.0;
        if (cost < best_cost) { best = c; best_cost = cost; }
    }
    if (best > ktiles) best = ktiles;
    if (best < 1) best = 1;
    return best;
}

template <bool GEN, bool GEN_FP16>
static cudaError_t launch_proj_t(dim3 grid, size_t smem, cudaStream_t st, const unsigned char* ah,
                                 const unsigned char* al, const unsigned char* bh, const unsigned char* bl,
                                 const TcEpilogue& ep, int M, int N, int ktiles, int per, uint32_t idesc, int* err,
                                 const TcGen& gen)
{
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel<GEN, GEN_FP16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e) return e;
    tc_gemm_kernel<GEN, GEN_FP16><<<grid, TC_THREADS, smem, st>>>(ah, al, bh, bl, ep, M, N, ktiles, per, idesc, err,
                                                                   gen);
    return cudaGetLastError();
}

template <bool GEN, bool GEN_FP16>
static cudaError_t launch_expand_t(int grid, size_t smem, cudaStream_t st, const unsigned char* ah,
                                   const unsigned char* al, const unsigned char* bh, const unsigned char* bl,
                                   const TcEpilogue& ep, int M, int N, int ktiles, uint32_t idesc, int* err,
                                   const TcGen& gen, int row0)
{
    cudaError_t e = cudaFuncSetAttribute(tc_expand_kernel<GEN, GEN_FP16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e) return e;
    tc_expand_kernel<GEN, GEN_FP16><<<grid, TCP_THREADS, smem, st>>>(ah, al, bh, bl, ep, M, N, ktiles, idesc, err,
                                                                      gen, row0);
    return cudaGetLastError();
}

// A: rows M, B: rows N (= tc_band_rows(nb)); one launch.  Mode 0: split-K
// partials (nsplit), mode 1: the persistent expansion.  With gen the A
// operand is generated from those tables (A.hi / A.lo unused).
static cudaError_t launch_tc(int mode, const TcOperand& A, int M, const TcOperand& B, int N, int nsplit, bool fp16,
                             const TcEpilogue& ep, int* err, cudaStream_t st, const TcGen* gen = nullptr, int row0 = 0)
{
    if (A.ldk != B.ldk || A.ldk % BK) return cudaErrorInvalidValue;
    const int ktiles = (int)(A.ldk / BK);
    const size_t smem = tc_gemm_smem_bytes();
    const uint32_t idesc = idesc_f16(BM, BN, fp16 ? 0u : 1u);
    const unsigned char *ah = (const unsigned char*)A.hi, *al = (const unsigned char*)A.lo;
    const unsigned char *bh = (const unsigned char*)B.hi, *bl = (const unsigned char*)B.lo;
    const TcGen none{};
    const TcGen& g = gen ? *gen : none;
    if (mode == 1) {
        if (row0 % BM || row0 >= M) return cudaErrorInvalidValue;
        const int tiles = ceil_div(M - row0, BM) * (N / BN);
        const int grid = std::min(tiles, sm_count());
        if (!gen)
            return launch_expand_t<false, true>(grid, smem, st, ah, al, bh, bl, ep, M, N, ktiles, idesc, err, g, row0);
        return fp16 ? launch_expand_t<true, true>(grid, smem, st, ah, al, bh, bl, ep, M, N, ktiles, idesc, err, g, row0)
                    : launch_expand_t<true, false>(grid, smem, st, ah, al, bh, bl, ep, M, N, ktiles, idesc, err, g,
                                                   row0);
    }
    const int per = ceil_div(ktiles, nsplit);
    const int nz = ceil_div(ktiles, per);
    dim3 grid(ceil_div(M, BM), N / BN, nz);
    if (!gen) return launch_proj_t<false, true>(grid, smem, st, ah, al, bh, bl, ep, M, N, ktiles, per, idesc, err, g);
    return fp16 ? launch_proj_t<true, true>(grid, smem, st, ah, al, bh, bl, ep, M, N, ktiles, per, idesc, err, g)
                : launch_proj_t<true, false>(grid, smem, st, ah, al, bh, bl, ep, M, N, ktiles, per, idesc, err, g);
}

cudaError_t tc_projection(const TcOperand& A, int P, const TcOperand& B, int nb, int nsplit, bool fp16, float* part,
                          const double* lam, int period, float2* W, int* err, cudaStream_t st, Prof* prof,
                          double* eterm, double* e_nl, const TcGen* gen)
{
    const int N = tc_band_rows(nb);
    TcEpilogue ep{};
    ep.part = part;
    ep.sa_scale = A.inv_scale;
    ep.sb_scale = B.inv_scale;
    int h = prof->open(PH_PROJ, st);
    cudaError_t e = launch_tc(0, A, P, B, N, nsplit, fp16, ep, err, st, gen);
    prof->close(h, st);
    if (e) return e;
    const int ktiles = (int)(A.ldk / BK);
    const int per = ceil_div(ktiles, nsplit);
    const int nz = ceil_div(ktiles, per);
    h = prof->open(PH_REDUCE, st);
    proj_reduce_kernel<float2><<<ceil_div((long)P * nb, 256), 256, 0, st>>>(P, nb, N, nz, part, lam, period, W,
                                                                            e_nl ? eterm : nullptr);
    if (e_nl) eterm_sum_kernel<<<nb, 256, 0, st>>>(P, nb, eterm, e_nl);
    prof->close(h, st, e_nl ? 2 : 1);
    return cudaGetLastError();
}

cudaError_t tc_rows_operand(const double2* x, int rows, int npw, bool fp16, TcOperand* A, cudaStream_t st)
{
    if (rows == 0) return cudaSuccess;
    if (fp16)
        split_rows_kernel<__half, double2><<<rows, 256, 0, st>>>(x, npw, A->ldk, (__half*)A->hi, (__half*)A->lo,
                                                                 A->inv_scale, true);
    else
        split_rows_kernel<__nv_bfloat16, double2><<<rows, 256, 0, st>>>(x, npw, A->ldk, (__nv_bfloat16*)A->hi,
                                                                        (__nv_bfloat16*)A->lo, A->inv_scale, false);
    return cudaGetLastError();
}

cudaError_t tc_gemm_c128(const TcOperand& A, int M, const TcOperand& B, int nb, int nsplit, bool fp16, float* part,
                         double2* out, int* err, cudaStream_t st)
{
    const int N = tc_band_rows(nb);
    TcEpilogue ep{};
    ep.part = part;
    ep.sa_scale = A.inv_scale;
    ep.sb_scale = B.inv_scale;
    cudaError_t e = launch_tc(0, A, M, B, N, nsplit, fp16, ep, err, st);
    if (e) return e;
    const int ktiles = (int)(A.ldk / BK);
    const int per = ceil_div(ktiles, nsplit);
    const int nz = ceil_div(ktiles, per);
    proj_reduce_kernel<double2><<<ceil_div((long)M * nb, 256), 256, 0, st>>>(M, nb, N, nz, part, nullptr, 1, out);
    return cudaGetLastError();
}

cudaError_t tc_expansion(const TcOperand& A, int npw, const TcOperand& B, int nb, bool fp16, double2* hpsi,
                         int* err, cudaStream_t st, Prof* prof, const float2* add32, const TcGen* gen, int row0,
                         int row1)
{
    const int N = tc_band_rows(nb);
    TcEpilogue ep{};
    ep.hpsi = hpsi;
    ep.add32 = add32;
    ep.ldh = npw;
    ep.nb = nb;
    ep.sa_scale = A.inv_scale;
    ep.sb_scale = B.inv_scale;
    int h = prof->open(PH_EXPAND, st);
    cudaError_t e = launch_tc(1, A, row1 < 0 ? npw : row1, B, N, 1, fp16, ep, err, st, gen, row0);
    prof->close(h, st);
    return e;
}

// ---------------------------------------------------------------- generator tables
// by[j][g] = beta_rad(j)[g] * Y_lm(j)[g] rounded to FP32 (zero past npw)
__global__ void gen_by_kernel(const int2* __restrict__ byinfo, const double* __restrict__ beta,
                              const double* __restrict__ ylm, int npw, int ldg, float* __restrict__ by)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (g >= ldg) return;
    const int2 bi = byinfo[j];
    by[(size_t)j * ldg + g] = g < npw ? (float)(beta[(size_t)bi.x * npw + g] * ylm[(size_t)bi.y * npw + g]) : 0.f;
}

__global__ void gen_sf_kernel(const double2* __restrict__ sf, int npw, int ldg, float2* __restrict__ out)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int a = blockIdx.y;
    if (g >= ldg) return;
    float2 v = make_float2(0.f, 0.f);
    if (g < npw) {
        const double2 x = sf[(size_t)a * npw + g];
        v = make_float2((float)x.x, (float)x.y);
    }
    out[(size_t)a * ldg + g] = v;
}

// rmax[j] = max_g |by[j][g]|: bounds |Re|, |Im| of every projector row on by row j (|S| = 1)
__global__ void gen_rowmax_kernel(const float* __restrict__ by, int ldg, float* __restrict__ rmax)
{
    __shared__ float red[32];
    const float* row = by + (size_t)blockIdx.x * ldg;
    float mx = 0.f;
    for (int g = threadIdx.x; g < ldg; g += blockDim.x) mx = fmaxf(mx, fabsf(row[g]));
    mx = block_max(mx, red);
    if (threadIdx.x == 0) rmax[blockIdx.x] = mx;
}

// split scales: per G row of the transposed operand (max over by rows) and per projector row
__global__ void gen_scales_kernel(const float* __restrict__ by, int nby, int ldg, const int2* __restrict__ rows,
                                  int P, const float* __restrict__ rmax, bool fp16, float* g_scale, float* g_inv,
                                  float* p_scale, float* p_inv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ldg) {
        float mx = 0.f;
        for (int j = 0; j < nby; ++j) mx = fmaxf(mx, fabsf(by[(size_t)j * ldg + i]));
        const float sc = row_scale(mx, fp16);
        g_scale[i] = sc;
        g_inv[i] = 1.f / sc;
    }
    if (i < P) {
        const float sc = row_scale(rmax[rows[i].y / ldg], fp16);
        p_scale[i] = sc;
        p_inv[i] = 1.f / sc;
    }
}

// leading dimension of the tables: whole 128-row tiles of the expansion operand
static int gen_ldg(int npw) { return (int)tc_rows_pad((size_t)npw); }
// entries of the offset table: the projection's K pairs (P rounded up to 16)
static int gen_ppad(int P) { return (int)(tc_round_k(2 * (size_t)P) / 2); }

struct GenLayout {
    size_t by, sf, rows, ps, pi, gs, gi, rmax, byinfo, bytes;
};

static GenLayout gen_layout(int P, int npw, int nby, int natom)
{
    const size_t ldg = (size_t)gen_ldg(npw);
    GenLayout o;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off += (bytes + 255) / 256 * 256;
        return at;
    };
    o.by = take((size_t)(nby + 1) * ldg * sizeof(float));  // + a zero row
    o.sf = take((size_t)natom * ldg * sizeof(float2));
    o.rows = take((size_t)gen_ppad(P) * sizeof(int2));
    o.ps = take((size_t)P * sizeof(float));
    o.pi = take((size_t)P * sizeof(float));
    o.gs = take(ldg * sizeof(float));
    o.gi = take(ldg * sizeof(float));
    o.rmax = take((size_t)nby * sizeof(float));
    o.byinfo = take((size_t)nby * sizeof(int2));
    o.bytes = off;
    return o;
}

size_t tc_gen_bytes(int P, int npw, int nby, int natom) { return gen_layout(P, npw, nby, natom).bytes; }

cudaError_t tc_build_gen(unsigned char* mem, int P, int npw, const int2* h_rows, const int2* h_byinfo, int nby,
                         int natom, const double* beta, const double* ylm, const double2* sf, bool fp16, TcGen* out,
                         cudaStream_t st)
{
    if (P <= 0 || npw <= 0 || nby <= 0 || natom <= 0) return cudaErrorInvalidValue;
    const GenLayout o = gen_layout(P, npw, nby, natom);
    const int ldg = gen_ldg(npw);
    // element offsets of table rows are 32-bit
    if ((double)(std::max(nby + 1, natom)) * ldg >= 2147483647.0) return cudaErrorInvalidValue;
    const int ppad = gen_ppad(P);
    // (sf offset, by offset) per projector; past P the zero by row
    std::vector<int2> off((size_t)ppad, make_int2(0, nby * ldg));
    for (int p = 0; p < P; ++p) off[(size_t)p] = make_int2(h_rows[p].x * ldg, h_rows[p].y * ldg);
    TcGen g;
    g.by = reinterpret_cast<const float*>(mem + o.by);
    g.sf = reinterpret_cast<const float2*>(mem + o.sf);
    g.rows = reinterpret_cast<const int2*>(mem + o.rows);
    g.p_scale = reinterpret_cast<const float*>(mem + o.ps);
    g.p_inv = reinterpret_cast<const float*>(mem + o.pi);
    g.g_scale = reinterpret_cast<const float*>(mem + o.gs);
    g.g_inv = reinterpret_cast<const float*>(mem + o.gi);
    g.P = P;
    g.npw = npw;
    g.ldg = ldg;
    g.zero_off = nby * ldg;
    cudaError_t e;
    int2* rows = reinterpret_cast<int2*>(mem + o.rows);
    int2* byinfo = reinterpret_cast<int2*>(mem + o.byinfo);
    if ((e = cudaMemcpyAsync(rows, off.data(), (size_t)ppad * sizeof(int2), cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(byinfo, h_byinfo, (size_t)nby * sizeof(int2), cudaMemcpyHostToDevice, st))) return e;
    float* by = reinterpret_cast<float*>(mem + o.by);
    float* rmax = reinterpret_cast<float*>(mem + o.rmax);
    if ((e = cudaMemsetAsync(by + (size_t)nby * ldg, 0, (size_t)ldg * sizeof(float), st))) return e;
    gen_by_kernel<<<dim3(ceil_div(ldg, 256), nby), 256, 0, st>>>(byinfo, beta, ylm, npw, ldg, by);
    gen_sf_kernel<<<dim3(ceil_div(ldg, 256), natom), 256, 0, st>>>(sf, npw, ldg, reinterpret_cast<float2*>(mem + o.sf));
    gen_rowmax_kernel<<<nby, 256, 0, st>>>(by, ldg, rmax);
    gen_scales_kernel<<<ceil_div(std::max(ldg, P), 256), 256, 0, st>>>(
        by, nby, ldg, rows, P, rmax, fp16, reinterpret_cast<float*>(mem + o.gs), reinterpret_cast<float*>(mem + o.gi),
        reinterpret_cast<float*>(mem + o.ps), reinterpret_cast<float*>(mem + o.pi));
    if ((e = cudaGetLastError())) return e;
    *out = g;
    return cudaSuccess;
}

int tc_chain_splits(size_t ldk, int chain_k)
{
    const int kt = (int)(ldk / BK), per = chain_k / BK > 0 ? chain_k / BK : 1;
    return ceil_div(kt, per);
}

// Test hook: the MMA issuer's poll limit (polls < 0: back to the default).
cudaError_t tc_set_issue_wait_limit(long polls)
{
    const uint32_t v = polls < 0 ? WAIT_LIMIT : (uint32_t)std::min<long>(polls, (long)WAIT_LIMIT);
    return cudaMemcpyToSymbol(g_tc_issue_wait_limit, &v, sizeof(v));
}

// ---------------------------------------------------------------- ragged (batched) GEMMs
// The batch plans' nonlocal term on the tensor cores: the items of a cell
// (k-points with their own projector tables and band blocks) share each
// launch; every CTA reads its item from the table.  Band operands use the
// compact layout of TcRagItem (re row j, im row nbp + j, N = 2 nbp).
namespace {

// band b of item I: max |re|, |im| over its len values (FROM_W: W [P][nb] column b)
template <bool FROM_W>
__global__ void rag_band_max_kernel(const TcRagItem* __restrict__ items, const int2* __restrict__ bands, int P)
{
    const int2 ib = bands[blockIdx.y];
    const TcRagItem& I = items[ib.x];
    const int b = ib.y;
    const int len = FROM_W ? P : I.npw;
    uint32_t mx = 0u;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        if (FROM_W) {
            const float2 v = I.W[(size_t)i * I.nb + b];
            mx = max(mx, max(abs_key(v.x), abs_key(v.y)));
        } else {
            const double2 v = I.psi[(size_t)b * I.npw + i];
            mx = max(mx, max(abs_key(v.x), abs_key(v.y)));
        }
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(I.rowmax + b, mx);
}

// K of the expansion: 2 P rounded up to the stage depth
__device__ __forceinline__ size_t rag_k2(int P) { return ((size_t)2 * P + BK - 1) / BK * BK; }

// Rows j (re) and nbp + j (im) of item I's band operand, k = 4q .. 4q+3 per
// thread: the projection's from psi (re row (x_r, x_i), im row (x_i, -x_r)),
// the expansion's from W (re row (w_r, -w_i), im row (w_i, w_r)); bands
// nb <= j < nbp are zero rows with unit factors.
template <typename T, bool FROM_W>
__global__ void rag_band_write_kernel(const TcRagItem* __restrict__ items, const int2* __restrict__ rows, int P,
                                      bool fp16)
{
    const int2 ij = rows[blockIdx.y];
    const TcRagItem& I = items[ij.x];
    const int j = ij.y;
    const size_t ldk = FROM_W ? rag_k2(P) : (size_t)I.k1t * BK;
    const int len = FROM_W ? P : I.npw;
    T* hi = reinterpret_cast<T*>(FROM_W ? I.b2h : I.b1h);
    T* lo = reinterpret_cast<T*>(FROM_W ? I.b2l : I.b1l);
    float* inv = FROM_W ? I.b2s : I.b1s;
    const bool real = j < I.nb;
    const float sc = real ? row_scale(__uint_as_float(I.rowmax[j]), fp16) : 1.f;
    const size_t rre = (size_t)j, rim = (size_t)(I.nbp + j);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        inv[rre] = 1.f / sc;
        inv[rim] = 1.f / sc;
    }
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const size_t k = 4 * (size_t)q;
    if (k >= ldk) return;
    float a[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
    if (real) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int i = 2 * q + e;
            if (i < len) {
                const float2 v = FROM_W ? I.W[(size_t)i * I.nb + j] : to_c64(I.psi[(size_t)j * I.npw + i]);
                const float r = v.x * sc, m = v.y * sc;  // sc: a power of two
                if (!FROM_W) { a[2 * e] = r; a[2 * e + 1] = m; c[2 * e] = m; c[2 * e + 1] = -r; }
                else { a[2 * e] = r; a[2 * e + 1] = -m; c[2 * e] = m; c[2 * e + 1] = r; }
            }
        }
    }
    __align__(8) T ah[4], al[4], ch[4], cl[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        split2<T>(a[e], ah[e], al[e]);
        split2<T>(c[e], ch[e], cl[e]);
    }
    const size_t ore = tile_off(rre, k, ldk), oim = tile_off(rim, k, ldk);
    *reinterpret_cast<uint2*>(hi + ore) = *reinterpret_cast<const uint2*>(ah);
    *reinterpret_cast<uint2*>(lo + ore) = *reinterpret_cast<const uint2*>(al);
    *reinterpret_cast<uint2*>(hi + oim) = *reinterpret_cast<const uint2*>(ch);
    *reinterpret_cast<uint2*>(lo + oim) = *reinterpret_cast<const uint2*>(cl);
}

// bulk copies of the first n rows of a band operand's k-tile kt (the tiled
// layout keeps rows 0-127 and 128-255 in separate 8 KB tiles)
__device__ __forceinline__ void rag_load_b(unsigned char* dst, const unsigned char* src, size_t KT, size_t kt, int n,
                                           uint64_t* bar)
{
    const int n0 = min(n, 128);
    bulk_load(dst, src + kt * A_TILE, (uint32_t)n0 * 64u, bar);
    if (n > 128) bulk_load(dst + A_TILE, src + (KT + kt) * A_TILE, (uint32_t)(n - 128) * 64u, bar);
}

// Split-K projection of every item: CTA (m tile, item, split).  Warp roles as
// tc_gemm_kernel<GEN>; N = 2 nbp of the item (idesc per CTA); partials
// row-major [z][P][N] through the same per-warp transpose.
template <bool GEN_FP16>
__global__ void __launch_bounds__(TC_THREADS, 1)
    rag_proj_kernel(const TcRagItem* __restrict__ items, int P, int* err)
{
    const TcRagItem& I = items[blockIdx.y];
    if ((int)blockIdx.z >= I.nz) return;  // uniform: before any barrier or TMEM allocation
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* tiles = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    TcSmem* sh = reinterpret_cast<TcSmem*>(tiles + STAGES * STAGE_BYTES);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM;
    const int N = 2 * I.nbp;
    const int KT = I.k1t;
    const int kt0 = blockIdx.z * I.per;
    const int nk = max(0, min(KT, kt0 + I.per) - kt0);
    const uint32_t idesc = idesc_f16(BM, N, GEN_FP16 ? 0u : 1u);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&sh->full[s], 1);
            mbar_init(&sh->gfull[s], GEN_THREADS / 32);
            mbar_init(&sh->empty[s], 1);
        }
        mbar_init(&sh->done, 1);
        sh->abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;

    if (warp == 0 && lane == 0) {
        int issued = 0;
        for (int it = 0; it < nk; ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (it / STAGES) & 1;
            if (!mbar_wait_abort(&sh->empty[s], ph ^ 1, &sh->abort_flag)) {
                if (!*(volatile uint32_t*)&sh->abort_flag) { atomicExch(err, 1); sh->abort_flag = 1; }
                break;
            }
            if (*(volatile uint32_t*)&sh->abort_flag) break;
            unsigned char* st = tiles + s * STAGE_BYTES;
            mbar_arrive_expect_tx(&sh->full[s], 2u * (uint32_t)N * 64u);
            const size_t kt = (size_t)(kt0 + it);
            rag_load_b(st + 2 * A_TILE, I.b1h, (size_t)KT, kt, N, &sh->full[s]);
            rag_load_b(st + 2 * A_TILE + B_TILE, I.b1l, (size_t)KT, kt, N, &sh->full[s]);
            issued = it + 1;
        }
        for (int it = max(0, issued - STAGES); it < issued; ++it) mbar_wait(&sh->full[it % STAGES], (it / STAGES) & 1);
    } else if (warp == 1 && lane == 0) {
        const uint32_t lim = g_tc_issue_wait_limit;
        for (int it = 0; it < nk; ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (it / STAGES) & 1;
            if (!mbar_wait_n(&sh->full[s], ph, lim) || !mbar_wait_n(&sh->gfull[s], ph, lim)) {
                atomicExch(err, 2);
                sh->abort_flag = 1;
                break;
            }
            tc_fence_after();
            const uint32_t st = smem_u32(tiles + s * STAGE_BYTES);
            const uint64_t ah = sdesc_sw64(st), al = sdesc_sw64(st + A_TILE);
            const uint64_t bh = sdesc_sw64(st + 2 * A_TILE), bl = sdesc_sw64(st + 2 * A_TILE + B_TILE);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
                const uint64_t adv = (uint64_t)((kk * 32) >> 4);
                const uint32_t acc = tmem + (uint32_t)((it & 1) * BN);
                const uint32_t first = (it < 2 && kk == 0) ? 0u : 1u;
                tc_mma(acc, ah + adv, bh + adv, idesc, first);
                tc_mma(acc, ah + adv, bl + adv, idesc, 1u);
                tc_mma(acc, al + adv, bh + adv, idesc, 1u);
            }
            tc_commit(&sh->empty[s]);
        }
        tc_commit(&sh->done);
    } else if (warp >= 2) {
        using GT = typename std::conditional<GEN_FP16, __half, __nv_bfloat16>::type;
        gen_loop_rows<GT>(I.gen, sh, tiles, m0, kt0, nk, threadIdx.x - 64, err);
        const int q = warp & 3;
        const int half = (warp - 2) >> 2;
        const int row = m0 + q * 32 + lane;
        bool ok = mbar_wait(&sh->done, 0);
        tc_fence_after();
        if (!ok) atomicExch(err, 3);
        const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16);
        const bool go = __all_sync(0xffffffffu, ok && nk > 0 && !*(volatile uint32_t*)&sh->abort_flag);
        if (go) {
            const float sa = (row < P) ? I.gen.p_inv[row] : 0.f;
            const bool two = nk > 1;
            float* tr = reinterpret_cast<float*>(tiles) + (warp - 2) * 32 * 33;
            const int rbase = m0 + q * 32;
            float* out = I.part + ((size_t)blockIdx.z * P + rbase) * (size_t)N;
#pragma unroll 1
            for (int c0 = half * (BN / 2); c0 < min(N, (half + 1) * (BN / 2)); c0 += 32) {
                float v[32], w[32];
                tmem_ld32(tbase + c0, v);
                if (two) {
                    tmem_ld32(tbase + BN + c0, w);
#pragma unroll
                    for (int i = 0; i < 32; ++i) v[i] += w[i];
                }
                const int col = c0 + lane;
                const float sbl = col < N ? I.b1s[col] : 0.f;
                __syncwarp();
#pragma unroll
                for (int i = 0; i < 32; ++i) tr[lane * 33 + i] = v[i] * sa;
                __syncwarp();
#pragma unroll 8
                for (int i = 0; i < 32; ++i)
                    if (rbase + i < P && col < N) out[(size_t)i * N + col] = tr[i * 33 + lane] * sbl;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// W[p][b] = lambda_p sum_z (C[z][p][b] + i C[z][p][nbp + b]), compensated FP32
__global__ void rag_reduce_kernel(const TcRagItem* __restrict__ items, int P)
{
    const TcRagItem& I = items[blockIdx.y];
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= P * I.nb) return;
    const int p = idx / I.nb, b = idx % I.nb;
    const int N = 2 * I.nbp;
    const size_t zs = (size_t)P * N;
    const float* pre = I.part + (size_t)p * N + b;
    const float* pim = pre + I.nbp;
    Sum2f re, im;
    for (int z = 0; z < I.nz; ++z) {
        re.add(pre[z * zs]);
        im.add(pim[z * zs]);
    }
    const float f = I.lam ? d2f_bits(I.lam[p]) : 1.f;
    I.W[idx] = make_float2(f * re.value(), f * im.value());
}

// Expansion of every item: CTA = one 128-row G tile (item, tile) of tiles.
// Warp 0 copies the W' tiles, warp 1 issues the MMAs (one accumulator),
// warps 2-9 generate Pr^T and then add into hpsi, the 16-band chunks of the
// item split between the two warp halves.
template <bool GEN_FP16>
__global__ void __launch_bounds__(TC_THREADS, 1)
    rag_exp_kernel(const TcRagItem* __restrict__ items, const int2* __restrict__ tiles_of, int P, int* err)
{
    const int2 it2 = tiles_of[blockIdx.x];
    const TcRagItem& I = items[it2.x];
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* tiles = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    TcSmem* sh = reinterpret_cast<TcSmem*>(tiles + STAGES * STAGE_BYTES);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = it2.y * BM;
    const int N = 2 * I.nbp;
    const int KT = (int)(rag_k2(P) / BK);
    const int nk = KT;
    const uint32_t idesc = idesc_f16(BM, N, GEN_FP16 ? 0u : 1u);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&sh->full[s], 1);
            mbar_init(&sh->gfull[s], GEN_THREADS / 32);
            mbar_init(&sh->empty[s], 1);
        }
        mbar_init(&sh->done, 1);
        sh->abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;

    if (warp == 0 && lane == 0) {
        int issued = 0;
        for (int it = 0; it < nk; ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (it / STAGES) & 1;
            if (!mbar_wait_abort(&sh->empty[s], ph ^ 1, &sh->abort_flag)) {
                if (!*(volatile uint32_t*)&sh->abort_flag) { atomicExch(err, 1); sh->abort_flag = 1; }
                break;
            }
            if (*(volatile uint32_t*)&sh->abort_flag) break;
            unsigned char* st = tiles + s * STAGE_BYTES;
            mbar_arrive_expect_tx(&sh->full[s], 2u * (uint32_t)N * 64u);
            rag_load_b(st + 2 * A_TILE, I.b2h, (size_t)KT, (size_t)it, N, &sh->full[s]);
            rag_load_b(st + 2 * A_TILE + B_TILE, I.b2l, (size_t)KT, (size_t)it, N, &sh->full[s]);
            issued = it + 1;
        }
        for (int it = max(0, issued - STAGES); it < issued; ++it) mbar_wait(&sh->full[it % STAGES], (it / STAGES) & 1);
    } else if (warp == 1 && lane == 0) {
        const uint32_t lim = g_tc_issue_wait_limit;
        for (int it = 0; it < nk; ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (it / STAGES) & 1;
            if (!mbar_wait_n(&sh->full[s], ph, lim) || !mbar_wait_n(&sh->gfull[s], ph, lim)) {
                atomicExch(err, 2);
                sh->abort_flag = 1;
                break;
            }
            tc_fence_after();
            const uint32_t st = smem_u32(tiles + s * STAGE_BYTES);
            const uint64_t ah = sdesc_sw64(st), al = sdesc_sw64(st + A_TILE);
            const uint64_t bh = sdesc_sw64(st + 2 * A_TILE), bl = sdesc_sw64(st + 2 * A_TILE + B_TILE);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
                const uint64_t adv = (uint64_t)((kk * 32) >> 4);
                const uint32_t first = (it == 0 && kk == 0) ? 0u : 1u;
                tc_mma(tmem, ah + adv, bh + adv, idesc, first);
                tc_mma(tmem, ah + adv, bl + adv, idesc, 1u);
                tc_mma(tmem, al + adv, bh + adv, idesc, 1u);
            }
            tc_commit(&sh->empty[s]);
        }
        tc_commit(&sh->done);
    } else if (warp >= 2) {
        using GT = typename std::conditional<GEN_FP16, __half, __nv_bfloat16>::type;
        gen_loop_cols<GT>(I.gen, sh, tiles, m0, 0, nk, threadIdx.x - 64, err);
        const int q = warp & 3;
        const int half = (warp - 2) >> 2;
        const int row = m0 + q * 32 + lane;
        bool ok = mbar_wait(&sh->done, 0);
        tc_fence_after();
        if (!ok) atomicExch(err, 3);
        const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16);
        const bool go = __all_sync(0xffffffffu, ok && !*(volatile uint32_t*)&sh->abort_flag);
        if (go) {
            TcEpilogue ep{};
            ep.hpsi = I.hpsi;
            ep.ldh = I.npw;
            ep.nb = I.nb;
            ep.sb_scale = I.b2s;
            const float sa = (row < I.npw) ? I.gen.g_inv[row] : 0.f;
            // column j: re of band j, nbp + j: its im; 16-band chunks alternate between the halves
#pragma unroll 1
            for (int c0 = 16 * half; c0 < I.nbp; c0 += 32) {
                float re[16], im[16];
                tmem_ld16(tbase + c0, re);
                tmem_ld16(tbase + I.nbp + c0, im);
                if (row < I.npw) expand_rmw(ep, row, sa, c0, c0, re, im);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

template <typename T>
static void rag_operands(bool from_w, const TcRagItem* d_items, const int2* d_bands, int nbands, const int2* d_rows,
                         int nrows, int P, int len_max, size_t ldk_max, unsigned* rowmax_all, size_t n_rowmax,
                         bool fp16, cudaStream_t st)
{
    cudaMemsetAsync(rowmax_all, 0, n_rowmax * sizeof(unsigned), st);
    const int chunks = min(64, ceil_div(len_max, 256 * 4));
    if (from_w) rag_band_max_kernel<true><<<dim3(chunks, nbands), 256, 0, st>>>(d_items, d_bands, P);
    else rag_band_max_kernel<false><<<dim3(chunks, nbands), 256, 0, st>>>(d_items, d_bands, P);
    const dim3 g(ceil_div((long)(ldk_max / 4), 256), nrows);
    if (from_w) rag_band_write_kernel<T, true><<<g, 256, 0, st>>>(d_items, d_rows, P, fp16);
    else rag_band_write_kernel<T, false><<<g, 256, 0, st>>>(d_items, d_rows, P, fp16);
}

}  // namespace

int tc_rag_nbp(int nb) { return (nb + 15) / 16 * 16; }

cudaError_t tc_rag_project(const TcRagItem* d_items, int n_items, const int2* d_bands, int nbands, const int2* d_rows,
                           int nrows, int P, int k1t_max, int nz_max, bool fp16, unsigned* rowmax_all,
                           size_t n_rowmax, int* err, cudaStream_t st)
{
    if (n_items == 0 || nbands == 0 || P == 0) return cudaSuccess;
    if (n_items > 65535 || nrows > 65535 || nbands > 65535 || nz_max > 65535) return cudaErrorInvalidValue;
    const size_t k1_max = (size_t)k1t_max * BK;
    const int npw_max = (int)(k1_max / 2);
    if (fp16) rag_operands<__half>(false, d_items, d_bands, nbands, d_rows, nrows, P, npw_max, k1_max, rowmax_all,
                                   n_rowmax, true, st);
    else rag_operands<__nv_bfloat16>(false, d_items, d_bands, nbands, d_rows, nrows, P, npw_max, k1_max, rowmax_all,
                                     n_rowmax, false, st);
    cudaError_t e;
    const size_t smem = tc_gemm_smem_bytes();
    auto k = fp16 ? rag_proj_kernel<true> : rag_proj_kernel<false>;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) return e;
    k<<<dim3(ceil_div(P, BM), n_items, nz_max), TC_THREADS, smem, st>>>(d_items, P, err);
    rag_reduce_kernel<<<dim3(ceil_div((long)P * 128, 256), n_items), 256, 0, st>>>(d_items, P);
    const size_t k2 = tc_round_k(2 * (size_t)P);
    if (fp16) rag_operands<__half>(true, d_items, d_bands, nbands, d_rows, nrows, P, P, k2, rowmax_all, n_rowmax,
                                   true, st);
    else rag_operands<__nv_bfloat16>(true, d_items, d_bands, nbands, d_rows, nrows, P, P, k2, rowmax_all, n_rowmax,
                                     false, st);
    return cudaGetLastError();
}

cudaError_t tc_rag_expand(const TcRagItem* d_items, const int2* d_tiles, int ntiles, int P, bool fp16, int* err,
                          cudaStream_t st)
{
    if (ntiles == 0 || P == 0) return cudaSuccess;
    cudaError_t e;
    const size_t smem = tc_gemm_smem_bytes();
    auto k = fp16 ? rag_exp_kernel<true> : rag_exp_kernel<false>;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) return e;
    k<<<ntiles, TC_THREADS, smem, st>>>(d_items, d_tiles, P, err);
    return cudaGetLastError();
}
