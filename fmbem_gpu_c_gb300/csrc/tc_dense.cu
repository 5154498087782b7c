// Batched translation passes of the mixed path on the 5th-generation tensor cores
// (tcgen05.mma, kind::tf32) as dense operators: the M2L of the levels whose operators are small
// enough to store densely (p <= 16, the levels that carry most translations) and, on request,
// the M2M and L2L of those levels (one operator per octant).
//
// The translation of direction d is T_d = diag(e^{-i m' phi_d}) S_c diag(e^{i m phi_d}) (the RCR
// product of translation.cu:1864-1961 with its azimuthal phases taken out), where S_c (p^2 x p^2
// complex, formed once at plan time) depends only on the polar angle and the distance of d:
// the 316 directions fall into about 60 classes c of equal (dz, dx^2 + dy^2).  With the rows of
// a tile being 128 translations of one class (times right-hand sides), the pass is the real GEMM
//     D[t][o] = sum_k A[t][k] B[o][k],   A[t] = source expansion of translation t times e^{i m phi},
//                                         B    = S_c embedded as a real 2p^2 x 2p^2 matrix,
// k and o running over interleaved (re, im) parts, and the epilogue multiplies row t's outputs
// by e^{-i m' phi} of its own direction.  Split TF32 (3 products hi*hi + hi*lo + lo*hi of
// rounded 11-bit halves) gives close to FP32 accuracy.
//
// A persistent, warp-specialised kernel (one CTA per SM, 18 warps) runs over the tiles
// (128 translations x one output half):
//   warp 0     issues the MMAs (one thread) into one of two TMEM accumulators (2 x 256 columns)
//              and commits each K chunk to its stage's "empty" barrier, each tile to its
//              accumulator's "full" barrier;
//   warp 1     copies the operator's K chunks (hi and lo tiles, contiguous) with cp.async.bulk;
//   warps 2-9  gather the source expansions, two threads per row (translation), each half of
//              every 16-wide K chunk, apply the row's phases, split them into TF32 hi / lo and
//              store them in the no-swizzle K-major core-matrix layout;
//   warps 10-17 read a finished accumulator (tcgen05.ld; two warps per TMEM lane quarter, on
//              alternate 32-column blocks), stage 32 columns at a time in shared memory, apply
//              each row's phases and add them into the destination expansions with 16-byte FP32
//              atomics, overlapping the next tile's MMAs.
// Four shared-memory stages of KC = 16; every wait has a time limit, after which the thread sets
// the plan's error flag and stops.  Where one output half's whole operator fits beside the A
// stages (p <= 8), it stays resident instead: each CTA takes a contiguous range of tiles, warp 1
// copies a class's operator once per run of its tiles (operator-full barrier), and the MMA
// warp releases it after the run's last tile (a commit to the operator-empty barrier).
#include "plan.h"
#include "tc_common.cuh"
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace fmm {

constexpr int TC_M = 128;               // translations per tile (MMA M)
constexpr int TC_KC = 16;               // K per stage (2 MMA K-steps of 8)
constexpr int TC_STAGES = 4;
constexpr int TC_AWARPS = 8;            // source-gather warps (2..9)
constexpr int TC_EPI0 = 2 + TC_AWARPS;  // first epilogue warp
constexpr int TC_EWARPS = 8;            // epilogue warps (10..17), two per TMEM lane quarter
constexpr int TC_THREADS = 32 * (TC_EPI0 + TC_EWARPS);
// orders up to 16: at p = 20 (K = 800) the dense form's rounding (FP32 accumulation of 300
// split products per output) raised the iterations of the refined 64-column solve on the
// 200,000-triangle head-like body from 48 to 56, which cost more than its faster M2L saved
constexpr int TC_MAXP = 16;
constexpr int TC_MTAB = TC_MAXP * TC_MAXP + 8;  // order m of every coefficient (int8), zero padded
constexpr int TC_EPI_LD = 33;           // staging row stride (floats) of the epilogue
constexpr size_t TC_SMEM_MAX = 232448;  // 227 KB of dynamic shared memory per CTA

struct TcPass {
    const int4 *items;
    const int *g_src, *g_dst, *g_dir;    // per translation (class order): boxes and direction
    const float2 *PH;                    // phases e^{i m phi} of direction d at d phstride + phoff + m
    int phstride, phoff;
    int phased;                          // M2L: phases per row (pin = pout); M2M / L2L: none (PH a
                                         // table of ones, phstride 0)
    int nrhs, nsrc, ndst;
    int pin, P2o, K, nch, nhalf, CH, Nmma, ntiles;  // K = 2 pin^2 inputs, P2o = pout^2 outputs
    int res;                      // operator resident: one output half, whole operator in shared memory
    const float *B;
    const float2 *src;
    float2 *dst;
    int *err;
};

static size_t tc_stage_bytes(int Nmma) { return (size_t)8 * TC_KC * (TC_M + Nmma); }
// res = 0: stages of (A hi, A lo, B hi, B lo); res = 1: stages of (A hi, A lo) and the whole
// operator of one direction (nch chunks of B hi, B lo) resident
static size_t tc_smem_bytes(int Nmma, int res, int nch)
{
    size_t main = res ? TC_STAGES * (size_t)8 * TC_KC * TC_M + (size_t)nch * 8 * TC_KC * Nmma : TC_STAGES * tc_stage_bytes(Nmma);
    return main + TC_EWARPS * 32 * TC_EPI_LD * sizeof(float) + (2 * TC_STAGES + 6) * 8 + 16 + TC_MTAB;
}

// Output halves and MMA width for source order pin and destination order pout: each half holds
// CH coefficients (2 CH real outputs, Nmma = that rounded up to 16, <= 256); K = 2 pin^2 in
// chunks of 16.
static bool tc_geometry(int pin, int pout, TcDense &g)
{
    if (pin < 4 || pin > TC_MAXP || pout < 4 || pout > TC_MAXP) return false;
    const int P2 = pout * pout, K = 2 * pin * pin;
    for (g.nhalf = 1;; g.nhalf++) {
        g.CH = (P2 + g.nhalf - 1) / g.nhalf;
        g.Nmma = (2 * g.CH + 15) / 16 * 16;
        if (g.Nmma <= 256) break;
    }
    g.KC = TC_KC;
    g.nch = (K + TC_KC - 1) / TC_KC;
    if (tc_smem_bytes(g.Nmma, 0, g.nch) > TC_SMEM_MAX) return false;
    // one output half whose whole operator fits beside the A stages (p <= 8): the operator
    // stays in shared memory while a CTA's consecutive tiles keep its class
    g.res = g.nhalf == 1 && tc_smem_bytes(g.Nmma, 1, g.nch) <= TC_SMEM_MAX ? 1 : 0;
    return true;
}

// degree n and order m of coefficient i = n^2 + n + m
__device__ __forceinline__ void tc_nm(int i, int &n, int &m)
{
    int q = (int)sqrtf((float)i);
    while (q * q > i) q--;
    while ((q + 1) * (q + 1) <= i) q++;
    n = q;
    m = i - q * q - q;
}

// destination / source expansion of row r of tile (it): column e = translation t x nrhs + r,
// expansions stored [box][rhs][p^2]
__device__ __forceinline__ int tile_box(const TcPass &ps, int4 it, int r, bool source)
{
    if (r >= it.z) return -1;
    int e = it.y + r, t = e / ps.nrhs, rr = e - t * ps.nrhs;
    return (source ? ps.g_src[t] : ps.g_dst[t]) * ps.nrhs + rr;
}

__global__ void __launch_bounds__(TC_THREADS, 1) tc_dense_kernel(TcPass ps)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int Nmma = ps.Nmma, K = ps.K, P2 = ps.pin * ps.pin, P2o = ps.P2o, nch = ps.nch, res = ps.res;
    const uint32_t tA = (uint32_t)TC_M * TC_KC * 4, tB = (uint32_t)Nmma * TC_KC * 4, stage = 2 * tA + (res ? 0 : 2 * tB);
    unsigned char *bres = smem + TC_STAGES * stage;  // resident operator (res)
    float *epi = reinterpret_cast<float *>(bres + (res ? (size_t)nch * 2 * tB : 0));
    uint64_t *bars = reinterpret_cast<uint64_t *>(epi + TC_EWARPS * 32 * TC_EPI_LD);
    uint64_t *full = bars, *empty = bars + TC_STAGES, *accf = bars + 2 * TC_STAGES, *acce = accf + 2;
    uint64_t *bfull = acce + 2, *bempty = bfull + 1;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bempty + 1);
    signed char *s_m = reinterpret_cast<signed char *>(tslot + 4);  // m of coefficient i, 0 beyond p^2
    for (int i = threadIdx.x; i < TC_MTAB; i += blockDim.x) {
        int n, m;
        tc_nm(i, n, m);
        s_m[i] = i < P2 ? (signed char)m : (signed char)0;
    }
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // tiles of this CTA: strided over the grid, or (res) one contiguous range, so that
    // consecutive tiles share their class and its resident operator
    const int q_first = res ? (int)((long long)blockIdx.x * ps.ntiles / gridDim.x) : (int)blockIdx.x;
    const int q_end = res ? (int)((long long)(blockIdx.x + 1) * ps.ntiles / gridDim.x) : ps.ntiles;
    const int q_step = res ? 1 : (int)gridDim.x;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 32) {
        for (int s = 0; s < TC_STAGES; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(full + s)), "r"(TC_AWARPS + (res ? 0 : 1)));  // A warps (+ B copy)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(empty + s)));  // MMA commit
        }
        for (int a = 0; a < 2; a++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(accf + a)));   // MMA commit
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(acce + a)), "r"(TC_EWARPS));  // epilogue warps
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bfull)));   // operator copy (res)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bempty)));  // MMA commit (res)
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (warp == 0) {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc =
                (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(Nmma >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
            const uint32_t lbo = 128, sbo = 32 * TC_KC;
            int g = 0, i = 0, loads = 0, cur = -1;
            for (int q = q_first; q < q_end && ok; q += q_step, i++) {
                const int a = i & 1;
                ok = mbar_wait(smem_u32(acce + a), ((i >> 1) & 1) ^ 1);
                if (ok && res && ps.items[q].x != cur) {
                    // this tile's operator: the copy of the next class run
                    ok = mbar_wait(smem_u32(bfull), loads & 1);
                    loads++;
                    cur = ps.items[q].x;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t d_tmem = tmem + (uint32_t)(a * 256);
                for (int c = 0; c < nch && ok; c++, g++) {
                    const int s = g % TC_STAGES;
                    ok = mbar_wait(smem_u32(full + s), (g / TC_STAGES) & 1);
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t a_hi = smem_u32(smem + s * stage), a_lo = a_hi + tA;
                    const uint32_t b_hi = res ? smem_u32(bres) + (uint32_t)c * 2 * tB : a_hi + 2 * tA, b_lo = b_hi + tB;
#pragma unroll
                    for (int ks = 0; ks < TC_KC / 8; ks++)
#pragma unroll
                        for (int pass = 0; pass < 3; pass++) {
                            uint64_t ad = smem_desc((pass == 2 ? a_lo : a_hi) + ks * 256, lbo, sbo);
                            uint64_t bd = smem_desc((pass == 1 ? b_lo : b_hi) + ks * 256, lbo, sbo);
                            uint32_t acc = (c > 0 || ks > 0 || pass > 0) ? 1u : 0u;
                            asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %4, 0;\n\t"
                                         "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n\t}" ::"r"(d_tmem),
                                         "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                        }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_u32(empty + s))
                                 : "memory");
                }
                if (ok)
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_u32(accf + a))
                                 : "memory");
                // the last tile of a class run releases the resident operator once its MMAs are done
                if (ok && res && (q + 1 >= q_end || ps.items[q + 1].x != cur))
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_u32(bempty))
                                 : "memory");
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------------- operator copies
        if (lane == 0 && res) {
            // one copy of a class's whole operator per class run
            const uint32_t bytes = (uint32_t)nch * 2 * tB;
            int loads = 0, cur = -1;
            for (int q = q_first; q < q_end && ok; q += q_step) {
                const int4 it = ps.items[q];
                if (it.x == cur) continue;
                if (loads > 0) {
                    ok = mbar_wait(smem_u32(bempty), (loads - 1) & 1);
                    if (!ok) break;
                }
                const uint32_t bar = smem_u32(bfull), dst = smem_u32(bres);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
                asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                             "l"(ps.B + (size_t)it.x * nch * 2 * Nmma * TC_KC), "r"(bytes), "r"(bar)
                             : "memory");
                loads++;
                cur = it.x;
            }
        } else if (lane == 0) {
            const uint32_t bytes = 2 * tB;
            int g = 0;
            for (int q = q_first; q < q_end && ok; q += q_step) {
                const int item = q / ps.nhalf, h = q - item * ps.nhalf;
                const int4 it = ps.items[item];
                const float *Bd = ps.B + (size_t)(it.x * ps.nhalf + h) * nch * 2 * Nmma * TC_KC;
                for (int c = 0; c < nch && ok; c++, g++) {
                    const int s = g % TC_STAGES;
                    ok = mbar_wait(smem_u32(empty + s), ((g / TC_STAGES) & 1) ^ 1);
                    if (!ok) break;
                    const uint32_t bar = smem_u32(full + s), dst = smem_u32(smem + s * stage + 2 * tA);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
                    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                                 "l"(Bd + (size_t)c * 2 * Nmma * TC_KC), "r"(bytes), "r"(bar)
                                 : "memory");
                }
            }
        }
    } else if (warp < TC_EPI0) {
        // ---------------------------------------------------------------- source gather
        // two threads per row (translation), each 8 of every 16-wide K chunk; the loads of the
        // next two chunks are in flight while a chunk waits for its stage and is stored
        constexpr int KH = TC_KC / 2;
        static_assert(KH == 8, "four complex coefficients per thread and chunk half");
        const int at = tid - 64, r = at & (TC_M - 1), kh = (at >> 7) * KH;
        const float *srcf = reinterpret_cast<const float *>(ps.src);
        const bool vec4 = (K & 3) == 0;
        // The CTA's tiles as one stream of chunks u = (tile, chunk); the loads run two chunks
        // ahead of the stores, also across tile boundaries.  The row of the tile after the one
        // being loaded is looked up in two steps while the loads cross the current tile: its
        // work item when they enter it, its translation's source box and direction half way
        // through, so that neither lookup stalls the stream.
        const int ntile = q_first < q_end ? (q_end - q_first + q_step - 1) / q_step : 0;
        const int U = ntile * nch, cmid = nch / 2;
        struct RowSrc {
            const float *row;
            const float2 *ph;
            bool v;
        };
        auto tile_item = [&](int i) -> int4 {
            return i < ntile ? ps.items[(q_first + i * q_step) / ps.nhalf] : make_int4(0, 0, 0, 0);
        };
        // row r of a tile from its translation's raw source box / direction (box < 0: empty row)
        auto row_src = [&](int box, int rr, int dir) -> RowSrc {
            RowSrc o{srcf, ps.PH + ps.phoff, false};
            if (box < 0) return o;
            o.row = srcf + (size_t)(box * ps.nrhs + rr) * K;
            o.ph = ps.PH + (size_t)dir * ps.phstride + ps.phoff;
            o.v = true;
            return o;
        };
        int lt = 0, lc = 0;          // tile and chunk of the next load
        int nbox = -1, nrr = 0, ndir = 0;
        auto lookup = [&](int4 it) {  // the translation of row r of item it
            nbox = -1;
            if (r < it.z) {
                const int e = it.y + r, t = e / ps.nrhs;
                nrr = e - t * ps.nrhs;
                nbox = ps.g_src[t];
                ndir = ps.g_dir[t];
            }
        };
        lookup(tile_item(0));
        RowSrc cur = row_src(nbox, nrr, ndir);
        int4 itn = tile_item(1);
        // the row's source coefficients of chunk u and their phases e^{i m phi}: KH / 2 = 4
        // complex coefficients from i0 = k0 / 2 on (i0 a multiple of 4, so their four orders
        // are one 32-bit word of the m table)
        auto load = [&](float(&x)[KH], float2(&f)[KH / 2]) {
            if (lc == nch) {
                lc = 0;
                lt++;
                cur = row_src(nbox, nrr, ndir);
                itn = tile_item(lt + 1);
            }
            if (lc == cmid) lookup(itn);
            const int k0 = lc * TC_KC + kh;
            lc++;
            {
                const uint32_t mm = *reinterpret_cast<const uint32_t *>(s_m + (k0 >> 1));
#pragma unroll
                for (int j = 0; j < KH / 2; j++) f[j] = __ldg(cur.ph + (int)(signed char)(mm >> (8 * j)));
            }
#pragma unroll
            for (int j = 0; j < KH; j += 4) {
                const int k = k0 + j;
                if (cur.v && vec4 && k + 3 < K) {
                    float4 v = __ldg(reinterpret_cast<const float4 *>(cur.row + k));
                    x[j] = v.x; x[j + 1] = v.y; x[j + 2] = v.z; x[j + 3] = v.w;
                } else {
                    float2 v0 = make_float2(0.f, 0.f), v1 = make_float2(0.f, 0.f);
                    if (cur.v && k + 1 < K) v0 = __ldg(reinterpret_cast<const float2 *>(cur.row + k));
                    if (cur.v && k + 3 < K) v1 = __ldg(reinterpret_cast<const float2 *>(cur.row + k + 2));
                    x[j] = v0.x; x[j + 1] = v0.y; x[j + 2] = v1.x; x[j + 3] = v1.y;
                }
            }
        };
        auto store = [&](float(&x)[KH], const float2(&f)[KH / 2], int u) -> bool {
            const int s = u % TC_STAGES;
#pragma unroll
            for (int j = 0; j < KH / 2; j++) {
                const float xr = x[2 * j], xi = x[2 * j + 1];
                x[2 * j] = xr * f[j].x - xi * f[j].y;
                x[2 * j + 1] = xr * f[j].y + xi * f[j].x;
            }
            if (!mbar_wait(smem_u32(empty + s), ((u / TC_STAGES) & 1) ^ 1)) return false;
            unsigned char *Ahi = smem + s * stage, *Alo = Ahi + tA;
#pragma unroll
            for (int j = 0; j < KH; j += 4) {
                float4 hi, lo;
                hi.x = tf32_round(x[j]); lo.x = tf32_round(x[j] - hi.x);
                hi.y = tf32_round(x[j + 1]); lo.y = tf32_round(x[j + 1] - hi.y);
                hi.z = tf32_round(x[j + 2]); lo.z = tf32_round(x[j + 2] - hi.z);
                hi.w = tf32_round(x[j + 3]); lo.w = tf32_round(x[j + 3] - hi.w);
                const uint32_t o = core_off(r, kh + j, TC_KC);
                *reinterpret_cast<float4 *>(Ahi + o) = hi;
                *reinterpret_cast<float4 *>(Alo + o) = lo;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(full + s));
            return true;
        };
        float xa[KH], xb[KH], xc[KH];
        float2 fa[KH / 2], fb[KH / 2], fc[KH / 2];
        if (U > 0) load(xa, fa);
        if (U > 1) load(xb, fb);
        for (int u = 0; u < U && ok; u += 3) {
            if (u + 2 < U) load(xc, fc);
            ok = store(xa, fa, u);
            if (!ok || u + 1 >= U) break;
            if (u + 3 < U) load(xa, fa);
            ok = store(xb, fb, u + 1);
            if (!ok || u + 2 >= U) break;
            if (u + 4 < U) load(xb, fb);
            ok = store(xc, fc, u + 2);
        }
    } else {
        // ---------------------------------------------------------------- epilogue
        // warp w reads TMEM lane quarter w % 4; the two warps of a quarter take alternate
        // 32-column blocks
        const int wq = warp & 3, eh = (warp - TC_EPI0) >> 2;
        float *st = epi + (warp - TC_EPI0) * 32 * TC_EPI_LD;
        // destinations of coefficient pairs 16-byte aligned: p^2 and the half width even
        const bool pairs = (P2o % 2 == 0) && (ps.CH % 2 == 0);
        int i = 0;
        for (int q = q_first; q < q_end && ok; q += q_step, i++) {
            const int a = i & 1, item = q / ps.nhalf, h = q - item * ps.nhalf;
            const int4 it = ps.items[item];
            const int row = wq * 32 + lane;
            const int dbox = tile_box(ps, it, row, false);
            const int drow = row < it.z ? ps.g_dir[(it.y + row) / ps.nrhs] : 0;
            // rows of one class run hold each direction's translations contiguously, so a tile
            // whose first and last rows share a direction has one direction (one set of phases);
            // passes without phases read a table of ones (phstride 0)
            const int d0 = ps.g_dir[it.y / ps.nrhs];
            const bool uni = !ps.phased || d0 == ps.g_dir[(it.y + it.z - 1) / ps.nrhs];
            const float2 *ph0 = ps.PH + (size_t)d0 * ps.phstride + ps.phoff;
            const int co0 = h * ps.CH, nco = min(ps.CH, P2o - co0);
            ok = mbar_wait(smem_u32(accf + a), (i >> 1) & 1);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            for (int cb = 32 * eh; cb < Nmma; cb += 64) {
                uint32_t v[32];
                const uint32_t ta = tmem + ((uint32_t)(wq * 32) << 16) + (uint32_t)(a * 256 + cb);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                             "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                             : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                               "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                               "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]),
                               "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]),
                               "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                             : "r"(ta));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 32; j++) st[lane * TC_EPI_LD + j] = __uint_as_float(v[j]);
                __syncwarp();
                if (pairs) {
                    // four rows per step, 8 pairs of coefficients per row, each pair added with one
                    // 16-byte atomic; coefficient co of row rr times e^{-i m' phi} of its direction
                    const int jq = lane & 7, co = co0 + cb / 2 + 2 * jq;
                    const bool cv = cb + 4 * jq < 2 * nco;
                    const int m0 = s_m[cv ? co : 0], m1 = s_m[cv ? co + 1 : 0];
                    const float2 u0 = __ldg(ph0 + m0), u1 = __ldg(ph0 + m1);
#pragma unroll 4
                    for (int rq = 0; rq < 8; rq++) {
                        const int rr = 4 * rq + (lane >> 3);
                        const int d = __shfl_sync(0xffffffffu, dbox, rr);
                        const int dr = __shfl_sync(0xffffffffu, drow, rr);
                        if (d >= 0 && cv) {
                            const float2 *pr = ps.PH + (size_t)dr * ps.phstride + ps.phoff;
                            const float2 e0 = uni ? u0 : __ldg(pr + m0), e1 = uni ? u1 : __ldg(pr + m1);
                            const float *y = st + rr * TC_EPI_LD + 4 * jq;
                            const float4 w = make_float4(y[0] * e0.x + y[1] * e0.y, y[1] * e0.x - y[0] * e0.y,
                                                         y[2] * e1.x + y[3] * e1.y, y[3] * e1.x - y[2] * e1.y);
                            atomicAdd(reinterpret_cast<float4 *>(ps.dst + (size_t)d * P2o + co), w);
                        }
                    }
                } else {
                    // two rows per step, 16 coefficients (32 columns) per row
                    const int jc = lane & 15, c2 = cb + 2 * jc, co = co0 + c2 / 2;
                    const bool cv = c2 < 2 * nco;
                    const int mo = s_m[cv ? co : 0];
                    const float2 fu = __ldg(ph0 + mo);
#pragma unroll 4
                    for (int rp = 0; rp < 16; rp++) {
                        const int rr = 2 * rp + (lane >> 4);
                        const int d = __shfl_sync(0xffffffffu, dbox, rr);
                        const int dr = __shfl_sync(0xffffffffu, drow, rr);
                        if (d >= 0 && cv) {
                            const float2 e = uni ? fu : __ldg(ps.PH + (size_t)dr * ps.phstride + ps.phoff + mo);
                            const float yr = st[rr * TC_EPI_LD + 2 * jc], yi = st[rr * TC_EPI_LD + 2 * jc + 1];
                            atomicAdd(ps.dst + (size_t)d * P2o + co, make_float2(yr * e.x + yi * e.y, yi * e.x - yr * e.y));
                        }
                    }
                }
                __syncwarp();
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(acce + a));
        }
    }
    if (!ok) atomicExch(ps.err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// The real-embedded operators of a pass, split into TF32 hi/lo, in the tile layout: element
// (o, k) of half h, chunk c holds  Re T (o, k even-even / odd-odd), -Im T (o even, k odd) or
// Im T (o odd, k even) of coefficient (h CH + o/2, (c KC + k)/2).
// fout / fin (plans with scaled FP32 expansions, else null): per-degree factors of the
// destination and source coefficients, so that the operator maps the scaled expansions
// (multipoles d_n M_n, locals L_n / d_n of their own levels).
__global__ void tc_split_kernel(const double2 *__restrict__ T, int pin, int pout, int KC, int nch, int nhalf, int CH,
                                int Nmma, const double *__restrict__ fout, const double *__restrict__ fin,
                                float *__restrict__ B, size_t total)
{
    const int P2i = pin * pin, P2o = pout * pout, K = 2 * P2i;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
        size_t z = q;
        int kcol = (int)(z % KC); z /= KC;
        int nr = (int)(z % Nmma); z /= Nmma;
        int part = (int)(z % 2); z /= 2;
        int c = (int)(z % nch); z /= nch;
        int h = (int)(z % nhalf);
        int d = (int)(z / nhalf);
        int k = c * KC + kcol, nco = min(CH, P2o - h * CH);
        double v = 0.0;
        if (nr < 2 * nco && k < K) {
            const int io = h * CH + nr / 2, ii = k / 2;
            double2 t = T[((size_t)d * P2o + io) * P2i + ii];
            int po = nr & 1, pi = k & 1;
            v = po == 0 ? (pi == 0 ? t.x : -t.y) : (pi == 0 ? t.y : t.x);
            if (fout) v *= fout[(int)sqrtf((float)io + 0.5f)] * fin[(int)sqrtf((float)ii + 0.5f)];
        }
        float hi = tf32_round((float)v);
        float lo = tf32_round((float)(v - (double)hi));
        size_t base = ((((size_t)d * nhalf + h) * nch + c) * 2 + part) * (size_t)Nmma * KC;
        B[base + core_off(nr, kcol, KC) / 4] = part ? lo : hi;
    }
}

// The list of a pass and its orders: M2L of level l, M2M of level l into its parents, L2L of
// the parents into level l.
static RcrList *dense_list(Plan *P, int l, int which, int &pin, int &pout)
{
    LevelDev &L = P->lev[l];
    if (which == PASS_M2L) {
        pin = pout = L.p;
        return &L.m2l;
    }
    if (l <= P->lmin) return nullptr;
    const int pp = P->lev[l - 1].p;
    pin = which == PASS_M2M ? L.p : pp;
    pout = which == PASS_M2M ? pp : L.p;
    return which == PASS_M2M ? &L.m2m : &L.l2l;
}

static int build_tc_dense(Plan *P, int l, int which)
{
    int pin = 0, pout = 0;
    RcrList *Lst = dense_list(P, l, which, pin, pout);
    if (!Lst || Lst->key_beg.empty() || Lst->key_beg.back() == 0) return FMM_OK;
    TcDense &g = Lst->td;
    if (!tc_geometry(pin, pout, g)) return FMM_OK;
    g.pin = pin;
    g.pout = pout;
    const int nkeys = (int)Lst->key_beg.size() - 1, P2i = pin * pin, P2o = pout * pout;
    std::vector<int> rep;
    if (which == PASS_M2L) {
        g.phased = 1;
        direction_classes(P, PASS_M2L, nkeys, g.cls_of_dir, rep);
    } else {
        g.phased = 0;  // eight octant operators, phases included
        g.cls_of_dir.resize(nkeys);
        for (int d = 0; d < nkeys; d++) g.cls_of_dir[d] = d;
        rep = g.cls_of_dir;
    }
    g.ncls = (int)rep.size();
    size_t total = (size_t)g.ncls * g.nhalf * g.nch * 2 * g.Nmma * g.KC;
    double2 *T = nullptr;
    int *rep_dev = nullptr;
    double *fdev = nullptr;
    auto fail = [&](cudaError_t e) {
        cudaFree(T);
        cudaFree(rep_dev);
        cudaFree(fdev);
        fmm_set_error("tensor-core pass tables: %s", cudaGetErrorString(e));
        return FMM_ERR_CUDA;
    };
    cudaError_t e = cudaMalloc(&T, sizeof(double2) * (size_t)g.ncls * P2o * P2i);
    if (e == cudaSuccess) e = cudaMalloc(&rep_dev, sizeof(int) * rep.size());
    if (e == cudaSuccess) e = cudaMemcpy(rep_dev, rep.data(), sizeof(int) * rep.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(e);
    int st = gen_dense_rcr(P, l, which, rep_dev, g.ncls, T);
    if (st) {
        cudaFree(T);
        cudaFree(rep_dev);
        return st;
    }
    // degree factors of the scaled expansions: M2L 1/d^l both sides; M2M d^{l-1} out, 1/d^l
    // in; L2L 1/d^l out, d^{l-1} in
    const double *fo = nullptr, *fi = nullptr;
    if (P->scaled) {
        const int pm = std::max(pin, pout);
        std::vector<double> h(2 * pm, 1.0);
        for (int n = 0; n < pm; n++) {
            const double inv = 1.0 / P->dsc[l][n], par = which == PASS_M2L ? 1.0 : P->dsc[l - 1][n];
            h[n] = which == PASS_M2M ? par : inv;           // out
            h[pm + n] = which == PASS_L2L ? par : inv;      // in
        }
        e = cudaMalloc(&fdev, sizeof(double) * h.size());
        if (e == cudaSuccess) e = cudaMemcpy(fdev, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(e);
        fo = fdev;
        fi = fdev + pm;
    }
    e = dev_alloc(P, (void **)&g.B, sizeof(float) * total);
    if (e != cudaSuccess) return fail(e);
    g.B_bytes = sizeof(float) * total;
    tc_split_kernel<<<152 * 16, 256, 0, P->stream>>>(T, pin, pout, g.KC, g.nch, g.nhalf, g.CH, g.Nmma, fo, fi, g.B, total);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
    cudaFree(T);
    cudaFree(rep_dev);
    cudaFree(fdev);
    T = nullptr;
    rep_dev = nullptr;
    fdev = nullptr;
    if (e != cudaSuccess) return fail(e);
    return FMM_OK;
}

__global__ void tc_permute_kernel(int n, const int *__restrict__ perm, const int *__restrict__ src,
                                  const int *__restrict__ dst, int *__restrict__ psrc, int *__restrict__ pdst)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int t = perm[i];
        psrc[i] = src[t];
        pdst[i] = dst[t];
    }
}

// The pass's translations in class order and the tiles over them, rebuilt when nrhs changes:
// where the expansions of nrhs columns are more than L2 keeps, the destination boxes are cut
// into Morton ranges first (as for the SIMT tiles); within a range, class by class, the runs
// of the class's keys one after another (each run sorted by destination).  Tiles are (class,
// first column, count) of at most 128 columns e = t nrhs + r.
static int ensure_td_items(RcrList &Lst, size_t ws, int nrhs, cudaStream_t st)
{
    TcDense &g = Lst.td;
    if (g.items_nrhs == nrhs) return FMM_OK;
    const int nkeys = (int)Lst.key_beg.size() - 1, T = Lst.key_beg.back(), nd = std::max(Lst.ndst_rank, 1);
    const size_t budget = 48u << 20;
    const long long nblk = std::min<long long>(nd, std::max<long long>(1, (long long)((ws + budget - 1) / budget)));
    std::vector<std::vector<int>> dirs(g.ncls);
    for (int d = 0; d < nkeys; d++) dirs[g.cls_of_dir[d]].push_back(d);
    std::vector<int> perm, pdir;
    std::vector<int4> items;
    perm.reserve(T);
    pdir.reserve(T);
    const int *rk = Lst.dst_rank.data();
    for (long long k = 0; k < nblk; k++) {
        const int lo = (int)(k * nd / nblk), hi = (int)((k + 1) * nd / nblk);
        for (int c = 0; c < g.ncls; c++) {
            const long long r0 = (long long)perm.size();
            for (int d : dirs[c]) {
                int a0 = Lst.key_beg[d], a1 = Lst.key_beg[d + 1];
                if (nblk > 1) {
                    a0 = (int)(std::lower_bound(rk + Lst.key_beg[d], rk + Lst.key_beg[d + 1], lo) - rk);
                    a1 = (int)(std::lower_bound(rk + Lst.key_beg[d], rk + Lst.key_beg[d + 1], hi) - rk);
                }
                for (int a = a0; a < a1; a++) {
                    perm.push_back(a);
                    pdir.push_back(d);
                }
            }
            const long long e0 = r0 * nrhs, e1 = (long long)perm.size() * nrhs;
            for (long long a = e0; a < e1; a += TC_M)
                items.push_back(make_int4(c, (int)a, (int)std::min<long long>(TC_M, e1 - a), 0));
        }
    }
    if ((int)perm.size() != T) {
        fmm_set_error("tensor-core pass: the class order covers %d of %d translations", (int)perm.size(), T);
        return FMM_ERR_ARG;
    }
    if (!g.src && T > 0) {
        FMM_CUDA_TRY(cudaMalloc(&g.src, sizeof(int) * T));
        FMM_CUDA_TRY(cudaMalloc(&g.dst, sizeof(int) * T));
        FMM_CUDA_TRY(cudaMalloc(&g.dir, sizeof(int) * T));
    }
    if (T > 0) {
        int *perm_dev = nullptr;
        FMM_CUDA_TRY(cudaMalloc(&perm_dev, sizeof(int) * T));
        cudaError_t e = cudaMemcpy(perm_dev, perm.data(), sizeof(int) * T, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(g.dir, pdir.data(), sizeof(int) * T, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            tc_permute_kernel<<<(T + 255) / 256, 256, 0, st>>>(T, perm_dev, Lst.src, Lst.dst, g.src, g.dst);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(perm_dev);
        if (e != cudaSuccess) { fmm_set_error("tensor-core pass lists: %s", cudaGetErrorString(e)); return FMM_ERR_CUDA; }
    }
    if (items.size() > g.items_cap) {
        if (g.items) cudaFree(g.items);
        g.items = nullptr;
        FMM_CUDA_TRY(cudaMalloc(&g.items, sizeof(int4) * items.size()));
        g.items_cap = items.size();
    }
    if (!items.empty()) FMM_CUDA_TRY(cudaMemcpy(g.items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
    g.n_items = (int)items.size();
    g.items_nrhs = nrhs;
    return FMM_OK;
}

int launch_tc_dense(Plan *P, int l, int which, int nrhs, cudaStream_t st)
{
    int pin = 0, pout = 0;
    RcrList *Lst = dense_list(P, l, which, pin, pout);
    if (!Lst || Lst->key_beg.empty() || Lst->key_beg.back() == 0) return FMM_OK;
    TcDense &g = Lst->td;
    RcrPass rp;
    pass32_desc(P, l, which, nrhs, rp);
    const size_t ws = ((size_t)rp.nsrc * pin * pin + (size_t)rp.ndst * pout * pout) * sizeof(float2) * nrhs;
    int e = ensure_td_items(*Lst, ws, nrhs, st);
    if (e) return e;
    if (!P->tc_ones) {
        std::vector<float2> ones(2 * TC_MAXP + 1, make_float2(1.f, 0.f));
        FMM_CUDA_TRY(dev_alloc(P, (void **)&P->tc_ones, sizeof(float2) * ones.size()));
        FMM_CUDA_TRY(cudaMemcpy(P->tc_ones, ones.data(), sizeof(float2) * ones.size(), cudaMemcpyHostToDevice));
    }
    TcPass ps;
    ps.items = g.items;
    ps.g_src = g.src;
    ps.g_dst = g.dst;
    ps.g_dir = g.dir;
    ps.phased = g.phased;
    ps.PH = g.phased ? P->PHsr32 : P->tc_ones;
    ps.phstride = g.phased ? 2 * P->pmax - 1 : 0;
    ps.phoff = g.phased ? P->pmax - 1 : TC_MAXP;
    ps.nrhs = nrhs;
    ps.nsrc = rp.nsrc;
    ps.ndst = rp.ndst;
    ps.pin = pin;
    ps.P2o = pout * pout;
    ps.K = 2 * pin * pin;
    ps.nch = g.nch;
    ps.nhalf = g.nhalf;
    ps.CH = g.CH;
    ps.Nmma = g.Nmma;
    ps.ntiles = g.n_items * g.nhalf;
    ps.res = g.res;
    ps.B = g.B;
    ps.src = rp.src;
    ps.dst = rp.dst;
    ps.err = P->tc_err;
    size_t sm = tc_smem_bytes(g.Nmma, g.res, g.nch);
    static size_t attr = 0;
    e = raise_smem_limit((const void *)tc_dense_kernel, sm, &attr);
    if (e) return e;
    // persistent: one CTA per SM (its shared memory and 512 TMEM columns take the SM)
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (nsm <= 0) nsm = 152;
    }
    tc_dense_kernel<<<std::min(ps.ntiles, nsm), TC_THREADS, sm, st>>>(ps);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

// The bounded wait on its own: an mbarrier that expects one arrival nobody makes is waited on
// with a limit of `cycles` (out[0] = 1 if that wait gave up), then completed and waited on again
// (out[1] = 1 if that wait saw the phase complete).
__global__ void wait_probe_kernel(long long cycles, int *out)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x != 0) return;
    const uint32_t b = smem_u32(&bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b));
    out[0] = mbar_wait_limit(b, 0, cycles) ? 0 : 1;
    mbar_arrive(b);
    out[1] = mbar_wait_limit(b, 0, cycles) ? 1 : 0;
}

} // namespace fmm

extern "C" int fmm_selftest_bounded_wait(int device, int *gave_up, int *completed)
{
    using namespace fmm;
    if (!gave_up || !completed) { fmm_set_error("fmm_selftest_bounded_wait: null argument"); return FMM_ERR_ARG; }
    FMM_CUDA_TRY(cudaSetDevice(device));
    int *d = nullptr, h[2] = {0, 0};
    FMM_CUDA_TRY(cudaMalloc(&d, sizeof(h)));
    wait_probe_kernel<<<1, 32>>>(2000000LL, d);  // ~1 ms at 2 GHz
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) { fmm_set_error("fmm_selftest_bounded_wait: %s", cudaGetErrorString(e)); return FMM_ERR_CUDA; }
    *gave_up = h[0];
    *completed = h[1];
    return FMM_OK;
}

namespace fmm {

int check_tc_error(Plan *P)
{
    if (!P->tc_err) return FMM_OK;
    int h = 0;
    FMM_CUDA_TRY(cudaMemcpy(&h, P->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        fmm_set_error("tensor-core M2L: a wait on its MMA barriers gave up");
        return FMM_ERR_CUDA;
    }
    return FMM_OK;
}

static void td_free(Plan *P, TcDense &g)
{
    cudaFree(g.B);
    P->device_bytes -= g.B_bytes;
    cudaFree(g.items);
    cudaFree(g.src);
    cudaFree(g.dst);
    cudaFree(g.dir);
    g = TcDense();
}

// For every pass whose source and destination orders are both <= 16 (M2L of a level, M2M
// into and L2L out of its parent level): build the dense split operators and keep the
// tensor-core pass where it beats the SIMT tiles on this plan (4 timed runs each), else free
// its tables.  FMMBEM_TENSOR_M2L (M2L) and FMMBEM_TENSOR_M2M (M2M and L2L) = 0 keep the SIMT
// tiles, = 1 take the tensor cores wherever they apply.  M2M and L2L stay on the SIMT tiles
// unless FMMBEM_TENSOR_M2M is set: their dense form is twice as fast but about ten times
// less accurate on the 81,920-triangle sphere (mixed against FP64 8.9e-7 against 7.7e-8),
// which costs the refined solves more iterations than it saves.
int tune_tc_dense(Plan *P)
{
    const char *env_l = getenv("FMMBEM_TENSOR_M2L"), *env_m = getenv("FMMBEM_TENSOR_M2M");
    const int mode_l = env_l ? atoi(env_l) : -1, mode_m = env_m ? atoi(env_m) : 0;
    if (mode_l == 0 && mode_m == 0) return FMM_OK;
    if (!P->tc_err) {
        FMM_CUDA_TRY(dev_alloc(P, (void **)&P->tc_err, sizeof(int)));
        FMM_CUDA_TRY(cudaMemset(P->tc_err, 0, sizeof(int)));
    }
    cudaEvent_t a, b;
    FMM_CUDA_TRY(cudaEventCreate(&a));
    FMM_CUDA_TRY(cudaEventCreate(&b));
    int rc = FMM_OK;
    for (int l = P->lmin; l <= P->lmax && rc == FMM_OK; l++) {
        for (int which = PASS_M2M; which <= PASS_L2L && rc == FMM_OK; which++) {
            const int mode = which == PASS_M2L ? mode_l : mode_m;
            if (mode == 0) continue;
            int pin = 0, pout = 0;
            RcrList *Lst = dense_list(P, l, which, pin, pout);
            if (!Lst || Lst->key_beg.empty() || Lst->key_beg.back() == 0) continue;
            rc = build_tc_dense(P, l, which);
            if (rc) break;
            if (!Lst->td.B) continue;  // orders beyond the dense form
            float ms[2] = {0.f, 0.f};
            for (int on = 0; on < 2 && rc == FMM_OK && mode != 1; on++) {
                Lst->td.on = on;
                for (int rep = 0; rep < 4 && rc == FMM_OK; rep++) {
                    if (cudaEventRecord(a, P->stream) != cudaSuccess) rc = FMM_ERR_CUDA;
                    if (rc == FMM_OK) rc = launch_pass32(P, l, which, 1, P->stream);
                    if (rc == FMM_OK && cudaEventRecord(b, P->stream) != cudaSuccess) rc = FMM_ERR_CUDA;
                    if (rc == FMM_OK && cudaEventSynchronize(b) != cudaSuccess) rc = FMM_ERR_CUDA;
                    float t = 0.f;
                    cudaEventElapsedTime(&t, a, b);
                    if (rep > 0) ms[on] += t;
                }
            }
            if (rc == FMM_OK) rc = check_tc_error(P);
            if (rc) break;
            Lst->td.on = (mode == 1 || ms[1] < ms[0]) ? 1 : 0;
            if (!Lst->td.on) td_free(P, Lst->td);
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc == FMM_ERR_CUDA && !fmm_last_error()[0]) fmm_set_error("tensor-core pass tuning: %s", cudaGetErrorString(cudaGetLastError()));
    return rc;
}

} // namespace fmm
