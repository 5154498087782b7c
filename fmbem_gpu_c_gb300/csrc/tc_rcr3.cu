// Batched RCR translations of the mixed path on the 5th-generation tensor cores
// (tcgen05.mma kind::tf32, split TF32), in three stages with the intermediates in a device
// scratch that stays in L2.
//
// One translation is rotate - coaxial - rotate (transMatsVecsMul_SR_rcr, reference
// translation.cu:1864-1961; the per-translation kernels cuSparseRotsVecsMul and
// cuSparseCoaxTransMatsVecsMul, translation.cu:1623, 1644):
//   R1  W_n = H_n (Phi x)_n          for every degree n (H_n real (2n+1)^2, Phi = e^{i m phi})
//   C   Z_m = C_|m| W_m              for every order m (C complex (p-|m|)^2, +m and -m share it)
//   R2  y_n += conj(Phi) H_n Z_n     for every degree n, added into the destination expansion
// H depends only on the polar angle of the translation, C only on its length.  So each stage
// is a batched GEMM over the translations that share its operator: the rotation stages group
// the translations of a pass by polar-angle class (e.g. all M2L offsets with the same dz and
// dx^2+dy^2; their azimuths only enter through the phases, applied while gathering and while
// writing), the coaxial stage by length class.  Classes hold many more translations than one
// direction, which keeps the tiles full at the coarse levels.
//
// Each tile is 64 columns (translation x right-hand side) of one class; the GEMM puts the data
// on the MMA's M side, 128 rows = 64 columns x 2 parts (re, im in the rotation stages, the +m and
// -m orders in the coaxial stage), and one operator block (one degree, or one order) on the N
// side: D[row][o] = sum_k A[row][k] B[o][k], K and N the block's size padded to 8 and 16, so the
// block-diagonal structure costs no MMA work.  Operands are split into TF32 hi and lo halves,
// each rounded to nearest, and multiplied as hi*hi + hi*lo + lo*hi with FP32 accumulation in
// TMEM (FP32-level accuracy).
//
// A persistent kernel per stage (one CTA per SM, 14 warps) runs over (tile, block range) items:
//   warp 0     issues the MMAs (one thread) of each block into one of four TMEM accumulators
//              (128 columns each), committing every K chunk to its stage's "empty" barrier and
//              every block to its accumulator's "full" barrier;
//   warp 1     copies the operator's K chunks (hi and lo tiles, precomputed in the core-matrix
//              layout) with cp.async.bulk;
//   warps 2-9  gather the data rows of every K chunk (source expansions with their phases, or the
//              previous stage's scratch), split them into TF32 hi / lo in shared memory;
//   warps 10-13 read finished accumulators (tcgen05.ld, one TMEM lane quarter per warp) and write
//              the stage's output: the scratch, or (R2) the destination expansions with their
//              phases, by FP32 atomics where several translations reach one box.
// Four shared-memory stages of K = 16; every wait has a time limit, after which the thread sets
// the plan's error flag and stops.  Passes are cut into chunks of translations whose scratch (W
// and Z, p^2 FP32 complex per column) fits the budget, three launches per chunk.
#include "plan.h"
#include "tc_common.cuh"
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

namespace fmm {

constexpr int T3_M = 128;
constexpr int T3_COLS = 64;
constexpr int T3_KC = 16;
constexpr int T3_SA = 4;            // data stages (A hi / lo)
constexpr int T3_SBMAX = 8;         // operator stages (B hi / lo) at most
constexpr int T3_SLOTS = 4;         // TMEM accumulators of 128 columns
constexpr int T3_NMAX = 128;
constexpr int T3_THREADS = 448;
constexpr int T3_GWARPS = 8;
constexpr int T3_EPI0 = 2 + T3_GWARPS;
constexpr uint32_t T3_TA = T3_M * T3_KC * 4;
constexpr size_t T3_SMEM_MAX = 227 * 1024 - 2048;  // dynamic shared memory beside the static tables
constexpr size_t T3_BAR_BYTES = (2 * T3_SA + 2 * T3_SBMAX + 2 * T3_SLOTS) * 8 + 16;
constexpr size_t T3_SCRATCH_BYTES = (size_t)32 << 20; // per scratch buffer (W, Z) of one pass
constexpr int T3_MAXP = 64;

enum { T3_R1 = 0, T3_C = 1, T3_R2 = 2 };

struct T3Args {
    int p, pinr, nq, nrhs, n_items, t0, nblk;
    int sb, s2;              // operator stages; staging row stride (float2) of the epilogue, 0 if none
    uint32_t bstage;         // bytes of one operator stage
    const int4 *items;       // (class, first column, count, b0 | b1 << 16)
    const int4 *blk;         // per block: (operator offset in floats, K, Npad, valid N); nblk of them
    const int *list;         // stage position -> translation of the chunk (chunk-local)
    const int *g_src, *g_dst, *t_dir;  // g_src set for R1 only
    const float2 *PH;
    int phstride, phoff;
    const float *ops;
    long long ops_stride;    // floats per class
    const float2 *src;       // R1: source expansions [box][rhs][src_stride]
    int src_stride;
    const float2 *in;        // C: W, R2: Z, [column][p^2] in the paired order
    float2 *out;             // R1: W, C: Z
    float2 *dst;             // R2: destination expansions [box][rhs][dst_stride]
    int dst_stride, atomic;
    int *err;
};

// Scratch order within degree n: m = 0 first, then the pairs (m, -m) for m = 1..n, so that the
// coaxial stage, which reads and writes +m and -m together, touches one sector for both.
__host__ __device__ __forceinline__ int t3_pm(int m) { return m == 0 ? 0 : (m > 0 ? 2 * m - 1 : -2 * m); }

// dynamic shared memory of a launch: data stages, operator stages, epilogue staging, barriers
static inline size_t t3_smem(uint32_t bstage, int sb, int s2)
{
    return (size_t)T3_SA * 2 * T3_TA + (size_t)sb * bstage + (size_t)4 * 16 * s2 * 8 + T3_BAR_BYTES;
}

__device__ __forceinline__ void t3_store(unsigned char *Ahi, unsigned char *Alo, int row, int k, const float (&v)[4])
{
    float4 hi, lo;
    hi.x = tf32_round(v[0]); lo.x = tf32_round(v[0] - hi.x);
    hi.y = tf32_round(v[1]); lo.y = tf32_round(v[1] - hi.y);
    hi.z = tf32_round(v[2]); lo.z = tf32_round(v[2] - hi.z);
    hi.w = tf32_round(v[3]); lo.w = tf32_round(v[3] - hi.w);
    const uint32_t o = core_off(row, k, T3_KC);
    *reinterpret_cast<float4 *>(Ahi + o) = hi;
    *reinterpret_cast<float4 *>(Alo + o) = lo;
}

// Position (item, block, K chunk) in a CTA's sequence of chunks (q >= n_items past the end),
// with what the gathering thread of column ci needs of the item, resolved once per item: the
// scratch column (-1 where the tile has no column ci), and for R1 the source box and the
// direction's phases.
struct T3Cursor {
    int q, b, c, b1, nch;
    int col, box;
    const float2 *ph;
};

__device__ __forceinline__ void t3_cur_item(T3Cursor &u, const T3Args &a, const int4 *blk, int ci)
{
    u.c = 0;
    u.col = -1;
    if (u.q < a.n_items) {
        const int4 it = a.items[u.q];
        u.b = it.w & 0xffff;
        u.b1 = it.w >> 16;
        u.nch = (blk[u.b].y + T3_KC - 1) / T3_KC;
        if (ci < it.z) {
            const int pos = it.y + ci, tl = a.list[pos / a.nrhs], rr = pos - (pos / a.nrhs) * a.nrhs;
            u.col = tl * a.nrhs + rr;
            if (a.g_src) {
                const int t = a.t0 + tl;
                u.box = a.g_src[t] * a.nrhs + rr;
                u.ph = a.PH + (size_t)a.t_dir[t] * a.phstride + a.phoff;
            }
        }
    }
}

__device__ __forceinline__ void t3_cur_next(T3Cursor &u, const T3Args &a, const int4 *blk, int ci)
{
    if (u.q >= a.n_items) return;
    if (++u.c < u.nch) return;
    u.c = 0;
    if (++u.b < u.b1) {
        u.nch = (blk[u.b].y + T3_KC - 1) / T3_KC;
        return;
    }
    u.q += gridDim.x;
    t3_cur_item(u, a, blk, ci);
}

// one thread's loads for one chunk (valid = 0 past the end of the CTA's sequence): R1 source
// values and their phases, R2 the Z values, C the W values of order +m (x[0..1]) and -m (x[2..3])
struct T3Raw {
    float2 x[4], e[4];
    int valid;
};

template <int ST>
__device__ __forceinline__ void t3_load(const T3Args &a, const T3Cursor &u, const int4 *blk, int qk, T3Raw &r)
{
#pragma unroll
    for (int j = 0; j < 4; j++) r.x[j] = r.e[j] = make_float2(0.f, 0.f);
    r.valid = u.q < a.n_items;
    if (!r.valid || u.col < 0) return;
    const int P2 = a.p * a.p, K = blk[u.b].y, k0 = u.c * T3_KC + 4 * qk;
    if (ST == T3_C) {
        // order m = b; K entries (n, part) for n = m + k/2 < pinr
        const int m = u.b;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (k0 + 2 * h < K) {
                const int n = m + k0 / 2 + h;
                const float2 *row = a.in + (size_t)u.col * P2 + n * n;
                r.x[h] = __ldg(row + t3_pm(m));
                if (m > 0) r.x[2 + h] = __ldg(row + t3_pm(-m));
            }
        }
    } else {
        // degree n = b; K entries m + n for |m| <= n, |m| < pinr
        const int n = u.b;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int k = k0 + j, m = k - n;
            if (k < K && m < a.pinr && -m < a.pinr) {
                if (ST == T3_R1) {
                    r.x[j] = __ldg(a.src + (size_t)u.box * a.src_stride + n * n + k);
                    r.e[j] = __ldg(u.ph + m);
                } else {
                    r.x[j] = __ldg(a.in + (size_t)u.col * P2 + n * n + t3_pm(m));
                }
            }
        }
    }
}

// the two data rows of a thread's chunk from its loads
template <int ST>
__device__ __forceinline__ void t3_values(const T3Raw &r, float (&v0)[4], float (&v1)[4])
{
    if (ST == T3_C) {
        v0[0] = r.x[0].x; v0[1] = r.x[0].y; v0[2] = r.x[1].x; v0[3] = r.x[1].y;
        v1[0] = r.x[2].x; v1[1] = r.x[2].y; v1[2] = r.x[3].x; v1[3] = r.x[3].y;
    } else if (ST == T3_R1) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            v0[j] = r.x[j].x * r.e[j].x - r.x[j].y * r.e[j].y;
            v1[j] = r.x[j].x * r.e[j].y + r.x[j].y * r.e[j].x;
        }
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            v0[j] = r.x[j].x;
            v1[j] = r.x[j].y;
        }
    }
}

template <int ST>
__global__ void __launch_bounds__(T3_THREADS, 1) rcr3_kernel(T3Args a)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *aring = smem;
    unsigned char *bring = aring + (size_t)T3_SA * 2 * T3_TA;
    float2 *stg_all = reinterpret_cast<float2 *>(bring + (size_t)a.sb * a.bstage);
    uint64_t *bars = reinterpret_cast<uint64_t *>(stg_all + (size_t)4 * 16 * a.s2);
    uint64_t *fulla = bars, *emptya = fulla + T3_SA, *fullb = emptya + T3_SA, *emptyb = fullb + T3_SBMAX;
    uint64_t *accf = emptyb + T3_SBMAX, *acce = accf + T3_SLOTS;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(acce + T3_SLOTS);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int P2 = a.p * a.p, SB = a.sb;
    __shared__ int4 s_blk[T3_MAXP];
    __shared__ int4 s_cinfo[4][16];  // epilogue: per warp, its 16 columns (scratch column, box, direction)
    for (int b = tid; b < a.nblk; b += blockDim.x) s_blk[b] = a.blk[b];
    const int4 *blk = s_blk;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 32) {
        for (int s = 0; s < T3_SA; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(fulla + s)), "r"(T3_GWARPS));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(emptya + s)));
        }
        for (int s = 0; s < SB; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(fullb + s)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(emptyb + s)));
        }
        for (int j = 0; j < T3_SLOTS; j++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(accf + j)));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(smem_u32(acce + j)));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (warp == 0) {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0) {
            const uint32_t lbo = 128, sbo = 32 * T3_KC;
            int g = 0, i = 0;
            for (int q = blockIdx.x; q < a.n_items && ok; q += gridDim.x) {
                const int4 it = a.items[q];
                const int b1 = it.w >> 16;
                for (int b = it.w & 0xffff; b < b1 && ok; b++, i++) {
                    const int4 bk = blk[b];
                    const int K = bk.y, Npad = bk.z, slot = i % T3_SLOTS;
                    ok = mbar_wait(smem_u32(acce + slot), ((i / T3_SLOTS) & 1) ^ 1);
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t d_tmem = tmem + (uint32_t)(slot * T3_NMAX);
                    const uint32_t idesc =
                        (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(Npad >> 3) << 17) | ((uint32_t)(T3_M >> 4) << 24);
                    const int nch = (K + T3_KC - 1) / T3_KC;
                    for (int c = 0; c < nch && ok; c++, g++) {
                        const int sa = g % T3_SA, sbi = g % SB;
                        ok = mbar_wait(smem_u32(fulla + sa), (g / T3_SA) & 1) &&
                             mbar_wait(smem_u32(fullb + sbi), (g / SB) & 1);
                        if (!ok) break;
                        asm volatile("tcgen05.fence::after_thread_sync;");
                        const uint32_t a_hi = smem_u32(aring + (size_t)sa * 2 * T3_TA), a_lo = a_hi + T3_TA;
                        const uint32_t b_hi = smem_u32(bring + (size_t)sbi * a.bstage), b_lo = b_hi + (uint32_t)Npad * T3_KC * 4;
                        const int nks = K - c * T3_KC > 8 ? 2 : 1;
                        for (int ks = 0; ks < nks; ks++)
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
                                         smem_u32(emptya + sa))
                                     : "memory");
                        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                         smem_u32(emptyb + sbi))
                                     : "memory");
                    }
                    if (ok)
                        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                         smem_u32(accf + slot))
                                     : "memory");
                }
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------------- operator copies
        if (lane == 0) {
            int g = 0;
            for (int q = blockIdx.x; q < a.n_items && ok; q += gridDim.x) {
                const int4 it = a.items[q];
                const int b1 = it.w >> 16;
                const float *opc = a.ops + (long long)it.x * a.ops_stride;
                for (int b = it.w & 0xffff; b < b1 && ok; b++) {
                    const int4 bk = blk[b];
                    const int K = bk.y, Npad = bk.z, nch = (K + T3_KC - 1) / T3_KC;
                    const uint32_t bytes = 2u * (uint32_t)Npad * T3_KC * 4;
                    for (int c = 0; c < nch && ok; c++, g++) {
                        const int s = g % SB;
                        ok = mbar_wait(smem_u32(emptyb + s), ((g / SB) & 1) ^ 1);
                        if (!ok) break;
                        const uint32_t bar = smem_u32(fullb + s), dst = smem_u32(bring + (size_t)s * a.bstage);
                        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
                        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                                     "l"(opc + bk.x + (size_t)c * 2 * Npad * T3_KC), "r"(bytes), "r"(bar)
                                     : "memory");
                    }
                }
            }
        }
    } else if (warp < T3_EPI0) {
        // ---------------------------------------------------------------- data gather
        // thread (column ci, K quarter qk): rows 2 ci and 2 ci + 1, four K entries of every chunk.
        // Four chunks of loads are in flight: a buffer is reloaded right after it is stored.
        const int gt = tid - 64, ci = gt >> 2, qk = gt & 3;
        T3Cursor ul;
        ul.q = blockIdx.x;
        t3_cur_item(ul, a, blk, ci);
        T3Raw r[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            t3_load<ST>(a, ul, blk, qk, r[j]);
            t3_cur_next(ul, a, blk, ci);
        }
        for (int g = 0; ok; g += 4) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (!ok || !r[j].valid) {
                    ok = false;
                    break;
                }
                float v0[4], v1[4];
                t3_values<ST>(r[j], v0, v1);
                const int s = (g + j) % T3_SA;
                if (!mbar_wait(smem_u32(emptya + s), (((g + j) / T3_SA) & 1) ^ 1)) {
                    ok = false;
                    atomicExch(a.err, 1);
                    break;
                }
                unsigned char *Ahi = aring + (size_t)s * 2 * T3_TA, *Alo = Ahi + T3_TA;
                t3_store(Ahi, Alo, 2 * ci, 4 * qk, v0);
                t3_store(Ahi, Alo, 2 * ci + 1, 4 * qk, v1);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(fulla + s));
                t3_load<ST>(a, ul, blk, qk, r[j]);
                t3_cur_next(ul, a, blk, ci);
            }
        }
        ok = true; // the end of the sequence is not an error; a failed wait set the flag above
    } else {
        // ---------------------------------------------------------------- epilogue
        // Warp w reads TMEM lane quarter w & 3: rows of 16 columns, re and im (or +m and -m) in
        // adjacent lanes.  The rotation stages stage a block's outputs for their 16 columns in
        // shared memory and write them out with consecutive lanes on consecutive entries of a
        // column (several columns per pass when a column has fewer than 32 entries); the coaxial
        // stage writes its +m and -m rows to adjacent scratch entries directly.
        const int wq = warp & 3, row = wq * 32 + lane, ci = row >> 1, part = row & 1, cl = lane >> 1;
        const int ew = warp - T3_EPI0;
        float2 *stg = stg_all + (size_t)ew * 16 * a.s2;
        float *stgf = reinterpret_cast<float *>(stg);
        int4 *cinfo = s_cinfo[ew];
        int i = 0;
        for (int q = blockIdx.x; q < a.n_items && ok; q += gridDim.x) {
            const int4 it = a.items[q];
            const int b1 = it.w >> 16;
            const bool valid = ci < it.z;
            int col = -1;
            const float2 *ph = a.PH + a.phoff;
            if (valid) {
                const int pos = it.y + ci, tl = a.list[pos / a.nrhs], r = pos - (pos / a.nrhs) * a.nrhs;
                col = tl * a.nrhs + r;
                if (ST == T3_R2) ph = a.PH + (size_t)a.t_dir[a.t0 + tl] * a.phstride + a.phoff;
                if (ST != T3_C && part == 0) {
                    int dbox = 0, dir = 0;
                    if (ST == T3_R2) {
                        const int t = a.t0 + tl;
                        dbox = a.g_dst[t] * a.nrhs + r;
                        dir = a.t_dir[t];
                    }
                    cinfo[cl] = make_int4(col, dbox, dir, 0);
                }
            } else if (ST != T3_C && part == 0) {
                cinfo[cl] = make_int4(-1, 0, 0, 0);
            }
            __syncwarp();
            for (int b = it.w & 0xffff; b < b1 && ok; b++, i++) {
                const int4 bk = blk[b];
                const int Npad = bk.z, nout = bk.w, slot = i % T3_SLOTS;
                ok = mbar_wait(smem_u32(accf + slot), (i / T3_SLOTS) & 1);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                for (int j0 = 0; j0 < Npad; j0 += 32) {
                    uint32_t v[32];
                    const uint32_t ta = tmem + ((uint32_t)(wq * 32) << 16) + (uint32_t)(slot * T3_NMAX + j0);
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                                   "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                                   "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]),
                                   "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]),
                                   "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                                 : "r"(ta));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (ST == T3_C) {
                        // row (column ci, sign part): Z_{+-m}(n') = (v[2j'], v[2j'+1]), n' = m + j'
                        const int m = b;
                        if (valid && !(part && m == 0)) {
                            float2 *zc = a.out + (size_t)col * P2 + t3_pm(part ? -m : m);
#pragma unroll
                            for (int j = 0; j < 32; j += 2) {
                                const int jj = j0 + j;
                                if (jj < nout) {
                                    const int n = m + jj / 2;
                                    zc[n * n] = make_float2(__uint_as_float(v[j]), __uint_as_float(v[j + 1]));
                                }
                            }
                        }
                    } else if (ST == T3_R1) {
                        // output j of degree n (m' = j - n), staged at its paired position
                        const int n = b;
#pragma unroll
                        for (int j = 0; j < 32; j++) {
                            const int jj = j0 + j;
                            if (jj < nout) stgf[2 * (cl * a.s2 + t3_pm(jj - n)) + part] = __uint_as_float(v[j]);
                        }
                    } else {
                        // y e^{-i m' phi}: re and im from the lane pair, the column's phases loaded
                        // together for the piece; staged in natural order
                        const int n = b;
                        float2 e[32];
#pragma unroll
                        for (int j = 0; j < 32; j++) {
                            const int m = min(j0 + j, nout - 1) - n;
                            e[j] = __ldg(ph + m);
                        }
#pragma unroll
                        for (int j = 0; j < 32; j++) {
                            const float mine = __uint_as_float(v[j]);
                            const float other = __shfl_xor_sync(0xffffffffu, mine, 1);
                            const float yr = part ? other : mine, yi = part ? mine : other;
                            const float w = part ? e[j].x * yi - e[j].y * yr : e[j].x * yr + e[j].y * yi;
                            if (j0 + j < nout) stgf[2 * (cl * a.s2 + j0 + j) + part] = w;
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;");
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(acce + slot));
                if (ST != T3_C) {
                    const int n = b;
                    // columns per pass: 32 / nout when a column's run is shorter than a warp
                    const int cpp = nout < 32 ? 32 / nout : 1, coff = nout < 32 ? lane / nout : 0;
                    const int e0 = nout < 32 ? lane - coff * nout : lane;
                    for (int c0 = 0; c0 < 16; c0 += cpp) {
                        const int c = c0 + coff;
                        if (c >= 16 || coff >= cpp) continue;
                        const int4 inf = cinfo[c];
                        if (inf.x < 0) continue;
                        for (int e = e0; e < nout; e += 32) {
                            const float2 y = stg[c * a.s2 + e];
                            if (ST == T3_R1) {
                                a.out[(size_t)inf.x * P2 + n * n + e] = y;
                            } else {
                                float2 *d = a.dst + (size_t)inf.y * a.dst_stride + n * n + e;
                                if (a.atomic) {
                                    atomicAdd(d, y);
                                } else {
                                    const float2 o = *d;
                                    *d = make_float2(o.x + y.x, o.y + y.y);
                                }
                            }
                        }
                    }
                    __syncwarp();
                }
            }
            __syncwarp();
        }
    }
    if (!ok) atomicExch(a.err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// ----------------------------------------------------------------------------- host side

static int t3_npad(int n) { return (n + 15) / 16 * 16; }

// block layout of a stage's operator table: per block, nch = ceil(K/16) chunks of [hi | lo]
// tiles of Npad x 16 floats in the core-matrix layout
static long long t3_layout(std::vector<int4> &blk)
{
    long long off = 0;
    for (auto &b : blk) {
        b.x = (int)off;
        off += (long long)((b.y + T3_KC - 1) / T3_KC) * 2 * b.z * T3_KC;
    }
    return off;
}

static inline void t3_put(float *tab, long long base, int Npad, int o, int k, double v)
{
    const int c = k / T3_KC, kc = k % T3_KC;
    // TF32 halves rounded to nearest, as the device splits its data
    float hi = (float)v;
    uint32_t u;
    memcpy(&u, &hi, 4);
    u = tf32_round_bits(u);
    memcpy(&hi, &u, 4);
    float lo = (float)((double)(float)v - (double)hi);
    memcpy(&u, &lo, 4);
    u = tf32_round_bits(u);
    memcpy(&lo, &u, 4);
    const long long t = base + (long long)c * 2 * Npad * T3_KC;
    tab[t + core_off(o, kc, T3_KC) / 4] = hi;
    tab[t + (long long)Npad * T3_KC + core_off(o, kc, T3_KC) / 4] = lo;
}

// polar-angle class of every key (direction or octant) of a pass
void direction_classes(const Plan *P, int which, int nkeys, std::vector<int> &cls, std::vector<int> &rep)
{
    cls.assign(nkeys, -1);
    rep.clear();
    std::map<long long, int> seen;
    for (int d = 0; d < nkeys; d++) {
        long long key;
        if (which == PASS_M2L) {
            int s = -1;
            for (int q = 0; q < 343; q++)
                if (P->dir_slot[q] == d) s = q;
            int dx = s / 49 - 3, dy = (s / 7) % 7 - 3, dz = s % 7 - 3;
            key = (long long)(dz + 8) * 1000 + dx * dx + dy * dy;
        } else {
            key = d & 1; // octant: the z bit fixes the polar angle
        }
        auto itc = seen.find(key);
        if (itc == seen.end()) {
            int id = (int)rep.size();
            seen[key] = id;
            rep.push_back(d);
            cls[d] = id;
        } else {
            cls[d] = itc->second;
        }
    }
}

int build_tc3(Plan *P, int l, int which)
{
    RcrPass ps;
    RcrList *Lst = pass32_desc(P, l, which, 1, ps);
    if (!Lst || Lst->key_beg.empty() || Lst->key_beg.back() == 0) return FMM_OK;
    Tc3 &t = Lst->t3;
    if (t.built) return FMM_OK;
    const int p = ps.p;
    if (p < 2 || p > T3_MAXP) return FMM_OK;
    t.p = p;
    t.pinr = std::min(ps.pin, p);
    t.nq = std::min(ps.pout, p);
    const int nkeys = (int)Lst->key_beg.size() - 1;
    t.T = Lst->key_beg.back();
    // direction of every translation, classes
    std::vector<int> tdir(t.T);
    for (int d = 0; d < nkeys; d++)
        for (int q = Lst->key_beg[d]; q < Lst->key_beg[d + 1]; q++) tdir[q] = d;
    std::vector<int> clsR, rep;
    direction_classes(P, which, nkeys, clsR, rep);
    t.nclsR = (int)rep.size();
    int nclsC = 0;
    for (int d = 0; d < nkeys; d++) nclsC = std::max(nclsC, Lst->key_w[d] + 1);
    t.nclsC = nclsC;
    t.clsR_of_t.resize(t.T);
    t.clsC_of_t.resize(t.T);
    for (int q = 0; q < t.T; q++) {
        t.clsR_of_t[q] = clsR[tdir[q]];
        t.clsC_of_t[q] = Lst->key_w[tdir[q]];
    }
    // block descriptors: rotation blocks n < p (K = N = 2n+1), coaxial blocks m < min(nq, pinr)
    t.hblkR.clear();
    for (int n = 0; n < p; n++) t.hblkR.push_back(make_int4(0, 2 * n + 1, t3_npad(2 * n + 1), 2 * n + 1));
    t.strideR = t3_layout(t.hblkR);
    t.hblkC.clear();
    for (int m = 0; m < std::min(t.nq, t.pinr); m++)
        t.hblkC.push_back(make_int4(0, 2 * (t.pinr - m), t3_npad(2 * (t.nq - m)), 2 * (t.nq - m)));
    t.strideC = t3_layout(t.hblkC);
    // operator tables from the pass's own FP32 tables (the same ones the SIMT tiles read)
    const int rs = rot_size(p), cs = coax_size(p);
    std::vector<float> Hh((size_t)t.nclsR * rs);
    for (int c = 0; c < t.nclsR; c++)
        FMM_CUDA_TRY(cudaMemcpy(Hh.data() + (size_t)c * rs, ps.H + (size_t)rep[c] * ps.hstride, sizeof(float) * rs,
                                cudaMemcpyDeviceToHost));
    std::vector<float2> Ch((size_t)nclsC * cs);
    FMM_CUDA_TRY(cudaMemcpy(Ch.data(), ps.Cc, sizeof(float2) * Ch.size(), cudaMemcpyDeviceToHost));
    std::vector<float> tabR((size_t)t.nclsR * t.strideR, 0.f), tabC((size_t)nclsC * t.strideC, 0.f);
    for (int c = 0; c < t.nclsR; c++) {
        const float *H = Hh.data() + (size_t)c * rs;
        for (int n = 0; n < p; n++) {
            const int r = 2 * n + 1;
            const int4 &bk = t.hblkR[n];
            for (int m = 0; m < r; m++)
                for (int o = 0; o < r; o++)
                    t3_put(tabR.data(), (long long)c * t.strideR + bk.x, bk.z, o, m, H[rot_off(n) + m * r + o]);
        }
    }
    for (int q = 0; q < nclsC; q++) {
        const float2 *C = Ch.data() + (size_t)q * cs;
        for (size_t mb = 0; mb < t.hblkC.size(); mb++) {
            const int m = (int)mb, sz = p - m;
            const int4 &bk = t.hblkC[mb];
            const long long base = (long long)q * t.strideC + bk.x;
            for (int n = m; n < t.pinr; n++)
                for (int np = m; np < t.nq; np++) {
                    const float2 v = C[coax_off(p, m) + (n - m) * sz + (np - m)];
                    const int o = 2 * (np - m), k = 2 * (n - m);
                    t3_put(tabC.data(), base, bk.z, o, k, v.x);
                    t3_put(tabC.data(), base, bk.z, o, k + 1, -v.y);
                    t3_put(tabC.data(), base, bk.z, o + 1, k, v.y);
                    t3_put(tabC.data(), base, bk.z, o + 1, k + 1, v.x);
                }
        }
    }
    FMM_CUDA_TRY(dev_alloc(P, (void **)&t.opsR, sizeof(float) * tabR.size()));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&t.opsC, sizeof(float) * std::max<size_t>(1, tabC.size())));
    FMM_CUDA_TRY(cudaMemcpy(t.opsR, tabR.data(), sizeof(float) * tabR.size(), cudaMemcpyHostToDevice));
    if (!tabC.empty()) FMM_CUDA_TRY(cudaMemcpy(t.opsC, tabC.data(), sizeof(float) * tabC.size(), cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&t.blkR, sizeof(int4) * t.hblkR.size()));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&t.blkC, sizeof(int4) * std::max<size_t>(1, t.hblkC.size())));
    FMM_CUDA_TRY(cudaMemcpy(t.blkR, t.hblkR.data(), sizeof(int4) * t.hblkR.size(), cudaMemcpyHostToDevice));
    if (!t.hblkC.empty())
        FMM_CUDA_TRY(cudaMemcpy(t.blkC, t.hblkC.data(), sizeof(int4) * t.hblkC.size(), cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&t.t_dir, sizeof(int) * t.T));
    FMM_CUDA_TRY(cudaMemcpy(t.t_dir, tdir.data(), sizeof(int) * t.T, cudaMemcpyHostToDevice));
    t.built = 1;
    return FMM_OK;
}

// items of one stage for one chunk: tiles of 64 columns over the runs of equal class in
// `order` (chunk-local translations sorted by class), each cut into block ranges of about
// equal MMA work so that a launch has a few items per SM
static void t3_items(const std::vector<int> &order, const std::vector<int> &cls_of_t, int t0, int nrhs,
                     const std::vector<int4> &blk, int nb, int target, std::vector<int4> &items)
{
    std::vector<int4> tiles;
    size_t a = 0;
    while (a < order.size()) {
        const int c = cls_of_t[t0 + order[a]];
        size_t b = a;
        while (b < order.size() && cls_of_t[t0 + order[b]] == c) b++;
        for (long long e = (long long)a * nrhs; e < (long long)b * nrhs; e += T3_COLS)
            tiles.push_back(make_int4(c, (int)e, (int)std::min<long long>(T3_COLS, (long long)b * nrhs - e), 0));
        a = b;
    }
    if (nb <= 0) return;
    std::vector<long long> cost(nb + 1, 0);
    for (int b = 0; b < nb; b++) cost[b + 1] = cost[b] + (long long)((blk[b].y + T3_KC - 1) / T3_KC) * blk[b].z + 64;
    int ns = (int)std::min<long long>(nb, std::max<long long>(1, (target + (long long)tiles.size() - 1) / std::max<size_t>(1, tiles.size())));
    // block range boundaries by equal cost, heaviest ranges first
    std::vector<int> cut(1, 0);
    for (int k = 1; k < ns; k++) {
        long long goal = cost[nb] * k / ns;
        int b = (int)(std::lower_bound(cost.begin(), cost.end(), goal) - cost.begin());
        b = std::max(b, cut.back() + 1);
        if (b < nb) cut.push_back(b);
    }
    cut.push_back(nb);
    for (size_t k = cut.size() - 1; k-- > 0;)
        for (const int4 &tl : tiles) items.push_back(make_int4(tl.x, tl.y, tl.z, cut[k] | (cut[k + 1] << 16)));
}

// chunks, class orders and items for nrhs columns
static int t3_prepare(Plan *P, Tc3 &t, int nrhs)
{
    if (t.items_nrhs == nrhs) return FMM_OK;
    const size_t colbytes = (size_t)t.p * t.p * sizeof(float2);
    const long long cap_cols = std::max<long long>(nrhs, (long long)(T3_SCRATCH_BYTES / colbytes));
    const int ct = (int)std::max<long long>(1, cap_cols / nrhs);
    t.chunk_t0.clear();
    for (int a = 0; a < t.T; a += ct) t.chunk_t0.push_back(a);
    t.chunk_t0.push_back(t.T);
    const int nchunk = (int)t.chunk_t0.size() - 1;
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int target = 2 * nsm;
    std::vector<int> listR, listC;
    std::vector<int4> itR1, itC, itR2;
    t.it_beg.assign(3 * (nchunk + 1), 0);
    const int nbR1 = t.pinr, nbR2 = t.nq, nbC = (int)t.hblkC.size();
    for (int k = 0; k < nchunk; k++) {
        const int t0 = t.chunk_t0[k], n = t.chunk_t0[k + 1] - t0;
        std::vector<int> oR(n), oC(n);
        for (int i = 0; i < n; i++) oR[i] = oC[i] = i;
        std::stable_sort(oR.begin(), oR.end(), [&](int x, int y) { return t.clsR_of_t[t0 + x] < t.clsR_of_t[t0 + y]; });
        std::stable_sort(oC.begin(), oC.end(), [&](int x, int y) { return t.clsC_of_t[t0 + x] < t.clsC_of_t[t0 + y]; });
        t.it_beg[3 * k] = (int)itR1.size();
        t.it_beg[3 * k + 1] = (int)itC.size();
        t.it_beg[3 * k + 2] = (int)itR2.size();
        t3_items(oR, t.clsR_of_t, t0, nrhs, t.hblkR, nbR1, target, itR1);
        t3_items(oC, t.clsC_of_t, t0, nrhs, t.hblkC, nbC, target, itC);
        t3_items(oR, t.clsR_of_t, t0, nrhs, t.hblkR, nbR2, target, itR2);
        listR.insert(listR.end(), oR.begin(), oR.end());
        listC.insert(listC.end(), oC.begin(), oC.end());
    }
    t.it_beg[3 * nchunk] = (int)itR1.size();
    t.it_beg[3 * nchunk + 1] = (int)itC.size();
    t.it_beg[3 * nchunk + 2] = (int)itR2.size();
    auto upload = [&](const std::vector<int4> &v, int4 *&ptr, size_t &cap) -> int {
        if (v.size() > cap) {
            if (ptr) cudaFree(ptr);
            ptr = nullptr;
            FMM_CUDA_TRY(cudaMalloc(&ptr, sizeof(int4) * v.size()));
            cap = v.size();
        }
        if (!v.empty()) FMM_CUDA_TRY(cudaMemcpy(ptr, v.data(), sizeof(int4) * v.size(), cudaMemcpyHostToDevice));
        return FMM_OK;
    };
    int e = upload(itR1, t.itR1, t.capR1);
    if (!e) e = upload(itC, t.itC, t.capC);
    if (!e) e = upload(itR2, t.itR2, t.capR2);
    if (e) return e;
    if (!t.listR) {
        FMM_CUDA_TRY(dev_alloc(P, (void **)&t.listR, sizeof(int) * t.T));
        FMM_CUDA_TRY(dev_alloc(P, (void **)&t.listC, sizeof(int) * t.T));
    }
    FMM_CUDA_TRY(cudaMemcpy(t.listR, listR.data(), sizeof(int) * t.T, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(t.listC, listC.data(), sizeof(int) * t.T, cudaMemcpyHostToDevice));
    const size_t need = (size_t)ct * nrhs * t.p * t.p;
    if (need > t.scratch_cap) {
        if (t.W) cudaFree(t.W);
        if (t.Z) cudaFree(t.Z);
        t.W = t.Z = nullptr;
        FMM_CUDA_TRY(cudaMalloc(&t.W, sizeof(float2) * need));
        FMM_CUDA_TRY(cudaMalloc(&t.Z, sizeof(float2) * need));
        t.scratch_cap = need;
    }
    t.items_nrhs = nrhs;
    return FMM_OK;
}

// Ring and staging sizes of a launch from its blocks: the rotation stages stage each block's
// outputs (up to 2p-1 complex per column, row stride 1 mod 16 float2 so that the 16 columns of a
// warp hit different banks); the operator stages take what is left, up to eight.
template <int ST>
static int t3_launch(T3Args &a, const std::vector<int4> &hblk, int nsm, cudaStream_t st)
{
    static size_t attr = 0;
    int npmax = 16, nomax = 1;
    for (const int4 &b : hblk) {
        npmax = std::max(npmax, b.z);
        nomax = std::max(nomax, b.w);
    }
    a.bstage = 2u * (uint32_t)npmax * T3_KC * 4;
    a.s2 = ST == T3_C ? 0 : (nomax + 15) / 16 * 16 + 1;
    a.sb = T3_SBMAX;
    while (a.sb > 2 && t3_smem(a.bstage, a.sb, a.s2) > T3_SMEM_MAX) a.sb--;
    const size_t sm = t3_smem(a.bstage, a.sb, a.s2);
    if (sm > T3_SMEM_MAX) {
        fmm_set_error("three-stage tensor-core pass: %zu bytes of shared memory needed", sm);
        return FMM_ERR_ARG;
    }
    int e = raise_smem_limit((const void *)rcr3_kernel<ST>, T3_SMEM_MAX, &attr);
    if (e) return e;
    if (a.n_items <= 0) return FMM_OK;
    rcr3_kernel<ST><<<std::min(a.n_items, nsm), T3_THREADS, sm, st>>>(a);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int launch_tc3_pass(Plan *P, int l, int which, int nrhs, cudaStream_t st)
{
    RcrPass ps;
    RcrList *Lst = pass32_desc(P, l, which, nrhs, ps);
    if (!Lst || Lst->key_beg.empty() || Lst->key_beg.back() == 0) return FMM_OK;
    Tc3 &t = Lst->t3;
    if (!t.built) {
        fmm_set_error("three-stage tensor-core pass of level %d not built", l);
        return FMM_ERR_ARG;
    }
    int e = t3_prepare(P, t, nrhs);
    if (e) return e;
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    T3Args a;
    memset(&a, 0, sizeof(a));
    a.p = t.p;
    a.pinr = t.pinr;
    a.nq = t.nq;
    a.nrhs = nrhs;
    a.g_dst = Lst->dst;
    a.t_dir = t.t_dir;
    a.PH = ps.PH;
    a.phstride = ps.phstride;
    a.phoff = ps.phoff;
    a.src = ps.src;
    a.src_stride = ps.pin * ps.pin;
    a.dst = ps.dst;
    a.dst_stride = ps.pout * ps.pout;
    a.atomic = ps.atomic;
    a.err = P->tc_err;
    const int nchunk = (int)t.chunk_t0.size() - 1;
    for (int k = 0; k < nchunk; k++) {
        a.t0 = t.chunk_t0[k];
        // R1: sources -> W
        a.items = t.itR1 + t.it_beg[3 * k];
        a.n_items = t.it_beg[3 * (k + 1)] - t.it_beg[3 * k];
        a.list = t.listR + a.t0;
        a.blk = t.blkR;
        a.nblk = (int)t.hblkR.size();
        a.ops = t.opsR;
        a.ops_stride = t.strideR;
        a.g_src = Lst->src;
        a.in = nullptr;
        a.out = t.W;
        if ((e = t3_launch<T3_R1>(a, t.hblkR, nsm, st))) return e;
        // C: W -> Z
        a.items = t.itC + t.it_beg[3 * k + 1];
        a.n_items = t.it_beg[3 * (k + 1) + 1] - t.it_beg[3 * k + 1];
        a.list = t.listC + a.t0;
        a.blk = t.blkC;
        a.nblk = (int)t.hblkC.size();
        a.ops = t.opsC;
        a.ops_stride = t.strideC;
        a.g_src = nullptr;
        a.in = t.W;
        a.out = t.Z;
        if ((e = t3_launch<T3_C>(a, t.hblkC, nsm, st))) return e;
        // R2: Z -> destinations
        a.items = t.itR2 + t.it_beg[3 * k + 2];
        a.n_items = t.it_beg[3 * (k + 1) + 2] - t.it_beg[3 * k + 2];
        a.list = t.listR + a.t0;
        a.blk = t.blkR;
        a.nblk = (int)t.hblkR.size();
        a.ops = t.opsR;
        a.ops_stride = t.strideR;
        a.g_src = nullptr;
        a.in = t.Z;
        a.out = nullptr;
        if ((e = t3_launch<T3_R2>(a, t.hblkR, nsm, st))) return e;
    }
    return FMM_OK;
}

static void t3_free(Plan *P, Tc3 &t)
{
    for (void *q : {(void *)t.opsR, (void *)t.opsC, (void *)t.blkR, (void *)t.blkC, (void *)t.t_dir, (void *)t.itR1,
                    (void *)t.itC, (void *)t.itR2, (void *)t.listR, (void *)t.listC, (void *)t.W, (void *)t.Z})
        if (q) cudaFree(q);
    P->device_bytes -= sizeof(float) * (size_t)(t.nclsR * t.strideR + std::max<long long>(1, t.nclsC * t.strideC));
    t = Tc3();
}

// Plan-time choice per batched pass: the three-stage tensor-core form where it beats the
// pass's current form (SIMT tiles, or the dense tensor-core M2L) on this plan, timed with one
// right-hand side.  FMMBEM_TC3=0 keeps the current forms, FMMBEM_TC3=1 takes the three-stage
// form wherever it applies.
int tune_tc3(Plan *P)
{
    const char *env = getenv("FMMBEM_TC3");
    const int mode = env ? atoi(env) : -1;
    if (mode == 0) return FMM_OK;
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
            RcrPass ps;
            RcrList *Lst = pass32_desc(P, l, which, 1, ps);
            if (!Lst || Lst->key_beg.empty() || Lst->key_beg.back() == 0) continue;
            rc = build_tc3(P, l, which);
            if (rc || !Lst->t3.built) break;
            float ms[2] = {0.f, 0.f};
            for (int on = 0; on < 2 && rc == FMM_OK && mode != 1; on++) {
                Lst->t3.on = on;
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
            Lst->t3.on = (mode == 1 || ms[1] < ms[0]) ? 1 : 0;
            if (!Lst->t3.on) t3_free(P, Lst->t3);
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc == FMM_ERR_CUDA && !fmm_last_error()[0]) fmm_set_error("three-stage tensor-core tuning: %s", cudaGetErrorString(cudaGetLastError()));
    return rc;
}

} // namespace fmm
