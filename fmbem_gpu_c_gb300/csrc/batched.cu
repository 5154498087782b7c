// Batched translations for the mixed-precision matvec: M2M, M2L and L2L as direction-grouped
// tiles of register-blocked small matrix products.
//
// Every translation is rotation - coaxial - rotation (RCR) as in transMatsVecsMul_SR_rcr
// (reference translation.cu:1864-1961).  All translations of one level that share a
// direction (one of 316 M2L offsets, or one of 8 octants for M2M/L2L) use the same real
// rotation block H, the same phases e^{i m phi} and the same coaxial blocks.  A CTA takes TC
// of them as the columns of a matrix:
//   stage 0  gather the TC source vectors into shared memory as X[nm][t] and apply
//            e^{i m phi} (zero-padded to order p, zero columns beyond the item's count);
//   stage 1  W_n = H_n X_n for every degree n (H_n is (2n+1) x (2n+1), real);
//   stage 2  X_m = C_|m| W_m for every order m (C_|m| is the (p-|m|)^2 coaxial block, complex;
//            +m and -m share it);
//   stage 3  Y_n = H_n X_n for n < pout, times e^{-i m' phi}, added into the destinations.
// A thread computes R rows x CG columns of one block per unit of work (CG = TC, or 16-column
// groups when TC is 32 or 64): the CG-wide rows of X and W are read as shared-memory
// broadcasts and every H or C entry loaded from L1/L2 feeds 2 CG (real H) or 4 CG (complex
// C) FMAs.  Units are ordered by cost within each column group so the long blocks start
// first.  Destinations are added with FP32 vector atomics where several items reach
// the same box (M2M, M2L), and with a plain read-add-write where every box is reached once
// (L2L).
#include "plan.h"
#include <algorithm>
#include <cstdlib>
#include <vector>

namespace fmm {

static __device__ __forceinline__ void nm_of(int i, int &n, int &m)
{
    int q = (int)sqrtf((float)i);
    while (q * q > i) q--;
    while ((q + 1) * (q + 1) <= i) q++;
    n = q;
    m = i - q * q - q;
}

// Tiles X and W hold p^2 rows of TC complex columns.  The 16-byte chunks of row q are
// XOR-swizzled by q mod 8 (mod TC/2 for TC = 8) so that units reading rows of different
// degrees in one warp hit different banks.
template <int TC>
static __device__ __forceinline__ float4 *chunk(float2 *base, int row, int ch)
{
    constexpr int M = (TC / 2 < 8 ? TC / 2 : 8) - 1;
    return reinterpret_cast<float4 *>(base + (size_t)row * TC) + (ch ^ (row & M));
}

// rows row0..row0+R-1 of W_n = H_n X_n (r = 2n+1 rows) for the CG columns starting at chunk
// ch0; X row of step m is rb + m; Hn column-major (m', m).  The H entries of step m+1 are
// loaded while step m computes.
template <int TC, int CG, int R>
static __device__ __forceinline__ void rot_rows(const float *__restrict__ Hn, int r, int row0, float2 *X, int rb,
                                                int ch0, float2 (&acc)[R][CG])
{
#pragma unroll
    for (int k = 0; k < R; k++)
#pragma unroll
        for (int t = 0; t < CG; t++) acc[k][t] = make_float2(0.f, 0.f);
    float hn[R];
#pragma unroll
    for (int k = 0; k < R; k++) hn[k] = (row0 + k < r) ? Hn[row0 + k] : 0.f;
    for (int m = 0; m < r; m++) {
        float h[R];
#pragma unroll
        for (int k = 0; k < R; k++) {
            h[k] = hn[k];
            hn[k] = (m + 1 < r && row0 + k < r) ? Hn[(m + 1) * r + row0 + k] : 0.f;
        }
#pragma unroll
        for (int c = 0; c < CG / 2; c++) {
            float4 x = *chunk<TC>(X, rb + m, ch0 + c);
#pragma unroll
            for (int k = 0; k < R; k++) {
                acc[k][2 * c].x = fmaf(h[k], x.x, acc[k][2 * c].x);
                acc[k][2 * c].y = fmaf(h[k], x.y, acc[k][2 * c].y);
                acc[k][2 * c + 1].x = fmaf(h[k], x.z, acc[k][2 * c + 1].x);
                acc[k][2 * c + 1].y = fmaf(h[k], x.w, acc[k][2 * c + 1].y);
            }
        }
    }
}

static __device__ __forceinline__ void cmac(float2 &acc, float2 c, float ar, float ai)
{
    acc.x = fmaf(c.x, ar, acc.x);
    acc.x = fmaf(-c.y, ai, acc.x);
    acc.y = fmaf(c.x, ai, acc.y);
    acc.y = fmaf(c.y, ar, acc.y);
}

// One tile: item it = (direction, first column, count, coaxial block) of pass ps, with the
// CTA's dynamic shared memory smem4 and its column indices s_src / s_dst.  SHC also stages
// the direction's rotation block and coaxial block in shared memory, after the two tiles.
//
// A stage lasts as long as its busiest thread.  The units of a stage are ordered by cost
// (longest first); without BAL thread t takes units t, t + B, t + 2B, ... (B threads), which
// leaves most threads idle while the few longest units finish when the units barely outnumber
// the threads.  BAL takes them in boustrophedon order (t, 2B - 1 - t, 2B + t, ...), so a thread
// that drew a long unit in one round draws a short one in the next, ranks the column groups
// inside each cost class, and gives +m and -m of the coaxial stage units of their own; with
// one- or two-row units the busiest thread does about 1.05-1.15 times the average work at
// p = 20-40 (counting each unit's FMAs and loads), against about 1.8 times with the default
// schedule.  Every output is still summed in the same order, so the results do not depend on
// BAL, R1 or R2.
template <int TC, int CG, int R1, int R2, bool SHC, bool BAL = false>
static __device__ __forceinline__ void rcr_tile(const RcrPass &ps, const int4 it, float4 *smem4, int *s_src, int *s_dst)
{
    const int p = ps.p, pp = p * p;
    float2 *X = reinterpret_cast<float2 *>(smem4);
    float2 *W = X + (size_t)pp * TC;
    float2 *sC = W + (size_t)pp * TC;
    float *sH = reinterpret_cast<float *>(sC + coax_size(p));
    const int cnt = it.z;
    const float *Hg = ps.H + (size_t)(ps.hrep ? ps.hrep[it.x] : it.x) * ps.hstride;
    const float2 *ph = ps.PH + (size_t)it.x * ps.phstride + ps.phoff;
    const float2 *Cg = ps.Cc + (size_t)it.w * coax_size(p);
    const float *H = SHC ? sH : Hg;
    const float2 *Cc = SHC ? sC : Cg;
    if (threadIdx.x < TC) {
        // column e = translation t x nrhs + right-hand side r; the expansions hold the columns
        // of a box next to each other ([box][rhs][p^2]), so a tile's sources are contiguous runs
        bool v = (int)threadIdx.x < cnt;
        int e = it.y + threadIdx.x, t = e / ps.nrhs, r = e - t * ps.nrhs;
        s_src[threadIdx.x] = v ? ps.g_src[t] * ps.nrhs + r : -1;
        s_dst[threadIdx.x] = v ? ps.g_dst[t] * ps.nrhs + r : -1;
    }
    if (SHC) {
        const int rs = rot_size(p), cs = coax_size(p);
        for (int i = threadIdx.x; i < rs; i += blockDim.x) sH[i] = __ldg(Hg + i);
        for (int i = threadIdx.x; i < cs; i += blockDim.x) sC[i] = __ldg(Cg + i);
    }
    __syncthreads();

    // stage 0: gather, phase, zero padding
    const int pin = min(ps.pin, p), pin2 = pin * pin, sstride = ps.pin * ps.pin;
    for (int i = threadIdx.x; i < pp * TC; i += blockDim.x) {
        int nm = i / TC, t = i % TC;
        float2 v = make_float2(0.f, 0.f);
        int s = s_src[t];
        if (s >= 0 && nm < pin2) {
            int n, m;
            nm_of(nm, n, m);
            v = cmul(__ldg(ps.src + (size_t)s * sstride + nm), ph[m]);
        }
        reinterpret_cast<float2 *>(chunk<TC>(X, nm, t >> 1))[t & 1] = v;
    }
    __syncthreads();

    // stage 1: W_n = H_n X_n, n < p; a unit is R1 rows x CG columns, longest blocks first
    constexpr int G = TC / CG, HC = CG / 2;
    const int B = blockDim.x, tid = threadIdx.x;
    int U = 0;
    for (int n = 0; n < p; n++) U += (2 * n + R1) / R1;
    for (int k = 0;; k++) {
        const int u = k * B + ((BAL && (k & 1)) ? B - 1 - tid : tid);
        if (u >= U * G) break;
        const int g = BAL ? u % G : u / U;
        int n = p - 1, q = BAL ? u / G : u - g * U;
        while (q >= (2 * n + R1) / R1) {
            q -= (2 * n + R1) / R1;
            n--;
        }
        const int r = 2 * n + 1, row0 = q * R1;
        float2 acc[R1][CG];
        rot_rows<TC, CG, R1>(H + rot_off(n), r, row0, X, n * n, g * HC, acc);
#pragma unroll
        for (int k = 0; k < R1; k++)
            if (row0 + k < r) {
#pragma unroll
                for (int c = 0; c < HC; c++)
                    *chunk<TC>(W, n * n + row0 + k, g * HC + c) =
                        make_float4(acc[k][2 * c].x, acc[k][2 * c].y, acc[k][2 * c + 1].x, acc[k][2 * c + 1].y);
            }
    }
    __syncthreads();

    // stage 2: X_{+-m} = C_|m| W_{+-m} for the rows n' < nq (the ones stage 3 reads)
    const int nq = min(ps.pout, p);
    if constexpr (!BAL) {
        U = 0;
        for (int am = 0; am < nq; am++) U += (nq - am + R2 - 1) / R2;
        for (int u = threadIdx.x; u < U * G; u += blockDim.x) {
            const int g = u / U;
            int am = 0, q = u - g * U;
            while (q >= (nq - am + R2 - 1) / R2) {
                q -= (nq - am + R2 - 1) / R2;
                am++;
            }
            const int sz = p - am, nrow = nq - am, j0 = q * R2;
            const float2 *Cb = Cc + coax_off(p, am);
            float2 accP[R2][CG], accM[R2][CG];
#pragma unroll
            for (int k = 0; k < R2; k++)
#pragma unroll
                for (int t = 0; t < CG; t++) accP[k][t] = accM[k][t] = make_float2(0.f, 0.f);
            float2 cn[R2];
#pragma unroll
            for (int k = 0; k < R2; k++) cn[k] = (j0 + k < nrow) ? Cb[j0 + k] : make_float2(0.f, 0.f);
            for (int j = 0; j < sz; j++) {
                float2 c[R2];
#pragma unroll
                for (int k = 0; k < R2; k++) {
                    c[k] = cn[k];
                    cn[k] = (j + 1 < sz && j0 + k < nrow) ? Cb[(j + 1) * sz + j0 + k] : make_float2(0.f, 0.f);
                }
                const int n = am + j, rp = n * n + n + am, rm = n * n + n - am;
#pragma unroll
                for (int cc = 0; cc < HC; cc++) {
                    float4 a = *chunk<TC>(W, rp, g * HC + cc), b = *chunk<TC>(W, rm, g * HC + cc);
#pragma unroll
                    for (int k = 0; k < R2; k++) {
                        cmac(accP[k][2 * cc], c[k], a.x, a.y);
                        cmac(accP[k][2 * cc + 1], c[k], a.z, a.w);
                        cmac(accM[k][2 * cc], c[k], b.x, b.y);
                        cmac(accM[k][2 * cc + 1], c[k], b.z, b.w);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < R2; k++)
                if (j0 + k < nrow) {
                    const int np = am + j0 + k;
#pragma unroll
                    for (int cc = 0; cc < HC; cc++) {
                        *chunk<TC>(X, np * np + np + am, g * HC + cc) =
                            make_float4(accP[k][2 * cc].x, accP[k][2 * cc].y, accP[k][2 * cc + 1].x, accP[k][2 * cc + 1].y);
                        if (am > 0)
                            *chunk<TC>(X, np * np + np - am, g * HC + cc) = make_float4(
                                accM[k][2 * cc].x, accM[k][2 * cc].y, accM[k][2 * cc + 1].x, accM[k][2 * cc + 1].y);
                    }
                }
        }
    } else {
        // units (|m|, row block, sign, column group), |m| ascending = cost descending
        U = 0;
        for (int am = 0; am < nq; am++) U += (am > 0 ? 2 : 1) * ((nq - am + R2 - 1) / R2);
        for (int k = 0;; k++) {
            const int u = k * B + ((k & 1) ? B - 1 - tid : tid);
            if (u >= U * G) break;
            const int g = u % G;
            int am = 0, q = u / G;
            while (q >= (am > 0 ? 2 : 1) * ((nq - am + R2 - 1) / R2)) {
                q -= (am > 0 ? 2 : 1) * ((nq - am + R2 - 1) / R2);
                am++;
            }
            const int sg = am > 0 ? (q & 1) : 0, m = sg ? -am : am;
            const int sz = p - am, nrow = nq - am, j0 = (am > 0 ? q >> 1 : q) * R2;
            const float2 *Cb = Cc + coax_off(p, am);
            float2 acc[R2][CG];
#pragma unroll
            for (int r = 0; r < R2; r++)
#pragma unroll
                for (int t = 0; t < CG; t++) acc[r][t] = make_float2(0.f, 0.f);
            float2 cn[R2];
#pragma unroll
            for (int r = 0; r < R2; r++) cn[r] = (j0 + r < nrow) ? Cb[j0 + r] : make_float2(0.f, 0.f);
            for (int j = 0; j < sz; j++) {
                float2 c[R2];
#pragma unroll
                for (int r = 0; r < R2; r++) {
                    c[r] = cn[r];
                    cn[r] = (j + 1 < sz && j0 + r < nrow) ? Cb[(j + 1) * sz + j0 + r] : make_float2(0.f, 0.f);
                }
                const int n = am + j, row = n * n + n + m;
#pragma unroll
                for (int cc = 0; cc < HC; cc++) {
                    const float4 a = *chunk<TC>(W, row, g * HC + cc);
#pragma unroll
                    for (int r = 0; r < R2; r++) {
                        cmac(acc[r][2 * cc], c[r], a.x, a.y);
                        cmac(acc[r][2 * cc + 1], c[r], a.z, a.w);
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < R2; r++)
                if (j0 + r < nrow) {
                    const int np = am + j0 + r;
#pragma unroll
                    for (int cc = 0; cc < HC; cc++)
                        *chunk<TC>(X, np * np + np + m, g * HC + cc) =
                            make_float4(acc[r][2 * cc].x, acc[r][2 * cc].y, acc[r][2 * cc + 1].x, acc[r][2 * cc + 1].y);
                }
        }
    }
    __syncthreads();

    // stage 3: Y_n = e^{-i m' phi} H_n X_n for n < nq, into the destinations
    const int po2 = ps.pout * ps.pout;
    U = 0;
    for (int n = 0; n < nq; n++) U += (2 * n + R1) / R1;
    for (int k = 0;; k++) {
        const int u = k * B + ((BAL && (k & 1)) ? B - 1 - tid : tid);
        if (u >= U * G) break;
        const int g = BAL ? u % G : u / U;
        int n = nq - 1, q = BAL ? u / G : u - g * U;
        while (q >= (2 * n + R1) / R1) {
            q -= (2 * n + R1) / R1;
            n--;
        }
        const int r = 2 * n + 1, row0 = q * R1;
        float2 acc[R1][CG];
        rot_rows<TC, CG, R1>(H + rot_off(n), r, row0, X, n * n, g * HC, acc);
#pragma unroll
        for (int k = 0; k < R1; k++) {
            if (row0 + k >= r) continue;
            const float2 e = ph[row0 + k - n];
            const int idx = n * n + row0 + k;
#pragma unroll
            for (int c = 0; c < CG; c++) {
                const int t = g * CG + c;
                if (t >= cnt) break;
                float2 a = acc[k][c];
                float2 v = make_float2(e.x * a.x + e.y * a.y, e.x * a.y - e.y * a.x);
                float2 *d = ps.dst + (size_t)s_dst[t] * po2 + idx;
                if (ps.atomic) {
                    atomicAdd(d, v);
                } else {
                    float2 o = *d;
                    *d = make_float2(o.x + v.x, o.y + v.y);
                }
            }
        }
    }
}

template <int TC, int CG, int R1, int R2, bool SHC, bool BAL = false>
__global__ void __launch_bounds__(256, 2) rcr_tile_kernel(RcrPass ps)
{
    extern __shared__ float4 smem4[];
    __shared__ int s_src[TC], s_dst[TC];
    rcr_tile<TC, CG, R1, R2, SHC, BAL>(ps, ps.items[blockIdx.x], smem4, s_src, s_dst);
}

// Persistent form for many passes at once (the translation passes of many plans, one phase
// of a lockstep matvec): a grid of resident CTAs takes work items (pass, tile) from a device
// queue, in the order given (longest first), until it is empty.  The queue head is an
// atomic counter, zeroed before the launch; no CTA waits on another.
template <int TC, int CG, int R1, int R2, bool SHC, bool BAL = false>
__global__ void __launch_bounds__(256, 2) rcr_queue_kernel(const RcrPass *__restrict__ passes, const int *__restrict__ work_pass,
                                                           const int4 *__restrict__ work_item, const int *__restrict__ nwork,
                                                           int *head)
{
    extern __shared__ float4 smem4[];
    __shared__ int s_src[TC], s_dst[TC];
    __shared__ int s_w;
    const int n = *nwork;
    for (;;) {
        if (threadIdx.x == 0) s_w = atomicAdd(head, 1);
        __syncthreads();
        const int w = s_w;
        if (w >= n) break;
        rcr_tile<TC, CG, R1, R2, SHC, BAL>(passes[work_pass[w]], work_item[w], smem4, s_src, s_dst);
        __syncthreads();
    }
}

size_t rcr_tile_smem(int p, int tc, int shc)
{
    size_t s = 2 * (size_t)p * p * tc * sizeof(float2);
    if (shc) s += (size_t)coax_size(p) * sizeof(float2) + (size_t)rot_size(p) * sizeof(float);
    return s;
}

template <int TC, int CG, int R1, int R2, bool SHC, bool BAL = false>
static int launch_tile(const RcrPass &ps, int n_items, size_t sm, cudaStream_t st)
{
    static size_t attr = 0;
    int e = raise_smem_limit((const void *)rcr_tile_kernel<TC, CG, R1, R2, SHC, BAL>, sm, &attr);
    if (e) return e;
    rcr_tile_kernel<TC, CG, R1, R2, SHC, BAL><<<n_items, 256, sm, st>>>(ps);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

// The tile shapes, as template arguments: Tile<TC, CG, R1, R2, SHC, BAL>
template <int TC_, int CG_, int R1_, int R2_, bool SHC_, bool BAL_>
struct Tile {
    static constexpr int TC = TC_, CG = CG_, R1 = R1_, R2 = R2_;
    static constexpr bool SHC = SHC_, BAL = BAL_;
};

// Calls f(Tile<...>{}) for the shape that serves (columns tc, staged blocks shc, schedule bal):
// bal 0 the default schedule, 1 the balanced one with narrow column groups where they pay, 2 the
// balanced one with the default groups; a (tc, shc, bal) without a balanced shape runs bal 0.
template <class F>
static int with_tile(int tc, int shc, int bal, F &&f)
{
    if (bal == 2) {
        if (shc) {
            if (tc == 32) return f(Tile<32, 16, 1, 1, true, true>{});
        } else {
            switch (tc) {
            case 32: return f(Tile<32, 16, 1, 1, false, true>{});
            case 16: return f(Tile<16, 16, 1, 1, false, true>{});
            case 8: return f(Tile<8, 8, 1, 1, false, true>{});
            case 4: return f(Tile<4, 4, 1, 1, false, true>{});
            default: break;
            }
        }
    }
    if (bal == 1) {
        if (shc) {
            switch (tc) {
            case 64: return f(Tile<64, 16, 1, 1, true, true>{});
            case 32: return f(Tile<32, 8, 1, 1, true, true>{});
            default: break;
            }
        } else {
            switch (tc) {
            case 64: return f(Tile<64, 16, 1, 1, false, true>{});
            case 32: return f(Tile<32, 8, 1, 1, false, true>{});
            case 16: return f(Tile<16, 8, 1, 1, false, true>{});
            case 8: return f(Tile<8, 8, 2, 1, false, true>{});
            case 4: return f(Tile<4, 4, 2, 1, false, true>{});
            default: break;
            }
        }
    }
    if (shc) {
        switch (tc) {
        case 64: return f(Tile<64, 16, 2, 1, true, false>{});
        case 32: return f(Tile<32, 16, 2, 1, true, false>{});
        case 16: return f(Tile<16, 16, 2, 1, true, false>{});
        default: return f(Tile<8, 8, 4, 2, true, false>{});
        }
    }
    switch (tc) {
    case 64: return f(Tile<64, 16, 2, 1, false, false>{});
    case 32: return f(Tile<32, 16, 2, 1, false, false>{});
    case 16: return f(Tile<16, 16, 2, 1, false, false>{});
    case 4: return f(Tile<4, 4, 8, 4, false, false>{});
    default: return f(Tile<8, 8, 4, 2, false, false>{});
    }
}

// Raise the queue kernel's shared-memory limit and size its grid: every CTA resident at once
// (SMs x CTAs per SM at this shared memory), no more than the items.
int rcr_queue_prepare(int tc, int shc, int bal, size_t sm, int nwork, int *grid)
{
    return with_tile(tc, shc, bal, [&](auto t) -> int {
        using T = decltype(t);
        static size_t attr = 0;
        const void *fn = (const void *)rcr_queue_kernel<T::TC, T::CG, T::R1, T::R2, T::SHC, T::BAL>;
        int e = raise_smem_limit(fn, sm, &attr);
        if (e) return e;
        int dev = 0, nsm = 0, per_sm = 0;
        FMM_CUDA_TRY(cudaGetDevice(&dev));
        FMM_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        FMM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, sm));
        *grid = std::max(1, std::min(nwork, nsm * std::max(per_sm, 1)));
        return FMM_OK;
    });
}

int launch_rcr_queue(int tc, int shc, int bal, const RcrPass *passes, const int *work_pass, const int4 *work_item,
                     const int *nwork, int *head, size_t sm, int grid, cudaStream_t st)
{
    return with_tile(tc, shc, bal, [&](auto t) -> int {
        using T = decltype(t);
        rcr_queue_kernel<T::TC, T::CG, T::R1, T::R2, T::SHC, T::BAL><<<grid, 256, sm, st>>>(passes, work_pass, work_item,
                                                                                         nwork, head);
        FMM_CUDA_TRY(cudaGetLastError());
        return FMM_OK;
    });
}

void rcr_list_items(const RcrList &Lst, std::vector<int4> &items) { build_items(Lst, 1, Lst.tc, 0, true, items); }

// Work items over the columns e = t nrhs + r of a list: tiles of at most `width` columns of
// one direction (or octant), item .w = the direction's coaxial block when coax_w.  Where the
// expansions a pass touches for nrhs columns (ws_bytes) are more than L2 keeps, the
// destination boxes are cut into Morton ranges and the items ordered range by range, so that
// the tiles in flight share their sources and destinations in L2.  Each direction's
// translations are sorted by the Morton rank of their destination, so a range is one
// contiguous run of every direction.
static const size_t L2_BUDGET = 48u << 20;

void build_items(const RcrList &Lst, int nrhs, int width, size_t ws_bytes, bool coax_w, std::vector<int4> &items)
{
    items.clear();
    const int nkeys = (int)Lst.key_beg.size() - 1, nd = std::max(Lst.ndst_rank, 1);
    const long long nblk = std::min<long long>(nd, std::max<long long>(1, (long long)((ws_bytes + L2_BUDGET - 1) / L2_BUDGET)));
    const int *rk = Lst.dst_rank.data();
    for (long long k = 0; k < nblk; k++) {
        const int lo = (int)(k * nd / nblk), hi = (int)((k + 1) * nd / nblk);
        for (int d = 0; d < nkeys; d++) {
            int a0 = Lst.key_beg[d], a1 = Lst.key_beg[d + 1];
            if (nblk > 1) {
                a0 = (int)(std::lower_bound(rk + Lst.key_beg[d], rk + Lst.key_beg[d + 1], lo) - rk);
                a1 = (int)(std::lower_bound(rk + Lst.key_beg[d], rk + Lst.key_beg[d + 1], hi) - rk);
            }
            const long long e0 = (long long)a0 * nrhs, e1 = (long long)a1 * nrhs;
            for (long long a = e0; a < e1; a += width)
                items.push_back(make_int4(d, (int)a, (int)std::min<long long>(width, e1 - a), coax_w ? Lst.key_w[d] : 0));
        }
    }
}

// Device items of a SIMT pass for nrhs right-hand sides, rebuilt when nrhs changes.
static int ensure_items(RcrList &Lst, int nrhs, size_t ws_bytes)
{
    if (Lst.items_nrhs == nrhs) return FMM_OK;
    std::vector<int4> items;
    build_items(Lst, nrhs, Lst.tc, ws_bytes, true, items);
    if (items.size() > Lst.items_cap) {
        if (Lst.items) cudaFree(Lst.items);
        Lst.items = nullptr;
        FMM_CUDA_TRY(cudaMalloc(&Lst.items, sizeof(int4) * items.size()));
        Lst.items_cap = items.size();
    }
    if (!items.empty())
        FMM_CUDA_TRY(cudaMemcpy(Lst.items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
    Lst.n_items = (int)items.size();
    Lst.items_nrhs = nrhs;
    return FMM_OK;
}

int launch_rcr_pass(RcrList &Lst, RcrPass ps, cudaStream_t st)
{
    if (Lst.key_beg.empty() || Lst.key_beg.back() == 0) return FMM_OK;
    {
        size_t ws = ((size_t)ps.nsrc * ps.pin * ps.pin + (size_t)ps.ndst * ps.pout * ps.pout) * sizeof(float2) * ps.nrhs;
        int e = ensure_items(Lst, ps.nrhs, ws);
        if (e) return e;
    }
    ps.items = Lst.items;
    ps.g_src = Lst.src;
    ps.g_dst = Lst.dst;
    const int p = ps.p;
    size_t sm = rcr_tile_smem(p, Lst.tc, Lst.shc);
    return with_tile(Lst.tc, Lst.shc, Lst.bal, [&](auto t) -> int {
        using T = decltype(t);
        return launch_tile<T::TC, T::CG, T::R1, T::R2, T::SHC, T::BAL>(ps, Lst.n_items, sm, st);
    });
}

// Shared memory that keeps two CTAs on an SM: 228 KB per SM, 1 KB reserved and the static
// arrays per CTA.
static const size_t TWO_CTA_SMEM = (228 * 1024) / 2 - 1024 - 1024;
// and the most one CTA may take (227 KB less the static column indices)
const size_t MAX_TILE_SMEM = 227 * 1024 - 1024;

// Columns per CTA: the largest of 64, 32, 16 whose tiles (and, where they also fit, the
// staged rotation and coaxial blocks) keep two CTAs per SM, else 8 (one CTA per SM, p <= 42),
// else 4 (p <= 60).  With 16-column groups that gives every thread of the CTA a unit of work
// down to p = 10.
static void pick_tile(int p, int &tc, int &shc)
{
    for (tc = 64; tc >= 16; tc /= 2) {
        if (rcr_tile_smem(p, tc, 1) <= TWO_CTA_SMEM) { shc = 1; return; }
        if (rcr_tile_smem(p, tc, 0) <= TWO_CTA_SMEM) { shc = 0; return; }
    }
    tc = rcr_tile_smem(p, 8, 0) <= MAX_TILE_SMEM ? 8 : 4;
    shc = 0;
}

// drank: Morton rank of each destination box among the ndst boxes of its level.  The list is
// sorted by key, and within a key by the destination's Morton rank (two stable counting sorts).
static int upload_list(Plan *P, RcrList &Lst, const std::vector<int> &key, const std::vector<int> &src,
                       const std::vector<int> &dst, int nkeys, const std::vector<int> &key_w, int p,
                       const std::vector<int> &drank, int ndst)
{
    int tc, shc;
    pick_tile(p, tc, shc);
    size_t T = key.size();
    std::vector<int> byrank(std::max<size_t>(T, 1));
    {
        std::vector<int> rc(ndst + 1, 0);
        for (size_t i = 0; i < T; i++) rc[drank[dst[i]] + 1]++;
        for (int r = 0; r < ndst; r++) rc[r + 1] += rc[r];
        for (size_t i = 0; i < T; i++) byrank[rc[drank[dst[i]]]++] = (int)i;
    }
    std::vector<int> cnt(nkeys + 1, 0);
    for (size_t i = 0; i < T; i++) cnt[key[i] + 1]++;
    for (int d = 0; d < nkeys; d++) cnt[d + 1] += cnt[d];
    std::vector<int> gs(std::max<size_t>(T, 1)), gd(std::max<size_t>(T, 1)), fill(nkeys, 0);
    Lst.dst_rank.assign(T, 0);
    for (size_t q = 0; q < T; q++) {
        const int i = byrank[q];
        int pos = cnt[key[i]] + fill[key[i]]++;
        gs[pos] = src[i];
        gd[pos] = dst[i];
        Lst.dst_rank[pos] = drank[dst[i]];
    }
    Lst.ndst_rank = ndst;
    Lst.key_beg.assign(cnt.begin(), cnt.end());
    Lst.key_w = key_w;
    Lst.tc = tc;
    Lst.shc = shc;
    Lst.items_nrhs = 0;
    if (T == 0) return FMM_OK;
    int e = ensure_items(Lst, 1, 0);
    if (e) return e;
    FMM_CUDA_TRY(dev_alloc(P, (void **)&Lst.src, sizeof(int) * T));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&Lst.dst, sizeof(int) * T));
    FMM_CUDA_TRY(cudaMemcpy(Lst.src, gs.data(), sizeof(int) * T, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(Lst.dst, gd.data(), sizeof(int) * T, cudaMemcpyHostToDevice));
    return FMM_OK;
}

// Work lists of the batched passes: per level, the M2L translations grouped by direction,
// the M2M pairs (box -> parent) and the L2L pairs (parent -> box) grouped by octant.
int build_rcr_lists(Plan *P)
{
    // Morton rank of every box of every level (the level sets hold the boxes' Morton numbers
    // in first-occurrence order)
    std::vector<std::vector<int>> rank(P->lmax + 1);
    for (int l = P->lmin; l <= P->lmax; l++) {
        const std::vector<long long> &keys = P->tree.sets[l];
        std::vector<int> ord(keys.size());
        for (size_t i = 0; i < ord.size(); i++) ord[i] = (int)i;
        std::sort(ord.begin(), ord.end(), [&](int a, int b) { return keys[a] < keys[b]; });
        rank[l].assign(keys.size(), 0);
        for (size_t r = 0; r < ord.size(); r++) rank[l][ord[r]] = (int)r;
    }
    for (int l = P->lmin; l <= P->lmax; l++) {
        LevelDev &L = P->lev[l];
        if (L.num_sr > 0) {
            long long T = L.num_sr;
            std::vector<int> beg(L.nb + 1), src(T), dst(T), key(T);
            std::vector<short> dir(T);
            FMM_CUDA_TRY(cudaMemcpy(beg.data(), L.sr_beg, sizeof(int) * (L.nb + 1), cudaMemcpyDeviceToHost));
            FMM_CUDA_TRY(cudaMemcpy(src.data(), L.sr_src, sizeof(int) * T, cudaMemcpyDeviceToHost));
            FMM_CUDA_TRY(cudaMemcpy(dir.data(), L.sr_dir, sizeof(short) * T, cudaMemcpyDeviceToHost));
            for (int b = 0; b < L.nb; b++)
                for (int t = beg[b]; t < beg[b + 1]; t++) {
                    dst[t] = b;
                    key[t] = dir[t];
                }
            std::vector<int> kw(P->dir_dist, P->dir_dist + NDIR);
            int st = upload_list(P, L.m2l, key, src, dst, NDIR, kw, L.p, rank[l], L.nb);
            if (st) return st;
        }
        if (l > P->lmin) {
            LevelDev &PL = P->lev[l - 1];
            std::vector<int> par(L.nb), key(L.nb), self(L.nb);
            std::vector<unsigned char> oct(L.nb);
            FMM_CUDA_TRY(cudaMemcpy(par.data(), L.parent, sizeof(int) * L.nb, cudaMemcpyDeviceToHost));
            FMM_CUDA_TRY(cudaMemcpy(oct.data(), L.octant, L.nb, cudaMemcpyDeviceToHost));
            for (int b = 0; b < L.nb; b++) {
                key[b] = oct[b];
                self[b] = b;
            }
            std::vector<int> kw(8, 0);
            int st = upload_list(P, L.m2m, key, self, par, 8, kw, PL.p, rank[l - 1], PL.nb);
            if (st) return st;
            st = upload_list(P, L.l2l, key, par, self, 8, kw, PL.p, rank[l], L.nb);
            if (st) return st;
        }
    }
    return FMM_OK;
}

} // namespace fmm

namespace fmm {
// Tile width and schedule per pass, chosen at plan creation by timing the candidates on this
// plan's own lists and tables (one right-hand side): the default from pick_tile and a narrower
// tile -- 4 columns where the default is 8 (large p, few items per direction: more CTAs, two
// per SM), half the width where it is 16, 32 or 64 -- each with the default and the balanced
// unit schedule (BAL).  The winner is kept; matvec results do not depend on the choice beyond the
// order of the FP32 atomic additions.
int tune_rcr_tiles(Plan *P)
{
    // FMMBEM_TILE_BAL=0/1/2 forces one schedule on every pass (default tile width; a shape
    // without that schedule runs the default one), for tests
    if (const char *env = getenv("FMMBEM_TILE_BAL")) {
        const int bal = std::max(0, std::min(2, atoi(env)));
        for (int l = P->lmin; l <= P->lmax; l++)
            for (RcrList *R : {&P->lev[l].m2m, &P->lev[l].m2l, &P->lev[l].l2l}) {
                R->bal = bal;
                R->items_nrhs = 0;
            }
        return FMM_OK;
    }
    cudaEvent_t a, b;
    FMM_CUDA_TRY(cudaEventCreate(&a));
    FMM_CUDA_TRY(cudaEventCreate(&b));
    int rc = FMM_OK;
    for (int l = P->lmin; l <= P->lmax && rc == FMM_OK; l++) {
        LevelDev &L = P->lev[l];
        for (int which = PASS_M2M; which <= PASS_L2L && rc == FMM_OK; which++) {
            if (which != PASS_M2L && l == P->lmin) continue;
            RcrList &Lst = which == PASS_M2M ? L.m2m : which == PASS_M2L ? L.m2l : L.l2l;
            if (Lst.key_beg.empty() || Lst.key_beg.back() == 0) continue;
            int p = which == PASS_M2L ? L.p : P->lev[l - 1].p;
            std::vector<int3> cand = {{Lst.tc, Lst.shc, 0}};
            if (Lst.tc == 8) cand.push_back({4, 0, 0});
            if (Lst.tc == 16) cand.push_back({8, 0, 0});
            if (Lst.tc >= 32) cand.push_back({Lst.tc / 2, rcr_tile_smem(p, Lst.tc / 2, 1) <= TWO_CTA_SMEM ? 1 : 0, 0});
            // balanced variants (1: narrow column groups where they pay, 2: the default groups, one-row
            // units) exist for every width without staged blocks, and for 32 (and 64: 1 only) with
            for (size_t i = 0, n0 = cand.size(); i < n0; i++) {
                if (cand[i].y == 0 || cand[i].x >= 32) cand.push_back({cand[i].x, cand[i].y, 1});
                if (cand[i].x <= 32 && (cand[i].y == 0 || cand[i].x == 32)) cand.push_back({cand[i].x, cand[i].y, 2});
            }
            float best = 1e30f;
            int3 pick = cand[0];
            for (auto &c : cand) {
                Lst.tc = c.x;
                Lst.shc = c.y;
                Lst.bal = c.z;
                Lst.items_nrhs = 0;
                float tot = 0.f;
                for (int rep = 0; rep < 4 && rc == FMM_OK; rep++) {
                    if (cudaEventRecord(a, P->stream) != cudaSuccess) rc = FMM_ERR_CUDA;
                    if (rc == FMM_OK) rc = launch_pass32(P, l, which, 1, P->stream);
                    if (rc == FMM_OK && cudaEventRecord(b, P->stream) != cudaSuccess) rc = FMM_ERR_CUDA;
                    if (rc == FMM_OK && cudaEventSynchronize(b) != cudaSuccess) rc = FMM_ERR_CUDA;
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, a, b);
                    if (rep > 0) tot += ms;
                }
                if (rc != FMM_OK) break;
                if (tot < best) {
                    best = tot;
                    pick = c;
                }
            }
            Lst.tc = pick.x;
            Lst.shc = pick.y;
            Lst.bal = pick.z;
            Lst.items_nrhs = 0;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc == FMM_ERR_CUDA) fmm_set_error("tile tuning: %s", cudaGetErrorString(cudaGetLastError()));
    return rc;
}
} // namespace fmm
