// M2L of the mixed path on the 5th-generation tensor cores (tcgen05.mma, kind::tf32) for the
// levels whose translation operators are small enough to store densely (p <= 16, the levels
// that carry most translations).
//
// The translations of one direction share one operator T_d (p^2 x p^2 complex; the RCR
// product of translation.cu:1864-1961 formed once at plan time).  With the columns of a tile
// being 128 translations of that direction (times right-hand sides), the pass is the real GEMM
//     D[t][o] = sum_k A[t][k] B[o][k],   A[t] = source expansion of translation t,
//                                         B    = T_d embedded as a real 2p^2 x 2p^2 matrix,
// k and o running over interleaved (re, im) parts, so A is the expansion as it lies in memory.
// Split TF32 (3 products hi*hi + hi*lo + lo*hi of 11-bit halves) gives FP32-level accuracy.
//
// One CTA per (128-translation tile, output half): 256 threads gather A and copy B, chunk by
// chunk (KC of K), into two shared-memory stages in the no-swizzle K-major core-matrix layout;
// one thread issues the MMAs into a TMEM accumulator (128 lanes x Nmma columns) and commits
// them to the stage's mbarrier; at the end the 8 warps read the accumulator back
// (tcgen05.ld), stage it in shared memory and add it into the destination local expansions
// with coalesced FP32 atomics.  Every wait has a time limit; a wait that gives up sets the
// plan's error flag and the CTA skips its output.
#include "plan.h"
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace fmm {

constexpr int TC_M = 128;          // translations per tile (MMA M)
constexpr int TC_THREADS = 256;
constexpr int TC_MAXP = 16;
constexpr size_t TC_SMEM_MAX = 232448;  // 227 KB of dynamic shared memory per CTA
constexpr size_t TC_EXTRA = 16 + 16 + 2 * TC_M * sizeof(int);

struct TcPass {
    const int4 *items;
    const int *g_src, *g_dst;
    int nrhs, nsrc, ndst;
    int p, K, KC, nch, nhalf, CH, Nmma;
    const float *B;
    const float2 *src;
    float2 *dst;
    int *err;
};

static size_t tc_stage_bytes(int KC, int Nmma) { return (size_t)8 * KC * (TC_M + Nmma); }
static size_t tc_smem_bytes(int KC, int Nmma) { return 2 * tc_stage_bytes(KC, Nmma) + TC_EXTRA; }

// Output halves, MMA width and K chunk for order p: each half holds CH coefficients
// (2 CH real outputs, Nmma = that rounded up to 16, <= 256); KC from {40, 32} with the
// least padding of K = 2p^2 that fits two stages.
static bool tc_geometry(int p, TcM2L &g)
{
    if (p < 4 || p > TC_MAXP) return false;
    const int P2 = p * p, K = 2 * P2;
    for (g.nhalf = 1;; g.nhalf++) {
        g.CH = (P2 + g.nhalf - 1) / g.nhalf;
        g.Nmma = (2 * g.CH + 15) / 16 * 16;
        if (g.Nmma <= 256) break;
    }
    int best = 0;
    for (int kc : {40, 32}) {
        if (tc_smem_bytes(kc, g.Nmma) > TC_SMEM_MAX) continue;
        int kp = (K + kc - 1) / kc * kc;
        if (!best || kp < (K + best - 1) / best * best) best = kc;
    }
    if (!best) return false;
    g.KC = best;
    g.nch = (K + best - 1) / best;
    return true;
}

// byte offset of element (row r, k) in a no-swizzle K-major tile of KC columns: 8-row x 16-byte
// core matrices, K-adjacent cores 128 B apart (leading byte offset), 8-row groups 32 KC apart
// (stride byte offset)
__host__ __device__ __forceinline__ uint32_t core_off(int r, int k, int KC)
{
    return (uint32_t)((r >> 3) * 32 * KC + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ float tf32_trunc(float x) { return __int_as_float(__float_as_int(x) & (int)0xffffe000); }

__device__ __forceinline__ uint32_t smem_u32(const void *ptr) { return (uint32_t)__cvta_generic_to_shared(ptr); }

// shared-memory matrix descriptor (no swizzle): start, leading and stride byte offsets (>> 4),
// descriptor version 1 at bits 46-47
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// wait for the phase of the given parity of an mbarrier, at most ~1 s of SM clock
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.u32 %0, 1, 0, q;\n\t}"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
        if (clock64() - t0 > 2000000000LL) return false;
    }
}

__global__ void __launch_bounds__(TC_THREADS, 1) m2l_tc_kernel(TcPass ps)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int KC = ps.KC, Nmma = ps.Nmma, K = ps.K, P2 = ps.p * ps.p;
    const uint32_t tA = (uint32_t)TC_M * KC * 4, tB = (uint32_t)Nmma * KC * 4, stage = 2 * tA + 2 * tB;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + 2 * stage);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 2);
    int *s_src = reinterpret_cast<int *>(tslot + 4), *s_dst = s_src + TC_M;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int item = blockIdx.x / ps.nhalf, h = blockIdx.x - item * ps.nhalf;
    const int4 it = ps.items[item];

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)), "r"(256));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar + 1)));
    }
    if (tid < TC_M) {
        // column e = translation t x nrhs + right-hand side r, as in the batched tiles
        bool v = tid < it.z;
        int e = it.y + tid, t = e / ps.nrhs, r = e - t * ps.nrhs;
        s_src[tid] = v ? ps.g_src[t] + r * ps.nsrc : -1;
        s_dst[tid] = v ? ps.g_dst[t] + r * ps.ndst : -1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tslot;
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(Nmma >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
    const uint32_t lbo = 128, sbo = 32 * KC;
    const float *Bd = ps.B + (size_t)(it.x * ps.nhalf + h) * ps.nch * 2 * Nmma * KC;
    const float *srcf = reinterpret_cast<const float *>(ps.src);
    bool ok = true;

    for (int c = 0; c < ps.nch; c++) {
        const int buf = c & 1;
        unsigned char *Ahi = smem + buf * stage, *Alo = Ahi + tA, *Bst = Ahi + 2 * tA;
        if (c >= 2) ok = mbar_wait(smem_u32(mbar + buf), ((c >> 1) - 1) & 1) && ok;
        // A: 4 consecutive k of one row per task -> one 16-byte core row, split into hi / lo
        const int kq = KC / 4;
        for (int task = tid; task < TC_M * kq; task += TC_THREADS) {
            int r = task / kq, kg = task - r * kq, k0 = c * KC + 4 * kg, s = s_src[r];
            float x[4] = {0.f, 0.f, 0.f, 0.f};
            if (s >= 0) {
                const float *row = srcf + (size_t)s * K + k0;
                if (k0 + 1 < K) {
                    float2 v = __ldg(reinterpret_cast<const float2 *>(row));
                    x[0] = v.x; x[1] = v.y;
                }
                if (k0 + 3 < K) {
                    float2 v = __ldg(reinterpret_cast<const float2 *>(row + 2));
                    x[2] = v.x; x[3] = v.y;
                }
            }
            float4 hi, lo;
            hi.x = tf32_trunc(x[0]); lo.x = tf32_trunc(x[0] - hi.x);
            hi.y = tf32_trunc(x[1]); lo.y = tf32_trunc(x[1] - hi.y);
            hi.z = tf32_trunc(x[2]); lo.z = tf32_trunc(x[2] - hi.z);
            hi.w = tf32_trunc(x[3]); lo.w = tf32_trunc(x[3] - hi.w);
            uint32_t o = core_off(r, 4 * kg, KC);
            *reinterpret_cast<float4 *>(Ahi + o) = hi;
            *reinterpret_cast<float4 *>(Alo + o) = lo;
        }
        // B: the chunk's hi and lo tiles are stored contiguously in this layout
        const float4 *bsrc = reinterpret_cast<const float4 *>(Bd + (size_t)c * 2 * Nmma * KC);
        float4 *bdst = reinterpret_cast<float4 *>(Bst);
        for (int i = tid; i < (int)(2 * tB / 16); i += TC_THREADS) bdst[i] = __ldg(bsrc + i);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t a_hi = smem_u32(Ahi), a_lo = a_hi + tA, b_hi = smem_u32(Bst), b_lo = b_hi + tB;
            for (int ks = 0; ks < KC / 8; ks++)
                for (int pass = 0; pass < 3; pass++) {
                    uint64_t ad = smem_desc((pass == 2 ? a_lo : a_hi) + ks * 256, lbo, sbo);
                    uint64_t bd = smem_desc((pass == 1 ? b_lo : b_hi) + ks * 256, lbo, sbo);
                    uint32_t acc = (c > 0 || ks > 0 || pass > 0) ? 1u : 0u;
                    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %4, 0;\n\t"
                                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, q;\n\t}" ::"r"(tmem),
                                 "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(mbar + buf))
                         : "memory");
        }
    }
    {
        const int last = ps.nch - 1;
        ok = mbar_wait(smem_u32(mbar + (last & 1)), (last >> 1) & 1) && ok;
    }
    ok = __syncthreads_and(ok);
    asm volatile("tcgen05.fence::after_thread_sync;");
    float *sD = reinterpret_cast<float *>(smem);
    const int ld = Nmma + 1;
    if (ok) {
        // accumulator -> shared memory: warp w reads lanes 32 (w % 4)..+31 (its rows), warps
        // 0-3 the first half of the columns, warps 4-7 the second
        const int wq = warp & 3, row = wq * 32 + lane, half = Nmma / 2, c0 = (warp >> 2) * half;
        for (int cc = c0; cc < c0 + half; cc += 8) {
            uint32_t v[8];
            uint32_t ta = tmem + ((uint32_t)(wq * 32) << 16) + (uint32_t)cc;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                         : "r"(ta));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 8; j++) sD[row * ld + cc + j] = __uint_as_float(v[j]);
        }
    } else if (tid == 0) {
        atomicExch(ps.err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
    if (!ok) return;
    // coalesced adds into the destination locals: one row (translation) per warp at a time
    const int co0 = h * ps.CH, nco = min(ps.CH, P2 - co0);
    for (int r = warp; r < TC_M; r += TC_THREADS / 32) {
        const int d = s_dst[r];
        if (d < 0) continue;
        float2 *out = ps.dst + (size_t)d * P2 + co0;
        for (int j = lane; j < nco; j += 32) atomicAdd(out + j, make_float2(sD[r * ld + 2 * j], sD[r * ld + 2 * j + 1]));
    }
}

// The real-embedded operators of one level, split into TF32 hi/lo, in the tile layout:
// element (o, k) of half h, chunk c holds  Re T (o, k even-even / odd-odd), -Im T (o even, k
// odd) or Im T (o odd, k even) of coefficient (h CH + o/2, (c KC + k)/2).
__global__ void tc_split_kernel(const double2 *__restrict__ T, int p, int KC, int nch, int nhalf, int CH, int Nmma,
                                float *__restrict__ B, size_t total)
{
    const int P2 = p * p, K = 2 * P2;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
        size_t z = q;
        int kcol = (int)(z % KC); z /= KC;
        int nr = (int)(z % Nmma); z /= Nmma;
        int part = (int)(z % 2); z /= 2;
        int c = (int)(z % nch); z /= nch;
        int h = (int)(z % nhalf);
        int d = (int)(z / nhalf);
        int k = c * KC + kcol, nco = min(CH, P2 - h * CH);
        double v = 0.0;
        if (nr < 2 * nco && k < K) {
            double2 t = T[((size_t)d * P2 + h * CH + nr / 2) * P2 + k / 2];
            int po = nr & 1, pi = k & 1;
            v = po == 0 ? (pi == 0 ? t.x : -t.y) : (pi == 0 ? t.y : t.x);
        }
        float hi = tf32_trunc((float)v);
        float lo = tf32_trunc((float)(v - (double)hi));
        size_t base = ((((size_t)d * nhalf + h) * nch + c) * 2 + part) * (size_t)Nmma * KC;
        B[base + core_off(nr, kcol, KC) / 4] = part ? lo : hi;
    }
}

static int build_tc_level(Plan *P, int l)
{
    LevelDev &L = P->lev[l];
    TcM2L &g = L.tc;
    if (!tc_geometry(L.p, g)) return FMM_OK;
    const int P2 = L.p * L.p;
    size_t total = (size_t)NDIR * g.nhalf * g.nch * 2 * g.Nmma * g.KC;
    double2 *T = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&T, sizeof(double2) * (size_t)NDIR * P2 * P2));
    int st = gen_dense_m2l(P, l, T);
    if (st) { cudaFree(T); return st; }
    cudaError_t e = dev_alloc(P, (void **)&g.B, sizeof(float) * total);
    if (e != cudaSuccess) { cudaFree(T); fmm_set_error("tensor-core M2L tables: %s", cudaGetErrorString(e)); return FMM_ERR_CUDA; }
    g.B_bytes = sizeof(float) * total;
    tc_split_kernel<<<152 * 16, 256, 0, P->stream>>>(T, L.p, g.KC, g.nch, g.nhalf, g.CH, g.Nmma, g.B, total);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
    cudaFree(T);
    if (e != cudaSuccess) { fmm_set_error("tensor-core M2L tables: %s", cudaGetErrorString(e)); return FMM_ERR_CUDA; }
    return FMM_OK;
}

static int ensure_tc_items(LevelDev &L, int nrhs)
{
    TcM2L &g = L.tc;
    if (g.items_nrhs == nrhs) return FMM_OK;
    const RcrList &Lst = L.m2l;
    std::vector<int4> items;
    int nkeys = (int)Lst.key_beg.size() - 1;
    for (int d = 0; d < nkeys; d++) {
        long long e0 = (long long)Lst.key_beg[d] * nrhs, e1 = (long long)Lst.key_beg[d + 1] * nrhs;
        for (long long a = e0; a < e1; a += TC_M)
            items.push_back(make_int4(d, (int)a, (int)std::min<long long>(TC_M, e1 - a), 0));
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

int launch_tc_m2l(Plan *P, int l, int nrhs, cudaStream_t st)
{
    LevelDev &L = P->lev[l];
    TcM2L &g = L.tc;
    if (L.m2l.key_beg.empty() || L.m2l.key_beg.back() == 0) return FMM_OK;
    int e = ensure_tc_items(L, nrhs);
    if (e) return e;
    TcPass ps;
    ps.items = g.items;
    ps.g_src = L.m2l.src;
    ps.g_dst = L.m2l.dst;
    ps.nrhs = nrhs;
    ps.nsrc = L.nb;
    ps.ndst = L.nb;
    ps.p = L.p;
    ps.K = 2 * L.p * L.p;
    ps.KC = g.KC;
    ps.nch = g.nch;
    ps.nhalf = g.nhalf;
    ps.CH = g.CH;
    ps.Nmma = g.Nmma;
    ps.B = g.B;
    ps.src = L.Cm32;
    ps.dst = L.Dl32;
    ps.err = P->tc_err;
    size_t sm = tc_smem_bytes(g.KC, g.Nmma);
    static size_t attr = 0;
    e = raise_smem_limit((const void *)m2l_tc_kernel, sm, &attr);
    if (e) return e;
    m2l_tc_kernel<<<g.n_items * g.nhalf, TC_THREADS, sm, st>>>(ps);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

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

// For every level with p <= 16: build the dense split operators and keep the tensor-core
// pass where it beats the SIMT tiles on this plan (4 timed runs each), else free its tables.
// FMMBEM_TENSOR_M2L=0 keeps the SIMT tiles, =1 takes the tensor cores wherever they apply.
int tune_tc_m2l(Plan *P)
{
    const char *env = getenv("FMMBEM_TENSOR_M2L");
    int mode = env ? atoi(env) : -1;
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
        LevelDev &L = P->lev[l];
        if (L.num_sr == 0 || L.p > TC_MAXP) continue;
        rc = build_tc_level(P, l);
        if (rc || !L.tc.B) break;
        float ms[2] = {0.f, 0.f};
        for (int on = 0; on < 2 && rc == FMM_OK; on++) {
            L.tc.on = on;
            for (int rep = 0; rep < 4 && rc == FMM_OK; rep++) {
                if (cudaEventRecord(a, P->stream) != cudaSuccess) rc = FMM_ERR_CUDA;
                if (rc == FMM_OK) rc = launch_pass32(P, l, PASS_M2L, 1, P->stream);
                if (rc == FMM_OK && cudaEventRecord(b, P->stream) != cudaSuccess) rc = FMM_ERR_CUDA;
                if (rc == FMM_OK && cudaEventSynchronize(b) != cudaSuccess) rc = FMM_ERR_CUDA;
                float t = 0.f;
                cudaEventElapsedTime(&t, a, b);
                if (rep > 0) ms[on] += t;
            }
        }
        if (rc == FMM_OK) rc = check_tc_error(P);
        if (rc) break;
        L.tc.on = (mode == 1 || ms[1] < ms[0]) ? 1 : 0;
        if (!L.tc.on) {
            cudaFree(L.tc.B);
            P->device_bytes -= L.tc.B_bytes;
            L.tc.B = nullptr;
            L.tc.B_bytes = 0;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc == FMM_ERR_CUDA && !fmm_last_error()[0]) fmm_set_error("tensor-core M2L tuning: %s", cudaGetErrorString(cudaGetLastError()));
    return rc;
}

} // namespace fmm
