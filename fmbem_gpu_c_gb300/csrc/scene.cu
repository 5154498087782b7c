// Scenes: many plans (bodies, or one body at many frequencies) solved in lockstep.
//
// The plans of a scene keep their own octrees, orders and tables; the scene joins their
// unknowns into one vector (plan i at off[i]) and applies all their mixed-precision operators
// with one set of launches per matvec, whatever the number of bodies:
//   1. one kernel zeroes every plan's FP32 expansions (and the work-queue heads);
//   2. one P2M kernel over all plans' leaf boxes;
//   3. per level from the deepest up: the M2M passes of every plan that has the level, as
//      persistent work-queue launches (one per tile shape; the shapes run side by side);
//   4. the M2L passes of every plan and level, the same way;
//   5. per level from the top down: the L2L passes;
//   6. one fused L2P + near-field + identity kernel over all elements.
// Each phase's queue holds (pass, tile) items longest first; the resident CTAs of the
// persistent kernel take them from an atomic head, so uneven bodies share the GPU without a
// host round trip per body.  Phases follow one another in stream order: nothing waits on
// the device.  From the second call on the whole matvec replays as one CUDA graph.  Plans
// can be switched off (converged bodies of a solve): a compaction kernel at the start of the
// graph keeps, in order, the queue, P2M and L2P items of the switched-on plans only.
// The lockstep GMRES (gmres_core.h) then costs one scene matvec, three batched dot
// launches and one host synchronisation per Krylov step for all bodies together; a body
// whose residual is below tol stops extending its basis while the others continue.
//
// The tensor-core M2L is not used here (its tiles are per plan); the scene runs the SIMT
// tiles the plan tuned for every level.
#include "plan.h"
#include "gmres_core.h"
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

namespace fmm {

struct BodyDev {
    long long off;                // first unknown of this plan in the scene vector
    int nf, pl;                   // elements; leaf truncation order
    double k;
    double2 a;                    // identity coefficient
    const int *leaf_beg, *leaf_elem, *elem_leaf, *near_beg, *near_col;
    const float2 *U, *Rv, *nearv; // FP32 element tables and near-field matrix
    float2 *Cm, *Dl;              // leaf-level expansions (one column)
};

struct QueueGroup {               // one persistent launch: the passes of one tile shape in a phase
    int tc = 8, shc = 0, bal = 0, nwork = 0, head = 0, grid = 1;
    size_t smem = 0;
    int *work_pass = nullptr;         // the items of the switched-on plans (compacted per matvec)
    int4 *work_item = nullptr;
};

// One list that the compaction kernel filters by the plans' switches, order kept: n items of
// w0 (and w1) 32-bit words from src0 (src1) to dst0 (dst1); the count to *count.
struct CompactJob {
    int n, w0, w1;
    const int *owner;
    const int *src0, *src1;
    int *dst0, *dst1;
    int *count;
};

constexpr int SCENE_SIDE = 4;

struct Scene {
    std::vector<Plan *> plans;
    std::vector<int> buf_gen;         // each plan's expansion-buffer generation the scene was built on
    std::vector<long long> off;
    long long N = 0;
    int device = 0;
    cudaStream_t stream = nullptr, side[SCENE_SIDE] = {};
    std::vector<cudaEvent_t> events;  // fork / join per phase, and per plan for FP64 matvecs
    BodyDev *bodies = nullptr;
    RcrPass *passes = nullptr;
    int2 *p2m_items = nullptr, *l2p_items = nullptr;
    int n_p2m = 0, n_l2p = 0;
    float2 **zero_ptr = nullptr;
    long long *zero_len = nullptr;
    int2 *zero_items = nullptr;       // (segment, first float2) in chunks of ZERO_CHUNK
    int *zero_owner = nullptr;        // plan of each segment
    int n_zero = 0;
    CompactJob *jobs = nullptr;       // the queue groups, then the P2M and L2P item lists
    int n_jobs = 0;
    int *counts = nullptr;            // items left after compaction, per job
    int2 *p2m_all = nullptr, *l2p_all = nullptr;
    int *active = nullptr;            // per plan: 1 = apply its operator, 0 = skip it (y = 0)
    std::vector<int> active_host;
    std::vector<int> user_active;     // fmm_scene_set_active (empty: all) for fmm_scene_matvec
    int *heads = nullptr;
    int n_heads = 0;
    std::vector<std::vector<QueueGroup>> phases;
    int4 *chunks = nullptr;           // (plan, begin, end) over the scene vector for the BLAS
    int n_chunks = 0;
    double2 *xin = nullptr, *yout = nullptr;
    float2 *xin32 = nullptr;          // xin in FP32, written by the P2M pass for the near-field gathers
    cudaGraphExec_t graph = nullptr;
    int calls = 0;
    // solver workspace
    double2 *V = nullptr, *r = nullptr, *w = nullptr, *b = nullptr, *x = nullptr, *d = nullptr, *dev_h = nullptr;
    double *alpha = nullptr;
    int restart_cap = 0;
    std::vector<void *> allocs;
    // device time of the last solve's matvecs (events around each, read at the next sync)
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    int pending = -1;                 // precision of an unread event pair, -1 none
    double ms[2] = {0.0, 0.0};
    int calls_by_prec[2] = {0, 0};
    double solve_s = 0.0;
};

static const int ZERO_CHUNK = 8192;
static const int BLAS_CHUNK = 4096;

template <typename Tp>
static cudaError_t salloc(Scene *S, Tp **p, size_t bytes)
{
    cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(bytes, 16));
    if (e == cudaSuccess) S->allocs.push_back((void *)*p);
    return e;
}

template <typename Tp>
static int upload(Scene *S, Tp **dst, const std::vector<Tp> &src)
{
    FMM_CUDA_TRY(salloc(S, dst, sizeof(Tp) * src.size()));
    if (!src.empty()) FMM_CUDA_TRY(cudaMemcpy(*dst, src.data(), sizeof(Tp) * src.size(), cudaMemcpyHostToDevice));
    return FMM_OK;
}

// ------------------------------------------------------------------------------ kernels
__global__ void scene_zero_kernel(float2 *const *ptr, const long long *len, const int *owner, const int2 *items, int nitems,
                                  int *heads, int nheads, const int *active)
{
    if (blockIdx.x == 0)
        for (int i = threadIdx.x; i < nheads; i += blockDim.x) heads[i] = 0;
    if ((int)blockIdx.x >= nitems) return;
    const int2 it = items[blockIdx.x];
    if (!active[owner[it.x]]) return;
    float2 *p = ptr[it.x];
    long long end = min(len[it.x], (long long)it.y + ZERO_CHUNK);
    for (long long i = it.y + threadIdx.x; i < end; i += blockDim.x) p[i] = make_float2(0.f, 0.f);
}

// Order-keeping compaction of every job's items to those of switched-on plans: one CTA of
// 1024 threads per job, a block-wide prefix count per 1024 items.
__global__ void __launch_bounds__(1024) scene_compact_kernel(const CompactJob *__restrict__ jobs,
                                                             const int *__restrict__ active)
{
    const CompactJob J = jobs[blockIdx.x];
    __shared__ int warp_sum[32], base_s;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) base_s = 0;
    __syncthreads();
    for (int b0 = 0; b0 < J.n; b0 += 1024) {
        const int i = b0 + tid;
        const bool keep = i < J.n && active[J.owner[i]];
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) warp_sum[wid] = __popc(m);
        __syncthreads();
        if (wid == 0) {
            int v = warp_sum[lane], x = v;
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            warp_sum[lane] = x - v; // exclusive
        }
        __syncthreads();
        const int base = base_s;
        if (keep) {
            const int pos = base + warp_sum[wid] + __popc(m & ((1u << lane) - 1));
            for (int q = 0; q < J.w0; q++) J.dst0[(size_t)pos * J.w0 + q] = J.src0[(size_t)i * J.w0 + q];
            for (int q = 0; q < J.w1; q++) J.dst1[(size_t)pos * J.w1 + q] = J.src1[(size_t)i * J.w1 + q];
        }
        __syncthreads();
        if (tid == 1023) base_s = base + warp_sum[31] + __popc(m);
        __syncthreads();
    }
    if (tid == 0) *J.count = base_s;
}

// C_b[n,m] = ik sum_e x_e U_e[n,m] for leaf box b of plan it.x (the plan's p2m_kernel for one
// column in FP32): the box's elements and their i k x_e staged in shared memory once per item,
// and x_e in FP32 written to x32 for the near-field gathers of scene_l2p_kernel (every element
// lies in one leaf box)
__global__ void scene_p2m_kernel(const BodyDev *__restrict__ bodies, const int2 *__restrict__ items,
                                 const int *__restrict__ nitems, const double2 *__restrict__ x, float2 *__restrict__ x32)
{
    constexpr int MAXE = 64;
    __shared__ int s_e[MAXE];
    __shared__ float2 s_x[MAXE];
    const int n = *nitems;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const int2 it = items[w];
        const BodyDev &bd = bodies[it.x];
        const int b = it.y, ppl = bd.pl * bd.pl;
        float2 *out = bd.Cm + (size_t)b * ppl;
        const double2 *xb = x + bd.off;
        const int s0 = bd.leaf_beg[b], ne = bd.leaf_beg[b + 1] - s0;
        __syncthreads(); // the previous item's readers of s_e / s_x are done
        for (int j = threadIdx.x; j < ne; j += blockDim.x) {
            const int e = bd.leaf_elem[s0 + j];
            const double2 xe = xb[e];
            if (j < MAXE) {
                s_e[j] = e;
                s_x[j] = make_float2((float)(-bd.k * xe.y), (float)(bd.k * xe.x));
            }
            x32[bd.off + e] = make_float2((float)xe.x, (float)xe.y);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < ppl; i += blockDim.x) {
            float ar = 0.f, ai = 0.f;
#pragma unroll 4
            for (int j = 0; j < ne && j < MAXE; j++) {
                const float2 xe = s_x[j];
                const float2 u = bd.U[(size_t)s_e[j] * ppl + i];
                ar += xe.x * u.x - xe.y * u.y;
                ai += xe.x * u.y + xe.y * u.x;
            }
            for (int j = MAXE; j < ne; j++) {
                const int e = bd.leaf_elem[s0 + j];
                const double2 xe = xb[e];
                const float xr = (float)(-bd.k * xe.y), xi = (float)(bd.k * xe.x);
                const float2 u = bd.U[(size_t)e * ppl + i];
                ar += xr * u.x - xi * u.y;
                ai += xr * u.y + xi * u.x;
            }
            out[i] = make_float2(ar, ai);
        }
    }
}

static __device__ __forceinline__ void l2p_element(const BodyDev &bd, int e, const double2 *__restrict__ x,
                                                   const float2 *__restrict__ x32, double2 *__restrict__ y)
{
    const int lane = threadIdx.x & 31;
    const double2 *xb = x + bd.off;
    const float2 *xb32 = x32 + bd.off;
    float ar = 0.f, ai = 0.f;
    for (int s = bd.near_beg[e] + lane; s < bd.near_beg[e + 1]; s += 32) {
        const float2 v = bd.nearv[s];
        const float2 xf = xb32[bd.near_col[s]];
        const float xr = xf.x, xi = xf.y;
        ar += v.x * xr - v.y * xi;
        ai += v.x * xi + v.y * xr;
    }
    const int ppl = bd.pl * bd.pl;
    const float2 *D = bd.Dl + (size_t)bd.elem_leaf[e] * ppl, *R = bd.Rv + (size_t)e * ppl;
    for (int i = lane; i < ppl; i += 32) {
        float2 d = D[i], r = R[i];
        ar += d.x * r.x - d.y * r.y;
        ai += d.x * r.y + d.y * r.x;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ar += __shfl_xor_sync(0xffffffffu, ar, o);
        ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    if (lane == 0) {
        double2 xe = xb[e];
        y[bd.off + e] = make_double2(bd.a.x * xe.x - bd.a.y * xe.y + (double)ar, bd.a.x * xe.y + bd.a.y * xe.x + (double)ai);
    }
}

// y_e = a x_e + sum_near A_ej x_j + sum_nm D[n,m] Rv_e[n,m]: one warp per element, eight
// elements of one plan per item (the plan's l2p_near_kernel for one column), over the items of
// the switched-on plans (y of the others is zeroed before)
__global__ void scene_l2p_kernel(const BodyDev *__restrict__ bodies, const int2 *__restrict__ items,
                                 const int *__restrict__ nitems, const double2 *__restrict__ x,
                                 const float2 *__restrict__ x32, double2 *__restrict__ y)
{
    const int n = *nitems;
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        const int2 it = items[w];
        const BodyDev &bd = bodies[it.x];
        const int e = it.y + (threadIdx.x >> 5);
        if (e < bd.nf) l2p_element(bd, e, x, x32, y);
    }
}


// out[plan * nvec + j] += conj(V_j) . W over the chunk's range (grid: x = chunk, y = j); the
// chunks of switched-off plans (whose W is zero) are skipped
__global__ void scene_dot_kernel(const double2 *V, size_t vj, const double2 *W, const int4 *chunks, int nvec,
                                 double2 *out, const int *__restrict__ active)
{
    const int4 c = chunks[blockIdx.x];
    if (!active[c.x]) return;
    const int j = blockIdx.y;
    const double2 *v = V + (size_t)j * vj;
    double ar = 0, ai = 0;
    for (int i = c.y + threadIdx.x; i < c.z; i += blockDim.x) {
        double2 a = v[i], b = W[i];
        ar += a.x * b.x + a.y * b.y;
        ai += a.x * b.y - a.y * b.x;
    }
    __shared__ double sr[256], si[256];
    sr[threadIdx.x] = ar;
    si[threadIdx.x] = ai;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) { sr[threadIdx.x] += sr[threadIdx.x + s]; si[threadIdx.x] += si[threadIdx.x + s]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(&out[(size_t)c.x * nvec + j].x, sr[0]);
        atomicAdd(&out[(size_t)c.x * nvec + j].y, si[0]);
    }
}

// W -= sum_{j < nvec} V_j h[plan * nvec + j] over the chunk's range (only for switched-on plans
// where active is given)
__global__ void scene_sub_kernel(const double2 *V, size_t vj, int nvec, const double2 *h, double2 *W, const int4 *chunks,
                                 const int *__restrict__ active)
{
    const int4 c = chunks[blockIdx.x];
    if (active && !active[c.x]) return;
    const double2 *hc = h + (size_t)c.x * nvec;
    for (int i = c.y + threadIdx.x; i < c.z; i += blockDim.x) {
        double2 acc = W[i];
        for (int j = 0; j < nvec; j++) {
            double2 a = V[(size_t)j * vj + i], b = hc[j];
            acc.x -= a.x * b.x - a.y * b.y;
            acc.y -= a.x * b.y + a.y * b.x;
        }
        W[i] = acc;
    }
}

// Y = alpha[plan] X over the chunk's range
__global__ void scene_scale_kernel(const double *alpha, const double2 *X, double2 *Y, const int4 *chunks)
{
    const int4 c = chunks[blockIdx.x];
    const double a = alpha[c.x];
    for (int i = c.y + threadIdx.x; i < c.z; i += blockDim.x) {
        double2 v = X[i];
        Y[i] = make_double2(a * v.x, a * v.y);
    }
}

// ------------------------------------------------------------------------------ build
static void free_scene(Scene *S)
{
    if (!S) return;
    if (S->graph) cudaGraphExecDestroy(S->graph);
    for (void *p : S->allocs) cudaFree(p);
    for (double2 **q : {&S->V, &S->r, &S->w, &S->b, &S->x, &S->d, &S->dev_h}) cudaFree(*q);
    cudaFree(S->alpha);
    for (cudaEvent_t e : S->events) cudaEventDestroy(e);
    for (int i = 0; i < SCENE_SIDE; i++)
        if (S->side[i]) cudaStreamDestroy(S->side[i]);
    if (S->stream) cudaStreamDestroy(S->stream);
    if (S->t0) cudaEventDestroy(S->t0);
    if (S->t1) cudaEventDestroy(S->t1);
    delete S;
}

static int build_scene(Scene *S)
{
    const int n = (int)S->plans.size();
    std::vector<BodyDev> bodies(n);
    std::vector<int2> p2m, l2p, zitems;
    std::vector<int> zowner, powner;
    std::vector<float2 *> zptr;
    std::vector<long long> zlen;
    std::vector<int4> chunks;
    int Lmax = 0;
    S->off.assign(n + 1, 0);
    for (int i = 0; i < n; i++) {
        Plan *P = S->plans[i];
        S->off[i + 1] = S->off[i] + P->nf;
        Lmax = std::max(Lmax, P->lmax);
        LevelDev &LL = P->lev[P->lmax];
        BodyDev &bd = bodies[i];
        bd.off = S->off[i];
        bd.nf = P->nf;
        bd.pl = LL.p;
        bd.k = P->opt.k;
        bd.a = make_double2(P->opt.a_re, P->opt.a_im);
        bd.leaf_beg = P->leaf_beg;
        bd.leaf_elem = P->leaf_elem;
        bd.elem_leaf = P->elem_leaf;
        bd.near_beg = P->near_beg;
        bd.near_col = P->near_col;
        bd.U = P->U32;
        bd.Rv = P->Rv32;
        bd.nearv = P->near32;
        bd.Cm = LL.Cm32;
        bd.Dl = LL.Dl32;
        for (int b = 0; b < LL.nb; b++) p2m.push_back(make_int2(i, b));
        for (int e = 0; e < P->nf; e += 8) l2p.push_back(make_int2(i, e));
        for (int l = P->lmin; l <= P->lmax; l++) {
            long long len = (long long)P->lev[l].nb * P->lev[l].p * P->lev[l].p;
            if (l < P->lmax) { zptr.push_back(P->lev[l].Cm32); zlen.push_back(len); zowner.push_back(i); }
            zptr.push_back(P->lev[l].Dl32);
            zlen.push_back(len);
            zowner.push_back(i);
        }
        for (long long a = S->off[i]; a < S->off[i + 1]; a += BLAS_CHUNK)
            chunks.push_back(make_int4(i, (int)a, (int)std::min<long long>(a + BLAS_CHUNK, S->off[i + 1]), 0));
    }
    S->N = S->off[n];
    if (S->N >= (1LL << 31)) { fmm_set_error("fmm_scene_create: %lld unknowns in all, more than 2^31 - 1", S->N); return FMM_ERR_ARG; }
    for (size_t s = 0; s < zptr.size(); s++)
        for (long long a = 0; a < zlen[s]; a += ZERO_CHUNK) zitems.push_back(make_int2((int)s, (int)a));
    // translation passes and their queues: phase q = 0..Lmax-3 M2M of level Lmax-q, then M2L,
    // then L2L of levels 3..Lmax
    std::vector<RcrPass> passes;
    struct Work { int pass; int4 item; double cost; };
    struct Key { int phase, tc, shc, bal, cls; };
    std::vector<Key> keys;
    std::vector<std::vector<Work>> work;
    std::vector<size_t> smem;
    // passes of one tile shape are grouped further by the CTAs per SM their shared memory
    // allows, so that a few high-order passes do not set the occupancy of all the others
    auto group_of = [&](int phase, int tc, int shc, int bal, int cls) {
        for (size_t g = 0; g < keys.size(); g++)
            if (keys[g].phase == phase && keys[g].tc == tc && keys[g].shc == shc && keys[g].bal == bal && keys[g].cls == cls)
                return (int)g;
        keys.push_back({phase, tc, shc, bal, cls});
        work.emplace_back();
        smem.push_back(0);
        return (int)keys.size() - 1;
    };
    const int n_up = std::max(Lmax - 2, 0), ph_m2l = n_up;
    std::vector<int4> items;
    for (int i = 0; i < n; i++) {
        Plan *P = S->plans[i];
        for (int l = P->lmin; l <= P->lmax; l++)
            for (int which = PASS_M2M; which <= PASS_L2L; which++) {
                RcrPass ps;
                RcrList *Lst = pass32_desc(P, l, which, 1, ps);
                if (!Lst || Lst->key_beg.empty() || Lst->key_beg.back() == 0) continue;
                ps.g_src = Lst->src;
                ps.g_dst = Lst->dst;
                int phase = which == PASS_M2M ? Lmax - l : which == PASS_M2L ? ph_m2l : ph_m2l + (l - 2);
                size_t sm = rcr_tile_smem(ps.p, Lst->tc, Lst->shc);
                int cls = sm <= 76 * 1024 ? 3 : sm <= 113 * 1024 ? 2 : 1;
                int g = group_of(phase, Lst->tc, Lst->shc, Lst->bal, cls);
                smem[g] = std::max(smem[g], sm);
                int pi = (int)passes.size();
                passes.push_back(ps);
                powner.push_back(i);
                rcr_list_items(*Lst, items);
                double pc = (double)ps.p * ps.p * ps.p;
                for (const int4 &it : items) work[g].push_back({pi, it, pc * it.z});
            }
    }
    {
        int st;
        if ((st = upload(S, &S->bodies, bodies))) return st;
        if ((st = upload(S, &S->passes, passes))) return st;
        if ((st = upload(S, &S->p2m_all, p2m))) return st;
        if ((st = upload(S, &S->l2p_all, l2p))) return st;
        FMM_CUDA_TRY(salloc(S, &S->p2m_items, sizeof(int2) * p2m.size()));
        FMM_CUDA_TRY(salloc(S, &S->l2p_items, sizeof(int2) * l2p.size()));
        if ((st = upload(S, &S->zero_ptr, zptr))) return st;
        if ((st = upload(S, &S->zero_len, zlen))) return st;
        if ((st = upload(S, &S->zero_items, zitems))) return st;
        if ((st = upload(S, &S->zero_owner, zowner))) return st;
        S->active_host.assign(n, 1);
        if ((st = upload(S, &S->active, S->active_host))) return st;
        if ((st = upload(S, &S->chunks, chunks))) return st;
    }
    S->n_p2m = (int)p2m.size();
    S->n_l2p = (int)l2p.size();
    S->n_zero = (int)zitems.size();
    S->n_chunks = (int)chunks.size();
    S->n_heads = (int)keys.size();
    FMM_CUDA_TRY(salloc(S, &S->heads, sizeof(int) * std::max(S->n_heads, 1)));
    int nphase = ph_m2l + 1 + n_up;
    S->phases.assign(nphase, {});
    const int ng = (int)keys.size();
    S->n_jobs = ng + 2;
    FMM_CUDA_TRY(salloc(S, &S->counts, sizeof(int) * S->n_jobs));
    std::vector<CompactJob> jobs(S->n_jobs);
    for (size_t g = 0; g < keys.size(); g++) {
        std::vector<Work> &W = work[g];
        std::stable_sort(W.begin(), W.end(), [](const Work &a, const Work &b) { return a.cost > b.cost; });
        std::vector<int> wp(W.size());
        std::vector<int4> wi(W.size());
        for (size_t q = 0; q < W.size(); q++) {
            wp[q] = W[q].pass;
            wi[q] = W[q].item;
        }
        QueueGroup G;
        G.tc = keys[g].tc;
        G.shc = keys[g].shc;
        G.bal = keys[g].bal;
        G.nwork = (int)W.size();
        G.head = (int)g;
        G.smem = smem[g];
        int st;
        if ((st = rcr_queue_prepare(G.tc, G.shc, G.bal, G.smem, G.nwork, &G.grid))) return st;
        std::vector<int> own(W.size());
        for (size_t q = 0; q < W.size(); q++) own[q] = powner[wp[q]];
        int *wp_all = nullptr, *own_d = nullptr;
        int4 *wi_all = nullptr;
        if ((st = upload(S, &wp_all, wp))) return st;
        if ((st = upload(S, &wi_all, wi))) return st;
        if ((st = upload(S, &own_d, own))) return st;
        FMM_CUDA_TRY(salloc(S, &G.work_pass, sizeof(int) * wp.size()));
        FMM_CUDA_TRY(salloc(S, &G.work_item, sizeof(int4) * wi.size()));
        jobs[g] = CompactJob{G.nwork, 1, 4, own_d, wp_all, (const int *)wi_all, G.work_pass, (int *)G.work_item, S->counts + g};
        S->phases[keys[g].phase].push_back(G);
    }
    {
        std::vector<int> own_p(p2m.size()), own_l(l2p.size());
        for (size_t q = 0; q < p2m.size(); q++) own_p[q] = p2m[q].x;
        for (size_t q = 0; q < l2p.size(); q++) own_l[q] = l2p[q].x;
        int *op = nullptr, *ol = nullptr, st;
        if ((st = upload(S, &op, own_p))) return st;
        if ((st = upload(S, &ol, own_l))) return st;
        jobs[ng] = CompactJob{(int)p2m.size(), 2, 0, op, (const int *)S->p2m_all, nullptr, (int *)S->p2m_items, nullptr,
                              S->counts + ng};
        jobs[ng + 1] = CompactJob{(int)l2p.size(), 2, 0, ol, (const int *)S->l2p_all, nullptr, (int *)S->l2p_items, nullptr,
                                  S->counts + ng + 1};
        if ((st = upload(S, &S->jobs, jobs))) return st;
    }
    FMM_CUDA_TRY(salloc(S, &S->xin, sizeof(double2) * S->N));
    FMM_CUDA_TRY(salloc(S, &S->xin32, sizeof(float2) * S->N));
    FMM_CUDA_TRY(salloc(S, &S->yout, sizeof(double2) * S->N));
    S->events.resize(2 * nphase * SCENE_SIDE + 2 * n + 2);
    for (cudaEvent_t &e : S->events) FMM_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    FMM_CUDA_TRY(cudaEventCreate(&S->t0));
    FMM_CUDA_TRY(cudaEventCreate(&S->t1));
    return FMM_OK;
}

// ------------------------------------------------------------------------------ matvec
static int scene_translate(Scene *S)
{
    cudaStream_t st = S->stream;
    scene_zero_kernel<<<std::max(S->n_zero, 1), 256, 0, st>>>(S->zero_ptr, S->zero_len, S->zero_owner, S->zero_items,
                                                             S->n_zero, S->heads, S->n_heads, S->active);
    FMM_CUDA_TRY(cudaGetLastError());
    // the work of the switched-on plans only, in the same order; y = 0 for the others
    scene_compact_kernel<<<S->n_jobs, 1024, 0, st>>>(S->jobs, S->active);
    FMM_CUDA_TRY(cudaGetLastError());
    FMM_CUDA_TRY(cudaMemsetAsync(S->yout, 0, sizeof(double2) * S->N, st));
    const int ng = S->n_jobs - 2;
    if (S->n_p2m)
        scene_p2m_kernel<<<std::min(S->n_p2m, 152 * 16), 128, 0, st>>>(S->bodies, S->p2m_items, S->counts + ng, S->xin,
                                                                      S->xin32);
    FMM_CUDA_TRY(cudaGetLastError());
    int ev = 0;
    for (auto &groups : S->phases) {
        if (groups.empty()) continue;
        if (groups.size() == 1) {
            const QueueGroup &G = groups[0];
            int e = launch_rcr_queue(G.tc, G.shc, G.bal, S->passes, G.work_pass, G.work_item, S->counts + G.head,
                                     S->heads + G.head, G.smem, G.grid, st);
            if (e) return e;
            continue;
        }
        // the tile shapes of a phase run side by side
        cudaEvent_t fork = S->events[ev++];
        FMM_CUDA_TRY(cudaEventRecord(fork, st));
        int ns = std::min((int)groups.size(), SCENE_SIDE);
        for (int q = 0; q < ns; q++) FMM_CUDA_TRY(cudaStreamWaitEvent(S->side[q], fork, 0));
        for (size_t g = 0; g < groups.size(); g++) {
            const QueueGroup &G = groups[g];
            int e = launch_rcr_queue(G.tc, G.shc, G.bal, S->passes, G.work_pass, G.work_item, S->counts + G.head,
                                     S->heads + G.head, G.smem, G.grid, S->side[g % SCENE_SIDE]);
            if (e) return e;
        }
        for (int q = 0; q < ns; q++) {
            cudaEvent_t join = S->events[ev++];
            FMM_CUDA_TRY(cudaEventRecord(join, S->side[q]));
            FMM_CUDA_TRY(cudaStreamWaitEvent(st, join, 0));
        }
    }
    if (S->n_l2p)
        scene_l2p_kernel<<<std::min(S->n_l2p, 152 * 8), 256, 0, st>>>(S->bodies, S->l2p_items, S->counts + ng + 1, S->xin,
                                                                      S->xin32, S->yout);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

// The mixed matvec of every plan on xin -> yout: directly on the first call, captured as a
// graph on the second, replayed after that.
static int scene_mixed(Scene *S)
{
    if (S->graph) {
        FMM_CUDA_TRY(cudaGraphLaunch(S->graph, S->stream));
        return FMM_OK;
    }
    if (S->calls++ == 0) return scene_translate(S);
    cudaGraph_t g = nullptr;
    FMM_CUDA_TRY(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
    int e = scene_translate(S);
    cudaError_t ce = cudaStreamEndCapture(S->stream, &g);
    if (e) {
        if (g) cudaGraphDestroy(g);
        return e;
    }
    if (ce != cudaSuccess) {
        fmm_set_error("capturing the scene matvec: %s", cudaGetErrorString(ce));
        return FMM_ERR_CUDA;
    }
    ce = cudaGraphInstantiate(&S->graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
        S->graph = nullptr;
        fmm_set_error("instantiating the scene graph: %s", cudaGetErrorString(ce));
        return FMM_ERR_CUDA;
    }
    FMM_CUDA_TRY(cudaGraphLaunch(S->graph, S->stream));
    return FMM_OK;
}

// y = A x for every plan (device vectors of N entries) on the scene's stream.  FMM_MIXED: the
// lockstep launches above; FMM_FP64: each plan's own FP64 matvec on its own stream, forked
// from and joined back to the scene's stream.
static int scene_matvec_dev(Scene *S, const double2 *x, double2 *y, int precision)
{
    cudaStream_t st = S->stream;
    const int n = (int)S->plans.size();
    if (precision == FMM_MIXED) {
        // the scene's descriptors hold the plans' FP32 expansion addresses
        for (int i = 0; i < n; i++)
            if (S->plans[i]->buf_gen != S->buf_gen[i]) {
                fmm_set_error("scene: plan %d's expansion buffers were reallocated (a mixed matvec with more right-hand "
                              "sides) after fmm_scene_create; create the scene again", i);
                return FMM_ERR_ARG;
            }
        if (x != S->xin) FMM_CUDA_TRY(cudaMemcpyAsync(S->xin, x, sizeof(double2) * S->N, cudaMemcpyDeviceToDevice, st));
        int e = scene_mixed(S);
        if (e) return e;
        if (y != S->yout) FMM_CUDA_TRY(cudaMemcpyAsync(y, S->yout, sizeof(double2) * S->N, cudaMemcpyDeviceToDevice, st));
        return FMM_OK;
    }
    cudaEvent_t fork = S->events[S->events.size() - 1];
    FMM_CUDA_TRY(cudaEventRecord(fork, st));
    for (int i = 0; i < n; i++) {
        Plan *P = S->plans[i];
        if (!S->active_host[i]) {
            FMM_CUDA_TRY(cudaMemsetAsync(y + S->off[i], 0, sizeof(double2) * P->nf, st));
            continue;
        }
        FMM_CUDA_TRY(cudaStreamWaitEvent(P->stream, fork, 0));
        int e = run_matvec(P, x + S->off[i], y + S->off[i], precision == FMM_FLOAT2 ? FMM_FLOAT2 : FMM_FP64, 0, 1);
        if (e) return e;
        cudaEvent_t join = S->events[S->events.size() - 2 - i];
        FMM_CUDA_TRY(cudaEventRecord(join, P->stream));
        FMM_CUDA_TRY(cudaStreamWaitEvent(st, join, 0));
    }
    return FMM_OK;
}

// Adds the device time of the last timed matvec once its events have completed.
static void scene_read_timer(Scene *S)
{
    if (S->pending < 0) return;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, S->t0, S->t1) == cudaSuccess) S->ms[S->pending] += ms;
    else cudaGetLastError();
    S->pending = -1;
}

static int scene_matvec_timed(Scene *S, const double2 *x, double2 *y, int precision)
{
    scene_read_timer(S);
    FMM_CUDA_TRY(cudaEventRecord(S->t0, S->stream));
    int e = scene_matvec_dev(S, x, y, precision);
    if (e) return e;
    FMM_CUDA_TRY(cudaEventRecord(S->t1, S->stream));
    S->pending = precision == FMM_MIXED ? 1 : 0;
    S->calls_by_prec[S->pending]++;
    return FMM_OK;
}

// Which plans the next matvecs apply (the others give y = 0).
static int scene_set_active(Scene *S, const std::vector<int> &on)
{
    if (on == S->active_host) return FMM_OK;
    S->active_host = on;
    FMM_CUDA_TRY(cudaMemcpyAsync(S->active, S->active_host.data(), sizeof(int) * on.size(), cudaMemcpyHostToDevice,
                                 S->stream));
    return FMM_OK;
}

// ------------------------------------------------------------------------------ solver
// The bodies of a scene as the columns of gmres_core / solve_core: column i is the range
// [off[i], off[i+1]) of one vector of N entries; Krylov vector j at V + j N.
struct SceneOps {
    Scene *S;
    double2 *V(int j) { return S->V + (size_t)j * S->N; }
    double2 *r() { return S->r; }
    double2 *w() { return S->w; }
    double2 *b() { return S->b; }
    double2 *x() { return S->x; }
    double2 *d() { return S->d; }
    int nb() const { return (int)S->plans.size(); }
    int matvec(const double2 *x, double2 *y, int precision) { return status ? status : scene_matvec_timed(S, x, y, precision); }
    void axpby(double a, const double2 *x, double b, double2 *y) { launch_axpby(a, x, b, y, S->N, S->stream); }
    int dots_into(const double2 *Vb, size_t vj, const double2 *W, int nvec, std::vector<double2> &out)
    {
        FMM_CUDA_TRY(cudaMemsetAsync(S->dev_h, 0, sizeof(double2) * (size_t)nb() * nvec, S->stream));
        scene_dot_kernel<<<dim3(S->n_chunks, nvec), 256, 0, S->stream>>>(Vb, vj, W, S->chunks, nvec, S->dev_h, S->active);
        FMM_CUDA_TRY(cudaGetLastError());
        out.resize((size_t)nb() * nvec);
        FMM_CUDA_TRY(cudaMemcpyAsync(out.data(), S->dev_h, sizeof(double2) * out.size(), cudaMemcpyDeviceToHost, S->stream));
        FMM_CUDA_TRY(cudaStreamSynchronize(S->stream));
        return FMM_OK;
    }
    int norms(const double2 *W, std::vector<double> &out)
    {
        std::vector<double2> h;
        int st = dots_into(W, 0, W, 1, h);
        if (st) return st;
        out.resize(nb());
        for (int r = 0; r < nb(); r++) out[r] = sqrt(std::max(0.0, h[r].x));
        return FMM_OK;
    }
    int scale(const std::vector<double> &alpha, const double2 *X, double2 *Y)
    {
        FMM_CUDA_TRY(cudaMemcpyAsync(S->alpha, alpha.data(), sizeof(double) * nb(), cudaMemcpyHostToDevice, S->stream));
        scene_scale_kernel<<<S->n_chunks, 256, 0, S->stream>>>(S->alpha, X, Y, S->chunks);
        FMM_CUDA_TRY(cudaGetLastError());
        return FMM_OK;
    }
    int dots(int nvec, const double2 *W, std::vector<double2> &out) { return dots_into(S->V, S->N, W, nvec, out); }
    void sub_dots(int nvec, double2 *W)
    {
        scene_sub_kernel<<<S->n_chunks, 256, 0, S->stream>>>(S->V, S->N, nvec, S->dev_h, W, S->chunks, S->active);
    }
    int add_basis(std::vector<double2> &y, int kmax, double2 *X)
    {
        for (auto &v : y) v = make_double2(-v.x, -v.y); // the kernel subtracts
        FMM_CUDA_TRY(cudaMemcpyAsync(S->dev_h, y.data(), sizeof(double2) * y.size(), cudaMemcpyHostToDevice, S->stream));
        // every column: one that converged during this cycle still takes its update
        scene_sub_kernel<<<S->n_chunks, 256, 0, S->stream>>>(S->V, S->N, kmax, S->dev_h, X, S->chunks, nullptr);
        FMM_CUDA_TRY(cudaGetLastError());
        return FMM_OK;
    }
    int copy(double2 *dst, const double2 *src)
    {
        FMM_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double2) * S->N, cudaMemcpyDeviceToDevice, S->stream));
        return FMM_OK;
    }
    int zero(double2 *dst)
    {
        FMM_CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(double2) * S->N, S->stream));
        return FMM_OK;
    }
    double2 *tmp_alloc()
    {
        double2 *t = nullptr;
        cudaError_t e = cudaMallocAsync(&t, sizeof(double2) * S->N, S->stream);
        if (e != cudaSuccess) { fmm_set_error("scene solver workspace: %s", cudaGetErrorString(e)); return nullptr; }
        return t;
    }
    void tmp_free(double2 *t) { cudaFreeAsync(t, S->stream); }
    int sync()
    {
        FMM_CUDA_TRY(cudaStreamSynchronize(S->stream));
        return FMM_OK;
    }
    void active(const std::vector<int> &on) { status = status ? status : scene_set_active(S, on); }
    int status = FMM_OK;
};

static int ensure_scene_solver(Scene *S, int restart)
{
    if (S->restart_cap >= restart) return FMM_OK;
    for (double2 **q : {&S->V, &S->r, &S->w, &S->b, &S->x, &S->d, &S->dev_h}) {
        cudaFree(*q);
        *q = nullptr;
    }
    cudaFree(S->alpha);
    S->alpha = nullptr;
    S->restart_cap = 0;
    const size_t N = S->N, nb = S->plans.size();
    FMM_CUDA_TRY(cudaMalloc(&S->V, sizeof(double2) * N * (restart + 1)));
    for (double2 **q : {&S->r, &S->w, &S->b, &S->x, &S->d}) FMM_CUDA_TRY(cudaMalloc(q, sizeof(double2) * N));
    FMM_CUDA_TRY(cudaMalloc(&S->dev_h, sizeof(double2) * nb * (restart + 1)));
    FMM_CUDA_TRY(cudaMalloc(&S->alpha, sizeof(double) * nb));
    S->restart_cap = restart;
    return FMM_OK;
}

static bool is_dev(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

} // namespace fmm

using namespace fmm;

extern "C" int fmm_scene_create(fmm_plan *const *plans, int n, fmm_scene **scene)
{
    if (!plans || n < 1 || !scene) { fmm_set_error("fmm_scene_create: invalid argument"); return FMM_ERR_ARG; }
    *scene = nullptr;
    for (int i = 0; i < n; i++) {
        Plan *P = (Plan *)plans[i];
        if (!P) { fmm_set_error("fmm_scene_create: plan %d is null", i); return FMM_ERR_ARG; }
        if (!P->opt.build_mixed || !P->U32) {
            fmm_set_error("fmm_scene_create: plan %d has no mixed-precision tables (%s)", i, P->mixed_note);
            return FMM_ERR_ARG;
        }
        if (P->opt.device != ((Plan *)plans[0])->opt.device) {
            fmm_set_error("fmm_scene_create: plan %d is on device %d, plan 0 on %d", i, P->opt.device,
                          ((Plan *)plans[0])->opt.device);
            return FMM_ERR_ARG;
        }
        for (int j = 0; j < i; j++)
            if (plans[j] == plans[i]) { fmm_set_error("fmm_scene_create: plan %d appears twice", i); return FMM_ERR_ARG; }
    }
    Scene *S = new Scene();
    S->plans.assign((Plan *const *)plans, (Plan *const *)plans + n);
    S->device = S->plans[0]->opt.device;
    for (Plan *P : S->plans) S->buf_gen.push_back(P->buf_gen);
    int st = FMM_OK;
    if (cudaSetDevice(S->device) != cudaSuccess || cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) != cudaSuccess) {
        fmm_set_error("fmm_scene_create: %s", cudaGetErrorString(cudaGetLastError()));
        st = FMM_ERR_CUDA;
    }
    for (int i = 0; i < SCENE_SIDE && st == FMM_OK; i++)
        if (cudaStreamCreateWithFlags(&S->side[i], cudaStreamNonBlocking) != cudaSuccess) {
            fmm_set_error("fmm_scene_create: %s", cudaGetErrorString(cudaGetLastError()));
            st = FMM_ERR_CUDA;
        }
    if (st == FMM_OK) st = build_scene(S);
    if (st == FMM_OK && cudaDeviceSynchronize() != cudaSuccess) {
        fmm_set_error("fmm_scene_create: %s", cudaGetErrorString(cudaGetLastError()));
        st = FMM_ERR_CUDA;
    }
    if (st) { free_scene(S); return st; }
    for (Plan *P : S->plans) P->scene_refs++;
    *scene = (fmm_scene *)S;
    return FMM_OK;
}

extern "C" int fmm_scene_destroy(fmm_scene *scene)
{
    Scene *S = (Scene *)scene;
    if (S) {
        cudaSetDevice(S->device);
        for (Plan *P : S->plans) P->scene_refs--;
    }
    free_scene(S);
    return FMM_OK;
}

extern "C" int fmm_scene_unknowns(const fmm_scene *scene, long long *n, long long *offsets)
{
    const Scene *S = (const Scene *)scene;
    if (!S || !n) { fmm_set_error("fmm_scene_unknowns: null argument"); return FMM_ERR_ARG; }
    *n = S->N;
    if (offsets) memcpy(offsets, S->off.data(), sizeof(long long) * S->off.size());
    return FMM_OK;
}

extern "C" int fmm_scene_timings(const fmm_scene *scene, double *solve_s, double *mixed_ms, int *mixed_calls,
                                 double *fp64_ms, int *fp64_calls)
{
    const Scene *S = (const Scene *)scene;
    if (!S) { fmm_set_error("fmm_scene_timings: null scene"); return FMM_ERR_ARG; }
    if (solve_s) *solve_s = S->solve_s;
    if (mixed_ms) *mixed_ms = S->ms[1];
    if (mixed_calls) *mixed_calls = S->calls_by_prec[1];
    if (fp64_ms) *fp64_ms = S->ms[0];
    if (fp64_calls) *fp64_calls = S->calls_by_prec[0];
    return FMM_OK;
}

extern "C" int fmm_scene_set_active(fmm_scene *scene, const int *on)
{
    Scene *S = (Scene *)scene;
    if (!S) { fmm_set_error("fmm_scene_set_active: null scene"); return FMM_ERR_ARG; }
    S->user_active.clear();
    if (on)
        for (size_t i = 0; i < S->plans.size(); i++) S->user_active.push_back(on[i] ? 1 : 0);
    return FMM_OK;
}

extern "C" int fmm_scene_matvec(fmm_scene *scene, const cuDoubleComplex *x, cuDoubleComplex *y, int precision)
{
    Scene *S = (Scene *)scene;
    if (!S || !x || !y) { fmm_set_error("fmm_scene_matvec: null argument"); return FMM_ERR_ARG; }
    if (precision != FMM_FP64 && precision != FMM_MIXED && precision != FMM_FLOAT2) {
        fmm_set_error("unknown precision");
        return FMM_ERR_ARG;
    }
    FMM_CUDA_TRY(cudaSetDevice(S->device));
    bool xd = is_dev(x), yd = is_dev(y);
    const size_t bytes = sizeof(double2) * S->N;
    const double2 *xs = (const double2 *)x;
    double2 *ys = yd ? (double2 *)y : S->yout;
    if (!xd) {
        FMM_CUDA_TRY(cudaMemcpyAsync(S->xin, x, bytes, cudaMemcpyHostToDevice, S->stream));
        xs = S->xin;
    }
    int st = scene_set_active(S, S->user_active.empty() ? std::vector<int>(S->plans.size(), 1) : S->user_active);
    if (st) return st;
    st = scene_matvec_dev(S, xs, ys, precision);
    if (st) return st;
    if (!yd) FMM_CUDA_TRY(cudaMemcpyAsync(y, S->yout, bytes, cudaMemcpyDeviceToHost, S->stream));
    FMM_CUDA_TRY(cudaStreamSynchronize(S->stream));
    return FMM_OK;
}

extern "C" int fmm_scene_solve(fmm_scene *scene, const cuDoubleComplex *b, cuDoubleComplex *x, double tol, int maxit,
                               int restart, int precision, int *iters, double *relres)
{
    Scene *S = (Scene *)scene;
    if (!S || !b || !x || !(tol > 0) || maxit < 1 || restart < 1 || restart > 500) {
        fmm_set_error("fmm_scene_solve: invalid argument");
        return FMM_ERR_ARG;
    }
    if (precision != FMM_FP64 && precision != FMM_MIXED && precision != FMM_FLOAT2) {
        fmm_set_error("unknown precision");
        return FMM_ERR_ARG;
    }
    FMM_CUDA_TRY(cudaSetDevice(S->device));
    int st = ensure_scene_solver(S, restart);
    if (st) return st;
    const int n = (int)S->plans.size();
    const size_t bytes = sizeof(double2) * S->N;
    bool bd = is_dev(b), xd = is_dev(x);
    FMM_CUDA_TRY(cudaMemcpyAsync(S->b, b, bytes, bd ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, S->stream));
    FMM_CUDA_TRY(cudaMemcpyAsync(S->x, x, bytes, xd ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, S->stream));
    // norms of b and x at the start cover every plan
    if ((st = scene_set_active(S, std::vector<int>(n, 1)))) return st;
    SceneOps o{S};
    std::vector<int> it;
    std::vector<double> rr;
    S->ms[0] = S->ms[1] = 0.0;
    S->calls_by_prec[0] = S->calls_by_prec[1] = 0;
    S->pending = -1;
    auto w0 = std::chrono::steady_clock::now();
    if ((st = solve_core(o, n, tol, maxit, restart, precision, it, rr))) return st;
    if (o.status) return o.status;
    FMM_CUDA_TRY(cudaStreamSynchronize(S->stream));
    scene_read_timer(S);
    S->solve_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
    FMM_CUDA_TRY(cudaMemcpyAsync(x, S->x, bytes, xd ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, S->stream));
    FMM_CUDA_TRY(cudaStreamSynchronize(S->stream));
    bool ok = true;
    for (int r = 0; r < n; r++) {
        if (iters) iters[r] = it[r];
        if (relres) relres[r] = rr[r];
        ok = ok && rr[r] <= tol;
    }
    if (!ok) fmm_set_error("fmm_scene_solve: not every body reached tol %g", tol);
    return ok ? FMM_OK : FMM_ERR_NOT_CONVERGED;
}
