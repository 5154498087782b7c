// Plan creation, the public C ABI, and the GMRES / iterative-refinement solver.
#include "plan.h"
#include "gmres_core.h"
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <atomic>
#include <mutex>
#include <thread>

namespace fmm {
int set_dir_dist(const int *dd, const int *hrep);
}

using namespace fmm;

static thread_local char g_err[512] = "";

void fmm_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

extern "C" const char *fmm_last_error(void) { return g_err; }

namespace fmm {
// Kernels' dynamic shared-memory limits are process-wide while plans run on several host
// threads (fmm_solve_many): raise a limit under one lock and never lower it, so that no
// thread's launch sees a limit below what it set.
static std::mutex g_smem_mutex;

int raise_smem_limit(const void *func, size_t bytes, size_t *cache)
{
    std::lock_guard<std::mutex> lock(g_smem_mutex);
    if (*cache >= bytes) return FMM_OK;
    cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) {
        fmm_set_error("raising a kernel's shared-memory limit to %zu bytes: %s", bytes, cudaGetErrorString(e));
        return FMM_ERR_CUDA;
    }
    *cache = bytes;
    return FMM_OK;
}

cudaError_t dev_alloc(Plan *P, void **ptr, size_t bytes)
{
    cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 1);
    if (e == cudaSuccess) P->device_bytes += bytes;
    return e;
}

// truncNum (octree.c:777-796)
static int trunc_num(double k, double eps, double sigma, double a)
{
    double p_lo = 1 - log(eps * pow(1 - 1.0 / sigma, 1.5)) / log(sigma);
    double t0 = k * a, t1 = pow(3 * log(1.0 / eps), 1.5) / 2;
    double p_hi = t0 + t1 * pow(t0, 1.0 / 3);
    return (int)ceil(pow(pow(p_lo, 4) + pow(p_hi, 4), 0.25));
}
} // namespace fmm

extern "C" void fmm_default_options(fmm_options *opt)
{
    memset(opt, 0, sizeof(*opt));
    opt->k = 1.0;
    opt->depth = 0;
    opt->s = 5;
    opt->eps = 0.05;
    opt->rule = FMM_RULE_GAUSS3;
    opt->b_re = 1.0;
    opt->build_mixed = 1;
    opt->device = 0;
}

static void free_plan(Plan *P)
{
    if (!P) return;
    auto F = [](void *p) { if (p) cudaFree(p); };
    for (int l = 0; l <= FMM_MAX_LEVEL + 1; l++) {
        LevelDev &L = P->lev[l];
        F(L.parent); F(L.octant); F(L.child_beg); F(L.child_list); F(L.sr_beg); F(L.sr_src); F(L.sr_dir);
        F(L.Cm64); F(L.Dl64); F(L.Csr_ff); F(L.Crr_ff); F(L.CrrL_ff); F(L.Cm_ff); F(L.Dl_ff); F(L.Cm32); F(L.Dl32); F(L.Csr64); F(L.Csr32); F(L.Crr64); F(L.Crr32); F(L.Crr32L);
        for (RcrList *R : {&L.m2l, &L.m2m, &L.l2l}) {
            F(R->items); F(R->src); F(R->dst);
            Tc3 &t = R->t3;
            F(t.opsR); F(t.opsC); F(t.blkR); F(t.blkC); F(t.t_dir); F(t.itR1); F(t.itC); F(t.itR2);
            F(t.listR); F(t.listC); F(t.W); F(t.Z);
            F(R->td.B); F(R->td.items); F(R->td.src); F(R->td.dst); F(R->td.dir);
        }
    }
    F(P->tc_err); F(P->tc_ones); F(P->hrep_dev); F(P->m2l_part64); F(P->Hall_ff); F(P->PHall_ff); F(P->dsc_leaf_dev);
    F(P->Hsr64); F(P->PHsr64); F(P->Hsr32); F(P->PHsr32);
    F(P->V_dev); F(P->F_dev); F(P->elem_leaf); F(P->leaf_beg); F(P->leaf_elem);
    F(P->U64); F(P->Rv64); F(P->U32); F(P->Rv32); F(P->near_beg); F(P->near_col); F(P->near64); F(P->near32);
    F(P->nearT_beg); F(P->nearT_col); F(P->nearT64); F(P->nearT32);
    F(P->xbuf); F(P->ybuf); F(P->x32);
    F(P->gm_V); F(P->gm_w); F(P->gm_r); F(P->gm_x); F(P->gm_b); F(P->gm_d); F(P->gm_dev_h); F(P->gm_part); F(P->gm_alpha);
    if (P->timers_created)
        for (int i = 0; i < MAX_TIMERS; i++) { cudaEventDestroy(P->timers[i].beg); cudaEventDestroy(P->timers[i].end); }
    if (P->timers_created) {
        cudaEventDestroy(P->total.beg); cudaEventDestroy(P->total.end);
        cudaEventDestroy(P->phase.beg); cudaEventDestroy(P->phase.end);
    }
    drop_graph(P);
    if (P->stream) cudaStreamDestroy(P->stream);
    for (int i = 0; i < NSIDE; i++) {
        if (P->side[i]) cudaStreamDestroy(P->side[i]);
        if (P->join_ev[i]) cudaEventDestroy(P->join_ev[i]);
    }
    if (P->fork_ev) cudaEventDestroy(P->fork_ev);
    for (cudaEvent_t &e : P->m2l_ev)
        if (e) cudaEventDestroy(e);
    delete P;
}

static int plan_create_impl(std::vector<double> &&V, std::vector<int> &&F, const fmm_options *opt, fmm_plan **out)
{
    auto t0 = std::chrono::steady_clock::now();
    if (!opt || !out) { fmm_set_error("null argument"); return FMM_ERR_ARG; }
    *out = nullptr;
    int nv = (int)(V.size() / 3), nf = (int)(F.size() / 3);
    if (nf < 2 || nv < 3) { fmm_set_error("mesh too small (%d vertices, %d triangles)", nv, nf); return FMM_ERR_ARG; }
    if (!(opt->k > 0.0)) { fmm_set_error("wavenumber must be positive"); return FMM_ERR_ARG; }
    if (opt->rule != FMM_RULE_GAUSS3 && opt->rule != FMM_RULE_DUNAVANT7) { fmm_set_error("unknown rule %d", opt->rule); return FMM_ERR_ARG; }
    if (!std::isfinite(opt->alpha_re) || !std::isfinite(opt->alpha_im)) { fmm_set_error("coupling alpha is not finite"); return FMM_ERR_ARG; }
    if (opt->depth < -1 || opt->depth > FMM_MAX_LEVEL) { fmm_set_error("depth %d out of range", opt->depth); return FMM_ERR_ARG; }
    for (int e = 0; e < nf; e++)
        for (int t = 0; t < 3; t++)
            if (F[3 * e + t] < 0 || F[3 * e + t] >= nv) { fmm_set_error("element %d has vertex index %d out of range", e, F[3 * e + t]); return FMM_ERR_MESH; }
    for (int e = 0; e < nf; e++) {
        const double *a = &V[3 * F[3 * e]], *b = &V[3 * F[3 * e + 1]], *c = &V[3 * F[3 * e + 2]];
        double u[3] = {a[0] - c[0], a[1] - c[1], a[2] - c[2]}, v[3] = {b[0] - c[0], b[1] - c[1], b[2] - c[2]};
        double n0 = u[1] * v[2] - u[2] * v[1], n1 = u[2] * v[0] - u[0] * v[2], n2 = u[0] * v[1] - u[1] * v[0];
        if (!(n0 * n0 + n1 * n1 + n2 * n2 > 0.0)) { fmm_set_error("element %d has zero area", e); return FMM_ERR_MESH; }
    }
    Plan *P = new Plan();
    P->opt = *opt;
    P->nv = nv;
    P->nf = nf;
    P->V = std::move(V);
    P->F = std::move(F);
#define TRY(x) do { int s_ = (x); if (s_ != FMM_OK) { free_plan(P); return s_; } } while (0)
#define CTRY(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { fmm_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_)); free_plan(P); return FMM_ERR_CUDA; } } while (0)
    CTRY(cudaSetDevice(opt->device));
    // a blocking stream during setup: setup code mixes kernels on this stream with
    // default-stream cudaMemcpy read-backs (list counts), which must wait for those kernels;
    // replaced by a non-blocking stream once the plan is built
    CTRY(cudaStreamCreate(&P->stream));
    for (int i = 0; i < NSIDE; i++) {
        CTRY(cudaStreamCreateWithFlags(&P->side[i], cudaStreamNonBlocking));
        CTRY(cudaEventCreateWithFlags(&P->join_ev[i], cudaEventDisableTiming));
    }
    CTRY(cudaEventCreateWithFlags(&P->fork_ev, cudaEventDisableTiming));
    for (cudaEvent_t &e : P->m2l_ev) CTRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (const char *ns = getenv("FMMBEM_M2L_STREAMS")) P->nside = std::max(1, std::min(NSIDE, atoi(ns)));
    if (build_tree(P->V, P->F, opt->s, opt->depth, P->tree) != 0 || P->tree.lmax > FMM_MAX_LEVEL) {
        fmm_set_error("octree build failed (lmax=%d)", P->tree.lmax);
        free_plan(P);
        return FMM_ERR_MESH;
    }
    if (opt->depth < 0 && opt->p_level[P->tree.lmax] <= 0) {
        // the element-size cap gives way where the leaf order would exceed 40 (meshes coarse
        // against the wavelength): one level deeper at a time, no deeper than the plain rule
        HostTree plain;
        int lref = build_tree(P->V, P->F, opt->s, 0, plain) == 0 ? plain.lmax : P->tree.lmax;
        while (P->tree.lmax < std::min(lref, FMM_MAX_LEVEL) &&
               trunc_num(opt->k, opt->eps > 0 ? opt->eps : 0.05, 1.5, ldexp(P->tree.d, -P->tree.lmax)) > 40) {
            int next = P->tree.lmax + 1;
            if (build_tree(P->V, P->F, opt->s, next, P->tree) != 0) {
                fmm_set_error("octree build failed (lmax=%d)", next);
                free_plan(P);
                return FMM_ERR_MESH;
            }
        }
    }
    P->lmin = P->tree.lmin;
    P->lmax = P->tree.lmax;
    P->pmax = 0;
    for (int l = P->lmin; l <= P->lmax; l++) {
        int p = opt->p_level[l] > 0 ? opt->p_level[l] : trunc_num(opt->k, opt->eps > 0 ? opt->eps : 0.05, 1.5, ldexp(P->tree.d, -l));
        if (p < 1 || p > 64) { fmm_set_error("truncation order %d at level %d out of range [1, 64]", p, l); free_plan(P); return FMM_ERR_ARG; }
        P->lev[l].p = p;
        P->lev[l].nb = (int)P->tree.sets[l].size();
        P->pmax = std::max(P->pmax, p);
    }
    P->pleaf = P->lev[P->lmax].p;
    if (P->opt.build_mixed && rcr_tile_smem(P->pmax, 4, 0) > MAX_TILE_SMEM) {
        // the batched FP32 translations keep two p^2 x 4 complex tiles in shared memory at least
        P->opt.build_mixed = 0;
        snprintf(P->mixed_note, sizeof(P->mixed_note),
                 "mixed precision needs truncation orders <= 60 (this plan has %d); use FMM_FP64", P->pmax);
    }
    if (P->pleaf > 40) { fmm_set_error("leaf truncation order %d above 40", P->pleaf); free_plan(P); return FMM_ERR_ARG; }
    CTRY(dev_alloc(P, (void **)&P->V_dev, sizeof(double) * P->V.size()));
    CTRY(dev_alloc(P, (void **)&P->F_dev, sizeof(int) * P->F.size()));
    CTRY(dev_alloc(P, (void **)&P->elem_leaf, sizeof(int) * nf));
    CTRY(cudaMemcpy(P->V_dev, P->V.data(), sizeof(double) * P->V.size(), cudaMemcpyHostToDevice));
    CTRY(cudaMemcpy(P->F_dev, P->F.data(), sizeof(int) * P->F.size(), cudaMemcpyHostToDevice));
    CTRY(cudaMemcpy(P->elem_leaf, P->tree.elem_leaf.data(), sizeof(int) * nf, cudaMemcpyHostToDevice));
    TRY(gen_rotation_tables(P));
    TRY(set_dir_dist(P->dir_dist, P->dir_hrep));
    CTRY(dev_alloc(P, (void **)&P->hrep_dev, sizeof(int) * NDIR));
    CTRY(cudaMemcpy(P->hrep_dev, P->dir_hrep, sizeof(int) * NDIR, cudaMemcpyHostToDevice));
    TRY(build_lists(P));
    TRY(gen_coax_tables(P));
    for (int l = P->lmin; l <= P->lmax; l++) {
        LevelDev &L = P->lev[l];
        size_t n = (size_t)L.nb * L.p * L.p;
        CTRY(dev_alloc(P, (void **)&L.Cm64, sizeof(double2) * n));
        CTRY(dev_alloc(P, (void **)&L.Dl64, sizeof(double2) * n));
        if (P->opt.build_mixed) {
            CTRY(dev_alloc(P, (void **)&L.Cm32, sizeof(float2) * n));
            CTRY(dev_alloc(P, (void **)&L.Dl32, sizeof(float2) * n));
        }
    }
    {
        // FP64 M2L of levels with few boxes: split each box's sources over up to 16 CTAs so
        // that the level has ~4 CTAs per SM (each run keeps >= 8 translations)
        int dev = 0, nsm = 152;
        CTRY(cudaGetDevice(&dev));
        CTRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        size_t part = 0;
        for (int l = P->lmin; l <= P->lmax; l++) {
            LevelDev &L = P->lev[l];
            long long target = 4LL * nsm, per_box = L.nb ? L.num_sr / L.nb : 0;
            int S = L.nb > 0 && L.nb < target ? (int)std::min<long long>(16, (target + L.nb - 1) / L.nb) : 1;
            S = (int)std::max<long long>(1, std::min<long long>(S, per_box / 8));
            L.m2l_split = S;
            if (S > 1) part = std::max(part, (size_t)S * L.nb * L.p * L.p);
        }
        if (part) CTRY(dev_alloc(P, (void **)&P->m2l_part64, sizeof(double2) * part));
    }
    TRY(gen_element_tables(P));
    TRY(gen_near_field(P));
    if (P->opt.build_mixed) {
        TRY(build_rcr_lists(P));
        TRY(tune_rcr_tiles(P));
        TRY(tune_tc_dense(P));
        TRY(tune_tc3(P));
    }
    CTRY(dev_alloc(P, (void **)&P->xbuf, sizeof(double2) * nf));
    CTRY(dev_alloc(P, (void **)&P->ybuf, sizeof(double2) * nf));
    P->nrhs_cap = 1;
    for (int i = 0; i < MAX_TIMERS; i++) {
        CTRY(cudaEventCreate(&P->timers[i].beg));
        CTRY(cudaEventCreate(&P->timers[i].end));
    }
    CTRY(cudaEventCreate(&P->total.beg));
    CTRY(cudaEventCreate(&P->total.end));
    CTRY(cudaEventCreate(&P->phase.beg));
    CTRY(cudaEventCreate(&P->phase.end));
    P->timers_created = 1;
    CTRY(cudaStreamSynchronize(P->stream));
    // From here on the plan's work (matvecs, solves, graph captures) runs on a non-blocking
    // stream: the legacy default stream, which other threads may use (another plan's setup,
    // cudaMemcpy), must never come to depend on a stream that is capturing a graph.
    {
        cudaStream_t s2 = nullptr;
        CTRY(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
        CTRY(cudaStreamDestroy(P->stream));
        P->stream = s2;
    }
    P->setup_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = (fmm_plan *)P;
#undef TRY
#undef CTRY
    return FMM_OK;
}

extern "C" int fmm_plan_create(const double *V, int nv, const int *F, int nf, const fmm_options *opt, fmm_plan **plan)
{
    if (!V || !F || nv <= 0 || nf <= 0) { fmm_set_error("empty mesh"); return FMM_ERR_ARG; }
    std::vector<double> Vv(V, V + 3 * (size_t)nv);
    std::vector<int> Fv(F, F + 3 * (size_t)nf);
    return plan_create_impl(std::move(Vv), std::move(Fv), opt, plan);
}

extern "C" int fmm_plan_create_obj(const char *path, const fmm_options *opt, fmm_plan **plan)
{
    std::vector<double> V;
    std::vector<int> F;
    if (!path || read_obj(path, V, F) != 0) { fmm_set_error("cannot read %s", path ? path : "(null)"); return FMM_ERR_IO; }
    return plan_create_impl(std::move(V), std::move(F), opt, plan);
}

extern "C" int fmm_plan_destroy(fmm_plan *plan)
{
    Plan *P = (Plan *)plan;
    if (P && P->scene_refs > 0) {
        fmm_set_error("fmm_plan_destroy: %d scene(s) still use this plan; destroy them first", P->scene_refs);
        return FMM_ERR_ARG;
    }
    free_plan(P);
    return FMM_OK;
}

extern "C" int fmm_plan_info(const fmm_plan *plan, fmm_info *info)
{
    if (!plan || !info) { fmm_set_error("null argument"); return FMM_ERR_ARG; }
    const Plan *P = (const Plan *)plan;
    memset(info, 0, sizeof(*info));
    info->num_elem = P->nf;
    info->num_vert = P->nv;
    info->lmin = P->lmin;
    info->lmax = P->lmax;
    info->d = P->tree.d;
    for (int a = 0; a < 3; a++) info->pt_min[a] = P->tree.pt_min[a];
    for (int l = P->lmin; l <= P->lmax; l++) {
        info->p_level[l] = P->lev[l].p;
        info->num_box[l] = P->lev[l].nb;
        info->num_m2l[l] = P->lev[l].num_sr;
        // the form a pass runs in: three-stage, else dense tensor-core, else SIMT tiles
        auto dense = [](const RcrList &R) { return R.td.on && !R.t3.on; };
        const LevelDev &L = P->lev[l];
        info->m2l_columns[l] = P->opt.build_mixed ? (dense(L.m2l) ? 128 : L.m2l.tc) : 0;
        info->m2l_tensor[l] = P->opt.build_mixed && dense(L.m2l) ? 1 : 0;
        info->pass_dense[l] =
            P->opt.build_mixed ? (dense(L.m2m) ? 1 : 0) | (dense(L.m2l) ? 2 : 0) | (dense(L.l2l) ? 4 : 0) : 0;
        if (P->opt.build_mixed) {
            info->pass_tc3[l] = (P->lev[l].m2m.t3.on ? 1 : 0) | (P->lev[l].m2l.t3.on ? 2 : 0) | (P->lev[l].l2l.t3.on ? 4 : 0);
            // SIMT tiles with the balanced schedule: neither tensor-core form, and bal set
            auto bal = [&](const RcrList &R) { return !R.t3.on && !dense(R) && R.bal; };
            info->pass_balanced[l] = (bal(L.m2m) ? 1 : 0) | (bal(L.m2l) ? 2 : 0) | (bal(L.l2l) ? 4 : 0);
        }
    }
    info->expansions_scaled = P->opt.build_mixed && P->scaled ? 1 : 0;
    info->num_near = P->num_near;
    info->device_bytes = P->device_bytes;
    info->setup_seconds = P->setup_seconds;
    return FMM_OK;
}

extern "C" int fmm_plan_lists(const fmm_plan *plan, int level, long long *boxes, int *m2l_beg, int *m2l_src,
                              int *m2l_dir)
{
    if (!plan) { fmm_set_error("null plan"); return FMM_ERR_ARG; }
    const Plan *P = (const Plan *)plan;
    if (level < P->lmin || level > P->lmax) {
        fmm_set_error("fmm_plan_lists: level %d outside %d..%d", level, P->lmin, P->lmax);
        return FMM_ERR_ARG;
    }
    const LevelDev &L = P->lev[level];
    if (boxes)
        for (int i = 0; i < L.nb; i++) boxes[i] = P->tree.sets[level][i];
    if (m2l_beg) FMM_CUDA_TRY(cudaMemcpy(m2l_beg, L.sr_beg, sizeof(int) * (L.nb + 1), cudaMemcpyDeviceToHost));
    if (m2l_src && L.num_sr)
        FMM_CUDA_TRY(cudaMemcpy(m2l_src, L.sr_src, sizeof(int) * L.num_sr, cudaMemcpyDeviceToHost));
    if (m2l_dir && L.num_sr) {
        std::vector<short> d(L.num_sr);
        FMM_CUDA_TRY(cudaMemcpy(d.data(), L.sr_dir, sizeof(short) * L.num_sr, cudaMemcpyDeviceToHost));
        for (long long i = 0; i < L.num_sr; i++) m2l_dir[i] = d[i];
    }
    return FMM_OK;
}

extern "C" int fmm_plan_direction(const fmm_plan *plan, int dir, int *offset)
{
    if (!plan || !offset || dir < 0 || dir >= NDIR) { fmm_set_error("fmm_plan_direction: invalid argument"); return FMM_ERR_ARG; }
    const Plan *P = (const Plan *)plan;
    for (int s = 0; s < 343; s++)
        if (P->dir_slot[s] == dir) {
            offset[0] = s / 49 - 3;
            offset[1] = (s / 7) % 7 - 3;
            offset[2] = s % 7 - 3;
            return FMM_OK;
        }
    fmm_set_error("fmm_plan_direction: direction %d not found", dir);
    return FMM_ERR_ARG;
}

extern "C" int fmm_plan_near_lists(const fmm_plan *plan, int *box_beg, int *box_idx, long long *num_box_pairs,
                                   int *elem_beg, int *elem_col, long long *num_elem_pairs)
{
    if (!plan) { fmm_set_error("null plan"); return FMM_ERR_ARG; }
    const Plan *P = (const Plan *)plan;
    if (num_box_pairs) *num_box_pairs = (long long)P->near_box.size();
    if (num_elem_pairs) *num_elem_pairs = P->num_near;
    if (box_beg) std::copy(P->near_box_beg.begin(), P->near_box_beg.end(), box_beg);
    if (box_idx) std::copy(P->near_box.begin(), P->near_box.end(), box_idx);
    if (elem_beg) FMM_CUDA_TRY(cudaMemcpy(elem_beg, P->near_beg, sizeof(int) * (P->nf + 1), cudaMemcpyDeviceToHost));
    if (elem_col && P->num_near)
        FMM_CUDA_TRY(cudaMemcpy(elem_col, P->near_col, sizeof(int) * P->num_near, cudaMemcpyDeviceToHost));
    return FMM_OK;
}

static bool is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Staging buffers for host inputs and outputs, ncols columns of nf.
static int ensure_io(Plan *P, int ncols)
{
    if (ncols <= P->nrhs_cap) return FMM_OK;
    cudaFree(P->xbuf);
    cudaFree(P->ybuf);
    P->xbuf = P->ybuf = nullptr;
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->xbuf, sizeof(double2) * (size_t)P->nf * ncols));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->ybuf, sizeof(double2) * (size_t)P->nf * ncols));
    P->nrhs_cap = ncols;
    return FMM_OK;
}

// y = A x, A^T x or A^H x for nrhs columns; host or device buffers.  The mixed path applies
// the operator to all columns in one batched pass.
static int apply_operator(Plan *P, const cuDoubleComplex *x, cuDoubleComplex *y, int nrhs, int precision, int transpose,
                          int conjugate)
{
    if (!P || !x || !y || nrhs < 1) { fmm_set_error("invalid argument"); return FMM_ERR_ARG; }
    if (precision != FMM_FP64 && precision != FMM_MIXED && precision != FMM_FLOAT2) {
        fmm_set_error("unknown precision %d", precision);
        return FMM_ERR_ARG;
    }
    if (transpose) {
        int st = build_transpose(P);
        if (st) return st;
    }
    bool xd = is_device_ptr(x), yd = is_device_ptr(y);
    size_t n = (size_t)P->nf * nrhs;
    if (!xd || !yd || conjugate) {
        int st = ensure_io(P, nrhs);
        if (st) return st;
    }
    const double2 *xin = (const double2 *)x;
    double2 *yout = yd ? (double2 *)y : P->ybuf;
    if (!xd) {
        FMM_CUDA_TRY(cudaMemcpyAsync(P->xbuf, x, sizeof(double2) * n, cudaMemcpyHostToDevice, P->stream));
        xin = P->xbuf;
    }
    if (conjugate) {
        launch_conj(P, xin, P->xbuf, n);
        xin = P->xbuf;
    }
    int st = run_matvec(P, xin, yout, precision, transpose, nrhs);
    if (st) return st;
    if (conjugate) launch_conj(P, yout, yout, n);
    FMM_CUDA_TRY(cudaGetLastError());
    if (!yd) FMM_CUDA_TRY(cudaMemcpyAsync(y, P->ybuf, sizeof(double2) * n, cudaMemcpyDeviceToHost, P->stream));
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    return precision == FMM_MIXED ? check_tc_error(P) : FMM_OK;
}

extern "C" int fmm_matvec(fmm_plan *plan, const cuDoubleComplex *x, cuDoubleComplex *y, int nrhs, int precision)
{
    return apply_operator((Plan *)plan, x, y, nrhs, precision, 0, 0);
}

// Transposed operator: the sources become point sources at the centroids (multipole
// R_n^{-m}(y_i - c)) and the targets element integrals (local expansion integrated against
// b R + c dR/dn), with the same translation tables; the near field is the transposed CSR.
// A^H x = conj(A^T conj(x)).
extern "C" int fmm_matvec_adjoint(fmm_plan *plan, const cuDoubleComplex *x, cuDoubleComplex *y, int nrhs, int precision,
                                  int conjugate)
{
    return apply_operator((Plan *)plan, x, y, nrhs, precision, 1, conjugate ? 1 : 0);
}

extern "C" int fmm_set_profiling(fmm_plan *plan, int on)
{
    if (!plan) return FMM_ERR_ARG;
    if (on < 0 || on > 2) { fmm_set_error("profiling mode %d not in 0..2", on); return FMM_ERR_ARG; }
    ((Plan *)plan)->profiling = on;
    return FMM_OK;
}

extern "C" int fmm_last_timings(const fmm_plan *plan, const char **names, double *ms, int *count)
{
    const Plan *P = (const Plan *)plan;
    if (!P || !count) return FMM_ERR_ARG;
    std::vector<std::pair<const Timer *, const char *>> all;
    for (int i = 0; i < P->ntimers; i++) all.push_back({&P->timers[i], P->timers[i].name});
    if (P->have_phase) all.push_back({&P->phase, "translations"});
    if (P->have_total) all.push_back({&P->total, "matvec"});
    int total = (int)all.size();
    int n = std::min(*count, total);
    for (int i = 0; i < n; i++) {
        float t = 0.f;
        cudaEventSynchronize(all[i].first->end);
        cudaEventElapsedTime(&t, all[i].first->beg, all[i].first->end);
        if (names) names[i] = all[i].second;
        if (ms) ms[i] = t;
    }
    *count = total;
    return FMM_OK;
}

// ---------------------------------------------------------------------------- batched BLAS-1
// Column r of a batch of R vectors of length n; V holds Krylov vectors as [j][r][n].
namespace fmm {
// part[(r * nvec + j) * gridDim.x + block] = block's share of conj(V_j,r) . W_r   (grid: x over
// n, y = j, z = r); bdot_sum_kernel adds the shares in block order, so that the dots (and
// the solves built on them) do not depend on the schedule
__global__ void bdot_kernel(const double2 *V, size_t vj, size_t vr, const double2 *W, size_t wr, int n, int nvec,
                            double2 *part)
{
    int j = blockIdx.y, r = blockIdx.z;
    const double2 *v = V + (size_t)j * vj + (size_t)r * vr, *w = W + (size_t)r * wr;
    double ar = 0, ai = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 a = v[i], b = w[i];
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
    if (threadIdx.x == 0) part[((size_t)r * nvec + j) * gridDim.x + blockIdx.x] = make_double2(sr[0], si[0]);
}

__global__ void bdot_sum_kernel(const double2 *part, int nb, int m, double2 *out)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < m; q += gridDim.x * blockDim.x) {
        double ar = 0, ai = 0;
        for (int b = 0; b < nb; b++) {
            const double2 v = part[(size_t)q * nb + b];
            ar += v.x;
            ai += v.y;
        }
        out[q] = make_double2(ar, ai);
    }
}

// W_r -= sum_{j < nvec} V_j,r h[r * hs + j]   (grid: x over n, z = r)
__global__ void baxpy_kernel(const double2 *V, size_t vj, size_t vr, int nvec, const double2 *h, int hs, double2 *W,
                             size_t wr, int n)
{
    int r = blockIdx.z;
    const double2 *v = V + (size_t)r * vr, *c = h + (size_t)r * hs;
    double2 *w = W + (size_t)r * wr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 acc = w[i];
        for (int j = 0; j < nvec; j++) {
            double2 a = v[(size_t)j * vj + i], b = c[j];
            acc.x -= a.x * b.x - a.y * b.y;
            acc.y -= a.x * b.y + a.y * b.x;
        }
        w[i] = acc;
    }
}

// Y_r = alpha[r] X_r   (alpha real per column; grid: x over n, z = r)
__global__ void bscale_kernel(const double *alpha, const double2 *X, size_t xr, double2 *Y, size_t yr, int n)
{
    int r = blockIdx.z;
    double a = alpha[r];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 v = X[(size_t)r * xr + i];
        Y[(size_t)r * yr + i] = make_double2(a * v.x, a * v.y);
    }
}

// y = alpha x + beta y over n entries (alpha, beta real)
__global__ void axpby_kernel(double alpha, const double2 *x, double beta, double2 *y, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double2 a = x[i], b = y[i];
        y[i] = make_double2(alpha * a.x + beta * b.x, alpha * a.y + beta * b.y);
    }
}
} // namespace fmm

static const int BLAS_BLOCKS = 152 * 2;

static unsigned blas_grid(size_t n) { return (unsigned)std::min<size_t>(BLAS_BLOCKS, (n + 255) / 256); }

// Workspace of the batched solver for R columns and restart m.
static int ensure_gmres(Plan *P, int restart, int R)
{
    if (P->gm_restart >= restart && P->gm_cols >= R) return FMM_OK;
    restart = std::max(restart, P->gm_restart);
    R = std::max(R, P->gm_cols);
    for (double2 **q : {&P->gm_V, &P->gm_w, &P->gm_r, &P->gm_x, &P->gm_b, &P->gm_d, &P->gm_dev_h}) {
        cudaFree(*q);
        *q = nullptr;
    }
    cudaFree(P->gm_alpha);
    P->gm_alpha = nullptr;
    size_t n = (size_t)P->nf * R;
    FMM_CUDA_TRY(cudaMalloc(&P->gm_V, sizeof(double2) * n * (restart + 1)));
    FMM_CUDA_TRY(cudaMalloc(&P->gm_w, sizeof(double2) * n));
    FMM_CUDA_TRY(cudaMalloc(&P->gm_r, sizeof(double2) * n));
    FMM_CUDA_TRY(cudaMalloc(&P->gm_x, sizeof(double2) * n));
    FMM_CUDA_TRY(cudaMalloc(&P->gm_b, sizeof(double2) * n));
    FMM_CUDA_TRY(cudaMalloc(&P->gm_d, sizeof(double2) * n));
    FMM_CUDA_TRY(cudaMalloc(&P->gm_dev_h, sizeof(double2) * (size_t)R * (restart + 1)));
    cudaFree(P->gm_part);
    P->gm_part = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&P->gm_part, sizeof(double2) * (size_t)R * (restart + 1) * (BLAS_BLOCKS / 2)));
    FMM_CUDA_TRY(cudaMalloc(&P->gm_alpha, sizeof(double) * R));
    P->gm_restart = restart;
    P->gm_cols = R;
    return FMM_OK;
}

// out[r * nvec + j] = <V_j,r, W_r> for the R columns, copied to the host
static int bdots(Plan *P, const double2 *V, size_t vj, size_t vr, const double2 *W, size_t wr, int nvec, int R,
                 std::vector<double2> &out)
{
    dim3 grid(std::min(BLAS_BLOCKS / 2, (P->nf + 255) / 256), nvec, R);
    bdot_kernel<<<grid, 256, 0, P->stream>>>(V, vj, vr, W, wr, P->nf, nvec, P->gm_part);
    const int m = R * nvec;
    bdot_sum_kernel<<<(m + 255) / 256, 256, 0, P->stream>>>(P->gm_part, (int)grid.x, m, P->gm_dev_h);
    out.resize((size_t)R * nvec);
    FMM_CUDA_TRY(cudaMemcpyAsync(out.data(), P->gm_dev_h, sizeof(double2) * out.size(), cudaMemcpyDeviceToHost, P->stream));
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    return FMM_OK;
}

static int bnorms(Plan *P, const double2 *W, int R, std::vector<double> &out)
{
    std::vector<double2> h;
    int st = bdots(P, W, 0, P->nf, W, P->nf, 1, R, h);
    if (st) return st;
    out.resize(R);
    for (int r = 0; r < R; r++) out[r] = sqrt(std::max(0.0, h[r].x));
    return FMM_OK;
}

static int bscale(Plan *P, const std::vector<double> &alpha, const double2 *X, double2 *Y, int R)
{
    FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_alpha, alpha.data(), sizeof(double) * R, cudaMemcpyHostToDevice, P->stream));
    bscale_kernel<<<dim3(blas_grid(P->nf) / 2 + 1, 1, R), 256, 0, P->stream>>>(P->gm_alpha, X, P->nf, Y, P->nf, P->nf);
    return FMM_OK;
}

static void axpby(Plan *P, double a, const double2 *x, double b, double2 *y, size_t n)
{
    axpby_kernel<<<blas_grid(n), 256, 0, P->stream>>>(a, x, b, y, n);
}

namespace fmm {
void launch_axpby(double a, const double2 *x, double b, double2 *y, size_t n, cudaStream_t st)
{
    axpby_kernel<<<blas_grid(n), 256, 0, st>>>(a, x, b, y, n);
}
} // namespace fmm

// The columns of one plan for gmres_core / solve_core: R right-hand sides of nf entries one
// after another, Krylov vector j of column r at V + j R nf + r nf; the operator or its
// transpose.
struct PlanOps {
    Plan *P;
    int R, transpose;
    std::vector<int> on;          // columns whose matvec results are used (empty: all)
    size_t vj() const { return (size_t)R * P->nf; }
    double2 *V(int j) { return P->gm_V + (size_t)j * vj(); }
    double2 *r() { return P->gm_r; }
    double2 *w() { return P->gm_w; }
    double2 *b() { return P->gm_b; }
    double2 *x() { return P->gm_x; }
    double2 *d() { return P->gm_d; }
    // The FP64 matvec runs column by column, so columns that are switched off are skipped
    // (y = 0 for them); the mixed pass applies all columns at once.
    int matvec(const double2 *x, double2 *y, int precision)
    {
        bool all = true;
        for (int v : on) all = all && v;
        if (precision == FMM_MIXED || on.empty() || all) return run_matvec(P, x, y, precision, transpose, R);
        for (int r = 0; r < R; r++) {
            const size_t o = (size_t)r * P->nf;
            if (on[r]) {
                int st = run_matvec(P, x + o, y + o, precision, transpose, 1);
                if (st) return st;
            } else {
                FMM_CUDA_TRY(cudaMemsetAsync(y + o, 0, sizeof(double2) * P->nf, P->stream));
            }
        }
        return FMM_OK;
    }
    void axpby(double a, const double2 *x, double b, double2 *y) { ::axpby(P, a, x, b, y, vj()); }
    int norms(const double2 *W, std::vector<double> &out) { return bnorms(P, W, R, out); }
    int scale(const std::vector<double> &alpha, const double2 *X, double2 *Y) { return bscale(P, alpha, X, Y, R); }
    int dots(int nvec, const double2 *W, std::vector<double2> &out)
    {
        return bdots(P, P->gm_V, vj(), P->nf, W, P->nf, nvec, R, out);
    }
    void sub_dots(int nvec, double2 *W)
    {
        baxpy_kernel<<<dim3(blas_grid(P->nf) / 2 + 1, 1, R), 256, 0, P->stream>>>(P->gm_V, vj(), P->nf, nvec, P->gm_dev_h,
                                                                                  nvec, W, P->nf, P->nf);
    }
    int add_basis(std::vector<double2> &y, int kmax, double2 *X)
    {
        for (auto &v : y) v = make_double2(-v.x, -v.y); // baxpy subtracts
        FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_dev_h, y.data(), sizeof(double2) * y.size(), cudaMemcpyHostToDevice, P->stream));
        baxpy_kernel<<<dim3(blas_grid(P->nf) / 2 + 1, 1, R), 256, 0, P->stream>>>(P->gm_V, vj(), P->nf, kmax, P->gm_dev_h,
                                                                                  kmax, X, P->nf, P->nf);
        return FMM_OK;
    }
    int copy(double2 *dst, const double2 *src)
    {
        FMM_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double2) * vj(), cudaMemcpyDeviceToDevice, P->stream));
        return FMM_OK;
    }
    int zero(double2 *dst)
    {
        FMM_CUDA_TRY(cudaMemsetAsync(dst, 0, sizeof(double2) * vj(), P->stream));
        return FMM_OK;
    }
    double2 *tmp_alloc()
    {
        double2 *t = nullptr;
        cudaError_t e = cudaMallocAsync(&t, sizeof(double2) * vj(), P->stream);
        if (e != cudaSuccess) { fmm_set_error("solver workspace: %s", cudaGetErrorString(e)); return nullptr; }
        return t;
    }
    void tmp_free(double2 *t) { cudaFreeAsync(t, P->stream); }
    int sync()
    {
        FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
        return FMM_OK;
    }
    void active(const std::vector<int> &a) { on = a; }
};

static int solve_batch(Plan *P, int R, double tol, int maxit, int restart, int precision, std::vector<int> &iters,
                       std::vector<double> &relres, int transpose = 0)
{
    PlanOps o{P, R, transpose, {}};
    return solve_core(o, R, tol, maxit, restart, precision, iters, relres);
}

static int solve_entry(Plan *P, const cuDoubleComplex *b, cuDoubleComplex *x, int R, double tol, int maxit, int restart,
                       int precision, int *iters, double *relres)
{
    if (!P || !b || !x || R < 1 || !(tol > 0) || maxit < 1 || restart < 1 || restart > 500) { fmm_set_error("invalid argument"); return FMM_ERR_ARG; }
    if (precision != FMM_FP64 && precision != FMM_MIXED && precision != FMM_FLOAT2) {
        fmm_set_error("unknown precision");
        return FMM_ERR_ARG;
    }
    int st = ensure_gmres(P, restart, R);
    if (st) return st;
    size_t n = (size_t)P->nf * R;
    bool bd = is_device_ptr(b), xd = is_device_ptr(x);
    FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_b, b, sizeof(double2) * n, bd ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, P->stream));
    FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_x, x, sizeof(double2) * n, xd ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, P->stream));
    std::vector<int> it;
    std::vector<double> rr;
    if ((st = solve_batch(P, R, tol, maxit, restart, precision, it, rr))) return st;
    FMM_CUDA_TRY(cudaMemcpyAsync(x, P->gm_x, sizeof(double2) * n, xd ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, P->stream));
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    if (precision == FMM_MIXED && (st = check_tc_error(P))) return st;
    bool ok = true;
    for (int r = 0; r < R; r++) {
        if (iters) iters[r] = it[r];
        if (relres) relres[r] = rr[r];
        ok = ok && rr[r] <= tol;
    }
    return ok ? FMM_OK : FMM_ERR_NOT_CONVERGED;
}

namespace fmm {
// A^T x = rhs for one column, device buffers (the adjoint solve of fmm_vjp)
int solve_transposed(Plan *P, const double2 *rhs_dev, double2 *x_dev, double tol, int maxit, int restart, int precision,
                     int *iters, double *relres)
{
    int st = build_transpose(P);
    if (st) return st;
    if ((st = ensure_gmres(P, restart, 1))) return st;
    size_t n = P->nf;
    FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_b, rhs_dev, sizeof(double2) * n, cudaMemcpyDeviceToDevice, P->stream));
    FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_x, x_dev, sizeof(double2) * n, cudaMemcpyDeviceToDevice, P->stream));
    std::vector<int> it;
    std::vector<double> rr;
    if ((st = solve_batch(P, 1, tol, maxit, restart, precision, it, rr, 1))) return st;
    FMM_CUDA_TRY(cudaMemcpyAsync(x_dev, P->gm_x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, P->stream));
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    if (iters) *iters = it[0];
    if (relres) *relres = rr[0];
    return rr[0] <= tol ? FMM_OK : FMM_ERR_NOT_CONVERGED;
}
} // namespace fmm

extern "C" int fmm_gmres(fmm_plan *plan, const cuDoubleComplex *b, cuDoubleComplex *x, double tol, int maxit,
                         int restart, int precision, int *iters, double *relres)
{
    return solve_entry((Plan *)plan, b, x, 1, tol, maxit, restart, precision, iters, relres);
}

extern "C" int fmm_solve_batched(fmm_plan *plan, const cuDoubleComplex *B, cuDoubleComplex *X, int nrhs, double tol,
                                 int maxit, int restart, int precision, int *iters, double *relres)
{
    return solve_entry((Plan *)plan, B, X, nrhs, tol, maxit, restart, precision, iters, relres);
}

extern "C" int fmm_solve_many(fmm_plan *const *plans, int n, const cuDoubleComplex *const *b, cuDoubleComplex *const *x,
                              double tol, int maxit, int restart, int precision, int nthreads, int *iters, double *relres,
                              int *status)
{
    if (!plans || n < 0 || !b || !x || nthreads < 1) { fmm_set_error("fmm_solve_many: invalid argument"); return FMM_ERR_ARG; }
    for (int i = 0; i < n; i++)
        if (!plans[i] || !b[i] || !x[i]) { fmm_set_error("fmm_solve_many: null plan or buffer %d", i); return FMM_ERR_ARG; }
    // a plan is driven by one thread at a time (plans are not thread-safe)
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++)
            if (plans[i] == plans[j]) { fmm_set_error("fmm_solve_many: plan %d appears twice", i); return FMM_ERR_ARG; }
    std::atomic<int> next(0), worst(FMM_OK);
    std::vector<std::string> errs(n);
    auto work = [&]() {
        int i;
        while ((i = next.fetch_add(1)) < n) {
            int it = 0;
            double rr = 0.0;
            // FMM_MIXED where the plan has mixed-precision tables, FP64 where plan creation
            // could not build them
            int prec = (precision == FMM_MIXED && !((Plan *)plans[i])->U32) ? FMM_FP64 : precision;
            int st = fmm_gmres(plans[i], b[i], x[i], tol, maxit, restart, prec, &it, &rr);
            if (iters) iters[i] = it;
            if (relres) relres[i] = rr;
            if (status) status[i] = st;
            if (st != FMM_OK) {
                errs[i] = fmm_last_error();
                int w = worst.load();
                // a hard error outranks non-convergence
                while ((w == FMM_OK || (w == FMM_ERR_NOT_CONVERGED && st != FMM_ERR_NOT_CONVERGED)) &&
                       !worst.compare_exchange_weak(w, st)) {
                }
            }
        }
    };
    int nt = std::min(nthreads, std::max(n, 1));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    int w = worst.load();
    if (w != FMM_OK)
        for (int i = 0; i < n; i++)
            if (!errs[i].empty()) { fmm_set_error("fmm_solve_many: plan %d: %s", i, errs[i].c_str()); break; }
    return w;
}

extern "C" int fmm_far_field(fmm_plan *plan, const cuDoubleComplex *p, const double *pts, int npts, cuDoubleComplex *out)
{
    Plan *P = (Plan *)plan;
    if (!P || !p || !pts || !out || npts < 0) { fmm_set_error("invalid argument"); return FMM_ERR_ARG; }
    double2 *pd = nullptr, *od = nullptr;
    double *ptd = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&pd, sizeof(double2) * P->nf));
    FMM_CUDA_TRY(cudaMalloc(&od, sizeof(double2) * std::max(1, npts)));
    FMM_CUDA_TRY(cudaMalloc(&ptd, sizeof(double) * 3 * std::max(1, npts)));
    FMM_CUDA_TRY(cudaMemcpy(pd, p, sizeof(double2) * P->nf, cudaMemcpyDefault));
    FMM_CUDA_TRY(cudaMemcpy(ptd, pts, sizeof(double) * 3 * npts, cudaMemcpyDefault));
    int st = launch_far_field(P, pd, ptd, npts, od);
    if (st == FMM_OK) {
        FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
        FMM_CUDA_TRY(cudaMemcpy(out, od, sizeof(double2) * npts, cudaMemcpyDefault));
    }
    cudaFree(pd); cudaFree(od); cudaFree(ptd);
    return st;
}

extern "C" int fmm_plane_wave_rhs(fmm_plan *plan, const double *dir, cuDoubleComplex *rhs)
{
    Plan *P = (Plan *)plan;
    if (!P || !dir || !rhs) { fmm_set_error("invalid argument"); return FMM_ERR_ARG; }
    double2 *r = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&r, sizeof(double2) * P->nf));
    int st = launch_plane_wave(P, dir, r);
    if (st == FMM_OK) {
        FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
        FMM_CUDA_TRY(cudaMemcpy(rhs, r, sizeof(double2) * P->nf, cudaMemcpyDefault));
    }
    cudaFree(r);
    return st;
}

// Icosphere by midpoint subdivision of the icosahedron, vertices projected to the sphere,
// faces counter-clockwise from outside; coordinates rounded through "%.9g" text like the
// OBJ files this library writes.
extern "C" int fmm_mesh_icosphere(int subdiv, double radius, double *Vout, int *nv, int *Fout, int *nf)
{
    if (subdiv < 0 || subdiv > 9 || !(radius > 0) || !nv || !nf) { fmm_set_error("invalid argument"); return FMM_ERR_ARG; }
    double t = (1.0 + sqrt(5.0)) / 2.0;
    double base[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                          {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    int fb[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                     {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                     {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    std::vector<double> V;
    std::vector<int> F;
    for (int i = 0; i < 12; i++) {
        double *b = base[i];
        double nn = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        V.push_back(b[0] / nn); V.push_back(b[1] / nn); V.push_back(b[2] / nn);
    }
    for (int i = 0; i < 20; i++) for (int j = 0; j < 3; j++) F.push_back(fb[i][j]);
    for (int s = 0; s < subdiv; s++) {
        std::vector<int> NF;
        std::vector<std::pair<long long, int>> cache;
        std::vector<std::vector<std::pair<int, int>>> adj(V.size() / 3 + F.size());
        auto mid = [&](int a, int b) {
            int lo = std::min(a, b), hi = std::max(a, b);
            for (auto &pr : adj[lo]) if (pr.first == hi) return pr.second;
            double m[3];
            for (int q = 0; q < 3; q++) m[q] = 0.5 * (V[3 * a + q] + V[3 * b + q]);
            double nn = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
            for (int q = 0; q < 3; q++) V.push_back(m[q] / nn);
            int id = (int)(V.size() / 3) - 1;
            adj[lo].push_back({hi, id});
            return id;
        };
        for (size_t f = 0; f < F.size() / 3; f++) {
            int a = F[3 * f], b = F[3 * f + 1], c = F[3 * f + 2];
            int ab = mid(a, b), bc = mid(b, c), ca = mid(c, a);
            int nfaces[4][3] = {{a, ab, ca}, {b, bc, ab}, {c, ca, bc}, {ab, bc, ca}};
            for (int q = 0; q < 4; q++) for (int r = 0; r < 3; r++) NF.push_back(nfaces[q][r]);
        }
        F.swap(NF);
    }
    *nv = (int)(V.size() / 3);
    *nf = (int)(F.size() / 3);
    if (Vout) {
        char buf[64];
        for (size_t i = 0; i < V.size(); i++) {
            snprintf(buf, sizeof(buf), "%.9g", V[i] * radius);
            Vout[i] = strtod(buf, nullptr);
        }
    }
    if (Fout) memcpy(Fout, F.data(), sizeof(int) * F.size());
    return FMM_OK;
}
