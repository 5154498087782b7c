// Plan creation, the public C ABI, and the GMRES / iterative-refinement solver.
#include "plan.h"
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace fmm {
int set_dir_dist(const int *dd);
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
        F(L.Cm64); F(L.Dl64); F(L.Cm32); F(L.Dl32); F(L.Csr64); F(L.Csr32); F(L.Crr64); F(L.Crr32);
        for (RcrList *R : {&L.m2l, &L.m2m, &L.l2l}) { F(R->items); F(R->src); F(R->dst); }
    }
    F(P->Hsr64); F(P->PHsr64); F(P->Hsr32); F(P->PHsr32);
    F(P->V_dev); F(P->F_dev); F(P->elem_leaf); F(P->leaf_beg); F(P->leaf_elem);
    F(P->U64); F(P->Rv64); F(P->U32); F(P->Rv32); F(P->near_beg); F(P->near_col); F(P->near64); F(P->near32);
    F(P->nearT_beg); F(P->nearT_col); F(P->nearT64); F(P->nearT32);
    F(P->xbuf); F(P->ybuf);
    F(P->gm_V); F(P->gm_w); F(P->gm_r); F(P->gm_x); F(P->gm_b); F(P->gm_d); F(P->gm_dev_h);
    if (P->timers_created)
        for (int i = 0; i < MAX_TIMERS; i++) { cudaEventDestroy(P->timers[i].beg); cudaEventDestroy(P->timers[i].end); }
    if (P->timers_created) { cudaEventDestroy(P->total.beg); cudaEventDestroy(P->total.end); }
    if (P->stream) cudaStreamDestroy(P->stream);
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
    if (opt->depth < 0 || opt->depth > FMM_MAX_LEVEL) { fmm_set_error("depth %d out of range", opt->depth); return FMM_ERR_ARG; }
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
    // a blocking stream: setup code mixes kernels on this stream with default-stream
    // cudaMemcpy read-backs (list counts), which must wait for those kernels
    CTRY(cudaStreamCreate(&P->stream));
    if (build_tree(P->V, P->F, opt->s, opt->depth, P->tree) != 0 || P->tree.lmax > FMM_MAX_LEVEL) {
        fmm_set_error("octree build failed (lmax=%d)", P->tree.lmax);
        free_plan(P);
        return FMM_ERR_MESH;
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
    if (P->opt.build_mixed && rcr_tile_smem(P->pmax, 8, 0) > 227 * 1024) {
        // the batched FP32 translations keep two p^2 x 8 complex tiles in shared memory
        P->opt.build_mixed = 0;
        snprintf(P->mixed_note, sizeof(P->mixed_note),
                 "mixed precision needs truncation orders <= 42 (this plan has %d); use FMM_FP64", P->pmax);
    }
    if (P->pleaf > 40) { fmm_set_error("leaf truncation order %d above 40", P->pleaf); free_plan(P); return FMM_ERR_ARG; }
    CTRY(dev_alloc(P, (void **)&P->V_dev, sizeof(double) * P->V.size()));
    CTRY(dev_alloc(P, (void **)&P->F_dev, sizeof(int) * P->F.size()));
    CTRY(dev_alloc(P, (void **)&P->elem_leaf, sizeof(int) * nf));
    CTRY(cudaMemcpy(P->V_dev, P->V.data(), sizeof(double) * P->V.size(), cudaMemcpyHostToDevice));
    CTRY(cudaMemcpy(P->F_dev, P->F.data(), sizeof(int) * P->F.size(), cudaMemcpyHostToDevice));
    CTRY(cudaMemcpy(P->elem_leaf, P->tree.elem_leaf.data(), sizeof(int) * nf, cudaMemcpyHostToDevice));
    TRY(gen_rotation_tables(P));
    TRY(set_dir_dist(P->dir_dist));
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
    TRY(gen_element_tables(P));
    TRY(gen_near_field(P));
    if (P->opt.build_mixed) {
        TRY(build_rcr_lists(P));
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
    P->timers_created = 1;
    CTRY(cudaStreamSynchronize(P->stream));
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
    free_plan((Plan *)plan);
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
        info->m2l_columns[l] = P->opt.build_mixed ? P->lev[l].m2l.tc : 0;
    }
    info->num_near = P->num_near;
    info->device_bytes = P->device_bytes;
    info->setup_seconds = P->setup_seconds;
    return FMM_OK;
}

static bool is_device_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

extern "C" int fmm_matvec(fmm_plan *plan, const cuDoubleComplex *x, cuDoubleComplex *y, int nrhs, int precision)
{
    Plan *P = (Plan *)plan;
    if (!P || !x || !y || nrhs < 1) { fmm_set_error("invalid argument"); return FMM_ERR_ARG; }
    if (precision != FMM_FP64 && precision != FMM_MIXED) { fmm_set_error("unknown precision %d", precision); return FMM_ERR_ARG; }
    bool xd = is_device_ptr(x), yd = is_device_ptr(y);
    for (int r = 0; r < nrhs; r++) {
        const double2 *xs = (const double2 *)x + (size_t)r * P->nf;
        double2 *ys = (double2 *)y + (size_t)r * P->nf;
        const double2 *xin = xs;
        double2 *yout = ys;
        if (!xd) {
            FMM_CUDA_TRY(cudaMemcpyAsync(P->xbuf, xs, sizeof(double2) * P->nf, cudaMemcpyHostToDevice, P->stream));
            xin = P->xbuf;
        }
        if (!yd) yout = P->ybuf;
        int st = run_matvec(P, xin, yout, precision);
        if (st) return st;
        if (!yd) FMM_CUDA_TRY(cudaMemcpyAsync(ys, P->ybuf, sizeof(double2) * P->nf, cudaMemcpyDeviceToHost, P->stream));
    }
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    return FMM_OK;
}

// Transposed operator: the sources become point sources at the centroids (multipole
// R_n^{-m}(y_i - c)) and the targets element integrals (local expansion integrated against
// b R + c dR/dn), with the same translation tables; the near field is the transposed CSR.
// A^H x = conj(A^T conj(x)).
extern "C" int fmm_matvec_adjoint(fmm_plan *plan, const cuDoubleComplex *x, cuDoubleComplex *y, int nrhs, int precision,
                                  int conjugate)
{
    Plan *P = (Plan *)plan;
    if (!P || !x || !y || nrhs < 1) { fmm_set_error("invalid argument"); return FMM_ERR_ARG; }
    if (precision != FMM_FP64 && precision != FMM_MIXED) { fmm_set_error("unknown precision %d", precision); return FMM_ERR_ARG; }
    {
        int st = build_transpose(P);
        if (st) return st;
    }
    bool xd = is_device_ptr(x), yd = is_device_ptr(y);
    for (int r = 0; r < nrhs; r++) {
        const double2 *xs = (const double2 *)x + (size_t)r * P->nf;
        double2 *ys = (double2 *)y + (size_t)r * P->nf;
        const double2 *xin = xs;
        double2 *yout = yd ? ys : P->ybuf;
        if (!xd) {
            FMM_CUDA_TRY(cudaMemcpyAsync(P->xbuf, xs, sizeof(double2) * P->nf, cudaMemcpyHostToDevice, P->stream));
            xin = P->xbuf;
        }
        if (conjugate) {
            launch_conj(P, xin, P->xbuf);
            xin = P->xbuf;
        }
        int st = run_matvec(P, xin, yout, precision, 1);
        if (st) return st;
        if (conjugate) launch_conj(P, yout, yout);
        FMM_CUDA_TRY(cudaGetLastError());
        if (!yd) FMM_CUDA_TRY(cudaMemcpyAsync(ys, P->ybuf, sizeof(double2) * P->nf, cudaMemcpyDeviceToHost, P->stream));
    }
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    return FMM_OK;
}

extern "C" int fmm_set_profiling(fmm_plan *plan, int on)
{
    if (!plan) return FMM_ERR_ARG;
    ((Plan *)plan)->profiling = on ? 1 : 0;
    return FMM_OK;
}

extern "C" int fmm_last_timings(const fmm_plan *plan, const char **names, double *ms, int *count)
{
    const Plan *P = (const Plan *)plan;
    if (!P || !count) return FMM_ERR_ARG;
    int total = P->ntimers + (P->have_total ? 1 : 0);
    int n = std::min(*count, total);
    for (int i = 0; i < n; i++) {
        const Timer &tm = i < P->ntimers ? P->timers[i] : P->total;
        float t = 0.f;
        cudaEventSynchronize(tm.end);
        cudaEventElapsedTime(&t, tm.beg, tm.end);
        if (names) names[i] = i < P->ntimers ? tm.name : "matvec";
        if (ms) ms[i] = t;
    }
    *count = total;
    return FMM_OK;
}

// ---------------------------------------------------------------------------- BLAS-1 kernels
namespace fmm {
__global__ void multi_dot_kernel(const double2 *V, size_t ld, int nvec, const double2 *w, int n, double2 *out)
{
    int j = blockIdx.y;
    const double2 *v = V + (size_t)j * ld;
    double ar = 0, ai = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 a = v[i], b = w[i];
        ar += a.x * b.x + a.y * b.y; // conj(a) b
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
    if (threadIdx.x == 0) { atomicAdd(&out[j].x, sr[0]); atomicAdd(&out[j].y, si[0]); }
}

// w -= sum_j V_j h_j
__global__ void multi_axpy_kernel(const double2 *V, size_t ld, int nvec, const double2 *h, double2 *w, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 acc = w[i];
        for (int j = 0; j < nvec; j++) {
            double2 v = V[(size_t)j * ld + i], c = h[j];
            acc.x -= v.x * c.x - v.y * c.y;
            acc.y -= v.x * c.y + v.y * c.x;
        }
        w[i] = acc;
    }
}

// y = alpha x + beta y (alpha, beta complex)
__global__ void axpby_kernel(double2 alpha, const double2 *x, double2 beta, double2 *y, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 a = x[i], b = y[i];
        y[i] = make_double2(alpha.x * a.x - alpha.y * a.y + beta.x * b.x - beta.y * b.y,
                            alpha.x * a.y + alpha.y * a.x + beta.x * b.y + beta.y * b.x);
    }
}
} // namespace fmm

static const int BLAS_BLOCKS = 152 * 2;

static int dev_dots(Plan *P, const double2 *V, int nvec, const double2 *w, double2 *hdev, std::vector<double2> &hhost)
{
    FMM_CUDA_TRY(cudaMemsetAsync(hdev, 0, sizeof(double2) * nvec, P->stream));
    dim3 grid(std::min(BLAS_BLOCKS, (P->nf + 255) / 256), nvec);
    multi_dot_kernel<<<grid, 256, 0, P->stream>>>(V, P->nf, nvec, w, P->nf, hdev);
    hhost.resize(nvec);
    FMM_CUDA_TRY(cudaMemcpyAsync(hhost.data(), hdev, sizeof(double2) * nvec, cudaMemcpyDeviceToHost, P->stream));
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    return FMM_OK;
}

static int dev_norm(Plan *P, const double2 *w, double *out)
{
    std::vector<double2> h;
    int st = dev_dots(P, w, 1, w, P->gm_dev_h, h);
    if (st) return st;
    *out = sqrt(std::max(0.0, h[0].x));
    return FMM_OK;
}

static void axpby(Plan *P, double2 a, const double2 *x, double2 b, double2 *y)
{
    axpby_kernel<<<std::min(BLAS_BLOCKS, (P->nf + 255) / 256), 256, 0, P->stream>>>(a, x, b, y, P->nf);
}

static int ensure_gmres(Plan *P, int restart)
{
    if (P->gm_restart >= restart) return FMM_OK;
    if (P->gm_V) cudaFree(P->gm_V);
    if (!P->gm_w) {
        FMM_CUDA_TRY(cudaMalloc(&P->gm_w, sizeof(double2) * P->nf));
        FMM_CUDA_TRY(cudaMalloc(&P->gm_r, sizeof(double2) * P->nf));
        FMM_CUDA_TRY(cudaMalloc(&P->gm_x, sizeof(double2) * P->nf));
        FMM_CUDA_TRY(cudaMalloc(&P->gm_b, sizeof(double2) * P->nf));
        FMM_CUDA_TRY(cudaMalloc(&P->gm_d, sizeof(double2) * P->nf));
        FMM_CUDA_TRY(cudaMalloc(&P->gm_dev_h, sizeof(double2) * 512));
    }
    FMM_CUDA_TRY(cudaMalloc(&P->gm_V, sizeof(double2) * (size_t)P->nf * (restart + 1)));
    P->gm_restart = restart;
    return FMM_OK;
}

// Restarted GMRES with classical Gram-Schmidt applied twice (CGS2); all vectors FP64 on the
// device; Hessenberg least squares by Givens rotations on the host.  Solves A x = b where
// the matvec runs at `precision`; x (device) holds the initial guess.  Convergence is
// relative to bnorm_ref.
static int gmres_core(Plan *P, const double2 *b, double2 *x, double tol, int maxit, int restart, int precision,
                      double bnorm_ref, int *iters, double *relres)
{
    int n = P->nf, m = restart;
    std::vector<double2> H((size_t)(m + 1) * m), g(m + 1), cs(m), sn(m), hcol, h2;
    int total = 0;
    double res = 0.0;
    while (true) {
        // r = b - A x
        int st = run_matvec(P, x, P->gm_r, precision);
        if (st) return st;
        axpby(P, make_double2(1, 0), b, make_double2(-1, 0), P->gm_r);
        double beta;
        if ((st = dev_norm(P, P->gm_r, &beta))) return st;
        res = beta / bnorm_ref;
        if (!std::isfinite(res)) { fmm_set_error("GMRES residual is not finite"); return FMM_ERR_BREAKDOWN; }
        if (res <= tol || total >= maxit) break;
        axpby(P, make_double2(1.0 / beta, 0), P->gm_r, make_double2(0, 0), P->gm_V);
        std::fill(g.begin(), g.end(), make_double2(0, 0));
        g[0] = make_double2(beta, 0);
        int j = 0;
        for (; j < m && total < maxit; j++) {
            double2 *vj = P->gm_V + (size_t)j * n, *w = P->gm_w;
            if ((st = run_matvec(P, vj, w, precision))) return st;
            // two passes of classical Gram-Schmidt
            if ((st = dev_dots(P, P->gm_V, j + 1, w, P->gm_dev_h, hcol))) return st;
            multi_axpy_kernel<<<std::min(BLAS_BLOCKS, (n + 255) / 256), 256, 0, P->stream>>>(P->gm_V, n, j + 1, P->gm_dev_h, w, n);
            if ((st = dev_dots(P, P->gm_V, j + 1, w, P->gm_dev_h, h2))) return st;
            multi_axpy_kernel<<<std::min(BLAS_BLOCKS, (n + 255) / 256), 256, 0, P->stream>>>(P->gm_V, n, j + 1, P->gm_dev_h, w, n);
            for (int i = 0; i <= j; i++) { hcol[i].x += h2[i].x; hcol[i].y += h2[i].y; }
            double hn;
            if ((st = dev_norm(P, w, &hn))) return st;
            total++;
            for (int i = 0; i <= j; i++) H[(size_t)i * m + j] = hcol[i];
            H[(size_t)(j + 1) * m + j] = make_double2(hn, 0);
            // apply previous rotations
            for (int i = 0; i < j; i++) {
                double2 a = H[(size_t)i * m + j], bq = H[(size_t)(i + 1) * m + j];
                double2 c = cs[i], s = sn[i];
                // [c  s; -conj(s) c] with c real
                double2 na = make_double2(c.x * a.x + s.x * bq.x - s.y * bq.y, c.x * a.y + s.x * bq.y + s.y * bq.x);
                double2 nb = make_double2(-(s.x * a.x + s.y * a.y) + c.x * bq.x, -(s.x * a.y - s.y * a.x) + c.x * bq.y);
                H[(size_t)i * m + j] = na;
                H[(size_t)(i + 1) * m + j] = nb;
            }
            double2 a = H[(size_t)j * m + j];
            double an = hypot(a.x, a.y), den = hypot(an, hn);
            double2 c, s;
            if (den == 0.0) { fmm_set_error("GMRES breakdown"); return FMM_ERR_BREAKDOWN; }
            if (an == 0.0) { c = make_double2(0, 0); s = make_double2(1, 0); }
            else {
                c = make_double2(an / den, 0);
                // s = (a/|a|) * conj(hn) / den ; hn real
                s = make_double2(a.x / an * hn / den, a.y / an * hn / den);
            }
            cs[j] = c;
            sn[j] = s;
            H[(size_t)j * m + j] = make_double2(c.x * a.x + s.x * hn, c.x * a.y + s.y * hn);
            H[(size_t)(j + 1) * m + j] = make_double2(0, 0);
            double2 gj = g[j];
            g[j + 1] = make_double2(-(s.x * gj.x + s.y * gj.y), -(s.x * gj.y - s.y * gj.x));
            g[j] = make_double2(c.x * gj.x, c.x * gj.y);
            res = hypot(g[j + 1].x, g[j + 1].y) / bnorm_ref;
            if (hn == 0.0 || res <= tol) { j++; break; }
            axpby(P, make_double2(1.0 / hn, 0), w, make_double2(0, 0), P->gm_V + (size_t)(j + 1) * n);
        }
        // back substitution, x += V y
        int kdim = j;
        std::vector<double2> yv(kdim);
        for (int i = kdim - 1; i >= 0; i--) {
            double2 acc = g[i];
            for (int q = i + 1; q < kdim; q++) {
                double2 h = H[(size_t)i * m + q];
                acc.x -= h.x * yv[q].x - h.y * yv[q].y;
                acc.y -= h.x * yv[q].y + h.y * yv[q].x;
            }
            double2 d = H[(size_t)i * m + i];
            double dd = d.x * d.x + d.y * d.y;
            yv[i] = make_double2((acc.x * d.x + acc.y * d.y) / dd, (acc.y * d.x - acc.x * d.y) / dd);
        }
        FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_dev_h, yv.data(), sizeof(double2) * kdim, cudaMemcpyHostToDevice, P->stream));
        // x -= V (-y)
        for (int i = 0; i < kdim; i++) yv[i] = make_double2(-yv[i].x, -yv[i].y);
        FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_dev_h, yv.data(), sizeof(double2) * kdim, cudaMemcpyHostToDevice, P->stream));
        multi_axpy_kernel<<<std::min(BLAS_BLOCKS, (n + 255) / 256), 256, 0, P->stream>>>(P->gm_V, n, kdim, P->gm_dev_h, x, n);
        FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
        if (res <= tol || total >= maxit) {
            // recompute the true residual once more at the top of the loop
            int st2 = run_matvec(P, x, P->gm_r, precision);
            if (st2) return st2;
            axpby(P, make_double2(1, 0), b, make_double2(-1, 0), P->gm_r);
            double bt;
            if ((st2 = dev_norm(P, P->gm_r, &bt))) return st2;
            res = bt / bnorm_ref;
            break;
        }
    }
    if (iters) *iters = total;
    if (relres) *relres = res;
    return FMM_OK;
}

extern "C" int fmm_gmres(fmm_plan *plan, const cuDoubleComplex *b, cuDoubleComplex *x, double tol, int maxit,
                         int restart, int precision, int *iters, double *relres)
{
    Plan *P = (Plan *)plan;
    if (!P || !b || !x || !(tol > 0) || maxit < 1 || restart < 1 || restart > 500) { fmm_set_error("invalid argument"); return FMM_ERR_ARG; }
    if (precision != FMM_FP64 && precision != FMM_MIXED) { fmm_set_error("unknown precision"); return FMM_ERR_ARG; }
    int st = ensure_gmres(P, restart);
    if (st) return st;
    int n = P->nf;
    bool bd = is_device_ptr(b), xd = is_device_ptr(x);
    FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_b, b, sizeof(double2) * n, bd ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, P->stream));
    FMM_CUDA_TRY(cudaMemcpyAsync(P->gm_x, x, sizeof(double2) * n, xd ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, P->stream));
    double bnorm;
    if ((st = dev_norm(P, P->gm_b, &bnorm))) return st;
    if (bnorm == 0.0) bnorm = 1.0;
    int it = 0;
    double rr = 0.0;
    if (precision == FMM_FP64) {
        st = gmres_core(P, P->gm_b, P->gm_x, tol, maxit, restart, FMM_FP64, bnorm, &it, &rr);
    } else {
        // iterative refinement: r = b - A64 x (FP64), solve A32 d = r, x += d
        double2 *d = P->gm_d;
        int total = 0;
        for (int outer = 0; outer < 20; outer++) {
            if ((st = run_matvec(P, P->gm_x, P->gm_w, FMM_FP64))) return st;
            // gm_w = b - A x  (kept in gm_w; gmres_core uses gm_r and gm_w as work, so copy to d's rhs slot)
            axpby(P, make_double2(1, 0), P->gm_b, make_double2(-1, 0), P->gm_w);
            double rn;
            if ((st = dev_norm(P, P->gm_w, &rn))) return st;
            rr = rn / bnorm;
            if (rr <= tol || total >= maxit) break;
            // inner solve on a copy of the residual
            double2 *rhs = nullptr;
            FMM_CUDA_TRY(cudaMalloc(&rhs, sizeof(double2) * n));
            FMM_CUDA_TRY(cudaMemcpyAsync(rhs, P->gm_w, sizeof(double2) * n, cudaMemcpyDeviceToDevice, P->stream));
            FMM_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(double2) * n, P->stream));
            double inner_tol = std::max(1e-5, 0.5 * tol / rr);
            if (inner_tol > 0.1) inner_tol = 0.1;
            int iti = 0;
            double rri = 0;
            st = gmres_core(P, rhs, d, inner_tol, maxit - total, restart, FMM_MIXED, rn, &iti, &rri);
            cudaFree(rhs);
            if (st) return st;
            total += iti;
            axpby(P, make_double2(1, 0), d, make_double2(1, 0), P->gm_x);
        }
        it = total;
    }
    if (st) return st;
    FMM_CUDA_TRY(cudaMemcpyAsync(x, P->gm_x, sizeof(double2) * n, xd ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, P->stream));
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return rr <= tol ? FMM_OK : FMM_ERR_NOT_CONVERGED;
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
