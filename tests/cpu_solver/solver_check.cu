// Host-only check of the lockstep GMRES and iterative refinement of gmres_core.h (no kernels,
// no GPU): the solver runs over a column layout whose operator is a dense complex matrix per
// column, applied on the host.  FMM_FP64 and FMM_FLOAT2 (the FP64-quality matvec the
// refinement's residuals use) apply it in double precision; FMM_MIXED applies the matrix
// rounded to float with float accumulation, so the refinement has the same kind of noise
// floor as the mixed FMM.  One JSON line per case goes to stdout.
#include "../../fmbem_gpu_c_gb300/csrc/gmres_core.h"
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

static char g_err[256];
void fmm_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

typedef std::complex<double> cd;

// R columns, column r an n_r x n_r system; vectors are the columns one after another
struct HostOps {
    std::vector<int> n, off;
    int N = 0, R = 0, restart = 0;
    std::vector<std::vector<cd>> A;        // per column, row-major
    std::vector<double2> Vb, rb, wb, bb, xb, db;
    std::vector<double2> h;                // dots of the last dots() call, [r][nvec]
    int last_nvec = 0;
    std::vector<int> on;                   // active columns of the next matvec
    long long col_matvecs = 0;             // column applications, counted
    std::vector<double2 *> tmps;

    double2 *V(int j) { return Vb.data() + (size_t)j * N; }
    double2 *r() { return rb.data(); }
    double2 *w() { return wb.data(); }
    double2 *b() { return bb.data(); }
    double2 *x() { return xb.data(); }
    double2 *d() { return db.data(); }
    int matvec(const double2 *xv, double2 *yv, int precision)
    {
        for (int c = 0; c < R; c++) {
            const int m = n[c], o = off[c];
            if (!on.empty() && !on[c]) {
                for (int i = 0; i < m; i++) yv[o + i] = make_double2(0, 0);
                continue;
            }
            col_matvecs++;
            for (int i = 0; i < m; i++) {
                if (precision != FMM_MIXED) {
                    cd acc = 0;
                    for (int j = 0; j < m; j++) acc += A[c][(size_t)i * m + j] * cd(xv[o + j].x, xv[o + j].y);
                    yv[o + i] = make_double2(acc.real(), acc.imag());
                } else {
                    std::complex<float> acc = 0;
                    for (int j = 0; j < m; j++) {
                        cd a = A[c][(size_t)i * m + j];
                        acc += std::complex<float>((float)a.real(), (float)a.imag()) *
                               std::complex<float>((float)xv[o + j].x, (float)xv[o + j].y);
                    }
                    yv[o + i] = make_double2(acc.real(), acc.imag());
                }
            }
        }
        return FMM_OK;
    }
    void axpby(double a, const double2 *xv, double bcoef, double2 *y)
    {
        for (int i = 0; i < N; i++) y[i] = make_double2(a * xv[i].x + bcoef * y[i].x, a * xv[i].y + bcoef * y[i].y);
    }
    int dots_of(const double2 *Vbase, size_t vj, const double2 *W, int nvec, std::vector<double2> &out)
    {
        out.assign((size_t)R * nvec, make_double2(0, 0));
        for (int c = 0; c < R; c++)
            for (int j = 0; j < nvec; j++) {
                double ar = 0, ai = 0;
                for (int i = off[c]; i < off[c] + n[c]; i++) {
                    double2 a = Vbase[(size_t)j * vj + i], bq = W[i];
                    ar += a.x * bq.x + a.y * bq.y;
                    ai += a.x * bq.y - a.y * bq.x;
                }
                out[(size_t)c * nvec + j] = make_double2(ar, ai);
            }
        return FMM_OK;
    }
    int norms(const double2 *W, std::vector<double> &out)
    {
        std::vector<double2> t;
        dots_of(W, 0, W, 1, t);
        out.resize(R);
        for (int c = 0; c < R; c++) out[c] = sqrt(std::max(0.0, t[c].x));
        return FMM_OK;
    }
    int scale(const std::vector<double> &alpha, const double2 *X, double2 *Y)
    {
        for (int c = 0; c < R; c++)
            for (int i = off[c]; i < off[c] + n[c]; i++) Y[i] = make_double2(alpha[c] * X[i].x, alpha[c] * X[i].y);
        return FMM_OK;
    }
    int dots(int nvec, const double2 *W, std::vector<double2> &out)
    {
        dots_of(Vb.data(), N, W, nvec, out);
        h = out;
        last_nvec = nvec;
        return FMM_OK;
    }
    void sub_basis(int nvec, const std::vector<double2> &coef, double2 *W, int sign)
    {
        for (int c = 0; c < R; c++)
            for (int i = off[c]; i < off[c] + n[c]; i++)
                for (int j = 0; j < nvec; j++) {
                    double2 a = Vb[(size_t)j * N + i], q = coef[(size_t)c * nvec + j];
                    W[i].x -= sign * (a.x * q.x - a.y * q.y);
                    W[i].y -= sign * (a.x * q.y + a.y * q.x);
                }
    }
    void sub_dots(int nvec, double2 *W) { sub_basis(nvec, h, W, 1); }
    int add_basis(std::vector<double2> &y, int kmax, double2 *X)
    {
        sub_basis(kmax, y, X, -1);
        return FMM_OK;
    }
    int copy(double2 *dst, const double2 *src)
    {
        for (int i = 0; i < N; i++) dst[i] = src[i];
        return FMM_OK;
    }
    int zero(double2 *dst)
    {
        for (int i = 0; i < N; i++) dst[i] = make_double2(0, 0);
        return FMM_OK;
    }
    double2 *tmp_alloc()
    {
        double2 *t = new double2[N];
        tmps.push_back(t);
        return t;
    }
    void tmp_free(double2 *t) { delete[] t; }
    int sync() { return FMM_OK; }
    void active(const std::vector<int> &a) { on = a; }
};

// n_r x n_r systems I + s K with K random complex (entries ~ 1/sqrt(n)), s per column: larger s,
// more iterations
static void setup(HostOps &o, const std::vector<int> &sizes, const std::vector<double> &spread, int restart,
                  unsigned seed, bool zero_rhs_last)
{
    std::mt19937_64 g(seed);
    std::normal_distribution<double> nd;
    o.R = (int)sizes.size();
    o.n = sizes;
    o.off.assign(o.R + 1, 0);
    for (int c = 0; c < o.R; c++) o.off[c + 1] = o.off[c] + sizes[c];
    o.N = o.off[o.R];
    o.restart = restart;
    o.A.resize(o.R);
    for (int c = 0; c < o.R; c++) {
        const int m = sizes[c];
        o.A[c].assign((size_t)m * m, 0);
        for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++)
                o.A[c][(size_t)i * m + j] = (i == j ? 1.0 : 0.0) + spread[c] * cd(nd(g), nd(g)) / sqrt((double)m);
    }
    o.Vb.assign((size_t)(restart + 1) * o.N, make_double2(0, 0));
    for (auto *v : {&o.rb, &o.wb, &o.bb, &o.xb, &o.db}) v->assign(o.N, make_double2(0, 0));
    for (int c = 0; c < o.R; c++)
        for (int i = o.off[c]; i < o.off[c + 1]; i++)
            o.bb[i] = (zero_rhs_last && c == o.R - 1) ? make_double2(0, 0) : make_double2(nd(g), nd(g));
}

// true relative residual of column c in FP64
static double true_res(HostOps &o, int c)
{
    const int m = o.n[c], of = o.off[c];
    double rn = 0, bn = 0;
    for (int i = 0; i < m; i++) {
        cd acc = 0;
        for (int j = 0; j < m; j++) acc += o.A[c][(size_t)i * m + j] * cd(o.xb[of + j].x, o.xb[of + j].y);
        cd rr = cd(o.bb[of + i].x, o.bb[of + i].y) - acc;
        rn += std::norm(rr);
        bn += std::norm(cd(o.bb[of + i].x, o.bb[of + i].y));
    }
    return bn > 0 ? sqrt(rn / bn) : sqrt(rn);
}

static void run(const char *name, const std::vector<int> &sizes, const std::vector<double> &spread, int restart,
                double tol, int precision, bool zero_last)
{
    HostOps o;
    setup(o, sizes, spread, restart, 7, zero_last);
    std::vector<int> it;
    std::vector<double> rr;
    int st = fmm::solve_core(o, o.R, tol, 5000, restart, precision, it, rr);
    printf("{\"case\": \"%s\", \"status\": %d, \"error\": \"%s\", \"col_matvecs\": %lld, \"iters\": [", name, st, g_err,
           o.col_matvecs);
    for (int c = 0; c < o.R; c++) printf("%s%d", c ? ", " : "", it[c]);
    printf("], \"relres\": [");
    for (int c = 0; c < o.R; c++) printf("%s%.3e", c ? ", " : "", rr[c]);
    printf("], \"true_res\": [");
    for (int c = 0; c < o.R; c++) printf("%s%.3e", c ? ", " : "", true_res(o, c));
    printf("]}\n");
}

int main()
{
    // uneven columns (as the bodies of a scene), short restarts so that cycles end early
    std::vector<int> sizes = {40, 120, 64, 90};
    std::vector<double> spread = {0.2, 0.6, 0.4, 0.75};
    run("fp64", sizes, spread, 10, 1e-10, FMM_FP64, false);
    run("mixed", sizes, spread, 10, 1e-9, FMM_MIXED, false);
    run("mixed_zero_rhs", sizes, spread, 10, 1e-8, FMM_MIXED, true);
    run("fp64_long_restart", sizes, spread, 60, 1e-10, FMM_FP64, false);
    return 0;
}
