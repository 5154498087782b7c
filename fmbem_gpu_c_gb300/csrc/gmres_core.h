// Restarted GMRES on R columns in lockstep, and the FP64-refined mixed-precision solve around
// it, written once over a column layout `Ops`: the columns of one plan (right-hand sides of
// equal length) or the bodies of a scene (one column per plan, of unequal lengths).
//
// Ops provides, all on its stream:
//   double2 *V(int j), *r(), *w(), *b(), *x(), *d()   Krylov vector j; work and solve vectors
//   int matvec(const double2 *x, double2 *y, int precision)
//   void axpby(double a, const double2 *x, double b, double2 *y)          all columns
//   int norms(const double2 *W, std::vector<double> &out)                 per column, synchronizes
//   int scale(const std::vector<double> &alpha, const double2 *X, double2 *Y)   Y_r = alpha_r X_r
//   int dots(int nvec, const double2 *W, std::vector<double2> &out)      out[r nvec + j] = <V_j,r, W_r>,
//                                                                        kept on the device for sub_dots
//   void sub_dots(int nvec, double2 *W)                                  W_r -= sum_j V_j,r out[r nvec + j]
//   int add_basis(std::vector<double2> &y, int kmax, double2 *X)        X_r += sum_j V_j,r y[r kmax + j]
//                                                                        (may overwrite y)
//   int copy(double2 *dst, const double2 *src), zero(double2 *dst)       whole vectors
//   double2 *tmp_alloc(), void tmp_free(double2 *)                       a whole vector
//   int sync()
//   void active(const std::vector<int> &on)                              columns whose matvec results
//                                                                        are used (the others may be skipped)
#pragma once
#include "plan.h"
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

namespace fmm {

// Every Krylov step applies the operator to all R columns at once; classical Gram-Schmidt
// applied twice (CGS2), FP64 vectors on the device, Hessenberg least squares by Givens
// rotations on the host per column.  A column stops extending its basis once its residual
// estimate is below tol[r] (its new basis vectors are zero).  Solves A X = B at `precision`;
// X holds the initial guess.  Convergence of column r is relative to bref[r].
template <class Ops>
int gmres_core(Ops &o, const double2 *B, double2 *X, int R, const std::vector<double> &tol, int maxit, int restart,
               int precision, const std::vector<double> &bref, std::vector<int> &iters, std::vector<double> &res)
{
    const int m = restart;
    std::vector<std::vector<double2>> H(R, std::vector<double2>((size_t)(m + 1) * m)), g(R, std::vector<double2>(m + 1)),
        cs(R, std::vector<double2>(m)), sn(R, std::vector<double2>(m));
    std::vector<double2> h1, h2;
    std::vector<double> beta, hn, alpha(R);
    std::vector<int> kdim(R), running(R);
    iters.assign(R, 0);
    res.assign(R, 0.0);
    int total = 0;
    // columns whose X changed in the last restart cycle (all at first): only their residuals
    // are recomputed; the others keep the norm of the same X from before.  (Columns that stop
    // near the mixed operator's noise floor restart after a few steps, many times; recomputing
    // every column each time would cost a full matvec per restart.)
    std::vector<int> changed(R, 1);
    std::vector<double> beta_prev(R, 0.0);
    const std::vector<int> all(R, 1);
    while (true) {
        // R = B - A X, its norms, and which columns still need work
        o.active(changed);
        int st = o.matvec(X, o.r(), precision);
        if (st) return st;
        o.axpby(1.0, B, -1.0, o.r());
        o.active(all);
        if ((st = o.norms(o.r(), beta))) return st;
        for (int r = 0; r < R; r++)
            if (!changed[r]) beta[r] = beta_prev[r];
        beta_prev = beta;
        int any = 0;
        for (int r = 0; r < R; r++) {
            res[r] = bref[r] > 0 ? beta[r] / bref[r] : 0.0;
            if (!std::isfinite(res[r])) { fmm_set_error("GMRES residual of column %d is not finite", r); return FMM_ERR_BREAKDOWN; }
            running[r] = res[r] > tol[r];
            any |= running[r];
            alpha[r] = running[r] ? 1.0 / beta[r] : 0.0;
            kdim[r] = 0;
            std::fill(g[r].begin(), g[r].end(), make_double2(0, 0));
            g[r][0] = make_double2(beta[r], 0);
        }
        if (!any || total >= maxit) break;
        std::vector<int> ran(running);
        if ((st = o.scale(alpha, o.r(), o.V(0)))) return st;
        int j = 0;
        for (; j < m && total < maxit; j++) {
            double2 *W = o.w();
            o.active(running);
            if ((st = o.matvec(o.V(j), W, precision))) return st;
            if ((st = o.dots(j + 1, W, h1))) return st;
            o.sub_dots(j + 1, W);
            if ((st = o.dots(j + 1, W, h2))) return st;
            o.sub_dots(j + 1, W);
            if ((st = o.norms(W, hn))) return st;
            total++;
            any = 0;
            for (int r = 0; r < R; r++) {
                alpha[r] = 0.0;
                if (!running[r]) continue;
                iters[r]++;
                std::vector<double2> &Hr = H[r], &gr = g[r], &c_ = cs[r], &s_ = sn[r];
                for (int i = 0; i <= j; i++) {
                    double2 a = h1[(size_t)r * (j + 1) + i], b = h2[(size_t)r * (j + 1) + i];
                    Hr[(size_t)i * m + j] = make_double2(a.x + b.x, a.y + b.y);
                }
                double h = hn[r];
                // previous rotations [c s; -conj(s) c], c real
                for (int i = 0; i < j; i++) {
                    double2 a = Hr[(size_t)i * m + j], bq = Hr[(size_t)(i + 1) * m + j], c = c_[i], sv = s_[i];
                    Hr[(size_t)i * m + j] = make_double2(c.x * a.x + sv.x * bq.x - sv.y * bq.y, c.x * a.y + sv.x * bq.y + sv.y * bq.x);
                    Hr[(size_t)(i + 1) * m + j] =
                        make_double2(-(sv.x * a.x + sv.y * a.y) + c.x * bq.x, -(sv.x * a.y - sv.y * a.x) + c.x * bq.y);
                }
                double2 a = Hr[(size_t)j * m + j];
                double an = hypot(a.x, a.y), den = hypot(an, h);
                kdim[r] = j + 1;
                if (den == 0.0) { // the basis is exhausted: nothing more to add for this column
                    kdim[r] = j;
                    running[r] = 0;
                    continue;
                }
                double2 c, sv;
                if (an == 0.0) { c = make_double2(0, 0); sv = make_double2(1, 0); }
                else { c = make_double2(an / den, 0); sv = make_double2(a.x / an * h / den, a.y / an * h / den); }
                c_[j] = c;
                s_[j] = sv;
                Hr[(size_t)j * m + j] = make_double2(c.x * a.x + sv.x * h, c.x * a.y + sv.y * h);
                double2 gj = gr[j];
                gr[j + 1] = make_double2(-(sv.x * gj.x + sv.y * gj.y), -(sv.x * gj.y - sv.y * gj.x));
                gr[j] = make_double2(c.x * gj.x, c.x * gj.y);
                res[r] = hypot(gr[j + 1].x, gr[j + 1].y) / bref[r];
                if (h == 0.0 || res[r] <= tol[r]) { running[r] = 0; continue; }
                alpha[r] = 1.0 / h;
                any = 1;
            }
            if (j + 1 < m) {
                if ((st = o.scale(alpha, W, o.V(j + 1)))) return st;
            }
            if (!any) { j++; break; }
        }
        // X_r += V_r y_r, y_r from the triangular systems (zero beyond kdim[r])
        int kmax = 0;
        for (int r = 0; r < R; r++) kmax = std::max(kmax, kdim[r]);
        std::vector<double2> Y((size_t)R * std::max(kmax, 1), make_double2(0, 0));
        for (int r = 0; r < R; r++) {
            std::vector<double2> &Hr = H[r];
            for (int i = kdim[r] - 1; i >= 0; i--) {
                double2 acc = g[r][i];
                for (int q = i + 1; q < kdim[r]; q++) {
                    double2 hq = Hr[(size_t)i * m + q], yq = Y[(size_t)r * kmax + q];
                    acc.x -= hq.x * yq.x - hq.y * yq.y;
                    acc.y -= hq.x * yq.y + hq.y * yq.x;
                }
                double2 d = Hr[(size_t)i * m + i];
                double dd = d.x * d.x + d.y * d.y;
                Y[(size_t)r * kmax + i] = make_double2((acc.x * d.x + acc.y * d.y) / dd, (acc.y * d.x - acc.x * d.y) / dd);
            }
        }
        // a column that ran in this cycle may have a new X (and its residual vector is needed
        // if it runs again); one that did not run kept its X
        changed = ran;
        if (kmax > 0 && (st = o.add_basis(Y, kmax, X))) return st;
        if ((st = o.sync())) return st;
    }
    return FMM_OK;
}

// The precision of the refinement's residuals: the FP64 matvec with its M2L in float-float
// (FMM_FLOAT2: about 48 bits, about twice as fast as FP64 on GB300; plain FP64 where a plan has
// no mixed tables), or plain FP64 with FMMBEM_FF_RESIDUAL=0.
inline int residual_precision()
{
    const char *e = getenv("FMMBEM_FF_RESIDUAL");
    return (e && atoi(e) == 0) ? FMM_FP64 : FMM_FLOAT2;
}

// Solve A X = B (o.b() -> o.x(), X holding the initial guess) for R columns at `precision`.
// FMM_MIXED runs iterative refinement: residual B - A X in FP64 quality (residual_precision),
// inner lockstep GMRES on the mixed-precision matvec for the correction, X += D.
template <class Ops>
int solve_core(Ops &o, int R, double tol, int maxit, int restart, int precision, std::vector<int> &iters,
               std::vector<double> &relres)
{
    int st;
    std::vector<double> bnorm;
    if ((st = o.norms(o.b(), bnorm))) return st;
    for (auto &b : bnorm) if (b == 0.0) b = 1.0;
    std::vector<double> tolv(R, tol);
    // plain GMRES: FP64, or (FMM_FLOAT2) on the FP64-quality matvec with float-float translations
    if (precision == FMM_FP64 || precision == FMM_FLOAT2)
        return gmres_core(o, o.b(), o.x(), R, tolv, maxit, restart, precision, bnorm, iters, relres);
    iters.assign(R, 0);
    relres.assign(R, 0.0);
    std::vector<double> rn, itol(R);
    std::vector<int> it_in;
    std::vector<double> rr_in;
    int total = 0;
    // a zero initial guess needs no FP64 matvec for its residual: the FP64 matvec costs about
    // 20 mixed ones, so the first correction is solved to 0.5 tol (no lower than 5e-7, a few
    // times the mixed operator's noise: inner targets near that floor stall GMRES) and one or
    // two FP64 residuals confirm it
    std::vector<double> xn;
    if ((st = o.norms(o.x(), xn))) return st;
    bool x_zero = true;
    for (double v : xn) x_zero = x_zero && v == 0.0;
    // columns whose FP64 residual is still wanted: a column below tol gets no correction, so
    // its residual does not change and need not be recomputed
    std::vector<int> need(R, 1);
    std::vector<double> rn_prev(R, 0.0);
    for (int outer = 0; outer < 20; outer++) {
        // residual in FP64; columns already below tol get a zero right-hand side
        if (outer == 0 && x_zero) {
            if ((st = o.copy(o.w(), o.b()))) return st;
        } else {
            o.active(need);
            if ((st = o.matvec(o.x(), o.w(), residual_precision()))) return st;
            o.axpby(1.0, o.b(), -1.0, o.w());
        }
        o.active(std::vector<int>(R, 1));
        if ((st = o.norms(o.w(), rn))) return st;
        for (int r = 0; r < R; r++)
            if (!need[r]) rn[r] = rn_prev[r];
        rn_prev = rn;
        int any = 0;
        std::vector<double> keep(R);
        for (int r = 0; r < R; r++) {
            relres[r] = rn[r] / bnorm[r];
            need[r] = relres[r] > tol;
            keep[r] = relres[r] > tol ? 1.0 : 0.0;
            any |= relres[r] > tol;
            itol[r] = std::min(0.1, std::max(5e-7, 0.5 * tol / std::max(relres[r], 1e-300)));
        }
        if (!any || total >= maxit) break;
        if ((st = o.scale(keep, o.w(), o.w()))) return st;
        if ((st = o.zero(o.d()))) return st;
        std::vector<double> rref(rn);
        for (auto &v : rref) if (v == 0.0) v = 1.0;
        // gmres_core uses r(), w() (as W) and the basis: move the right-hand sides out of w()
        double2 *rhs = o.tmp_alloc();
        if (!rhs) return FMM_ERR_CUDA;
        if ((st = o.copy(rhs, o.w()))) { o.tmp_free(rhs); return st; }
        // the mixed matvec is not bitwise reproducible (FP32 atomics), so its residual floor is
        // ~1e-7; an inner solve that cannot get further hands back to an FP64 residual after a
        // few restart cycles instead of running to maxit
        int inner_cap = std::min(maxit - total, std::max(4 * restart, 200));
        st = gmres_core(o, rhs, o.d(), R, itol, inner_cap, restart, FMM_MIXED, rref, it_in, rr_in);
        o.tmp_free(rhs);
        if (st) return st;
        int step = 0;
        for (int r = 0; r < R; r++) {
            iters[r] += it_in[r];
            step = std::max(step, it_in[r]);
        }
        total += std::max(step, 1);
        o.axpby(1.0, o.d(), 1.0, o.x());
    }
    return FMM_OK;
}

} // namespace fmm
