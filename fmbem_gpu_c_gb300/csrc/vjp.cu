// fmm_vjp: reverse-mode derivative of a far-field objective with respect to the vertex
// positions (the adjoint path; the reference has none).
//
// With A(V) x = b(V) (b the plane wave at the centroids) and p = F(V) x the scattered field at
// fixed exterior points, a cotangent pbar of p (dJ = 2 Re pbar^H dp) gives
//     dJ/dV = 2 Re[ pbar^H (dF/dV) x ] + 2 Re[ mu^T (db/dV - (dA/dV) x) ],
// where mu = conj(lambda) solves A^T mu = F^T conj(pbar) (the adjoint system A^H lambda =
// F^H pbar, conjugated).  dA/dV is the derivative of the operator this library applies: the
// octree, truncation orders and box centres are held fixed and A is split as the matvec
// splits it:
//   near pairs (i, j)     direct quadrature, differentiated pair by pair;
//   far pairs, target i   sum_j A_ij x_j = sum_nm D_i[nm] R_n^m(c_i - C_i) with D the leaf
//                         local of the forward pass on x: differentiate in c_i;
//   far pairs, source j   sum_i mu_i A_ij = sum_nm Psi_j[nm] U_j[n,-m] with Psi the leaf local
//                         of the transposed pass on mu (U_j[n,-m] integrates R_n^m over T_j):
//                         differentiate the integral over T_j in its vertices.
// Every local derivative is exact to rounding: forward-mode dual numbers through the same
// quadrature rules, Green's function and regular basis.  The basis is evaluated through
// u = (x + i y)/r and polynomials in z/r (Q_n^m = st^m q_n^m), which stays smooth on the
// z-axis where (theta, phi) do not.
#include "plan.h"
#include <algorithm>
#include <vector>

namespace fmm {

// copies of the regular rules of tables.cu (rule_tables), uploaded on first use
__constant__ double v_rule_bary[2][16 * 3];
__constant__ double v_rule_w[2][16];
__constant__ int v_rule_n[2];
// the 8-point Gauss rule on [-1, 1] of the Burton-Miller edge integrals (tables.cu)
constexpr int V_LINE_PTS = 8;
__constant__ double v_line_x[V_LINE_PTS], v_line_w[V_LINE_PTS];

static int upload_vjp_rules()
{
    static int dev_done = -1;
    int dev = 0;
    FMM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev_done == dev) return FMM_OK;
    double bary[2][48], w[2][16];
    int n[2];
    rule_tables(bary, w, n);
    FMM_CUDA_TRY(cudaMemcpyToSymbol(v_rule_bary, bary, sizeof(bary)));
    FMM_CUDA_TRY(cudaMemcpyToSymbol(v_rule_w, w, sizeof(w)));
    FMM_CUDA_TRY(cudaMemcpyToSymbol(v_rule_n, n, sizeof(n)));
    double lx[V_LINE_PTS], lw[V_LINE_PTS];
    line_rule(V_LINE_PTS, lx, lw);
    FMM_CUDA_TRY(cudaMemcpyToSymbol(v_line_x, lx, sizeof(lx)));
    FMM_CUDA_TRY(cudaMemcpyToSymbol(v_line_w, lw, sizeof(lw)));
    dev_done = dev;
    return FMM_OK;
}

// ----------------------------------------------------------------------------- dual numbers
template <int N> struct Dn {
    double v, d[N];
};

template <int N> __device__ __forceinline__ Dn<N> dconst(double a)
{
    Dn<N> r;
    r.v = a;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = 0.0;
    return r;
}
template <int N> __device__ __forceinline__ Dn<N> dvar(double a, int slot)
{
    Dn<N> r = dconst<N>(a);
    r.d[slot] = 1.0;
    return r;
}
template <int N> __device__ __forceinline__ Dn<N> operator+(const Dn<N> &a, const Dn<N> &b)
{
    Dn<N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int N> __device__ __forceinline__ Dn<N> operator-(const Dn<N> &a, const Dn<N> &b)
{
    Dn<N> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int N> __device__ __forceinline__ Dn<N> operator-(const Dn<N> &a)
{
    Dn<N> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = -a.d[i];
    return r;
}
template <int N> __device__ __forceinline__ Dn<N> operator*(const Dn<N> &a, const Dn<N> &b)
{
    Dn<N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int N> __device__ __forceinline__ Dn<N> operator*(double s, const Dn<N> &a)
{
    Dn<N> r;
    r.v = s * a.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = s * a.d[i];
    return r;
}
template <int N> __device__ __forceinline__ Dn<N> operator/(const Dn<N> &a, const Dn<N> &b)
{
    Dn<N> r;
    double inv = 1.0 / b.v;
    r.v = a.v * inv;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
    return r;
}
template <int N> __device__ __forceinline__ Dn<N> dsqrt(const Dn<N> &a)
{
    Dn<N> r;
    r.v = sqrt(a.v);
    double h = 0.5 / r.v;
#pragma unroll
    for (int i = 0; i < N; i++) r.d[i] = a.d[i] * h;
    return r;
}
template <int N> __device__ __forceinline__ void dsincos(const Dn<N> &a, Dn<N> &s, Dn<N> &c)
{
    double sv, cv;
    sincos(a.v, &sv, &cv);
    s.v = sv;
    c.v = cv;
#pragma unroll
    for (int i = 0; i < N; i++) {
        s.d[i] = cv * a.d[i];
        c.d[i] = -sv * a.d[i];
    }
}

// complex dual
template <int N> struct CDn {
    Dn<N> re, im;
};
template <int N> __device__ __forceinline__ CDn<N> cdzero()
{
    CDn<N> r;
    r.re = dconst<N>(0.0);
    r.im = dconst<N>(0.0);
    return r;
}
template <int N> __device__ __forceinline__ CDn<N> cdmul(const CDn<N> &a, const CDn<N> &b)
{
    CDn<N> r;
    r.re = a.re * b.re - a.im * b.im;
    r.im = a.re * b.im + a.im * b.re;
    return r;
}
// acc += c * a  (c a plain complex constant)
template <int N> __device__ __forceinline__ void cdmac(CDn<N> &acc, double2 c, const CDn<N> &a)
{
    acc.re.v += c.x * a.re.v - c.y * a.im.v;
    acc.im.v += c.x * a.im.v + c.y * a.re.v;
#pragma unroll
    for (int i = 0; i < N; i++) {
        acc.re.d[i] += c.x * a.re.d[i] - c.y * a.im.d[i];
        acc.im.d[i] += c.x * a.im.d[i] + c.y * a.re.d[i];
    }
}
// derivative of Re(w * z) for a plain complex w, one slot
template <int N> __device__ __forceinline__ double re_wd(double2 w, const CDn<N> &z, int i)
{
    return w.x * z.re.d[i] - w.y * z.im.d[i];
}

// ----------------------------------------------------------------------------- kernels in duals
template <int N>
__device__ void tri_normal_d(const Dn<N> *nod, Dn<N> *nc, Dn<N> &J)
{
    Dn<N> u0 = nod[0] - nod[6], u1 = nod[1] - nod[7], u2 = nod[2] - nod[8];
    Dn<N> v0 = nod[3] - nod[6], v1 = nod[4] - nod[7], v2 = nod[5] - nod[8];
    nc[0] = u1 * v2 - u2 * v1;
    nc[1] = u2 * v0 - u0 * v2;
    nc[2] = u0 * v1 - u1 * v0;
    J = dsqrt(nc[0] * nc[0] + nc[1] * nc[1] + nc[2] * nc[2]);
}

// G(x, y) = exp(ikr)/(4 pi r) (kern 0) or dG/dn_x = G (ik - 1/r) (x - y).nh / r (kern 1); the
// caller passes the unit normal
template <int N>
__device__ CDn<N> green_d(double k, const Dn<N> *x, const Dn<N> *y, const Dn<N> *nh, int kern)
{
    Dn<N> d0 = x[0] - y[0], d1 = x[1] - y[1], d2 = x[2] - y[2];
    Dn<N> r = dsqrt(d0 * d0 + d1 * d1 + d2 * d2);
    Dn<N> s, c;
    dsincos(k * r, s, c);
    Dn<N> inv = dconst<N>(1.0 / (4.0 * FMM_PI)) / r;
    CDn<N> g;
    g.re = c * inv;
    g.im = s * inv;
    if (!kern) return g;
    Dn<N> dn = (d0 * nh[0] + d1 * nh[1] + d2 * nh[2]) / r;
    Dn<N> ar = -(dconst<N>(1.0) / r);
    CDn<N> f;
    f.re = ar * dn;
    f.im = k * dn;
    return cdmul(g, f);
}

template <int N>
__device__ CDn<N> elem_integral_d(double k, const Dn<N> *nod, const Dn<N> *y, int rule, int kern)
{
    Dn<N> nc[3], J;
    tri_normal_d(nod, nc, J);
    Dn<N> nh[3] = {nc[0] / J, nc[1] / J, nc[2] / J};
    CDn<N> acc = cdzero<N>();
    int nq = v_rule_n[rule];
    for (int q = 0; q < nq; q++) {
        const double *b = &v_rule_bary[rule][3 * q];
        Dn<N> x[3];
        for (int a = 0; a < 3; a++) x[a] = b[0] * nod[a] + b[1] * nod[3 + a] + b[2] * nod[6 + a];
        CDn<N> g = green_d(k, x, y, nh, kern);
        Dn<N> wq = v_rule_w[rule][q] * J;
        acc.re = acc.re + wq * g.re;
        acc.im = acc.im + wq * g.im;
    }
    return acc;
}

template <int N>
__device__ void centroid_d(const Dn<N> *nod, Dn<N> *y)
{
    for (int a = 0; a < 3; a++) {
        Dn<N> c23 = 0.5 * (nod[3 + a] + nod[6 + a]);
        y[a] = nod[a] + (2.0 / 3.0) * (c23 - nod[a]);
    }
}

// self term: centroid split into three sub-triangles with the collapsed rule
template <int N>
__device__ CDn<N> elem_integral_sgl_d(double k, const Dn<N> *nod, int kern)
{
    Dn<N> y[3];
    centroid_d(nod, y);
    CDn<N> acc = cdzero<N>();
    for (int s = 0; s < 3; s++) {
        Dn<N> sub[9];
        int a0 = 3 * s, b0 = 3 * ((s + 1) % 3);
        for (int t = 0; t < 3; t++) {
            sub[t] = nod[a0 + t];
            sub[3 + t] = nod[b0 + t];
            sub[6 + t] = y[t];
        }
        CDn<N> part = elem_integral_d(k, sub, y, 0, kern);
        acc.re = acc.re + part.re;
        acc.im = acc.im + part.im;
    }
    return acc;
}

// ---------------------------------------------------------------- Burton-Miller terms in duals
// The same forms as tables.cu (elem_integrals_fused, hyper_edges, elem_hyper_self); the numbers of
// edge segments follow from the values, as there, and are held fixed by the derivative.
__device__ __forceinline__ int edge_segments_v(double len, double dist)
{
    double m = ceil(len / fmax(dist, 1e-12 * len));
    return m > 64.0 ? 64 : (int)m;
}

// int_T dG(x, y)/dn_y dS_x, ny the unit normal at y
template <int N>
__device__ CDn<N> elem_dGdny_d(double k, const Dn<N> *nod, const Dn<N> *y, const Dn<N> *ny, int rule)
{
    Dn<N> nc[3], J;
    tri_normal_d(nod, nc, J);
    CDn<N> acc = cdzero<N>();
    int nq = v_rule_n[rule];
    for (int q = 0; q < nq; q++) {
        const double *b = &v_rule_bary[rule][3 * q];
        Dn<N> x[3];
        for (int a = 0; a < 3; a++) x[a] = b[0] * nod[a] + b[1] * nod[3 + a] + b[2] * nod[6 + a];
        CDn<N> g = green_d(k, x, y, ny, 1);   // G (ik - 1/r) (x - y).ny / r
        Dn<N> wq = v_rule_w[rule][q] * J;
        acc.re = acc.re - wq * g.re;
        acc.im = acc.im - wq * g.im;
    }
    return acc;
}

// int_T d2G/dn_x dn_y dS_x at y off T: k^2 (ny.nT) int_T G - oint (ny x grad_y G) . dl
template <int N>
__device__ CDn<N> elem_hyper_near_d(double k, const Dn<N> *nod, const Dn<N> *y, const Dn<N> *ny, int rule)
{
    Dn<N> nc[3], J;
    tri_normal_d(nod, nc, J);
    CDn<N> S = elem_integral_d(k, nod, y, rule, 0);
    Dn<N> dn = (ny[0] * nc[0] + ny[1] * nc[1] + ny[2] * nc[2]) / J;
    CDn<N> line = cdzero<N>();
    for (int e = 0; e < 3; e++) {
        const Dn<N> *va = nod + 3 * e, *vb = nod + 3 * ((e + 1) % 3);
        Dn<N> t[3] = {vb[0] - va[0], vb[1] - va[1], vb[2] - va[2]}, a[3] = {y[0] - va[0], y[1] - va[1], y[2] - va[2]};
        double tt = t[0].v * t[0].v + t[1].v * t[1].v + t[2].v * t[2].v, len = sqrt(tt);
        double sc = fmin(fmax((a[0].v * t[0].v + a[1].v * t[1].v + a[2].v * t[2].v) / tt, 0.0), 1.0);
        double e0 = a[0].v - sc * t[0].v, e1 = a[1].v - sc * t[1].v, e2 = a[2].v - sc * t[2].v;
        int nseg = edge_segments_v(len, sqrt(e0 * e0 + e1 * e1 + e2 * e2));
        Dn<N> tn0 = t[1] * ny[2] - t[2] * ny[1], tn1 = t[2] * ny[0] - t[0] * ny[2], tn2 = t[0] * ny[1] - t[1] * ny[0];
        for (int g = 0; g < nseg; g++)
            for (int q = 0; q < V_LINE_PTS; q++) {
                double s = (g + 0.5 + 0.5 * v_line_x[q]) / nseg, w = 0.5 * v_line_w[q] / nseg;
                Dn<N> d0 = a[0] - s * t[0], d1 = a[1] - s * t[1], d2 = a[2] - s * t[2];
                Dn<N> r2 = d0 * d0 + d1 * d1 + d2 * d2, r = dsqrt(r2);
                Dn<N> sn, cs;
                dsincos(k * r, sn, cs);
                Dn<N> f = (w / (4.0 * FMM_PI)) * (d0 * tn0 + d1 * tn1 + d2 * tn2) / r2;
                Dn<N> ar = -(dconst<N>(1.0) / r);
                // e^{ikr} (ik - 1/r) f
                line.re = line.re + f * (cs * ar - k * sn);
                line.im = line.im + f * (k * cs + sn * ar);
            }
    }
    Dn<N> kk = (k * k) * dn;
    CDn<N> out;
    out.re = kk * S.re - line.re;
    out.im = kk * S.im - line.im;
    return out;
}

// Hadamard finite part of int_T d2G/dn_x dn_y at the centroid of the flat element T
template <int N>
__device__ CDn<N> elem_hyper_self_d(double k, const Dn<N> *nod)
{
    Dn<N> c[3];
    centroid_d(nod, c);
    CDn<N> ang = cdzero<N>();
    for (int e = 0; e < 3; e++) {
        const Dn<N> *va = nod + 3 * e, *vb = nod + 3 * ((e + 1) % 3);
        Dn<N> t[3] = {vb[0] - va[0], vb[1] - va[1], vb[2] - va[2]}, u[3] = {va[0] - c[0], va[1] - c[1], va[2] - c[2]};
        Dn<N> c0 = u[1] * t[2] - u[2] * t[1], c1 = u[2] * t[0] - u[0] * t[2], c2 = u[0] * t[1] - u[1] * t[0];
        Dn<N> hL = dsqrt(c0 * c0 + c1 * c1 + c2 * c2);
        double len = sqrt(t[0].v * t[0].v + t[1].v * t[1].v + t[2].v * t[2].v);
        int nseg = edge_segments_v(len, hL.v / len);
        for (int g = 0; g < nseg; g++)
            for (int q = 0; q < V_LINE_PTS; q++) {
                double s = (g + 0.5 + 0.5 * v_line_x[q]) / nseg, w = 0.5 * v_line_w[q] / nseg;
                Dn<N> d0 = u[0] + s * t[0], d1 = u[1] + s * t[1], d2 = u[2] + s * t[2];
                Dn<N> r = dsqrt(d0 * d0 + d1 * d1 + d2 * d2);
                Dn<N> sn, cs;
                dsincos(k * r, sn, cs);
                Dn<N> f = w * hL / (r * r * r);
                ang.re = ang.re + f * cs;
                ang.im = ang.im + f * sn;
            }
    }
    CDn<N> out;
    out.re = (-1.0 / (4.0 * FMM_PI)) * ang.re;
    out.im = (-1.0 / (4.0 * FMM_PI)) * ang.im + dconst<N>(2.0 * FMM_PI * k / (4.0 * FMM_PI));
    return out;
}

// spherical Bessel j_n(x), n < NB, Miller's backward recurrence normalised by j0 or j1, in duals
template <int N>
__device__ void sph_jn_d(int NB, const Dn<N> &x, Dn<N> *j)
{
    Dn<N> s, c;
    dsincos(x, s, c);
    Dn<N> j0 = s / x, j1 = s / (x * x) - c / x;
    int big = NB > (int)x.v ? NB : (int)x.v;
    int start = big + 40 + (int)(4.0 * sqrt((double)big + 1.0));
    Dn<N> fp1 = dconst<N>(0.0), f = dconst<N>(1e-300), f1 = dconst<N>(0.0);
    for (int n = start; n >= 1; n--) {
        Dn<N> fm1 = ((2.0 * n + 1.0) * f) / x - fp1;
        fp1 = f;
        f = fm1;
        if (n - 1 < NB) j[n - 1] = f;
        if (n - 1 == 1) f1 = f;
        if (fabs(f.v) > 1e250) {
            f = 1e-250 * f;
            fp1 = 1e-250 * fp1;
            f1 = 1e-250 * f1;
            for (int q = (n - 1 < NB ? n - 1 : NB); q < NB; q++) j[q] = 1e-250 * j[q];
        }
    }
    Dn<N> scale = (fabs(j0.v) > fabs(j1.v)) ? j0 / f : j1 / f1;
    for (int n = 0; n < NB; n++) j[n] = j[n] * scale;
}

constexpr int VJP_PMAX = 24; // largest leaf order (plus one for gradient expansions) handled here

// out[e] = sum_{n < P, |m| <= n} coef[e][n^2+n+m] R_n^m(v), R_n^m = j_n(kr) q_n^|m|(z/r) u^m
// (u^{-m} read as conj(u)^m), for NE expansions at one dual point v
template <int N, int NE>
__device__ void eval_expansions_d(int P, double k, const Dn<N> *v, const double2 *const *coef, CDn<N> *out)
{
    Dn<N> r = dsqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    Dn<N> ct = v[2] / r;
    CDn<N> u;
    u.re = v[0] / r;
    u.im = v[1] / r;
    Dn<N> jn[VJP_PMAX];
    sph_jn_d(P, k * r, jn);
    for (int e = 0; e < NE; e++) out[e] = cdzero<N>();
    CDn<N> um = cdzero<N>();
    um.re = dconst<N>(1.0);
    double cmm = 0.28209479177387814; // q_0^0 = 1/sqrt(4 pi)
    for (int m = 0; m < P; m++) {
        if (m > 0) {
            cmm *= sqrt((2.0 * m + 1.0) / (2.0 * m));
            um = cdmul(um, u);
        }
        Dn<N> q2 = dconst<N>(0.0), q1 = dconst<N>(0.0);
        for (int n = m; n < P; n++) {
            Dn<N> q;
            if (n == m) q = dconst<N>(cmm);
            else if (n == m + 1) q = (sqrt(2.0 * m + 3.0) * cmm) * ct;
            else {
                double a = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
                double b = sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) / (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
                q = a * (ct * q1 - b * q2);
            }
            q2 = q1;
            q1 = q;
            Dn<N> base = jn[n] * q;
            CDn<N> Rp, Rm;
            Rp.re = base * um.re;
            Rp.im = base * um.im;
            Rm.re = Rp.re;
            Rm.im = -Rp.im;
            for (int e = 0; e < NE; e++) {
                cdmac(out[e], coef[e][n * n + n + m], Rp);
                if (m > 0) cdmac(out[e], coef[e][n * n + n - m], Rm);
            }
        }
    }
}

__device__ __forceinline__ void load_tri_d(const double *V, const int *F, int e, double *nod)
{
    for (int t = 0; t < 3; t++)
        for (int a = 0; a < 3; a++) nod[3 * t + a] = V[3 * F[3 * e + t] + a];
}

__device__ __forceinline__ void add_vertex_grad(double *grad, const int *F, int e, const double *g9)
{
    for (int t = 0; t < 3; t++)
        for (int a = 0; a < 3; a++) atomicAdd(&grad[3 * F[3 * e + t] + a], g9[3 * t + a]);
}

// ----------------------------------------------------------------------------- VJP kernels
// the far-field operator F_kj = -int_{T_j} (b G + c dG/dn_x)(x, p_k) dS (fmm_far_field) with
// dual-number vertex derivatives
template <int N>
__device__ __forceinline__ CDn<N> far_entry_d(double k, const Dn<N> *nod, const Dn<N> *y, int rule, double2 nb, double2 nc)
{
    CDn<N> f = cdzero<N>();
    if (nb.x != 0.0 || nb.y != 0.0) cdmac(f, nb, elem_integral_d(k, nod, y, rule, 0));
    if (nc.x != 0.0 || nc.y != 0.0) cdmac(f, nc, elem_integral_d(k, nod, y, rule, 1));
    return f;
}

// right-hand side of the conjugated adjoint system: rhs_j = sum_k F_kj conj(pbar_k)
__global__ void vjp_adjoint_rhs_kernel(const double *V, const int *F, int nf, double k, int rule, double2 nb, double2 nc,
                                       const double *pts, int npts, const double2 *pbar, double2 *rhs);

// 2 Re[ sum_k conj(pbar_k) x_j dF_kj/dV_j ] for the vertices of element j; nb = -b, nc = -c
__global__ void vjp_farpts_kernel(const double *V, const int *F, int nf, double k, int rule, double2 nb, double2 nc,
                                  const double *pts, int npts, const double2 *pbar, const double2 *x, double *grad)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nf; j += gridDim.x * blockDim.x) {
        double nd[9];
        load_tri_d(V, F, j, nd);
        Dn<9> nod[9];
        for (int i = 0; i < 9; i++) nod[i] = dvar<9>(nd[i], i);
        double g9[9] = {0};
        double2 xj = x[j];
        for (int t = 0; t < npts; t++) {
            Dn<9> y[3] = {dconst<9>(pts[3 * t]), dconst<9>(pts[3 * t + 1]), dconst<9>(pts[3 * t + 2])};
            CDn<9> f = far_entry_d(k, nod, y, rule, nb, nc);
            double2 pb = pbar[t];
            // w = conj(pbar) x_j
            double2 w = make_double2(pb.x * xj.x + pb.y * xj.y, pb.x * xj.y - pb.y * xj.x);
            for (int i = 0; i < 9; i++) g9[i] += 2.0 * re_wd(w, f, i);
        }
        add_vertex_grad(grad, F, j, g9);
    }
}

__global__ void vjp_adjoint_rhs_kernel(const double *V, const int *F, int nf, double k, int rule, double2 nb, double2 nc,
                                       const double *pts, int npts, const double2 *pbar, double2 *rhs)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nf; j += gridDim.x * blockDim.x) {
        double nd[9];
        load_tri_d(V, F, j, nd);
        Dn<1> nod[9];
        for (int i = 0; i < 9; i++) nod[i] = dconst<1>(nd[i]);
        double2 acc = make_double2(0.0, 0.0);
        for (int t = 0; t < npts; t++) {
            Dn<1> y[3] = {dconst<1>(pts[3 * t]), dconst<1>(pts[3 * t + 1]), dconst<1>(pts[3 * t + 2])};
            CDn<1> f = far_entry_d(k, nod, y, rule, nb, nc);
            double2 pb = pbar[t];
            acc.x += f.re.v * pb.x + f.im.v * pb.y; // F conj(pbar)
            acc.y += f.im.v * pb.x - f.re.v * pb.y;
        }
        rhs[j] = acc;
    }
}

// 2 Re[ mu_i db_i/dV ] with b_i = exp(i k dir.c_i), c_i the centroid (1/3 per vertex)
__global__ void vjp_rhs_kernel(const double *V, const int *F, int nf, double k, double dx, double dy, double dz,
                               const double2 *mu, double *grad)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x) {
        double nd[9], c[3];
        load_tri_d(V, F, i, nd);
        for (int a = 0; a < 3; a++) c[a] = nd[a] + (2.0 / 3.0) * (0.5 * (nd[3 + a] + nd[6 + a]) - nd[a]);
        double s, co;
        sincos(k * (dx * c[0] + dy * c[1] + dz * c[2]), &s, &co);
        // d b / d c_a = i k dir_a b ;  Re(mu * i k dir_a b) = -k dir_a Im(mu b)
        double2 m = mu[i];
        double imb = m.x * s + m.y * co;
        double d3[3] = {dx, dy, dz}, g9[9];
        for (int t = 0; t < 3; t++)
            for (int a = 0; a < 3; a++) g9[3 * t + a] = 2.0 * (-k * d3[a] * imb) / 3.0;
        add_vertex_grad(grad, F, i, g9);
    }
}

// near pairs: -2 Re[ mu_i x_j dA_ij ], A_ij = b int_Tj G(., c_i) + c int_Tj dG/dn(., c_i);
// slots 0..8 the vertices of T_j, 9..11 the centroid c_i (1/3 to each vertex of T_i)
__global__ void vjp_near_kernel(const double *V, const int *F, int nf, const int *near_beg, const int *near_col,
                                double k, double2 bco, double2 cco, int rule, const double2 *mu, const double2 *x,
                                double *grad)
{
    int lane = threadIdx.x & 31, warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nwt = (gridDim.x * blockDim.x) >> 5;
    for (int i = warp; i < nf; i += nwt) {
        double ndi[9], ci[3];
        load_tri_d(V, F, i, ndi);
        for (int a = 0; a < 3; a++) ci[a] = ndi[a] + (2.0 / 3.0) * (0.5 * (ndi[3 + a] + ndi[6 + a]) - ndi[a]);
        double2 mi = mu[i];
        double gi[9] = {0};
        for (int s = near_beg[i] + lane; s < near_beg[i + 1]; s += 32) {
            int j = near_col[s];
            double nd[9];
            load_tri_d(V, F, j, nd);
            double2 xj = x[j];
            // w = -(mu_i x_j)
            double2 w = make_double2(-(mi.x * xj.x - mi.y * xj.y), -(mi.x * xj.y + mi.y * xj.x));
            double g9[9];
            if (i == j) {
                Dn<9> nod[9];
                for (int q = 0; q < 9; q++) nod[q] = dvar<9>(nd[q], q);
                CDn<9> v = cdzero<9>();
                if (bco.x != 0.0 || bco.y != 0.0) cdmac(v, bco, elem_integral_sgl_d(k, nod, 0));
                if (cco.x != 0.0 || cco.y != 0.0) cdmac(v, cco, elem_integral_sgl_d(k, nod, 1));
                for (int q = 0; q < 9; q++) g9[q] = 2.0 * re_wd(w, v, q);
                add_vertex_grad(grad, F, j, g9);
            } else {
                Dn<12> nod[9], y[3];
                for (int q = 0; q < 9; q++) nod[q] = dvar<12>(nd[q], q);
                for (int a = 0; a < 3; a++) y[a] = dvar<12>(ci[a], 9 + a);
                CDn<12> v = cdzero<12>();
                if (bco.x != 0.0 || bco.y != 0.0) cdmac(v, bco, elem_integral_d(k, nod, y, rule, 0));
                if (cco.x != 0.0 || cco.y != 0.0) cdmac(v, cco, elem_integral_d(k, nod, y, rule, 1));
                for (int q = 0; q < 9; q++) g9[q] = 2.0 * re_wd(w, v, q);
                add_vertex_grad(grad, F, j, g9);
                for (int a = 0; a < 3; a++) {
                    double gc = 2.0 * re_wd(w, v, 9 + a) / 3.0;
                    for (int t = 0; t < 3; t++) gi[3 * t + a] += gc;
                }
            }
        }
        add_vertex_grad(grad, F, i, gi);
    }
}

// far pairs, target side: -2 Re[ mu_i d/dc_i sum_nm D_i[nm] R_n^m(c_i - C) ], 1/3 per vertex
__global__ void vjp_far_target_kernel(const double *V, const int *F, int nf, int pl, double k, const int *elem_leaf,
                                      const double *box_ctr, const double2 *D, const double2 *mu, double *grad)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x) {
        double nd[9];
        load_tri_d(V, F, i, nd);
        int b = elem_leaf[i];
        Dn<3> v[3];
        for (int a = 0; a < 3; a++) {
            double c = nd[a] + (2.0 / 3.0) * (0.5 * (nd[3 + a] + nd[6 + a]) - nd[a]);
            v[a] = dvar<3>(c - box_ctr[3 * b + a], a);
        }
        const double2 *coef[1] = {D + (size_t)b * pl * pl};
        CDn<3> t[1];
        eval_expansions_d<3, 1>(pl, k, v, coef, t);
        double2 m = mu[i], w = make_double2(-m.x, -m.y);
        double g9[9];
        for (int a = 0; a < 3; a++) {
            double gc = 2.0 * re_wd(w, t[0], a) / 3.0;
            for (int q = 0; q < 3; q++) g9[3 * q + a] = gc;
        }
        add_vertex_grad(grad, F, i, g9);
    }
}

// Burton-Miller near pairs: -2 Re[ mu_i x_j d/dV alpha (b K'_ij + c N_ij) ], both elements'
// vertices as dual slots (0..8 source j, 9..17 target i: its centroid and unit normal); the
// self term N_ii (K'_ii = 0) in the element's own 9 slots
__global__ void vjp_near_bm_kernel(const double *V, const int *F, int nf, const int *near_beg, const int *near_col,
                                   double k, double2 bco, double2 cco, double2 alpha, int rule, const double2 *mu,
                                   const double2 *x, double *grad)
{
    int lane = threadIdx.x & 31, warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nwt = (gridDim.x * blockDim.x) >> 5;
    const bool hb = bco.x != 0.0 || bco.y != 0.0, hc = cco.x != 0.0 || cco.y != 0.0;
    for (int i = warp; i < nf; i += nwt) {
        double ndi[9];
        load_tri_d(V, F, i, ndi);
        double2 mi = mu[i];
        double gi[9] = {0};
        for (int s = near_beg[i] + lane; s < near_beg[i + 1]; s += 32) {
            int j = near_col[s];
            double2 xj = x[j];
            // w = -(mu_i x_j alpha)
            double2 mx = make_double2(mi.x * xj.x - mi.y * xj.y, mi.x * xj.y + mi.y * xj.x);
            double2 w = make_double2(-(mx.x * alpha.x - mx.y * alpha.y), -(mx.x * alpha.y + mx.y * alpha.x));
            if (i == j) {
                if (!hc) continue;
                Dn<9> nod[9];
                for (int q = 0; q < 9; q++) nod[q] = dvar<9>(ndi[q], q);
                CDn<9> v = cdzero<9>();
                cdmac(v, cco, elem_hyper_self_d(k, nod));
                double g9[9];
                for (int q = 0; q < 9; q++) g9[q] = 2.0 * re_wd(w, v, q);
                add_vertex_grad(grad, F, j, g9);
            } else {
                double nd[9];
                load_tri_d(V, F, j, nd);
                Dn<18> nod[9], tgt[9], y[3], ncy[3], Jy;
                for (int q = 0; q < 9; q++) {
                    nod[q] = dvar<18>(nd[q], q);
                    tgt[q] = dvar<18>(ndi[q], 9 + q);
                }
                centroid_d(tgt, y);
                tri_normal_d(tgt, ncy, Jy);
                Dn<18> ny[3] = {ncy[0] / Jy, ncy[1] / Jy, ncy[2] / Jy};
                CDn<18> v = cdzero<18>();
                if (hb) cdmac(v, bco, elem_dGdny_d(k, nod, y, ny, rule));
                if (hc) cdmac(v, cco, elem_hyper_near_d(k, nod, y, ny, rule));
                double g9[9];
                for (int q = 0; q < 9; q++) g9[q] = 2.0 * re_wd(w, v, q);
                add_vertex_grad(grad, F, j, g9);
                for (int q = 0; q < 9; q++) gi[q] += 2.0 * re_wd(w, v, 9 + q);
            }
        }
        add_vertex_grad(grad, F, i, gi);
    }
}

// Burton-Miller far pairs, target side: -2 Re[ mu_i alpha d/dV (n_i . grad phi(c_i)) ] with
// phi = sum_nm D_i[nm] R_n^m(. - C), grad phi from its derivative expansions (Dz, Dp, Dm)
__global__ void vjp_far_target_bm_kernel(const double *V, const int *F, int nf, int pl, double k, double2 alpha,
                                         const int *elem_leaf, const double *box_ctr, const double2 *Dz,
                                         const double2 *Dp, const double2 *Dm, const double2 *mu, double *grad)
{
    const int po = pl + 1;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x) {
        double nd[9];
        load_tri_d(V, F, i, nd);
        int b = elem_leaf[i];
        Dn<9> nod[9], c[3], nc[3], J;
        for (int q = 0; q < 9; q++) nod[q] = dvar<9>(nd[q], q);
        centroid_d(nod, c);
        tri_normal_d(nod, nc, J);
        Dn<9> v[3];
        for (int a = 0; a < 3; a++) v[a] = c[a] - dconst<9>(box_ctr[3 * b + a]);
        const double2 *coef[3] = {Dz + (size_t)b * po * po, Dp + (size_t)b * po * po, Dm + (size_t)b * po * po};
        CDn<9> e[3];
        eval_expansions_d<9, 3>(po, k, v, coef, e);
        CDn<9> gx, gy;
        gx.re = 0.5 * (e[1].re + e[2].re);
        gx.im = 0.5 * (e[1].im + e[2].im);
        gy.re = 0.5 * (e[1].im - e[2].im);
        gy.im = -0.5 * (e[1].re - e[2].re);
        CDn<9> f;
        f.re = (gx.re * nc[0] + gy.re * nc[1] + e[0].re * nc[2]) / J;
        f.im = (gx.im * nc[0] + gy.im * nc[1] + e[0].im * nc[2]) / J;
        double2 m = mu[i];
        double2 w = make_double2(-(m.x * alpha.x - m.y * alpha.y), -(m.x * alpha.y + m.y * alpha.x));
        double g9[9];
        for (int q = 0; q < 9; q++) g9[q] = 2.0 * re_wd(w, f, q);
        add_vertex_grad(grad, F, i, g9);
    }
}

// 2 Re[ mu_i d/dV alpha i k (d.n_i) exp(i k d.c_i) ]: the Burton-Miller term of the plane-wave
// right-hand side
__global__ void vjp_rhs_bm_kernel(const double *V, const int *F, int nf, double k, double dx, double dy, double dz,
                                  double2 alpha, const double2 *mu, double *grad)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x) {
        double nd[9];
        load_tri_d(V, F, i, nd);
        Dn<9> nod[9], c[3], nc[3], J;
        for (int q = 0; q < 9; q++) nod[q] = dvar<9>(nd[q], q);
        centroid_d(nod, c);
        tri_normal_d(nod, nc, J);
        Dn<9> ph = k * (dx * c[0] + dy * c[1] + dz * c[2]);
        Dn<9> kd = k * ((dx * nc[0] + dy * nc[1] + dz * nc[2]) / J);
        Dn<9> sn, cs;
        dsincos(ph, sn, cs);
        // alpha i kd (cs + i sn) = alpha kd (-sn + i cs)
        CDn<9> t;
        t.re = -(kd * sn);
        t.im = kd * cs;
        CDn<9> f = cdzero<9>();
        cdmac(f, alpha, t);
        double2 m = mu[i];
        double g9[9];
        for (int q = 0; q < 9; q++) g9[q] = 2.0 * re_wd(m, f, q);
        add_vertex_grad(grad, F, i, g9);
    }
}

// Coefficients of the derivatives of a regular expansion sum Psi[nm] R_n^m of order pl as
// expansions of order pl + 1 (from the G&D recurrences of dR/dz and (d/dx +- i d/dy) R):
//   dz  : k [ a(n,m) Psi_{n+1}^m - a(n-1,m) Psi_{n-1}^m ]
//   d+  : k [ b(n,-m) Psi_{n-1}^{m-1} - b(n+1,m-1) Psi_{n+1}^{m-1} ]
//   d-  : k [ b(n,m) Psi_{n-1}^{m+1} - b(n+1,-m-1) Psi_{n+1}^{m+1} ]
__global__ void deriv_coef_kernel(int nb, int pl, double k, const double2 *Psi, double2 *Dz, double2 *Dp, double2 *Dm)
{
    int po = pl + 1, po2 = po * po;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < (size_t)nb * po2; idx += (size_t)gridDim.x * blockDim.x) {
        int b = (int)(idx / po2), i = (int)(idx % po2);
        int n = (int)sqrt((double)i);
        while (n * n > i) n--;
        while ((n + 1) * (n + 1) <= i) n++;
        int m = i - n * n - n;
        const double2 *S = Psi + (size_t)b * pl * pl;
        auto at = [&](int nn, int mm) -> double2 {
            if (nn < 0 || nn >= pl || mm > nn || mm < -nn) return make_double2(0.0, 0.0);
            return S[nn * nn + nn + mm];
        };
        double2 a1 = at(n + 1, m), a0 = at(n - 1, m);
        double ca1 = coefA(n, m), ca0 = coefA(n - 1, m);
        Dz[idx] = make_double2(k * (ca1 * a1.x - ca0 * a0.x), k * (ca1 * a1.y - ca0 * a0.y));
        double2 p0 = at(n - 1, m - 1), p1 = at(n + 1, m - 1);
        double cp0 = coefB(n, -m), cp1 = coefB(n + 1, m - 1);
        Dp[idx] = make_double2(k * (cp0 * p0.x - cp1 * p1.x), k * (cp0 * p0.y - cp1 * p1.y));
        double2 q0 = at(n - 1, m + 1), q1 = at(n + 1, m + 1);
        double cq0 = coefB(n, m), cq1 = coefB(n + 1, -m - 1);
        Dm[idx] = make_double2(k * (cq0 * q0.x - cq1 * q1.x), k * (cq0 * q0.y - cq1 * q1.y));
    }
}

// far pairs, source side: -2 Re[ x_j d/dV_j sum_q w_q (b phi(y_q) J + c grad phi(y_q) . Nc) ]
// with phi = sum_nm Psi_j[nm] R_n^m(. - C) and Nc = J nh the unnormalised normal
__global__ void vjp_far_source_kernel(const double *V, const int *F, int nf, int pl, double k, int rule, double2 bco,
                                      double2 cco, const int *elem_leaf, const double *box_ctr, const double2 *Psi,
                                      const double2 *Dz, const double2 *Dp, const double2 *Dm, const double2 *x,
                                      double *grad)
{
    const int po = pl + 1;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nf; j += gridDim.x * blockDim.x) {
        double nd[9];
        load_tri_d(V, F, j, nd);
        int b = elem_leaf[j];
        Dn<9> nod[9];
        for (int i = 0; i < 9; i++) nod[i] = dvar<9>(nd[i], i);
        Dn<9> nc[3], J;
        tri_normal_d(nod, nc, J);
        // the order pl expansion zero-padded to pl + 1 shares the evaluation with its derivatives
        const double2 *coef[4] = {nullptr, Dz + (size_t)b * po * po, Dp + (size_t)b * po * po, Dm + (size_t)b * po * po};
        CDn<9> S = cdzero<9>();
        int nq = v_rule_n[rule];
        for (int q = 0; q < nq; q++) {
            const double *bb = &v_rule_bary[rule][3 * q];
            Dn<9> v[3];
            for (int a = 0; a < 3; a++)
                v[a] = bb[0] * nod[a] + bb[1] * nod[3 + a] + bb[2] * nod[6 + a] - dconst<9>(box_ctr[3 * b + a]);
            CDn<9> e[4];
            const double2 *c1[1] = {Psi + (size_t)b * pl * pl};
            eval_expansions_d<9, 1>(pl, k, v, c1, e);
            eval_expansions_d<9, 3>(po, k, v, coef + 1, e + 1);
            // grad phi: dx = (d+ + d-)/2, dy = (d+ - d-)/(2i), dz
            CDn<9> gx, gy;
            gx.re = 0.5 * (e[2].re + e[3].re);
            gx.im = 0.5 * (e[2].im + e[3].im);
            gy.re = 0.5 * (e[2].im - e[3].im);
            gy.im = -0.5 * (e[2].re - e[3].re);
            CDn<9> dn;
            dn.re = gx.re * nc[0] + gy.re * nc[1] + e[1].re * nc[2];
            dn.im = gx.im * nc[0] + gy.im * nc[1] + e[1].im * nc[2];
            CDn<9> phiJ;
            phiJ.re = e[0].re * J;
            phiJ.im = e[0].im * J;
            double wq = v_rule_w[rule][q];
            CDn<9> t = cdzero<9>();
            cdmac(t, bco, phiJ);
            cdmac(t, cco, dn);
            S.re = S.re + wq * t.re;
            S.im = S.im + wq * t.im;
        }
        double2 xj = x[j], w = make_double2(-xj.x, -xj.y);
        double g9[9];
        for (int i = 0; i < 9; i++) g9[i] = 2.0 * re_wd(w, S, i);
        add_vertex_grad(grad, F, j, g9);
    }
}

// g_beta[j] = i k ( (w_j - z_j) x_j - (alpha/2) mu_j x_j ): the admittance derivative per
// element (see fmm_vjp_admittance)
__global__ void vjp_admittance_kernel(int nf, double k, double2 alpha, const double2 *w, const double2 *z,
                                      const double2 *mu, const double2 *x, double2 *g)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nf; j += gridDim.x * blockDim.x) {
        double2 gb = cmul(csub(w[j], z[j]), x[j]);
        double2 ga = cmul(mu[j], x[j]);
        double2 t = csub(gb, cscale(cmul(alpha, ga), 0.5));
        g[j] = make_double2(-k * t.y, k * t.x);
    }
}

} // namespace fmm

using namespace fmm;

static std::vector<double> leaf_centres(const Plan *P)
{
    const LevelDev &L = P->lev[P->lmax];
    std::vector<double> ctr(3 * (size_t)L.nb);
    double h = ldexp(1.0, -P->lmax), h2 = ldexp(1.0, -P->lmax - 1);
    for (int i = 0; i < L.nb; i++) {
        int x, y, z;
        box_xyz(P->tree.sets[P->lmax][i], P->lmax, &x, &y, &z);
        ctr[3 * i] = P->tree.d * (h * x + h2) + P->tree.pt_min[0];
        ctr[3 * i + 1] = P->tree.d * (h * y + h2) + P->tree.pt_min[1];
        ctr[3 * i + 2] = P->tree.d * (h * z + h2) + P->tree.pt_min[2];
    }
    return ctr;
}

namespace fmm {
int solve_transposed(Plan *P, const double2 *rhs_dev, double2 *x_dev, double tol, int maxit, int restart, int precision,
                     int *iters, double *relres);
}

extern "C" int fmm_vjp(fmm_plan *plan, const cuDoubleComplex *x, const double *dir, const double *pts, int npts,
                       const cuDoubleComplex *pbar, double tol, int precision, double *grad, cuDoubleComplex *lambda)
{
    Plan *P = (Plan *)plan;
    if (!P || !x || !pts || npts < 1 || !pbar || !grad || !(tol > 0)) { fmm_set_error("fmm_vjp: invalid argument"); return FMM_ERR_ARG; }
    if (precision != FMM_FP64 && precision != FMM_MIXED) { fmm_set_error("fmm_vjp: unknown precision"); return FMM_ERR_ARG; }
    if (P->pleaf + 1 > VJP_PMAX) { fmm_set_error("fmm_vjp: leaf order %d above %d", P->pleaf, VJP_PMAX - 1); return FMM_ERR_ARG; }

    int nf = P->nf, nv = P->nv, pl = P->pleaf, lmax = P->lmax;
    int nbl = P->lev[lmax].nb;
    cudaStream_t st = P->stream;
    int rc = build_transpose(P);
    if (rc) return rc;
    if ((rc = upload_vjp_rules())) return rc;
    size_t loc = (size_t)nbl * pl * pl, locd = (size_t)nbl * (pl + 1) * (pl + 1);
    double2 *xd = nullptr, *pb = nullptr, *rhs = nullptr, *mu = nullptr, *tmp = nullptr, *D = nullptr, *Dz = nullptr, *Dp = nullptr,
            *Dm = nullptr;
    double *ptd = nullptr, *gd = nullptr, *ctr = nullptr;
    std::vector<double> hctr = leaf_centres(P);
#define VTRY(call)                                                                                              \
    do {                                                                                                        \
        cudaError_t e_ = (call);                                                                                \
        if (e_ != cudaSuccess) { fmm_set_error("fmm_vjp: %s: %s", #call, cudaGetErrorString(e_)); rc = FMM_ERR_CUDA; goto done; } \
    } while (0)
    VTRY(cudaMalloc(&xd, sizeof(double2) * nf));
    VTRY(cudaMalloc(&pb, sizeof(double2) * npts));
    VTRY(cudaMalloc(&rhs, sizeof(double2) * nf));
    VTRY(cudaMalloc(&mu, sizeof(double2) * nf));
    VTRY(cudaMalloc(&tmp, sizeof(double2) * nf));
    VTRY(cudaMalloc(&D, sizeof(double2) * loc));
    VTRY(cudaMalloc(&Dz, sizeof(double2) * locd));
    VTRY(cudaMalloc(&Dp, sizeof(double2) * locd));
    VTRY(cudaMalloc(&Dm, sizeof(double2) * locd));
    VTRY(cudaMalloc(&ptd, sizeof(double) * 3 * npts));
    VTRY(cudaMalloc(&gd, sizeof(double) * 3 * nv));
    VTRY(cudaMalloc(&ctr, sizeof(double) * hctr.size()));
    VTRY(cudaMemcpyAsync(xd, x, sizeof(double2) * nf, cudaMemcpyDefault, st));
    VTRY(cudaMemcpyAsync(pb, pbar, sizeof(double2) * npts, cudaMemcpyDefault, st));
    VTRY(cudaMemcpyAsync(ptd, pts, sizeof(double) * 3 * npts, cudaMemcpyDefault, st));
    VTRY(cudaMemcpyAsync(ctr, hctr.data(), sizeof(double) * hctr.size(), cudaMemcpyHostToDevice, st));
    VTRY(cudaMemsetAsync(gd, 0, sizeof(double) * 3 * nv, st));
    VTRY(cudaMemsetAsync(mu, 0, sizeof(double2) * nf, st));
    {
        const int T = 128, B = std::min((nf + T - 1) / T, 152 * 8);
        // adjoint system A^T mu = F^T conj(pbar)
        double2 nb = make_double2(-P->opt.b_re, -P->opt.b_im), nc = make_double2(-P->opt.c_re, -P->opt.c_im);
        vjp_adjoint_rhs_kernel<<<B, T, 0, st>>>(P->V_dev, P->F_dev, nf, P->opt.k, P->opt.rule, nb, nc, ptd, npts, pb, rhs);
        VTRY(cudaGetLastError());
        int it = 0;
        double rr = 0.0;
        rc = solve_transposed(P, rhs, mu, tol, 1000, 60, precision, &it, &rr);
        if (rc != FMM_OK && rc != FMM_ERR_NOT_CONVERGED) goto done;
        if (rc == FMM_ERR_NOT_CONVERGED) { fmm_set_error("fmm_vjp: adjoint GMRES stopped at %.3g > %.3g", rr, tol); goto done; }
        // forward leaf locals D (FP64 pass on x), then the transposed leaf locals Psi (on mu)
        if ((rc = run_matvec(P, xd, tmp, FMM_FP64, 0, 1))) goto done;
        VTRY(cudaMemcpyAsync(D, P->lev[lmax].Dl64, sizeof(double2) * loc, cudaMemcpyDeviceToDevice, st));
        if ((rc = run_matvec(P, mu, tmp, FMM_FP64, 1, 1))) goto done;
        deriv_coef_kernel<<<(unsigned)std::min<size_t>((locd + 255) / 256, 152 * 8), 256, 0, st>>>(nbl, pl, P->opt.k,
                                                                                                 P->lev[lmax].Dl64, Dz, Dp, Dm);
        double2 bco = make_double2(P->opt.b_re, P->opt.b_im), cco = make_double2(P->opt.c_re, P->opt.c_im);
        vjp_far_source_kernel<<<B, T, 0, st>>>(P->V_dev, P->F_dev, nf, pl, P->opt.k, P->opt.rule, bco, cco, P->elem_leaf,
                                               ctr, P->lev[lmax].Dl64, Dz, Dp, Dm, xd, gd);
        vjp_far_target_kernel<<<B, T, 0, st>>>(P->V_dev, P->F_dev, nf, pl, P->opt.k, P->elem_leaf, ctr, D, mu, gd);
        const double2 alpha = make_double2(P->opt.alpha_re, P->opt.alpha_im);
        const bool bm = alpha.x != 0.0 || alpha.y != 0.0;
        if (bm) {
            // target-side normal derivative of the far field: the derivative expansions of D
            // (Dz, Dp, Dm are free again once the source kernel above has run)
            deriv_coef_kernel<<<(unsigned)std::min<size_t>((locd + 255) / 256, 152 * 8), 256, 0, st>>>(nbl, pl, P->opt.k,
                                                                                                     D, Dz, Dp, Dm);
            vjp_far_target_bm_kernel<<<B, T, 0, st>>>(P->V_dev, P->F_dev, nf, pl, P->opt.k, alpha, P->elem_leaf, ctr, Dz,
                                                      Dp, Dm, mu, gd);
            vjp_near_bm_kernel<<<std::min((nf + 3) / 4, 152 * 16), 128, 0, st>>>(
                P->V_dev, P->F_dev, nf, P->near_beg, P->near_col, P->opt.k, bco, cco, alpha, P->opt.rule, mu, xd, gd);
            if (dir)
                vjp_rhs_bm_kernel<<<B, T, 0, st>>>(P->V_dev, P->F_dev, nf, P->opt.k, dir[0], dir[1], dir[2], alpha, mu, gd);
        }
        vjp_near_kernel<<<std::min((nf + 7) / 8, 152 * 16), 256, 0, st>>>(P->V_dev, P->F_dev, nf, P->near_beg, P->near_col,
                                                                        P->opt.k, bco, cco, P->opt.rule, mu, xd, gd);
        vjp_farpts_kernel<<<B, T, 0, st>>>(P->V_dev, P->F_dev, nf, P->opt.k, P->opt.rule, nb, nc, ptd, npts, pb, xd, gd);
        if (dir)
            vjp_rhs_kernel<<<B, T, 0, st>>>(P->V_dev, P->F_dev, nf, P->opt.k, dir[0], dir[1], dir[2], mu, gd);
        VTRY(cudaGetLastError());
        VTRY(cudaMemcpyAsync(grad, gd, sizeof(double) * 3 * nv, cudaMemcpyDefault, st));
        if (lambda) {
            // lambda = conj(mu)
            launch_conj(P, mu, tmp, nf);
            VTRY(cudaMemcpyAsync(lambda, tmp, sizeof(double2) * nf, cudaMemcpyDefault, st));
        }
        VTRY(cudaStreamSynchronize(st));
        rc = FMM_OK;
    }
done:
#undef VTRY
    for (void *q : {(void *)xd, (void *)pb, (void *)rhs, (void *)mu, (void *)tmp, (void *)D, (void *)Dz, (void *)Dp, (void *)Dm,
                    (void *)ptd, (void *)gd, (void *)ctr})
        if (q) cudaFree(q);
    return rc;
}

// Admittance derivative of the far-field objective of fmm_vjp.  For a locally reacting surface
// dp/dn = i k beta_j p on element j the operator is A = a I + (1 + alpha d/dn_y)(L B + c M), with
// B = diag(b_j), b_j = i k beta_j at the source elements and, with the Burton-Miller coupling,
// a_i = (1 + alpha b_i)/2 at the targets; the far field is F x = M x - L_far (B x).  So
//     dJ = 2 Re sum_j g_j dbeta_j,
//     g_j = i k [ x_j (w_j - z_j) - (alpha/2) conj(lambda_j) x_j ],
// w = (dF/db)^T conj(pbar) (the far-field operator with b = 1, c = 0), z = S^T conj(lambda) with
// S = (1 + alpha d/dn_y) L: one transposed FP64 FMM pass of the plan with its element tables and
// near-field matrix regenerated for (a, b, c) = (0, 1, 0), on temporary buffers that stand in for
// the plan's own during the pass.
extern "C" int fmm_vjp_admittance(fmm_plan *plan, const cuDoubleComplex *x, const double *pts, int npts,
                                  const cuDoubleComplex *pbar, const cuDoubleComplex *lambda, cuDoubleComplex *g_beta,
                                  double *dJ_dbeta)
{
    Plan *P = (Plan *)plan;
    if (!P || !x || !pts || npts < 1 || !pbar || !lambda || (!g_beta && !dJ_dbeta)) {
        fmm_set_error("fmm_vjp_admittance: invalid argument");
        return FMM_ERR_ARG;
    }
    int nf = P->nf, pl = P->pleaf;
    cudaStream_t st = P->stream;
    int rc = build_transpose(P);
    if (rc) return rc;
    size_t tbl = (size_t)nf * pl * pl;
    long long nnz = P->num_near;
    double2 *xd = nullptr, *mu = nullptr, *pb = nullptr, *w = nullptr, *z = nullptr, *U = nullptr, *Rv = nullptr,
            *nearL = nullptr, *nearTL = nullptr, *g = nullptr;
    double *ptd = nullptr;
    std::vector<double2> hg;
#define ATRY(call)                                                                                                 \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) { fmm_set_error("fmm_vjp_admittance: %s: %s", #call, cudaGetErrorString(e_)); rc = FMM_ERR_CUDA; goto done; } \
    } while (0)
    ATRY(cudaMalloc(&xd, sizeof(double2) * nf));
    ATRY(cudaMalloc(&mu, sizeof(double2) * nf));
    ATRY(cudaMalloc(&w, sizeof(double2) * nf));
    ATRY(cudaMalloc(&z, sizeof(double2) * nf));
    ATRY(cudaMalloc(&g, sizeof(double2) * nf));
    ATRY(cudaMalloc(&pb, sizeof(double2) * npts));
    ATRY(cudaMalloc(&ptd, sizeof(double) * 3 * npts));
    ATRY(cudaMalloc(&U, sizeof(double2) * tbl));
    ATRY(cudaMalloc(&Rv, sizeof(double2) * tbl));
    ATRY(cudaMalloc(&nearL, sizeof(double2) * (nnz + 1)));
    ATRY(cudaMalloc(&nearTL, sizeof(double2) * (nnz + 1)));
    ATRY(cudaMemcpyAsync(xd, x, sizeof(double2) * nf, cudaMemcpyDefault, st));
    ATRY(cudaMemcpyAsync(w, lambda, sizeof(double2) * nf, cudaMemcpyDefault, st));
    ATRY(cudaMemcpyAsync(pb, pbar, sizeof(double2) * npts, cudaMemcpyDefault, st));
    ATRY(cudaMemcpyAsync(ptd, pts, sizeof(double) * 3 * npts, cudaMemcpyDefault, st));
    launch_conj(P, w, mu, nf); // mu = conj(lambda)
    ATRY(cudaGetLastError());
    if ((rc = gen_operator_part(P, make_double2(1.0, 0.0), make_double2(0.0, 0.0), U, Rv, nearL))) goto done;
    if ((rc = near_transpose_values(P, nearL, nearTL))) goto done;
    {
        // z = S^T mu with the single-layer part standing in for the plan's operator
        double2 *sU = P->U64, *sN = P->near64, *sNT = P->nearT64;
        fmm_options so = P->opt;
        P->U64 = U;
        P->near64 = nearL;
        P->nearT64 = nearTL;
        P->opt.a_re = P->opt.a_im = 0.0;
        P->opt.b_re = 1.0;
        P->opt.b_im = 0.0;
        P->opt.c_re = P->opt.c_im = 0.0;
        rc = run_matvec(P, mu, z, FMM_FP64, 1, 1);
        cudaError_t e2 = cudaStreamSynchronize(st);
        P->U64 = sU;
        P->near64 = sN;
        P->nearT64 = sNT;
        P->opt = so;
        if (rc) goto done;
        ATRY(e2);
    }
    {
        const int T = 128, B = std::min((nf + T - 1) / T, 152 * 8);
        // w = (dF/db)^T conj(pbar): the far-field operator -int G of unit b
        vjp_adjoint_rhs_kernel<<<B, T, 0, st>>>(P->V_dev, P->F_dev, nf, P->opt.k, P->opt.rule, make_double2(-1.0, 0.0),
                                                make_double2(0.0, 0.0), ptd, npts, pb, w);
        vjp_admittance_kernel<<<B, T, 0, st>>>(nf, P->opt.k, make_double2(P->opt.alpha_re, P->opt.alpha_im), w, z, mu, xd, g);
        ATRY(cudaGetLastError());
        hg.resize(nf);
        ATRY(cudaMemcpyAsync(hg.data(), g, sizeof(double2) * nf, cudaMemcpyDeviceToHost, st));
        ATRY(cudaStreamSynchronize(st));
        if (g_beta) ATRY(cudaMemcpy(g_beta, hg.data(), sizeof(double2) * nf, cudaMemcpyDefault));
        if (dJ_dbeta) {
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < nf; j++) { sr += hg[j].x; si += hg[j].y; }
            dJ_dbeta[0] = 2.0 * sr;  // dJ/dRe(beta) = 2 Re g
            dJ_dbeta[1] = -2.0 * si; // dJ/dIm(beta) = 2 Re(i g)
        }
        rc = FMM_OK;
    }
done:
#undef ATRY
    for (void *q : {(void *)xd, (void *)mu, (void *)pb, (void *)w, (void *)z, (void *)U, (void *)Rv, (void *)nearL,
                    (void *)nearTL, (void *)g, (void *)ptd})
        if (q) cudaFree(q);
    return rc;
}
