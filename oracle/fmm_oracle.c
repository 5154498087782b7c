/* FP64 CPU restatement of the reference FMM-BEM algorithm (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY -- the reference the GPU product is tested against, never linked by it.
 *
 * What each part restates (paths within the reference project):
 *   aCoeff/bCoeff              translation.cu:189-212
 *   spherical basis R, S       translation.cu:141-187 (sphHrmc with the Condon-Shortley
 *                              phase of GSL's Plm, R = j_n Y_n^m, S = h_n Y_n^m, h = j + i y)
 *   rotation coefficients      translation.cu:1064-1237.  orc_rot_H_recur() is the
 *                              reference's recurrence over m (rotMatsInit + sparseRotMatGen).
 *                              That recurrence loses orthogonality in FP64 (1e-5 at p=20,
 *                              diverges at p=40), so orc_rot_H() evaluates the same
 *                              coefficients H_n^{m'm}(beta) from Wigner's d^n_{m'm}(beta)
 *                              via the stable three-term recurrence in degree n, with
 *                              H = (-1)^{max(m',0)} (-1)^{max(-m,0)} d.  The two agree to
 *                              1e-12 where the reference's recurrence is accurate (p <= 10).
 *   coaxial matrices           translation.cu:555-771, 919-949 (rr/srCoaxTransMatsInit +
 *                              sparseCoaxTransMatGen), sparse layout translation.cu:17-32
 *   RCR product                translation.cu:1552-1611 (cuSparseRotVecMul,
 *                              cuSparseCoaxTransMatVecMul) composed as in
 *                              transMatsVecsMul_SR_rcr (translation.cu:1864-1961): rotate by
 *                              (phi, theta, 0), coaxial, rotate by (0, theta, phi)
 *   quadrature                 integral.cu:23-63 (Gauss-Legendre), 80-109 (collapsed rule),
 *                              202-249 (centroid split for the singular self term)
 *   G, dG/dn_x                 integral.cu:72-78, 391-402
 *   P2M element moments        integral.cu:251-365, 821-836 (triElemIntegral_R / pRpn with
 *                              the (n, -m) index; the reference's loop bug at 831 fixed)
 *   FMM passes                 translation.cu:3412-3769 (OprL): upward SS, downward SR and
 *                              RR with per-level truncation, plus the L2P and near field that
 *                              the reference leaves out.
 * The 7-point rule is Dunavant's degree-5 rule (Radon's formula).
 */
#include "fmm_oracle.h"
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;
#define NM(n, m) ((n) * (n) + (n) + (m))
static const double PI_D = 3.14159265358979323846;

/* ------------------------------------------------------------------ special functions */
void orc_sph_jn(int N, double x, double *j)
{
    if (N <= 0) return;
    if (x == 0.0) {
        j[0] = 1.0;
        for (int n = 1; n < N; n++) j[n] = 0.0;
        return;
    }
    double j0 = sin(x) / x;
    double j1 = sin(x) / (x * x) - cos(x) / x;
    int big = N > (int)x ? N : (int)x;
    int start = big + 40 + (int)(4.0 * sqrt((double)big + 1.0));
    double fp1 = 0.0, f = 1e-300, f1 = 0.0;
    for (int n = start; n >= 1; n--) {
        double fm1 = (2.0 * n + 1.0) / x * f - fp1;
        fp1 = f;
        f = fm1;
        /* f now holds the unnormalised value at index n-1 */
        if (n - 1 < N) j[n - 1] = f;
        if (n - 1 == 1) f1 = f;
        if (fabs(f) > 1e250) {
            f *= 1e-250; fp1 *= 1e-250; f1 *= 1e-250;
            for (int q = (n - 1 < N ? n - 1 : N); q < N; q++) j[q] *= 1e-250;
        }
    }
    double f0 = f;
    double scale = (fabs(j0) > fabs(j1)) ? j0 / f0 : j1 / f1;
    for (int n = 0; n < N; n++) j[n] *= scale;
}

void orc_sph_yn(int N, double x, double *y)
{
    if (N <= 0) return;
    y[0] = -cos(x) / x;
    if (N == 1) return;
    y[1] = -cos(x) / (x * x) - sin(x) / x;
    for (int n = 1; n + 1 < N; n++) y[n + 1] = (2.0 * n + 1.0) / x * y[n] - y[n - 1];
}

void orc_legendre_Q(int p, double ct, double *Q)
{
    double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    Q[0] = 1.0 / sqrt(4.0 * PI_D);
    for (int m = 1; m < p; m++)
        Q[m * (m + 1) / 2 + m] = sqrt((2.0 * m + 1.0) / (2.0 * m)) * st * Q[(m - 1) * m / 2 + (m - 1)];
    for (int m = 0; m < p; m++) {
        if (m + 1 < p) Q[(m + 1) * (m + 2) / 2 + m] = sqrt(2.0 * m + 3.0) * ct * Q[m * (m + 1) / 2 + m];
        for (int n = m + 2; n < p; n++) {
            double a = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
            double b = sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) / (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
            Q[n * (n + 1) / 2 + m] = a * (ct * Q[(n - 1) * n / 2 + m] - b * Q[(n - 2) * (n - 1) / 2 + m]);
        }
    }
}

static void basis_generic(int p, double k, const double *v, cplx *out, int singular)
{
    double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double *jn = (double *)malloc(sizeof(double) * (p + 1) * 2);
    double *yn = jn + (p + 1);
    double *Q = (double *)malloc(sizeof(double) * (p * (p + 1) / 2 + 1));
    if (r == 0.0) {
        for (int i = 0; i < p * p; i++) out[i] = 0.0;
        if (!singular) out[0] = 1.0 / sqrt(4.0 * PI_D);
        free(jn); free(Q);
        return;
    }
    double ct = v[2] / r, phi = atan2(v[1], v[0]);
    orc_sph_jn(p, k * r, jn);
    if (singular) orc_sph_yn(p, k * r, yn);
    orc_legendre_Q(p, ct, Q);
    for (int n = 0; n < p; n++) {
        cplx radial = singular ? (jn[n] + I * yn[n]) : jn[n];
        for (int m = -n; m <= n; m++) {
            int am = m < 0 ? -m : m;
            out[NM(n, m)] = radial * Q[n * (n + 1) / 2 + am] * (cos(m * phi) + I * sin(m * phi));
        }
    }
    free(jn); free(Q);
}

void orc_basis_R(int p, double k, const double *v, double *out) { basis_generic(p, k, v, (cplx *)out, 0); }
void orc_basis_S(int p, double k, const double *v, double *out) { basis_generic(p, k, v, (cplx *)out, 1); }

double orc_aC(int n, int m)
{
    if (n >= abs(m)) return sqrt((double)(n + 1 + m) * (n + 1 - m) / ((2.0 * n + 1.0) * (2.0 * n + 3.0)));
    return 0.0;
}
double orc_bC(int n, int m)
{
    if (m >= 0 && n >= m) return sqrt((double)(n - m - 1) * (n - m) / ((2.0 * n - 1.0) * (2.0 * n + 1.0)));
    if (-n <= m && m < 0) return -sqrt((double)(n - m - 1) * (n - m) / ((2.0 * n - 1.0) * (2.0 * n + 1.0)));
    return 0.0;
}

/* ------------------------------------------------------------------ tables */
int orc_rot_size(int p) { return p * (4 * p * p - 1) / 3; }
int orc_coax_size(int p) { return p * (2 * p * p + 3 * p + 1) / 6; }
static inline int rot_off(int n) { return n * (4 * n * n - 1) / 3; }
static inline int coax_off(int p, int m) { return m * (2 * m * m - (3 + 6 * p) * m + 1 + 6 * (p + p * p)) / 6; }

/* Wigner d^j_{m'm}(beta) at the lowest degree j = max(|m'|,|m|) (Wigner's sum has one term) */
static double wigner_start(int j, int mp, int m, double c, double s)
{
    int mu, sgn = 1;
    if (m == j) mu = mp;
    else if (mp == j) { mu = m; if ((m - j) & 1) sgn = -1; }
    else if (m == -j) { mu = -mp; if ((-mp - j) & 1) sgn = -1; }
    else mu = -m;
    /* sqrt(binom(2j, j+mu)) c^{j+mu} s^{j-mu} */
    double binom = 1.0;
    for (int i = 1; i <= j - mu; i++) binom = binom * (double)(j + mu + i) / (double)i;
    double v = sqrt(binom);
    for (int i = 0; i < j + mu; i++) v *= c;
    for (int i = 0; i < j - mu; i++) v *= s;
    return sgn * v;
}

void orc_rot_H(double beta, int p, double *H)
{
    double c = cos(0.5 * beta), s = sin(0.5 * beta), cb = cos(beta);
    for (int mp = -(p - 1); mp <= p - 1; mp++) {
        for (int m = -(p - 1); m <= p - 1; m++) {
            int j0 = abs(mp) > abs(m) ? abs(mp) : abs(m);
            double sign = (((mp > 0 ? mp : 0) + (m < 0 ? -m : 0)) & 1) ? -1.0 : 1.0;
            double dprev = 0.0, dcur = wigner_start(j0, mp, m, c, s);
            H[rot_off(j0) + (mp + j0) + (m + j0) * (2 * j0 + 1)] = sign * dcur;
            for (int j = j0; j + 1 < p; j++) {
                double dn;
                if (j == 0) {
                    dn = cb * dcur;
                } else {
                    double a = j * sqrt(((j + 1.0) * (j + 1.0) - (double)m * m) * ((j + 1.0) * (j + 1.0) - (double)mp * mp));
                    double b = (2.0 * j + 1.0) * (j * (j + 1.0) * cb - (double)m * mp);
                    double cc = (j + 1.0) * sqrt(((double)j * j - (double)m * m) * ((double)j * j - (double)mp * mp));
                    dn = (b * dcur - cc * dprev) / a;
                }
                dprev = dcur;
                dcur = dn;
                H[rot_off(j + 1) + (mp + j + 1) + (m + j + 1) * (2 * j + 3)] = sign * dcur;
            }
        }
    }
}

void orc_rot_H_recur(double beta, int p, double *H)
{
    /* translation.cu:1064-1237 restated in FP64: column m=0 from Legendre, then the
     * recurrence that advances m from degree n+1, then mirror to negative m */
    int N = 2 * p - 1;
    double *cur = (double *)calloc((size_t)N * N, sizeof(double));
    double *nxt = (double *)calloc((size_t)N * N, sizeof(double));
    double cb = cos(beta), sb = sin(beta);
    double *Q = (double *)malloc(sizeof(double) * (N * (N + 1) / 2 + 1));
    orc_legendre_Q(N, cb, Q);
    for (int n = 0; n < N; n++)
        for (int mp = -n; mp <= n; mp++) {
            int am = abs(mp);
            /* (-1)^m' sqrt((n-|m'|)!/(n+|m'|)!) P_n^{|m'|}, P with Condon-Shortley phase,
             * equals sqrt(4 pi/(2n+1)) Q_n^{|m'|} */
            cur[NM(n, mp)] = sqrt(4.0 * PI_D / (2.0 * n + 1.0)) * Q[n * (n + 1) / 2 + am];
        }
    for (int n = 0; n < p; n++)
        for (int mp = -n; mp <= n; mp++) H[rot_off(n) + (mp + n) + n * (2 * n + 1)] = cur[NM(n, mp)];
    for (int m = 0; m + 1 <= p - 1; m++) {
        memset(nxt, 0, sizeof(double) * N * N);
        for (int n = m + 1; n <= 2 * p - 2 - (m + 1); n++)
            for (int mp = -n; mp <= n; mp++) {
                double t0 = 0.5 * orc_bC(n + 1, -mp - 1) / orc_bC(n + 1, m) * (1 - cb);
                double t1 = 0.5 * orc_bC(n + 1, mp - 1) / orc_bC(n + 1, m) * (1 + cb);
                double t2 = orc_aC(n, mp) / orc_bC(n + 1, m) * sb;
                nxt[NM(n, mp)] = t0 * cur[NM(n + 1, mp + 1)] - t1 * cur[NM(n + 1, mp - 1)] - t2 * cur[NM(n + 1, mp)];
            }
        double *tmp = cur; cur = nxt; nxt = tmp;
        int mm = m + 1;
        for (int n = mm; n < p; n++)
            for (int mp = -n; mp <= n; mp++) H[rot_off(n) + (mp + n) + (mm + n) * (2 * n + 1)] = cur[NM(n, mp)];
    }
    for (int n = 1; n < p; n++)
        for (int m = -n; m < 0; m++)
            for (int mp = -n; mp <= n; mp++)
                H[rot_off(n) + (mp + n) + (m + n) * (2 * n + 1)] = H[rot_off(n) + (-mp + n) + (-m + n) * (2 * n + 1)];
    free(cur); free(nxt); free(Q);
}

void orc_rot_matrix(double alpha, double beta, double gamma, int p, double *Rout)
{
    cplx *R = (cplx *)Rout;
    double *H = (double *)malloc(sizeof(double) * orc_rot_size(p));
    orc_rot_H(beta, p, H);
    for (int n = 0; n < p; n++)
        for (int m = -n; m <= n; m++)
            for (int mp = -n; mp <= n; mp++) {
                int idx = rot_off(n) + (mp + n) + (m + n) * (2 * n + 1);
                R[idx] = cexp(I * (m * alpha - mp * gamma)) * H[idx];
            }
    free(H);
}

void orc_coax(double k, double t, int p, int sr, double *Cout)
{
    cplx *C = (cplx *)Cout;
    int R = 2 * p - 1; /* rows np = 0 .. 2p-2 */
    /* E[m][np][n], m >= 0 */
    cplx *E = (cplx *)calloc((size_t)p * R * p, sizeof(cplx));
#define EE(m, np, n) E[((size_t)(m) * R + (np)) * p + (n)]
    double *jn = (double *)malloc(sizeof(double) * R);
    double *yn = (double *)malloc(sizeof(double) * R);
    orc_sph_jn(R, k * t, jn);
    if (sr) orc_sph_yn(R, k * t, yn);
    for (int np = 0; np < R; np++) {
        cplx h = sr ? (jn[np] + I * yn[np]) : (cplx)jn[np];
        EE(0, np, 0) = ((np & 1) ? -1.0 : 1.0) * sqrt(2.0 * np + 1.0) * h;
    }
    for (int m = 0; m + 1 <= p - 1; m++)
        for (int np = m + 1; np <= 2 * p - 2 - (m + 1); np++) {
            double t0 = orc_bC(np, -m - 1) / orc_bC(m + 1, -m - 1);
            double t1 = orc_bC(np + 1, m) / orc_bC(m + 1, -m - 1);
            EE(m + 1, np, m + 1) = t0 * EE(m, np - 1, m) - t1 * EE(m, np + 1, m);
        }
    for (int m = 0; m <= p - 2; m++)
        for (int n = m; n + 1 <= p - 1; n++)
            for (int np = m; np <= 2 * p - 2 - (n + 1); np++) {
                double t0 = orc_aC(np - 1, m) / orc_aC(n, m);
                double t1 = orc_aC(np, m) / orc_aC(n, m);
                double t2 = orc_aC(n - 1, m) / orc_aC(n, m);
                cplx e0 = (np - 1 >= m) ? EE(m, np - 1, n) : 0.0;
                cplx e2 = (n - 1 >= m) ? EE(m, np, n - 1) : 0.0;
                EE(m, np, n + 1) = t0 * e0 - t1 * EE(m, np + 1, n) + t2 * e2;
            }
    /* (R|R): entries with n' < n come from the exact coaxial symmetry (R|R)_{n'n} =
     * (-1)^{n+n'} (R|R)_{nn'}.  The recurrence above (translation.cu:678-771) forms them by
     * cancellation and loses them at small k t (1e13 relative error at kt = 0.05, p = 14,
     * against a 60-digit run), which breaks L2L; its n' >= n side is accurate to 1e-15.
     * This is a deliberate deviation from the reference; (S|R) is accurate throughout. */
    for (int m = 0; m < p; m++) {
        int off = coax_off(p, m);
        for (int np = m; np < p; np++)
            for (int n = m; n < p; n++)
                C[off + (np - m) + (n - m) * (p - m)] =
                    (!sr && np < n) ? (((n + np) & 1) ? -1.0 : 1.0) * EE(m, n, np) : EE(m, np, n);
    }
#undef EE
    free(E); free(jn); free(yn);
}

/* y (first pout^2 entries, accumulated) += RCR(x with pin^2 entries, zero padded to p).
 * Work space: w1 holds p^2 entries, w2 holds p^2 + 2p - 1 entries. */
static void rcr_apply(int p, const double *H, double phi, const cplx *C, const cplx *x, int pin,
                      cplx *y, int pout, cplx *w1, cplx *w2)
{
    cplx *ph = w2 + p * p; /* 2p-1 phases */
    for (int m = -(p - 1); m <= p - 1; m++) ph[m + p - 1] = cexp(I * (m * phi));
    for (int n = 0; n < p; n++) {
        const double *Hn = H + rot_off(n);
        int w = 2 * n + 1;
        for (int mp = -n; mp <= n; mp++) w1[NM(n, mp)] = 0.0;
        if (n >= pin) continue;
        for (int m = -n; m <= n; m++) {
            cplx xv = ph[m + p - 1] * x[NM(n, m)];
            const double *col = Hn + (m + n) * w;
            for (int mp = -n; mp <= n; mp++) w1[NM(n, mp)] += col[mp + n] * xv;
        }
    }
    for (int m = -(p - 1); m <= p - 1; m++) {
        int am = abs(m), sz = p - am;
        const cplx *Cm = C + coax_off(p, am);
        for (int np = am; np < p; np++) {
            cplx acc = 0.0;
            for (int n = am; n < p; n++) acc += Cm[(np - am) + (n - am) * sz] * w1[NM(n, m)];
            w2[NM(np, m)] = acc;
        }
    }
    for (int n = 0; n < pout; n++) {
        const double *Hn = H + rot_off(n);
        int w = 2 * n + 1;
        for (int m = -n; m <= n; m++) {
            cplx xv = w2[NM(n, m)];
            const double *col = Hn + (m + n) * w;
            for (int mp = -n; mp <= n; mp++) y[NM(n, mp)] += conj(ph[mp + p - 1]) * col[mp + n] * xv;
        }
    }
}

void orc_rcr(double k, const double *t, int p, int sr, const double *x, double *yout)
{
    double r = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    double th = acos(t[2] / r), phi = atan2(t[1], t[0]);
    double *H = (double *)malloc(sizeof(double) * orc_rot_size(p));
    cplx *C = (cplx *)malloc(sizeof(cplx) * orc_coax_size(p));
    cplx *w = (cplx *)malloc(sizeof(cplx) * (3 * p * p + 2 * p));
    orc_rot_H(th, p, H);
    orc_coax(k, r, p, sr, (double *)C);
    cplx *y = (cplx *)yout;
    for (int i = 0; i < p * p; i++) y[i] = 0.0;
    rcr_apply(p, H, phi, C, (const cplx *)x, p, y, p, w, w + p * p);
    free(H); free(C); free(w);
}

/* ------------------------------------------------------------------ quadrature */
void orc_gauss_legendre(int n, double *x, double *w)
{
    for (int i = 0; i < n; i++) {
        double z = cos(PI_D * (i + 0.75) / (n + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= n; j++) {
                double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-16) break;
        }
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

/* collapsed Gauss rule of integral.cu:80-109: for GL order g, points in the order of the
 * reference loops (outer eta2 -> theta, inner eta1 -> rho).  Weight excludes J. */
static int collapsed_rule(int g, double *bary, double *w)
{
    double x[16], wt[16];
    orc_gauss_legendre(g, x, wt);
    int q = 0;
    for (int i = 0; i < g; i++) {
        double theta = 0.5 + 0.5 * x[i];
        for (int j = 0; j < g; j++) {
            double rho = 0.5 + 0.5 * x[j];
            double xi1 = rho * (1 - theta);
            double xi2 = rho - xi1;
            double xi3 = 1 - xi1 - xi2;
            bary[3 * q] = xi1; bary[3 * q + 1] = xi2; bary[3 * q + 2] = xi3;
            w[q] = 0.25 * wt[i] * wt[j] * rho;
            q++;
        }
    }
    return q;
}

int orc_rule(int rule, double *bary, double *w)
{
    if (rule == 1) {
        /* Dunavant degree 5 (Radon): centroid 9/40, two orbits */
        double s15 = sqrt(15.0);
        double b1 = (6.0 - s15) / 21.0, a1 = 1.0 - 2.0 * b1, w1 = (155.0 - s15) / 1200.0;
        double b2 = (6.0 + s15) / 21.0, a2 = 1.0 - 2.0 * b2, w2 = (155.0 + s15) / 1200.0;
        double pts[7][3] = {{1.0 / 3, 1.0 / 3, 1.0 / 3}, {a1, b1, b1}, {b1, a1, b1}, {b1, b1, a1},
                            {a2, b2, b2}, {b2, a2, b2}, {b2, b2, a2}};
        double ww[7] = {9.0 / 40, w1, w1, w1, w2, w2, w2};
        for (int q = 0; q < 7; q++) {
            bary[3 * q] = pts[q][0]; bary[3 * q + 1] = pts[q][1]; bary[3 * q + 2] = pts[q][2];
            w[q] = 0.5 * ww[q]; /* integral = J * sum w f, area = J/2 */
        }
        return 7;
    }
    return collapsed_rule(3, bary, w);
}

static inline void tri_point(const double *nod, const double *b, double *x)
{
    x[0] = nod[0] * b[0] + nod[3] * b[1] + nod[6] * b[2];
    x[1] = nod[1] * b[0] + nod[4] * b[1] + nod[7] * b[2];
    x[2] = nod[2] * b[0] + nod[5] * b[1] + nod[8] * b[2];
}

static inline void tri_normal(const double *nod, double *nrml, double *J)
{
    double u[3] = {nod[0] - nod[6], nod[1] - nod[7], nod[2] - nod[8]};
    double v[3] = {nod[3] - nod[6], nod[4] - nod[7], nod[5] - nod[8]};
    nrml[0] = u[1] * v[2] - u[2] * v[1];
    nrml[1] = u[2] * v[0] - u[0] * v[2];
    nrml[2] = u[0] * v[1] - u[1] * v[0];
    *J = sqrt(nrml[0] * nrml[0] + nrml[1] * nrml[1] + nrml[2] * nrml[2]);
}

static inline void tri_centroid(const double *nod, double *y)
{
    for (int a = 0; a < 3; a++) {
        double c23 = 0.5 * (nod[3 + a] + nod[6 + a]);
        y[a] = nod[a] + (2.0 / 3.0) * (c23 - nod[a]);
    }
}

static inline cplx green(double k, const double *x, const double *y)
{
    double d[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    return (cos(k * r) + I * sin(k * r)) / (4.0 * PI_D * r);
}

static inline cplx dgreen(double k, const double *x, const double *y, const double *n)
{
    double d[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    cplx g = (cos(k * r) + I * sin(k * r)) / (4.0 * PI_D * r);
    double dn = (d[0] * n[0] + d[1] * n[1] + d[2] * n[2]) / r;
    return g * (-1.0 / r + I * k) * dn;
}

/* kernel 0: G, 1: dG/dn_x (element normal) */
static cplx elem_integral(double k, const double *nod, const double *y, int rule, int kern)
{
    double bary[64 * 3], w[64], nrml[3], J;
    int nq = orc_rule(rule, bary, w);
    tri_normal(nod, nrml, &J);
    double nh[3] = {nrml[0] / J, nrml[1] / J, nrml[2] / J};
    cplx acc = 0.0;
    for (int q = 0; q < nq; q++) {
        double x[3];
        tri_point(nod, bary + 3 * q, x);
        acc += w[q] * J * (kern ? dgreen(k, x, y, nh) : green(k, x, y));
    }
    return acc;
}

/* centroid split of integral.cu:202-249 with the collapsed rule, singular vertex last */
static cplx elem_integral_sgl(double k, const double *nod, int kern)
{
    double y[3];
    tri_centroid(nod, y);
    cplx acc = 0.0;
    double bary[64 * 3], w[64];
    int nq = collapsed_rule(3, bary, w);
    for (int s = 0; s < 3; s++) {
        double sub[9];
        const double *a = nod + 3 * s, *b = nod + 3 * ((s + 1) % 3);
        for (int t = 0; t < 3; t++) { sub[t] = a[t]; sub[3 + t] = b[t]; sub[6 + t] = y[t]; }
        double nrml[3], J;
        tri_normal(sub, nrml, &J);
        double nh[3] = {nrml[0] / J, nrml[1] / J, nrml[2] / J};
        cplx part = 0.0;
        for (int q = 0; q < nq; q++) {
            double x[3];
            tri_point(sub, bary + 3 * q, x);
            part += w[q] * J * (kern ? dgreen(k, x, y, nh) : green(k, x, y));
        }
        acc += part;
    }
    return acc;
}

void orc_elem_G(double k, const double *nod9, const double *y, int rule, int sgl, double *out)
{
    cplx z = sgl ? elem_integral_sgl(k, nod9, 0) : elem_integral(k, nod9, y, rule, 0);
    out[0] = creal(z); out[1] = cimag(z);
}
void orc_elem_dG(double k, const double *nod9, const double *y, int rule, int sgl, double *out)
{
    cplx z = sgl ? elem_integral_sgl(k, nod9, 1) : elem_integral(k, nod9, y, rule, 1);
    out[0] = creal(z); out[1] = cimag(z);
}

/* directional derivative of R_n^m along unit u (integral.cu:284-331); Rb holds the basis
 * up to order p+1 */
static cplx dirdev_R(double k, int n, int m, const double *u, const cplx *Rb)
{
#define RB(nn, mm) (((nn) < 0 || abs(mm) > (nn)) ? (cplx)0.0 : Rb[NM(nn, mm)])
    cplx t0 = orc_bC(n + 1, -(m + 1)) * RB(n + 1, m + 1) - orc_bC(n, m) * RB(n - 1, m + 1);
    cplx t1 = orc_bC(n + 1, m - 1) * RB(n + 1, m - 1) - orc_bC(n, -m) * RB(n - 1, m - 1);
    cplx t2 = orc_aC(n - 1, m) * RB(n - 1, m) - orc_aC(n, m) * RB(n + 1, m);
#undef RB
    return 0.5 * k * (u[0] - I * u[1]) * t0 + 0.5 * k * (u[0] + I * u[1]) * t1 + k * u[2] * t2;
}

/* element moments: out[NM(n,m)] = int R_n^{-m}(x - c) dS  or  int dR_n^{-m}/dn dS */
void orc_elem_R(double k, const double *nod, const double *c, int p, int rule, int deriv, double *outp)
{
    cplx *out = (cplx *)outp;
    double bary[64 * 3], w[64], nrml[3], J;
    int nq = orc_rule(rule, bary, w);
    tri_normal(nod, nrml, &J);
    double nh[3] = {nrml[0] / J, nrml[1] / J, nrml[2] / J};
    cplx *Rb = (cplx *)malloc(sizeof(cplx) * (p + 1) * (p + 1));
    for (int i = 0; i < p * p; i++) out[i] = 0.0;
    for (int q = 0; q < nq; q++) {
        double x[3], v[3];
        tri_point(nod, bary + 3 * q, x);
        v[0] = x[0] - c[0]; v[1] = x[1] - c[1]; v[2] = x[2] - c[2];
        basis_generic(p + 1, k, v, Rb, 0);
        for (int n = 0; n < p; n++)
            for (int m = -n; m <= n; m++) {
                cplx val = deriv ? dirdev_R(k, n, -m, nh, Rb) : Rb[NM(n, -m)];
                out[NM(n, m)] += w[q] * J * val;
            }
    }
    free(Rb);
}

/* directional derivative of R_n^m(x) along nrml (dirDev_R, integral.cu:284-331) */
void orc_dirdev_R(double k, int n, int m, const double *nrml, const double *x, double *out)
{
    cplx *Rb = (cplx *)malloc(sizeof(cplx) * (n + 2) * (n + 2));
    basis_generic(n + 2, k, x, Rb, 0);
    cplx z = dirdev_R(k, n, m, nrml, Rb);
    free(Rb);
    out[0] = creal(z); out[1] = cimag(z);
}

/* dG(x, y)/dn_y (pGp2n, integral.cu:400-413): G (ik - 1/r) (y - x).n / r */
static inline cplx dgreen_y(double k, const double *x, const double *y, const double *n)
{
    double d[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    cplx g = (cos(k * r) + I * sin(k * r)) / (4.0 * PI_D * r);
    return g * (I * k - 1.0 / r) * (d[0] * n[0] + d[1] * n[1] + d[2] * n[2]) / r;
}

/* d2G(x, y)/dn_x dn_y (p2Gp1np2n, integral.cu:603-622):
 * e^{ikr}/(4 pi r^3) [(3 - 3ikr - k^2 r^2) ((x-y).n1/r) ((y-x).n2/r) + (1 - ikr) n1.n2] */
static inline cplx hyper_kernel(double k, const double *n1, const double *n2, const double *x, const double *y)
{
    double d[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double a1 = (d[0] * n1[0] + d[1] * n1[1] + d[2] * n1[2]) / r;
    double a2 = -(d[0] * n2[0] + d[1] * n2[1] + d[2] * n2[2]) / r;
    double n12 = n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2];
    cplx e = (cos(k * r) + I * sin(k * r)) / (4.0 * PI_D * r * r * r);
    return e * ((3.0 - k * k * r * r - 3.0 * I * k * r) * a1 * a2 + (1.0 - I * k * r) * n12);
}

/* int_T dG/dn_y dS_x with the collapsed rule: regular (triElemIntegral_pGp2n_nsgl,
 * integral.cu:509-537; the caller's normal at y) or self term (triElemIntegral_pGp2n_sgl,
 * integral.cu:539-601: centroid split, each sub-triangle's own normal, y = centroid) */
void orc_elem_dGdny(double k, const double *nod9, const double *nrml, const double *y, int sgl, double *out)
{
    double bary[64 * 3], w[64];
    int nq = collapsed_rule(3, bary, w);
    cplx acc = 0.0;
    if (!sgl) {
        double nn[3], J;
        tri_normal(nod9, nn, &J);
        for (int q = 0; q < nq; q++) {
            double x[3];
            tri_point(nod9, bary + 3 * q, x);
            acc += w[q] * J * dgreen_y(k, x, y, nrml);
        }
    } else {
        double c[3];
        tri_centroid(nod9, c);
        for (int s = 0; s < 3; s++) {
            double sub[9], nn[3], J;
            const double *a = nod9 + 3 * s, *b = nod9 + 3 * ((s + 1) % 3);
            for (int t = 0; t < 3; t++) { sub[t] = a[t]; sub[3 + t] = b[t]; sub[6 + t] = c[t]; }
            tri_normal(sub, nn, &J);
            double nh[3] = {nn[0] / J, nn[1] / J, nn[2] / J};
            for (int q = 0; q < nq; q++) {
                double x[3];
                tri_point(sub, bary + 3 * q, x);
                acc += w[q] * J * dgreen_y(k, x, c, nh);
            }
        }
    }
    out[0] = creal(acc); out[1] = cimag(acc);
}

/* distance from the centroid to the boundary of the triangle along the in-plane direction at
 * angle theta (theta2rho, integral.cu:668-736): node 1 on the polar axis, node 2 at the
 * positive angle 1c2, node 3 at 1c2 + 2c3; the ray meets edge 12, 23 or 31 */
static double centroid_ray(const double *nod9, double theta)
{
    double c[3], dc[3], de[3];
    tri_centroid(nod9, c);
    for (int i = 0; i < 3; i++) {
        const double *a = nod9 + 3 * i, *b = nod9 + 3 * ((i + 1) % 3);
        dc[i] = sqrt((a[0] - c[0]) * (a[0] - c[0]) + (a[1] - c[1]) * (a[1] - c[1]) + (a[2] - c[2]) * (a[2] - c[2]));
        de[i] = sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    }
    double th2 = acos((dc[0] * dc[0] + dc[1] * dc[1] - de[0] * de[0]) / (2.0 * dc[0] * dc[1]));
    double th3 = th2 + acos((dc[1] * dc[1] + dc[2] * dc[2] - de[1] * de[1]) / (2.0 * dc[1] * dc[2]));
    double P[3][2] = {{dc[0], 0.0}, {dc[1] * cos(th2), dc[1] * sin(th2)}, {dc[2] * cos(th3), dc[2] * sin(th3)}};
    int e = theta < th2 ? 0 : (theta < th3 ? 1 : 2);
    const double *A = P[e], *B = P[(e + 1) % 3];
    double u[2] = {cos(theta), sin(theta)}, v[2] = {B[0] - A[0], B[1] - A[1]};
    /* t u = A + s v  =>  t = (A x v) / (u x v) */
    double t = (A[0] * v[1] - A[1] * v[0]) / (u[0] * v[1] - u[1] * v[0]);
    return fabs(t);
}

/* int_T d2G/dn_x dn_y dS_x: regular (triElemIntegral_p2Gp1np2n_nsgl, integral.cu:624-660;
 * n_x the element's unit normal, n_y the caller's) or the finite part at the centroid of the
 * flat element (triElemIntegral_p2Gp1np2n_sgl, integral.cu:738-751):
 *   -1/(4 pi) [ int_0^{2 pi} e^{ik rho(theta)} / rho(theta) dtheta - 2 pi i k ]
 * with an nth-point Gauss rule in theta (the reference uses its 3-point rule). */
void orc_elem_hyper(double k, const double *nod9, const double *nrml, const double *y, int sgl, int nth, double *out)
{
    cplx acc = 0.0;
    if (!sgl) {
        double bary[64 * 3], w[64], nn[3], J;
        int nq = collapsed_rule(3, bary, w);
        tri_normal(nod9, nn, &J);
        double nh[3] = {nn[0] / J, nn[1] / J, nn[2] / J};
        for (int q = 0; q < nq; q++) {
            double x[3];
            tri_point(nod9, bary + 3 * q, x);
            acc += w[q] * J * hyper_kernel(k, nh, nrml, x, y);
        }
    } else {
        double *s = (double *)malloc(sizeof(double) * 2 * nth), *ws = s + nth;
        orc_gauss_legendre(nth, s, ws);
        cplx sum = 0.0;
        for (int i = 0; i < nth; i++) {
            double rho = centroid_ray(nod9, PI_D * s[i] + PI_D);
            sum += ws[i] * (cos(k * rho) + I * sin(k * rho)) / rho;
        }
        free(s);
        acc = -(PI_D * sum - 2.0 * PI_D * I * k) / (4.0 * PI_D);
    }
    out[0] = creal(acc); out[1] = cimag(acc);
}

/* coefficients of the normal derivative of a regular expansion (cmptDiffCoeff,
 * integral.cu:753-823): d/dn sum_{n<=p} c_n^m R_n^m = sum_{n<p} c'_n^m R_n^m + (orders >= p),
 * from the G&D recurrences of dirDev_R collected by output index; coeff holds (p+1)^2
 * entries (orders 0..p), coeff_n p^2. */
void orc_diff_coeff(double k, const double *coeffp, int p, const double *nrml, double *outp)
{
    const cplx *c = (const cplx *)coeffp;
    cplx *o = (cplx *)outp;
#define CF(nn, mm) (((nn) < 0 || abs(mm) > (nn)) ? (cplx)0.0 : c[NM(nn, mm)])
    for (int n = 0; n < p; n++)
        for (int m = -n; m <= n; m++) {
            cplx t0 = orc_bC(n, -m) * CF(n - 1, m - 1) - orc_bC(n + 1, m - 1) * CF(n + 1, m - 1);
            cplx t1 = orc_bC(n, m) * CF(n - 1, m + 1) - orc_bC(n + 1, -m - 1) * CF(n + 1, m + 1);
            cplx t2 = orc_aC(n, m) * CF(n + 1, m) - orc_aC(n - 1, m) * CF(n - 1, m);
            o[NM(n, m)] = 0.5 * k * (nrml[0] - I * nrml[1]) * t0 + 0.5 * k * (nrml[0] + I * nrml[1]) * t1 + k * nrml[2] * t2;
        }
#undef CF
}

/* int_T d2G/dn_x dn_y dS_y at the collocation point x with unit normal nx, T flat with unit
 * normal nT, in the regularised (Maue) form
 *     k^2 (nx.nT) int_T G dS_y  -  oint_{dT} (nx x grad_x G(x, y)) . dl_y,
 * the boundary traversed v0 -> v1 -> v2 (counter-clockwise about nT).  With x the centroid of
 * T itself (sgl) the finite part in polar form (elem_hyper_self). */
#define MAUE_LINE_PTS 8
/* distance from x to the segment [a, b] */
static double seg_dist(const double *x, const double *a, const double *b)
{
    double t[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, d[3] = {x[0] - a[0], x[1] - a[1], x[2] - a[2]};
    double tt = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
    double s = (d[0] * t[0] + d[1] * t[1] + d[2] * t[2]) / tt;
    s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
    double e[3] = {d[0] - s * t[0], d[1] - s * t[1], d[2] - s * t[2]};
    return sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
}

/* Hadamard finite part of int_T d2G/dn_x dn_y at the centroid c of the flat element T,
 *     -1/(4 pi) [ int_0^{2 pi} e^{ik rho(theta)} / rho(theta) dtheta - 2 pi i k ],
 * the angle integral taken edge by edge: along edge e (length L_e, distance h_e from c)
 * dtheta = h_e L_e / rho^3 ds, s in [0, 1], by Gauss on segments no longer than h_e. */
static cplx elem_hyper_self(double k, const double *nod)
{
    double c[3], gx[MAUE_LINE_PTS], gw[MAUE_LINE_PTS];
    tri_centroid(nod, c);
    orc_gauss_legendre(MAUE_LINE_PTS, gx, gw);
    cplx ang = 0.0;
    for (int e = 0; e < 3; e++) {
        const double *va = nod + 3 * e, *vb = nod + 3 * ((e + 1) % 3);
        double t[3] = {vb[0] - va[0], vb[1] - va[1], vb[2] - va[2]}, u[3] = {va[0] - c[0], va[1] - c[1], va[2] - c[2]};
        double cr[3] = {u[1] * t[2] - u[2] * t[1], u[2] * t[0] - u[0] * t[2], u[0] * t[1] - u[1] * t[0]};
        double hL = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);  /* h_e L_e */
        double len = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        int nseg = (int)ceil(len / fmax(hL / len, 1e-12 * len));
        if (nseg > 64) nseg = 64;
        for (int g = 0; g < nseg; g++)
            for (int q = 0; q < MAUE_LINE_PTS; q++) {
                double s = (g + 0.5 + 0.5 * gx[q]) / nseg, w = 0.5 * gw[q] / nseg;
                double d[3] = {u[0] + s * t[0], u[1] + s * t[1], u[2] + s * t[2]};
                double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                ang += w * hL * (cos(k * r) + I * sin(k * r)) / (r * r * r);
            }
    }
    return -(ang - 2.0 * PI_D * I * k) / (4.0 * PI_D);
}

static cplx elem_hyper_maue(double k, const double *nod, const double *x, const double *nx, int rule, int sgl)
{
    if (sgl) return elem_hyper_self(k, nod);
    double nT[3], J;
    tri_normal(nod, nT, &J);
    nT[0] /= J; nT[1] /= J; nT[2] /= J;
    double dotn = nx[0] * nT[0] + nx[1] * nT[1] + nx[2] * nT[2];
    cplx S = sgl ? elem_integral_sgl(k, nod, 0) : elem_integral(k, nod, x, rule, 0);
    double gx[MAUE_LINE_PTS], gw[MAUE_LINE_PTS];
    orc_gauss_legendre(MAUE_LINE_PTS, gx, gw);
    cplx line = 0.0;
    for (int e = 0; e < 3; e++) {
        const double *va = nod + 3 * e, *vb = nod + 3 * ((e + 1) % 3);
        double t[3] = {vb[0] - va[0], vb[1] - va[1], vb[2] - va[2]};
        double len = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        /* segments no longer than the distance from x: Gauss converges like 4.2^(-2n) */
        double dist = seg_dist(x, va, vb);
        int nseg = (int)ceil(len / fmax(dist, 1e-12 * len));
        if (nseg > 64) nseg = 64;
        for (int g = 0; g < nseg; g++)
            for (int q = 0; q < MAUE_LINE_PTS; q++) {
                double s = (g + 0.5 + 0.5 * gx[q]) / nseg, w = 0.5 * gw[q] / nseg;
                double d[3] = {x[0] - va[0] - s * t[0], x[1] - va[1] - s * t[1], x[2] - va[2] - s * t[2]};
                double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                cplx gr = (cos(k * r) + I * sin(k * r)) / (4.0 * PI_D * r);
                /* (nx x grad_x G) . t,  grad_x G = G (ik - 1/r) d / r */
                double cr[3] = {nx[1] * d[2] - nx[2] * d[1], nx[2] * d[0] - nx[0] * d[2], nx[0] * d[1] - nx[1] * d[0]};
                line += w * gr * (I * k - 1.0 / r) / r * (cr[0] * t[0] + cr[1] * t[1] + cr[2] * t[2]);
            }
    }
    return k * k * dotn * S - line;
}

/* int_T dG/dn_x dS_y at the collocation point x with unit normal nx (the normal derivative of
 * the single layer at x); zero on the flat element itself */
static cplx elem_dGdnx(double k, const double *nod, const double *x, const double *nx, int rule, int sgl)
{
    if (sgl) return 0.0;
    double bary[64 * 3], w[64], nn[3], J;
    int nq = orc_rule(rule, bary, w);
    tri_normal(nod, nn, &J);
    cplx acc = 0.0;
    for (int q = 0; q < nq; q++) {
        double y[3];
        tri_point(nod, bary + 3 * q, y);
        acc += w[q] * J * dgreen_y(k, y, x, nx);
    }
    return acc;
}

/* Near-field coefficient of source element j at collocation element i (centroid yc, unit
 * normal nh), without the diagonal a:
 *     b L + c M + alpha (b K' + c N)
 * L, M with the regular rule or the centroid split (self); K' the normal derivative of L at
 * yc; N the normal derivative of M in the Maue form.  alpha = 0 is the conventional operator. */
static cplx pair_value(double k, const double *nod, const double *yc, const double *nh, int sgl, int rule, cplx b, cplx c,
                       cplx alpha)
{
    cplx v = 0.0;
    if (b != 0.0) v += b * (sgl ? elem_integral_sgl(k, nod, 0) : elem_integral(k, nod, yc, rule, 0));
    if (c != 0.0) v += c * (sgl ? elem_integral_sgl(k, nod, 1) : elem_integral(k, nod, yc, rule, 1));
    if (alpha != 0.0) {
        cplx w = 0.0;
        if (b != 0.0) w += b * elem_dGdnx(k, nod, yc, nh, rule, sgl);
        if (c != 0.0) w += c * elem_hyper_maue(k, nod, yc, nh, rule, sgl);
        v += alpha * w;
    }
    return v;
}

/* the Maue-form element integral for the tests */
void orc_elem_hyper_maue(double k, const double *nod9, const double *x, const double *nx, int rule, int sgl, double *out)
{
    cplx z = elem_hyper_maue(k, nod9, x, nx, rule, sgl);
    out[0] = creal(z); out[1] = cimag(z);
}

static void unit_normal(const double *nod, double *nh)
{
    double J;
    tri_normal(nod, nh, &J);
    nh[0] /= J; nh[1] /= J; nh[2] /= J;
}

/* ------------------------------------------------------------------ FMM */
typedef struct {
    int nb, p;
    long long *box;         /* Morton numbers, level-set order */
    long long *sorted_key;  /* for lookup */
    int *sorted_idx;
    double *ctr;            /* 3 per box */
    int *parent;            /* l >= 3 */
    int *child_beg, *child_list; /* children in the next level, CSR */
    int *sr_beg, *sr_src, *sr_dir; /* CSR of M2L sources and direction slot */
    cplx *Cm, *Dl;          /* multipole / local coefficients, nb * p * p */
} orc_level;

struct orc_fmm {
    int nv, nf, lmax, rule, nthreads, pmax;
    double k, d, pt_min[3];
    cplx a, b, c, alpha;  /* y = a x + (1 + alpha d/dn_y)(b L + c M) x */
    double *Vc;
    int *F;
    orc_level lev[16];
    int *elem_leaf;
    int *leaf_beg, *leaf_elem;  /* elements per leaf box */
    cplx *U;      /* P2M vectors, nf * p_lmax^2 (already combined b V + c W) */
    cplx *Rv;     /* L2P vectors at centroids, nf * p_lmax^2 */
    int *near_beg, *near_col;   /* near-field CSR by element */
    cplx *near_val;
    double *Hsr;  /* 343 direction slots x rot_size(pmax) */
    double *Hss, *Hrr; /* 8 octants x rot_size(pmax) */
    double phi_sr[343], phi_ss[8], phi_rr[8];
    cplx *Csr[16];  /* per level: 28 squared-distance slots (index s2) x coax_size(p_l) */
    cplx *Crr[16];  /* per level l>=3: coax for M2M/L2L at p_{l-1} */
};

static int lookup(const orc_level *L, long long key)
{
    int lo = 0, hi = L->nb - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (L->sorted_key[mid] == key) return L->sorted_idx[mid];
        if (L->sorted_key[mid] < key) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

static void box_xyz(long long num, int l, int *x, int *y, int *z)
{
    int xx = 0, yy = 0, zz = 0;
    for (int b = 0; b < l; b++) {
        int digit = (int)((num >> (3 * (l - 1 - b))) & 7);
        xx = (xx << 1) | ((digit >> 2) & 1);
        yy = (yy << 1) | ((digit >> 1) & 1);
        zz = (zz << 1) | (digit & 1);
    }
    *x = xx; *y = yy; *z = zz;
}

static long long box_num(int x, int y, int z, int l)
{
    long long key = 0;
    for (int b = l - 1; b >= 0; b--) key = key * 8 + 4 * ((x >> b) & 1) + 2 * ((y >> b) & 1) + ((z >> b) & 1);
    return key;
}

static int cmp_ll_idx(const void *a, const void *b)
{
    const long long *x = (const long long *)a, *y = (const long long *)b;
    return (x[0] > y[0]) - (x[0] < y[0]);
}

static void rng_axis(int t, int top, int *lo, int *hi)
{
    *lo = t > 0 ? t - 1 : 0;
    *hi = t < top ? t + 1 : top;
}

orc_fmm *orc_fmm_create(int nv, const double *V, int nf, const int *F, double k,
                        double a_re, double a_im, double b_re, double b_im, double c_re, double c_im,
                        double al_re, double al_im, int rule, int lmax, const int *nbox, const long long *boxes,
                        const int *elem_leaf, const int *p_level, double d, const double *pt_min,
                        int nthreads)
{
    orc_fmm *f = (orc_fmm *)calloc(1, sizeof(orc_fmm));
    f->nv = nv; f->nf = nf; f->k = k; f->lmax = lmax; f->rule = rule; f->d = d;
    f->nthreads = nthreads > 0 ? nthreads : 1;
    f->a = a_re + I * a_im; f->b = b_re + I * b_im; f->c = c_re + I * c_im; f->alpha = al_re + I * al_im;
    memcpy(f->pt_min, pt_min, sizeof(double) * 3);
    f->Vc = (double *)malloc(sizeof(double) * 3 * nv);
    memcpy(f->Vc, V, sizeof(double) * 3 * nv);
    f->F = (int *)malloc(sizeof(int) * 3 * nf);
    memcpy(f->F, F, sizeof(int) * 3 * nf);
    f->pmax = 0;
    const long long *bp = boxes;
    for (int l = 2; l <= lmax; l++) {
        orc_level *L = &f->lev[l];
        L->nb = nbox[l - 2];
        L->p = p_level[l - 2];
        if (L->p > f->pmax) f->pmax = L->p;
        L->box = (long long *)malloc(sizeof(long long) * L->nb);
        memcpy(L->box, bp, sizeof(long long) * L->nb);
        bp += L->nb;
        long long *tmp = (long long *)malloc(sizeof(long long) * 2 * L->nb);
        for (int i = 0; i < L->nb; i++) { tmp[2 * i] = L->box[i]; tmp[2 * i + 1] = i; }
        qsort(tmp, L->nb, 2 * sizeof(long long), cmp_ll_idx);
        L->sorted_key = (long long *)malloc(sizeof(long long) * L->nb);
        L->sorted_idx = (int *)malloc(sizeof(int) * L->nb);
        for (int i = 0; i < L->nb; i++) { L->sorted_key[i] = tmp[2 * i]; L->sorted_idx[i] = (int)tmp[2 * i + 1]; }
        free(tmp);
        L->ctr = (double *)malloc(sizeof(double) * 3 * L->nb);
        double h = ldexp(1.0, -l), h2 = ldexp(1.0, -l - 1);
        for (int i = 0; i < L->nb; i++) {
            int x, y, z;
            box_xyz(L->box[i], l, &x, &y, &z);
            L->ctr[3 * i] = d * (h * x + h2) + pt_min[0];
            L->ctr[3 * i + 1] = d * (h * y + h2) + pt_min[1];
            L->ctr[3 * i + 2] = d * (h * z + h2) + pt_min[2];
        }
        size_t pp = (size_t)L->p * L->p;
        L->Cm = (cplx *)calloc((size_t)L->nb * pp, sizeof(cplx));
        L->Dl = (cplx *)calloc((size_t)L->nb * pp, sizeof(cplx));
    }
    /* parents and children */
    for (int l = 3; l <= lmax; l++) {
        orc_level *L = &f->lev[l], *P = &f->lev[l - 1];
        L->parent = (int *)malloc(sizeof(int) * L->nb);
        P->child_beg = (int *)calloc(P->nb + 1, sizeof(int));
        P->child_list = (int *)malloc(sizeof(int) * L->nb);
        for (int i = 0; i < L->nb; i++) {
            L->parent[i] = lookup(P, L->box[i] / 8);
            P->child_beg[L->parent[i] + 1]++;
        }
        for (int i = 0; i < P->nb; i++) P->child_beg[i + 1] += P->child_beg[i];
        int *fill = (int *)calloc(P->nb, sizeof(int));
        for (int i = 0; i < L->nb; i++) {
            int q = L->parent[i];
            P->child_list[P->child_beg[q] + fill[q]++] = i;
        }
        free(fill);
    }
    /* M2L lists: children of the parent's neighbourhood not adjacent to the box, parent's
     * neighbours first and the parent last as in I4 (octree.c:517-543) */
    for (int l = 2; l <= lmax; l++) {
        orc_level *L = &f->lev[l];
        int ptop = (1 << (l - 1)) - 1;
        L->sr_beg = (int *)calloc(L->nb + 1, sizeof(int));
        size_t cap = (size_t)L->nb * 189 + 1;
        L->sr_src = (int *)malloc(sizeof(int) * cap);
        L->sr_dir = (int *)malloc(sizeof(int) * cap);
        int cnt = 0;
        for (int i = 0; i < L->nb; i++) {
            int x, y, z;
            box_xyz(L->box[i], l, &x, &y, &z);
            int X = x >> 1, Y = y >> 1, Z = z >> 1, xl, xh, yl, yh, zl, zh;
            rng_axis(X, ptop, &xl, &xh);
            rng_axis(Y, ptop, &yl, &yh);
            rng_axis(Z, ptop, &zl, &zh);
            for (int pass = 0; pass < 2; pass++)
                for (int px = xl; px <= xh; px++)
                    for (int py = yl; py <= yh; py++)
                        for (int pz = zl; pz <= zh; pz++) {
                            int self = (px == X && py == Y && pz == Z);
                            if ((pass == 0) == self) continue;
                            for (int cc = 0; cc < 8; cc++) {
                                int cx = 2 * px + ((cc >> 2) & 1), cy = 2 * py + ((cc >> 1) & 1), cz = 2 * pz + (cc & 1);
                                if (abs(cx - x) <= 1 && abs(cy - y) <= 1 && abs(cz - z) <= 1) continue;
                                int s = lookup(L, box_num(cx, cy, cz, l));
                                if (s < 0) continue;
                                L->sr_src[cnt] = s;
                                L->sr_dir[cnt] = (x - cx + 3) * 49 + (y - cy + 3) * 7 + (z - cz + 3);
                                cnt++;
                            }
                        }
            L->sr_beg[i + 1] = cnt;
        }
    }
    /* elements per leaf box */
    orc_level *LL = &f->lev[lmax];
    f->elem_leaf = (int *)malloc(sizeof(int) * nf);
    memcpy(f->elem_leaf, elem_leaf, sizeof(int) * nf);
    f->leaf_beg = (int *)calloc(LL->nb + 1, sizeof(int));
    f->leaf_elem = (int *)malloc(sizeof(int) * nf);
    for (int e = 0; e < nf; e++) f->leaf_beg[elem_leaf[e] + 1]++;
    for (int i = 0; i < LL->nb; i++) f->leaf_beg[i + 1] += f->leaf_beg[i];
    {
        int *fill = (int *)calloc((size_t)LL->nb + 1, sizeof(int));
        for (int e = 0; e < nf; e++) f->leaf_elem[f->leaf_beg[elem_leaf[e]] + fill[elem_leaf[e]]++] = e;
        free(fill);
    }
    /* rotation tables at pmax (prefixes serve every level) */
    int rs = orc_rot_size(f->pmax);
    f->Hsr = (double *)calloc((size_t)343 * rs, sizeof(double));
    f->Hss = (double *)malloc(sizeof(double) * 8 * rs);
    f->Hrr = (double *)malloc(sizeof(double) * 8 * rs);
#pragma omp parallel for num_threads(f->nthreads) schedule(dynamic)
    for (int s = 0; s < 343; s++) {
        int dx = s / 49 - 3, dy = (s / 7) % 7 - 3, dz = s % 7 - 3;
        if (abs(dx) <= 1 && abs(dy) <= 1 && abs(dz) <= 1) continue;
        double r = sqrt((double)(dx * dx + dy * dy + dz * dz));
        orc_rot_H(acos(dz / r), f->pmax, f->Hsr + (size_t)s * rs);
        f->phi_sr[s] = atan2((double)dy, (double)dx);
    }
    for (int o = 0; o < 8; o++) {
        /* M2M: parent - child = (1/2 - b) * child size;  L2L: child - parent */
        double t[3] = {0.5 - ((o >> 2) & 1), 0.5 - ((o >> 1) & 1), 0.5 - (o & 1)};
        double r = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        orc_rot_H(acos(t[2] / r), f->pmax, f->Hss + (size_t)o * rs);
        f->phi_ss[o] = atan2(t[1], t[0]);
        orc_rot_H(acos(-t[2] / r), f->pmax, f->Hrr + (size_t)o * rs);
        f->phi_rr[o] = atan2(-t[1], -t[0]);
    }
    /* coaxial tables */
    for (int l = 2; l <= lmax; l++) {
        int p = f->lev[l].p, cs = orc_coax_size(p);
        double size = d * ldexp(1.0, -l);
        f->Csr[l] = (cplx *)calloc((size_t)28 * cs, sizeof(cplx));
        for (int s2 = 4; s2 <= 27; s2++)
            orc_coax(k, sqrt((double)s2) * size, p, 1, (double *)(f->Csr[l] + (size_t)s2 * cs));
        if (l >= 3) {
            int pp = f->lev[l - 1].p;
            f->Crr[l] = (cplx *)malloc(sizeof(cplx) * orc_coax_size(pp));
            orc_coax(k, 0.5 * sqrt(3.0) * size, pp, 0, (double *)f->Crr[l]);
        }
    }
    /* P2M and L2P vectors */
    int pl = LL->p;
    size_t ppl = (size_t)pl * pl;
    f->U = (cplx *)malloc(sizeof(cplx) * nf * ppl);
    f->Rv = (cplx *)malloc(sizeof(cplx) * nf * ppl);
#pragma omp parallel num_threads(f->nthreads)
    {
        cplx *tmp = (cplx *)malloc(sizeof(cplx) * ppl);
#pragma omp for schedule(dynamic, 64)
        for (int e = 0; e < nf; e++) {
            double nod[9], y[3], v[3];
            for (int t = 0; t < 3; t++)
                for (int a = 0; a < 3; a++) nod[3 * t + a] = V[3 * F[3 * e + t] + a];
            const double *c = LL->ctr + 3 * elem_leaf[e];
            cplx *U = f->U + e * ppl;
            for (size_t i = 0; i < ppl; i++) U[i] = 0.0;
            if (f->b != 0.0) {
                orc_elem_R(k, nod, c, pl, rule, 0, (double *)tmp);
                for (size_t i = 0; i < ppl; i++) U[i] += f->b * tmp[i];
            }
            if (f->c != 0.0) {
                orc_elem_R(k, nod, c, pl, rule, 1, (double *)tmp);
                for (size_t i = 0; i < ppl; i++) U[i] += f->c * tmp[i];
            }
            tri_centroid(nod, y);
            v[0] = y[0] - c[0]; v[1] = y[1] - c[1]; v[2] = y[2] - c[2];
            if (f->alpha == 0.0) {
                basis_generic(pl, k, v, f->Rv + e * ppl, 0);
            } else {
                /* L2P vector of R + alpha dR/dn at the centroid along the element normal */
                double nh[3];
                unit_normal(nod, nh);
                cplx *Rb = (cplx *)malloc(sizeof(cplx) * (pl + 1) * (pl + 1));
                basis_generic(pl + 1, k, v, Rb, 0);
                for (int n = 0; n < pl; n++)
                    for (int m = -n; m <= n; m++)
                        f->Rv[e * ppl + NM(n, m)] = Rb[NM(n, m)] + f->alpha * dirdev_R(k, n, m, nh, Rb);
                free(Rb);
            }
        }
        free(tmp);
    }
    /* near field CSR by target element: sources in I2 ∩ leaf set (octree.c:497-505) */
    f->near_beg = (int *)calloc(nf + 1, sizeof(int));
    {
        int top = (1 << lmax) - 1;
        int *nbrs = (int *)malloc(sizeof(int) * 27 * LL->nb);
        int *nnb = (int *)calloc(LL->nb, sizeof(int));
        for (int i = 0; i < LL->nb; i++) {
            int x, y, z, xl, xh, yl, yh, zl, zh;
            box_xyz(LL->box[i], lmax, &x, &y, &z);
            rng_axis(x, top, &xl, &xh); rng_axis(y, top, &yl, &yh); rng_axis(z, top, &zl, &zh);
            for (int px = xl; px <= xh; px++)
                for (int py = yl; py <= yh; py++)
                    for (int pz = zl; pz <= zh; pz++) {
                        int q = lookup(LL, box_num(px, py, pz, lmax));
                        if (q >= 0) nbrs[27 * i + nnb[i]++] = q;
                    }
        }
        for (int e = 0; e < nf; e++) {
            int b = elem_leaf[e], cnt = 0;
            for (int t = 0; t < nnb[b]; t++) cnt += f->leaf_beg[nbrs[27 * b + t] + 1] - f->leaf_beg[nbrs[27 * b + t]];
            f->near_beg[e + 1] = cnt;
        }
        for (int e = 0; e < nf; e++) f->near_beg[e + 1] += f->near_beg[e];
        long long total = f->near_beg[nf];
        f->near_col = (int *)malloc(sizeof(int) * (total + 1));
        f->near_val = (cplx *)malloc(sizeof(cplx) * (total + 1));
#pragma omp parallel for num_threads(f->nthreads) schedule(dynamic, 64)
        for (int e = 0; e < nf; e++) {
            int b = elem_leaf[e], pos = f->near_beg[e];
            double nodi[9], y[3], nh[3];
            for (int t = 0; t < 3; t++)
                for (int a = 0; a < 3; a++) nodi[3 * t + a] = V[3 * F[3 * e + t] + a];
            tri_centroid(nodi, y);
            unit_normal(nodi, nh);
            for (int t = 0; t < nnb[b]; t++) {
                int q = nbrs[27 * b + t];
                for (int s = f->leaf_beg[q]; s < f->leaf_beg[q + 1]; s++) {
                    int j = f->leaf_elem[s];
                    double nod[9];
                    for (int u = 0; u < 3; u++)
                        for (int a = 0; a < 3; a++) nod[3 * u + a] = V[3 * F[3 * j + u] + a];
                    cplx val = pair_value(k, nod, y, nh, j == e, rule, f->b, f->c, f->alpha);
                    f->near_col[pos] = j;
                    f->near_val[pos] = val;
                    pos++;
                }
            }
        }
        free(nbrs); free(nnb);
    }
    return f;
}

long long orc_fmm_num_sr(const orc_fmm *f, int l) { return f->lev[l].sr_beg[f->lev[l].nb]; }
long long orc_fmm_num_near(const orc_fmm *f) { return f->near_beg[f->nf]; }

/* Index of (n, -m) for the coefficient at nm_idx(n, m) = n^2 + n + m. */
static size_t flip_nm(size_t i)
{
    size_t n = (size_t)sqrt((double)i);
    while (n * n > i) n--;
    while ((n + 1) * (n + 1) <= i) n++;
    return 2 * (n * n + n) - i;
}

/* transpose = 0: y = A x as the reference's FMM pipeline computes it.
 * transpose = 1: y = A^T x.  The reference has no transposed operator; this one follows from
 * G(x, y) = G(y, x): the inputs become point sources at the element centroids (multipole
 * coefficients ik x_i R_n^{-m}(y_i - c), the centroid basis read at (n, -m)), every
 * translation is unchanged, the local expansion is integrated over the target element (the
 * element moments read at (n, -m)), and the near-field matrix is applied transposed. */
void orc_fmm_apply2(orc_fmm *f, const double *xin, double *yout, int transpose)
{
    const cplx *x = (const cplx *)xin;
    cplx *y = (cplx *)yout;
    int lmax = f->lmax, rs = orc_rot_size(f->pmax);
    orc_level *LL = &f->lev[lmax];
    int pl = LL->p;
    size_t ppl = (size_t)pl * pl;
    cplx ik = I * f->k;
    for (int l = 2; l <= lmax; l++) {
        size_t n = (size_t)f->lev[l].nb * f->lev[l].p * f->lev[l].p;
        memset(f->lev[l].Cm, 0, n * sizeof(cplx));
        memset(f->lev[l].Dl, 0, n * sizeof(cplx));
    }
    /* P2M */
#pragma omp parallel for num_threads(f->nthreads) schedule(dynamic, 16)
    for (int b = 0; b < LL->nb; b++) {
        cplx *C = LL->Cm + b * ppl;
        for (int s = f->leaf_beg[b]; s < f->leaf_beg[b + 1]; s++) {
            int e = f->leaf_elem[s];
            cplx xe = ik * x[e];
            if (transpose) {
                const cplx *Rv = f->Rv + e * ppl;
                for (size_t i = 0; i < ppl; i++) C[i] += xe * Rv[flip_nm(i)];
            } else {
                const cplx *U = f->U + e * ppl;
                for (size_t i = 0; i < ppl; i++) C[i] += xe * U[i];
            }
        }
    }
    /* M2M, the parent owns its sum */
    for (int l = lmax; l >= 3; l--) {
        orc_level *L = &f->lev[l], *P = &f->lev[l - 1];
        int pc = L->p, pp = P->p;
#pragma omp parallel num_threads(f->nthreads)
        {
            cplx *w = (cplx *)malloc(sizeof(cplx) * (2 * pp * pp + 2 * pp));
#pragma omp for schedule(dynamic, 8)
            for (int q = 0; q < P->nb; q++) {
                for (int s = P->child_beg[q]; s < P->child_beg[q + 1]; s++) {
                    int ch = P->child_list[s];
                    int o = (int)(L->box[ch] & 7);
                    rcr_apply(pp, f->Hss + (size_t)o * rs, f->phi_ss[o], f->Crr[l], L->Cm + (size_t)ch * pc * pc, pc,
                              P->Cm + (size_t)q * pp * pp, pp, w, w + pp * pp);
                }
            }
            free(w);
        }
    }
    /* M2L */
    for (int l = 2; l <= lmax; l++) {
        orc_level *L = &f->lev[l];
        int p = L->p, cs = orc_coax_size(p);
#pragma omp parallel num_threads(f->nthreads)
        {
            cplx *w = (cplx *)malloc(sizeof(cplx) * (2 * p * p + 2 * p));
#pragma omp for schedule(dynamic, 4)
            for (int b = 0; b < L->nb; b++) {
                for (int s = L->sr_beg[b]; s < L->sr_beg[b + 1]; s++) {
                    int src = L->sr_src[s], dir = L->sr_dir[s];
                    int dx = dir / 49 - 3, dy = (dir / 7) % 7 - 3, dz = dir % 7 - 3;
                    int s2 = dx * dx + dy * dy + dz * dz;
                    rcr_apply(p, f->Hsr + (size_t)dir * rs, f->phi_sr[dir], f->Csr[l] + (size_t)s2 * cs,
                              L->Cm + (size_t)src * p * p, p, L->Dl + (size_t)b * p * p, p, w, w + p * p);
                }
            }
            free(w);
        }
    }
    /* L2L, level by level after each level's locals are complete */
    for (int l = 3; l <= lmax; l++) {
        orc_level *L = &f->lev[l], *P = &f->lev[l - 1];
        int pc = L->p, pp = P->p;
#pragma omp parallel num_threads(f->nthreads)
        {
            cplx *w = (cplx *)malloc(sizeof(cplx) * (2 * pp * pp + 2 * pp));
#pragma omp for schedule(dynamic, 8)
            for (int b = 0; b < L->nb; b++) {
                int o = (int)(L->box[b] & 7);
                rcr_apply(pp, f->Hrr + (size_t)o * rs, f->phi_rr[o], f->Crr[l], P->Dl + (size_t)L->parent[b] * pp * pp, pp,
                          L->Dl + (size_t)b * pc * pc, pc, w, w + pp * pp);
            }
            free(w);
        }
    }
    /* near field + L2P + identity */
    if (transpose) {
        for (int e = 0; e < f->nf; e++) y[e] = f->a * x[e];
        for (int i = 0; i < f->nf; i++)
            for (int s = f->near_beg[i]; s < f->near_beg[i + 1]; s++) y[f->near_col[s]] += f->near_val[s] * x[i];
    }
#pragma omp parallel for num_threads(f->nthreads) schedule(dynamic, 64)
    for (int e = 0; e < f->nf; e++) {
        const cplx *D = LL->Dl + (size_t)f->elem_leaf[e] * ppl;
        cplx acc;
        if (transpose) {
            acc = y[e];
            const cplx *U = f->U + e * ppl;
            for (size_t i = 0; i < ppl; i++) acc += D[i] * U[flip_nm(i)];
        } else {
            acc = f->a * x[e];
            for (int s = f->near_beg[e]; s < f->near_beg[e + 1]; s++) acc += f->near_val[s] * x[f->near_col[s]];
            const cplx *R = f->Rv + e * ppl;
            for (size_t i = 0; i < ppl; i++) acc += D[i] * R[i];
        }
        y[e] = acc;
    }
}

void orc_fmm_apply(orc_fmm *f, const double *xin, double *yout) { orc_fmm_apply2(f, xin, yout, 0); }

void orc_fmm_destroy(orc_fmm *f)
{
    if (!f) return;
    for (int l = 2; l <= f->lmax; l++) {
        orc_level *L = &f->lev[l];
        free(L->box); free(L->sorted_key); free(L->sorted_idx); free(L->ctr); free(L->parent);
        free(L->child_beg); free(L->child_list); free(L->sr_beg); free(L->sr_src); free(L->sr_dir);
        free(L->Cm); free(L->Dl); free(f->Csr[l]); free(f->Crr[l]);
    }
    free(f->Vc); free(f->F); free(f->elem_leaf); free(f->leaf_beg); free(f->leaf_elem);
    free(f->U); free(f->Rv); free(f->near_beg); free(f->near_col); free(f->near_val);
    free(f->Hsr); free(f->Hss); free(f->Hrr);
    free(f);
}

void orc_dense_apply(int nv, const double *V, int nf, const int *F, double k,
                     double a_re, double a_im, double b_re, double b_im, double c_re, double c_im,
                     double al_re, double al_im, int rule, const double *xin, double *yout, int nthreads)
{
    (void)nv;
    const cplx *x = (const cplx *)xin;
    cplx *y = (cplx *)yout;
    cplx a = a_re + I * a_im, b = b_re + I * b_im, c = c_re + I * c_im, al = al_re + I * al_im;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(dynamic, 16)
    for (int i = 0; i < nf; i++) {
        double nodi[9], yc[3], nh[3];
        for (int t = 0; t < 3; t++)
            for (int q = 0; q < 3; q++) nodi[3 * t + q] = V[3 * F[3 * i + t] + q];
        tri_centroid(nodi, yc);
        unit_normal(nodi, nh);
        cplx acc = a * x[i];
        for (int j = 0; j < nf; j++) {
            double nod[9];
            for (int t = 0; t < 3; t++)
                for (int q = 0; q < 3; q++) nod[3 * t + q] = V[3 * F[3 * j + t] + q];
            acc += pair_value(k, nod, yc, nh, i == j, rule, b, c, al) * x[j];
        }
        y[i] = acc;
    }
}

/* The dense operator as an explicit nf x nf row-major matrix, entry (i, j) = a delta_ij +
 * the quadrature of element j at the centroid of element i: the coefficients orc_dense_apply
 * sums.  Used to check the transposed and adjoint operators on small meshes. */
void orc_dense_matrix(int nv, const double *V, int nf, const int *F, double k,
                      double a_re, double a_im, double b_re, double b_im, double c_re, double c_im,
                      double al_re, double al_im, int rule, double *out, int nthreads)
{
    (void)nv;
    cplx *A = (cplx *)out;
    cplx a = a_re + I * a_im, b = b_re + I * b_im, c = c_re + I * c_im, al = al_re + I * al_im;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(dynamic, 16)
    for (int i = 0; i < nf; i++) {
        double nodi[9], yc[3], nh[3];
        for (int t = 0; t < 3; t++)
            for (int q = 0; q < 3; q++) nodi[3 * t + q] = V[3 * F[3 * i + t] + q];
        tri_centroid(nodi, yc);
        unit_normal(nodi, nh);
        for (int j = 0; j < nf; j++) {
            double nod[9];
            for (int t = 0; t < 3; t++)
                for (int q = 0; q < 3; q++) nod[3 * t + q] = V[3 * F[3 * j + t] + q];
            cplx v = (i == j ? a : 0.0) + pair_value(k, nod, yc, nh, i == j, rule, b, c, al);
            A[(size_t)i * nf + j] = v;
        }
    }
}

void orc_far_field(int nv, const double *V, int nf, const int *F, double k, double b_re, double b_im, double c_re,
                   double c_im, int rule, const double *pin, int npts, const double *pts, double *out, int nthreads)
{
    (void)nv;
    const cplx *p = (const cplx *)pin;
    cplx *o = (cplx *)out;
    cplx b = b_re + I * b_im, c = c_re + I * c_im;
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1)
    for (int t = 0; t < npts; t++) {
        cplx acc = 0.0;
        for (int j = 0; j < nf; j++) {
            double nod[9];
            for (int u = 0; u < 3; u++)
                for (int q = 0; q < 3; q++) nod[3 * u + q] = V[3 * F[3 * j + u] + q];
            cplx v = 0.0;
            if (b != 0.0) v += b * elem_integral(k, nod, pts + 3 * t, rule, 0);
            if (c != 0.0) v += c * elem_integral(k, nod, pts + 3 * t, rule, 1);
            acc -= p[j] * v;
        }
        o[t] = acc;
    }
}

void orc_mie_rigid(double k, double a, int npts, const double *pts, double *out)
{
    cplx *o = (cplx *)out;
    int N = (int)(k * a) + 30;
    double *ja = (double *)malloc(sizeof(double) * (N + 2) * 4);
    double *ya = ja + (N + 2), *jr = ya + (N + 2), *yr = jr + (N + 2);
    for (int t = 0; t < npts; t++) {
        const double *P = pts + 3 * t;
        double r = sqrt(P[0] * P[0] + P[1] * P[1] + P[2] * P[2]);
        double ct = P[2] / r;
        orc_sph_jn(N + 2, k * a, ja); orc_sph_yn(N + 2, k * a, ya);
        orc_sph_jn(N + 2, k * r, jr); orc_sph_yn(N + 2, k * r, yr);
        cplx acc = 0.0, in = 1.0;
        double Pnm2 = 0.0, Pnm1 = 0.0;
        double x = k * a;
        for (int n = 0; n <= N; n++) {
            double Pn = (n == 0) ? 1.0 : (n == 1 ? ct : ((2.0 * n - 1.0) * ct * Pnm1 - (n - 1.0) * Pnm2) / n);
            Pnm2 = Pnm1;
            Pnm1 = Pn;
            /* f_n' = f_{n-1} - (n+1)/x f_n, and j_0' = -j_1 */
            double djn = (n == 0) ? -ja[1] : ja[n - 1] - (n + 1.0) / x * ja[n];
            double dyn = (n == 0) ? -ya[1] : ya[n - 1] - (n + 1.0) / x * ya[n];
            cplx dhn = djn + I * dyn;
            cplx hr = jr[n] + I * yr[n];
            acc += -in * (2.0 * n + 1.0) * (djn / dhn) * hr * Pn;
            in *= I;
        }
        o[t] = acc;
    }
    free(ja);
}

/* Mie series for a sphere of radius a with the locally reacting surface dp/dn = i k beta p
 * (n the outward normal, e^{ikz} incident): p_s = sum_n (2n+1) i^n A_n h_n(kr) P_n(cos theta),
 * A_n = -(j_n'(ka) - i beta j_n(ka)) / (h_n'(ka) - i beta h_n(ka)); beta = 0 is the rigid sphere. */
void orc_mie_impedance(double k, double a, double beta_re, double beta_im, int npts, const double *pts, double *out)
{
    cplx *o = (cplx *)out;
    cplx beta = beta_re + I * beta_im;
    int N = (int)(k * a) + 30;
    double *ja = (double *)malloc(sizeof(double) * (N + 2) * 4);
    double *ya = ja + (N + 2), *jr = ya + (N + 2), *yr = jr + (N + 2);
    double x = k * a;
    orc_sph_jn(N + 2, x, ja);
    orc_sph_yn(N + 2, x, ya);
    for (int t = 0; t < npts; t++) {
        const double *P = pts + 3 * t;
        double r = sqrt(P[0] * P[0] + P[1] * P[1] + P[2] * P[2]);
        double ct = P[2] / r;
        orc_sph_jn(N + 2, k * r, jr);
        orc_sph_yn(N + 2, k * r, yr);
        cplx acc = 0.0, in = 1.0;
        double Pnm2 = 0.0, Pnm1 = 0.0;
        for (int n = 0; n <= N; n++) {
            double Pn = (n == 0) ? 1.0 : (n == 1 ? ct : ((2.0 * n - 1.0) * ct * Pnm1 - (n - 1.0) * Pnm2) / n);
            Pnm2 = Pnm1;
            Pnm1 = Pn;
            double djn = (n == 0) ? -ja[1] : ja[n - 1] - (n + 1.0) / x * ja[n];
            double dyn = (n == 0) ? -ya[1] : ya[n - 1] - (n + 1.0) / x * ya[n];
            cplx hn = ja[n] + I * ya[n], dhn = djn + I * dyn;
            cplx An = -(djn - I * beta * ja[n]) / (dhn - I * beta * hn);
            acc += in * (2.0 * n + 1.0) * An * (jr[n] + I * yr[n]) * Pn;
            in *= I;
        }
        o[t] = acc;
    }
    free(ja);
}
