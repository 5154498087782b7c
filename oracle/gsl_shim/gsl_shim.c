/* Project-written implementations of the GSL routines the reference calls.
 *
 * TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/libfmmref.so so that the reference's
 * own sources can run as an oracle.  Nothing in the product links this file.
 *
 * Third-party boundary: GNU Scientific Library (system library, version not pinned by the
 * reference, linked with -lgsl -lgslcblas at makefile:174).  The routines restate the
 * published definitions:
 *   gsl_sf_bessel_jl/yl  spherical Bessel functions of the first/second kind,
 *                        j0 = sin x / x, y0 = -cos x / x, three-term recurrence
 *                        f_{l+1} = (2l+1)/x f_l - f_{l-1}; j_l uses Miller's backward
 *                        recurrence above the turning point (l > x).
 *   gsl_sf_legendre_Plm  associated Legendre P_l^m(x) including the Condon-Shortley
 *                        phase (-1)^m, as GSL documents for the unnormalised functions.
 *   gsl_eigen_symmv      symmetric eigen-decomposition (cyclic Jacobi rotations).
 */
#include "gsl/gsl_shim_decls.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

gsl_complex gsl_complex_rect(double x, double y) { gsl_complex z; z.dat[0] = x; z.dat[1] = y; return z; }
gsl_complex gsl_complex_mul(gsl_complex a, gsl_complex b)
{
    return gsl_complex_rect(a.dat[0] * b.dat[0] - a.dat[1] * b.dat[1], a.dat[0] * b.dat[1] + a.dat[1] * b.dat[0]);
}
gsl_complex gsl_complex_mul_real(gsl_complex a, double x) { return gsl_complex_rect(a.dat[0] * x, a.dat[1] * x); }

double gsl_sf_bessel_jl(const int l, const double x)
{
    if (l < 0) return 0.0;
    if (x == 0.0) return l == 0 ? 1.0 : 0.0;
    double ax = fabs(x);
    double j0 = sin(ax) / ax;
    if (l == 0) return j0;
    double j1 = sin(ax) / (ax * ax) - cos(ax) / ax;
    double val;
    if ((double)l < ax) {
        /* forward recurrence is stable below the turning point */
        double a = j0, b = j1;
        for (int n = 1; n < l; n++) {
            double c = (2.0 * n + 1.0) / ax * b - a;
            a = b; b = c;
        }
        val = b;
    } else {
        /* Miller: start well above max(l, x) and recur down, normalise with j0 or j1 */
        int big = (l > (int)ax ? l : (int)ax);
        int start = big + 40 + (int)(4.0 * sqrt((double)big + 1.0));
        double fp1 = 0.0, f = 1e-300, fl = 0.0, f0 = 0.0, f1 = 0.0;
        for (int n = start; n >= 1; n--) {
            double fm1 = (2.0 * n + 1.0) / ax * f - fp1;
            fp1 = f; f = fm1;
            if (n - 1 == l) fl = f;
            if (n - 1 == 1) f1 = f;
            if (fabs(f) > 1e250) { f *= 1e-250; fp1 *= 1e-250; fl *= 1e-250; f1 *= 1e-250; }
        }
        f0 = f;
        if (l == 1) fl = f1;
        double scale = (fabs(j0) > fabs(j1)) ? j0 / f0 : j1 / f1;
        val = fl * scale;
    }
    if (x < 0 && (l & 1)) val = -val;
    return val;
}

double gsl_sf_bessel_yl(const int l, const double x)
{
    if (l < 0) return 0.0;
    double y0 = -cos(x) / x;
    if (l == 0) return y0;
    double y1 = -cos(x) / (x * x) - sin(x) / x;
    double a = y0, b = y1;
    for (int n = 1; n < l; n++) {
        double c = (2.0 * n + 1.0) / x * b - a;
        a = b; b = c;
    }
    return b;
}

double gsl_sf_legendre_Plm(const int l, const int m, const double x)
{
    if (m < 0 || l < m) return 0.0;
    double pmm = 1.0;
    double root = sqrt(1.0 - x) * sqrt(1.0 + x);
    double fact = 1.0;
    for (int i = 1; i <= m; i++) { pmm *= -fact * root; fact += 2.0; }
    if (l == m) return pmm;
    double pmmp1 = x * (2.0 * m + 1.0) * pmm;
    if (l == m + 1) return pmmp1;
    double pll = 0.0;
    for (int ll = m + 2; ll <= l; ll++) {
        pll = (x * (2.0 * ll - 1.0) * pmmp1 - (ll + m - 1.0) * pmm) / (ll - m);
        pmm = pmmp1; pmmp1 = pll;
    }
    return pll;
}

gsl_vector *gsl_vector_alloc(const size_t n)
{
    gsl_vector *v = (gsl_vector *)malloc(sizeof(gsl_vector));
    v->size = n; v->data = (double *)calloc(n, sizeof(double));
    return v;
}
void gsl_vector_free(gsl_vector *v) { if (v) { free(v->data); free(v); } }
void gsl_vector_set(gsl_vector *v, const size_t i, double x) { v->data[i] = x; }
double gsl_vector_get(const gsl_vector *v, const size_t i) { return v->data[i]; }
gsl_matrix *gsl_matrix_alloc(const size_t n1, const size_t n2)
{
    gsl_matrix *m = (gsl_matrix *)malloc(sizeof(gsl_matrix));
    m->size1 = n1; m->size2 = n2; m->data = (double *)calloc(n1 * n2, sizeof(double));
    return m;
}
void gsl_matrix_free(gsl_matrix *m) { if (m) { free(m->data); free(m); } }
void gsl_matrix_set(gsl_matrix *m, const size_t i, const size_t j, double x) { m->data[i * m->size2 + j] = x; }
double gsl_matrix_get(const gsl_matrix *m, const size_t i, const size_t j) { return m->data[i * m->size2 + j]; }
gsl_eigen_symmv_workspace *gsl_eigen_symmv_alloc(const size_t n)
{
    gsl_eigen_symmv_workspace *w = (gsl_eigen_symmv_workspace *)malloc(sizeof(*w));
    w->size = n;
    return w;
}

/* cyclic Jacobi: A is destroyed, eval gets the eigenvalues, evec's columns the vectors */
int gsl_eigen_symmv(gsl_matrix *A, gsl_vector *eval, gsl_matrix *evec, gsl_eigen_symmv_workspace *w)
{
    (void)w;
    const size_t n = A->size1;
    double *a = A->data, *v = evec->data;
    for (size_t i = 0; i < n; i++)
        for (size_t j = 0; j < n; j++) v[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0;
        for (size_t i = 0; i < n; i++)
            for (size_t j = i + 1; j < n; j++) off += a[i * n + j] * a[i * n + j];
        if (off < 1e-300) break;
        for (size_t p = 0; p < n; p++) {
            for (size_t q = p + 1; q < n; q++) {
                double apq = a[p * n + q];
                if (fabs(apq) < 1e-300) continue;
                double app = a[p * n + p], aqq = a[q * n + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (size_t k = 0; k < n; k++) {
                    double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (size_t k = 0; k < n; k++) {
                    double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
                for (size_t k = 0; k < n; k++) {
                    double vkp = v[k * n + p], vkq = v[k * n + q];
                    v[k * n + p] = c * vkp - s * vkq;
                    v[k * n + q] = s * vkp + c * vkq;
                }
            }
        }
    }
    for (size_t i = 0; i < n; i++) eval->data[i] = a[i * n + i];
    return 0;
}
