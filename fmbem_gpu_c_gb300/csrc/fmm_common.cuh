// Shared definitions for the GB300 FMM-BEM kernels: index maps, complex helpers, special
// functions in FP64, and error plumbing.
#pragma once
#include <cuda_runtime.h>
#include <cuComplex.h>
#include <stdint.h>
#include <stdio.h>
#include <math.h>

#ifndef FMM_PI
#define FMM_PI 3.14159265358979323846
#endif

// coefficient index of (n, m) in the reference's order NM2IDX0 (translation.h:60-62)
__host__ __device__ __forceinline__ int nm_idx(int n, int m) { return n * n + n + m; }
// sparse rotation layout: block n at n(4n^2-1)/3, entry (m', m) column-major (translation.cu:12-15, 1221-1235)
__host__ __device__ __forceinline__ int rot_off(int n) { return n * (4 * n * n - 1) / 3; }
__host__ __device__ __forceinline__ int rot_size(int p) { return p * (4 * p * p - 1) / 3; }
// sparse coaxial layout: block m at m(2m^2-(3+6p)m+1+6(p+p^2))/6, entry (n', n) column-major (translation.cu:17-32)
__host__ __device__ __forceinline__ int coax_off(int p, int m) { return m * (2 * m * m - (3 + 6 * p) * m + 1 + 6 * (p + p * p)) / 6; }
__host__ __device__ __forceinline__ int coax_size(int p) { return p * (2 * p * p + 3 * p + 1) / 6; }

// G&D recurrence coefficients a_n^m, b_n^m (translation.cu:189-212), FP64
__host__ __device__ __forceinline__ double coefA(int n, int m)
{
    int am = m < 0 ? -m : m;
    if (n >= am) return sqrt((double)(n + 1 + m) * (double)(n + 1 - m) / ((2.0 * n + 1.0) * (2.0 * n + 3.0)));
    return 0.0;
}
__host__ __device__ __forceinline__ double coefB(int n, int m)
{
    if (m >= 0 && n >= m) return sqrt((double)(n - m - 1) * (double)(n - m) / ((2.0 * n - 1.0) * (2.0 * n + 1.0)));
    if (-n <= m && m < 0) return -sqrt((double)(n - m - 1) * (double)(n - m) / ((2.0 * n - 1.0) * (2.0 * n + 1.0)));
    return 0.0;
}

// ---------------------------------------------------------------- complex helpers
template <typename T> struct cplx_t;
template <> struct cplx_t<double> { typedef double2 type; };
template <> struct cplx_t<float> { typedef float2 type; };

__host__ __device__ __forceinline__ double2 mk2(double a, double b) { return make_double2(a, b); }
__host__ __device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { return mk2(a.x + b.x, a.y + b.y); }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { return mk2(a.x - b.x, a.y - b.y); }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) { return mk2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename C> __host__ __device__ __forceinline__ C cconjmul(C a, C b) { return mk2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); } // conj(a)*b
template <typename C, typename R> __host__ __device__ __forceinline__ C cscale(C a, R s) { return mk2(a.x * s, a.y * s); }

// ---------------------------------------------------------------- special functions (device, FP64)
// Spherical Bessel j_n(x), n = 0..N-1, by Miller's backward recurrence normalised with j0 or j1.
__host__ __device__ inline void sph_jn_array(int N, double x, double *j)
{
    if (N <= 0) return;
    if (x == 0.0) {
        j[0] = 1.0;
        for (int n = 1; n < N; n++) j[n] = 0.0;
        return;
    }
    double s = sin(x), c = cos(x);
    double j0 = s / x, j1 = s / (x * x) - c / x;
    int big = N > (int)x ? N : (int)x;
    int start = big + 40 + (int)(4.0 * sqrt((double)big + 1.0));
    double fp1 = 0.0, f = 1e-300, f1 = 0.0;
    for (int n = start; n >= 1; n--) {
        double fm1 = (2.0 * n + 1.0) / x * f - fp1;
        fp1 = f;
        f = fm1;
        if (n - 1 < N) j[n - 1] = f;
        if (n - 1 == 1) f1 = f;
        if (fabs(f) > 1e250) {
            f *= 1e-250; fp1 *= 1e-250; f1 *= 1e-250;
            for (int q = (n - 1 < N ? n - 1 : N); q < N; q++) j[q] *= 1e-250;
        }
    }
    double scale = (fabs(j0) > fabs(j1)) ? j0 / f : j1 / f1;
    for (int n = 0; n < N; n++) j[n] *= scale;
}

__host__ __device__ inline void sph_yn_array(int N, double x, double *y)
{
    if (N <= 0) return;
    y[0] = -cos(x) / x;
    if (N == 1) return;
    y[1] = -cos(x) / (x * x) - sin(x) / x;
    for (int n = 1; n + 1 < N; n++) y[n + 1] = (2.0 * n + 1.0) / x * y[n] - y[n - 1];
}

// Orthonormal associated Legendre Q_n^m(cos theta) without the Condon-Shortley phase, so that
// the reference's Y_n^m (sphHrmc with GSL's Plm, translation.cu:153-169) equals
// Q_n^{|m|} e^{i m phi}.  Index n(n+1)/2 + m, 0 <= m <= n < p.
__host__ __device__ inline void legendre_Q(int p, double ct, double *Q)
{
    double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    Q[0] = 0.28209479177387814; // 1/sqrt(4 pi)
    for (int m = 1; m < p; m++) Q[m * (m + 1) / 2 + m] = sqrt((2.0 * m + 1.0) / (2.0 * m)) * st * Q[(m - 1) * m / 2 + (m - 1)];
    for (int m = 0; m < p; m++) {
        if (m + 1 < p) Q[(m + 1) * (m + 2) / 2 + m] = sqrt(2.0 * m + 3.0) * ct * Q[m * (m + 1) / 2 + m];
        for (int n = m + 2; n < p; n++) {
            double a = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
            double b = sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) / (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
            Q[n * (n + 1) / 2 + m] = a * (ct * Q[(n - 1) * n / 2 + m] - b * Q[(n - 2) * (n - 1) / 2 + m]);
        }
    }
}

// ---------------------------------------------------------------- errors
#define FMM_CUDA_TRY(call)                                                                    \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            fmm_set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return FMM_ERR_CUDA;                                                              \
        }                                                                                     \
    } while (0)

void fmm_set_error(const char *fmt, ...);
