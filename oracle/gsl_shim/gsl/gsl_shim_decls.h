/* Project-written stand-in for the small part of the GNU Scientific Library that the
 * reference FMM-BEM sources call.  Test infrastructure only: it exists so the reference's
 * own translation.cu / integral.cu can be compiled here as an oracle.  The implementations
 * (oracle/gsl_shim/gsl_shim.c) restate the published algorithms; they are checked against
 * SciPy in tests/test_oracle_pins.py. */
#ifndef FMMBEM_GSL_SHIM_DECLS_H
#define FMMBEM_GSL_SHIM_DECLS_H
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { double dat[2]; } gsl_complex;
#define GSL_REAL(z) ((z).dat[0])
#define GSL_IMAG(z) ((z).dat[1])
gsl_complex gsl_complex_rect(double x, double y);
gsl_complex gsl_complex_mul(gsl_complex a, gsl_complex b);
gsl_complex gsl_complex_mul_real(gsl_complex a, double x);
double gsl_sf_bessel_jl(const int l, const double x);
double gsl_sf_bessel_yl(const int l, const double x);
double gsl_sf_legendre_Plm(const int l, const int m, const double x);
typedef struct { size_t size; double *data; } gsl_vector;
typedef struct { size_t size1, size2; double *data; } gsl_matrix;
typedef struct { size_t size; } gsl_eigen_symmv_workspace;
gsl_vector *gsl_vector_alloc(const size_t n);
void gsl_vector_free(gsl_vector *v);
void gsl_vector_set(gsl_vector *v, const size_t i, double x);
double gsl_vector_get(const gsl_vector *v, const size_t i);
gsl_matrix *gsl_matrix_alloc(const size_t n1, const size_t n2);
void gsl_matrix_free(gsl_matrix *m);
void gsl_matrix_set(gsl_matrix *m, const size_t i, const size_t j, double x);
double gsl_matrix_get(const gsl_matrix *m, const size_t i, const size_t j);
gsl_eigen_symmv_workspace *gsl_eigen_symmv_alloc(const size_t n);
int gsl_eigen_symmv(gsl_matrix *A, gsl_vector *eval, gsl_matrix *evec, gsl_eigen_symmv_workspace *w);
#ifdef __cplusplus
}
#endif
#endif
