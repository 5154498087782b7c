/* FP64 CPU restatement of the reference FMM-BEM algorithm (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  Built into oracle/_build/liboracle.so and loaded by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg, to test against.  The product
 * library never links or calls it.
 *
 * Complex numbers are interleaved (re, im) doubles.  Coefficient vectors of order p hold
 * p*p entries in the reference's order NM2IDX0(n,m) = n*n+n+m (translation.h:60-62).
 */
#ifndef FMMBEM_ORACLE_H
#define FMMBEM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* special functions */
void orc_sph_jn(int N, double x, double *out);           /* j_n(x), n = 0..N-1 */
void orc_sph_yn(int N, double x, double *out);           /* y_n(x), n = 0..N-1 */
void orc_legendre_Q(int p, double ct, double *out);      /* orthonormal Q_n^m, index n(n+1)/2+m */
void orc_basis_R(int p, double k, const double *v, double *out); /* R_n^m(v), p*p complex */
void orc_basis_S(int p, double k, const double *v, double *out); /* S_n^m(v), p*p complex */
double orc_aC(int n, int m);
double orc_bC(int n, int m);

/* translation tables (sparse layouts of translation.cu:12-20) */
int orc_rot_size(int p);
int orc_coax_size(int p);
void orc_rot_H(double beta, int p, double *H);           /* stable (Wigner-d) rotation coefficients */
void orc_rot_H_recur(double beta, int p, double *H);     /* the reference's H recurrence, restated */
void orc_coax(double k, double t, int p, int sr, double *C); /* complex, sparse coaxial layout */
void orc_rot_matrix(double alpha, double beta, double gamma, int p, double *R); /* complex sparse */
void orc_rcr(double k, const double *t, int p, int sr, const double *x, double *y);

/* quadrature and element integrals */
int orc_rule(int rule, double *bary, double *w);          /* returns point count */
void orc_gauss_legendre(int n, double *x, double *w);
void orc_elem_G(double k, const double *nod9, const double *y, int rule, int sgl, double *out);
void orc_elem_dG(double k, const double *nod9, const double *y, int rule, int sgl, double *out);
void orc_elem_R(double k, const double *nod9, const double *c, int p, int rule, int deriv, double *out);
void orc_dirdev_R(double k, int n, int m, const double *nrml, const double *x, double *out);
void orc_elem_dGdny(double k, const double *nod9, const double *nrml, const double *y, int sgl, double *out);
void orc_elem_hyper(double k, const double *nod9, const double *nrml, const double *y, int sgl, int nth, double *out);
void orc_diff_coeff(double k, const double *coeff, int p, const double *nrml, double *out);

void orc_elem_hyper_maue(double k, const double *nod9, const double *x, const double *nx, int rule, int sgl, double *out);

/* FMM operator  y = a x + (1 + alpha d/dn_y)(b L + c M) x  on collocation points y at the
 * triangle centroids (alpha: Burton-Miller coupling, 0 for the conventional operator) */
typedef struct orc_fmm orc_fmm;
orc_fmm *orc_fmm_create(int nv, const double *V, int nf, const int *F, double k,
                        double a_re, double a_im, double b_re, double b_im, double c_re, double c_im,
                        double al_re, double al_im, int rule, int lmax, const int *nbox, const long long *boxes,
                        const int *elem_leaf, const int *p_level, double d, const double *pt_min,
                        int nthreads);
void orc_fmm_apply(orc_fmm *f, const double *x, double *y);
/* y = A x (transpose = 0) or y = A^T x (transpose = 1) */
void orc_fmm_apply2(orc_fmm *f, const double *x, double *y, int transpose);
void orc_fmm_destroy(orc_fmm *f);
long long orc_fmm_num_sr(const orc_fmm *f, int l);
long long orc_fmm_num_near(const orc_fmm *f);

/* dense reference operator (all pairs by direct quadrature), same a, b, c, alpha */
void orc_dense_apply(int nv, const double *V, int nf, const int *F, double k,
                     double a_re, double a_im, double b_re, double b_im, double c_re, double c_im,
                     double al_re, double al_im, int rule, const double *x, double *y, int nthreads);

/* the same operator as an explicit row-major nf x nf matrix (entry (i, j): element j at
 * the centroid of element i) */
void orc_dense_matrix(int nv, const double *V, int nf, const int *F, double k,
                      double a_re, double a_im, double b_re, double b_im, double c_re, double c_im,
                      double al_re, double al_im, int rule, double *out, int nthreads);

/* field of the operator's layer potentials at exterior points, -(b L + c M) p: the scattered
 * pressure for the exterior problem (c = -1, b = dp/dn / p; rigid: b = 0) */
void orc_far_field(int nv, const double *V, int nf, const int *F, double k, double b_re, double b_im, double c_re,
                   double c_im, int rule,
                   const double *p, int npts, const double *pts, double *out, int nthreads);
/* Mie series: scattered pressure of a rigid sphere (radius a) for exp(ikz) */
void orc_mie_rigid(double k, double a, int npts, const double *pts, double *out);
/* Mie series for the sphere with dp/dn = i k beta p (n outward) */
void orc_mie_impedance(double k, double a, double beta_re, double beta_im, int npts, const double *pts, double *out);

#ifdef __cplusplus
}
#endif
#endif
