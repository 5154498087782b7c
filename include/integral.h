/* integral.h -- the reference's boundary-integral interface (integral.h:17-69 of
 * ZiqiFrancisFan/FMBEM_GPU_C) as implemented by libfmmbem.so: Gauss-Legendre parameters,
 * the Green's function, element integrals of G, dG/dn_x, dG/dn_y and d2G/dn_x dn_y with the
 * collapsed Gauss rule (regular) and the centroid split or the polar finite part (singular
 * self term), element moments of the regular basis R_n^m and of dR_n^m/dn, and the
 * multipole coefficients of one element.
 *
 * All are host routines on the reference's FP32 arguments.  green, triElemIntegral_G_* and
 * triElemIntegral_pGp1n_* repeat the reference's FP32 arithmetic; the others compute in FP64
 * and round the result to FP32 once.  pt/wgt are the INTORDER-point Gauss rule of
 * genGaussParams. */
#ifndef INTEGRAL_H
#define INTEGRAL_H

#ifndef INTORDER
#define INTORDER 3
#endif

#include "translation.h"

#ifdef __cplusplus
extern "C" {
#endif

extern float INTPT_h[INTORDER];
extern float INTWGT_h[INTORDER];

int genGaussParams(const int n, float *pt, float *wgt);               /* integral.cu:23 */
int gaussPtsToDevice(const float *pt, const float *wgt);              /* integral.cu:65 */
cuFloatComplex green(const float k, const cartCoord x, const cartCoord y);                         /* :72 */
cuFloatComplex triElemIntegral_G_nsgl(const float wavNum, const cartCoord nod[3], const cartCoord y,
                                      const float *pt, const float *wgt);                          /* :80 */
cuFloatComplex triElemIntegral_G_sgl(const float wavNum, const cartCoord nod[3], const float *pt,
                                     const float *wgt);                                            /* :202 */
cuFloatComplex triElemIntegral_pGp1n_nsgl(const float wavNum, const cartCoord nod[3], const cartCoord y,
                                          const float *pt, const float *wgt);                      /* :417 */
cuFloatComplex triElemIntegral_pGp1n_sgl(const float wavNum, const cartCoord nod[3], const float *pt,
                                         const float *wgt);                                        /* :485 */

/* int_T R_n^m(x - x_lp) dS_x; zero for |m| > n (integral.cu:251-282) */
cuFloatComplex triElemIntegral_R(const float wavNum, const cartCoord nod[3], const int n, const int m,
                                 const cartCoord x_lp, const float *pt, const float *wgt);
/* nrml . grad R_n^m at x (Gumerov-Duraiswami differentiation relations, integral.cu:284-331) */
cuFloatComplex dirDev_R(const float wavNum, const int n, const int m, const cartCoord nrml, const cartCoord x);
/* int_T dR_n^m(x - x_lp)/dn_x dS_x with the element's unit normal (integral.cu:333-367) */
cuFloatComplex triElemIntegral_pRpn(const float wavNum, const cartCoord nod[3], const int n, const int m,
                                    const cartCoord x_lp, const float *pt, const float *wgt);
/* int_T dG(x, y)/dn_y dS_x, nrml the normal at y (integral.cu:509-537) */
cuFloatComplex triElemIntegral_pGp2n_nsgl(const float wavNum, const cartCoord nod[3], const cartCoord nrml,
                                          const cartCoord y, const float *pt, const float *wgt);
/* the same at y = the centroid of T, centroid split (integral.cu:539-601) */
cuFloatComplex triElemIntegral_pGp2n_sgl(const float wavNum, const cartCoord nod[3], const float *pt,
                                         const float *wgt);
/* int_T d2G(x, y)/dn_x dn_y dS_x, n_x the element's unit normal, nrml_y the normal at y
 * (integral.cu:624-660) */
cuFloatComplex triElemIntegral_p2Gp1np2n_nsgl(const float wavNum, const cartCoord nod[3], const cartCoord nrml_y,
                                              const cartCoord y, const float *pt, const float *wgt);
/* the Hadamard finite part of the same at the centroid of the flat element,
 * -1/(4 pi) [int_0^{2 pi} e^{ik rho}/rho dtheta - 2 pi i k], INTORDER points in theta
 * (integral.cu:738-751) */
cuFloatComplex triElemIntegral_p2Gp1np2n_sgl(const float wavNum, const cartCoord nod[3], const float *pt,
                                             const float *wgt);
/* coeff_n (p^2 entries): the coefficients on R_n^m, n < p, of d/dn sum_{n<=p} coeff_n^m R_n^m;
 * coeff holds (p+1)^2 entries (integral.cu:753-823) */
void cmptDiffCoeff(const float wavNum, const cuFloatComplex *coeff, const int p, const cartCoord nrml,
                   cuFloatComplex *coeff_n);
/* coeff (p^2 entries) = i k q int_T R_n^{-m}(x - x_lp) dS_x for element elem of the node array
 * pt: its single layer's multipole coefficients about x_lp (integral.cu:825-840) */
void bottomLevelCoeff_L(const float wavNum, const triElem elem, const cuFloatComplex q, const cartCoord *pt,
                        const cartCoord x_lp, const float *intPt, const float *intWgt, cuFloatComplex *coeff,
                        const int p);

#ifdef __cplusplus
}
#endif
#endif /* INTEGRAL_H */
