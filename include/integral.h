/* integral.h -- the reference's boundary-integral interface (integral.h:17-69 of
 * ZiqiFrancisFan/FMBEM_GPU_C) as implemented by libfmmbem.so: Gauss-Legendre parameters,
 * the Green's function, and element integrals of G and dG/dn with the collapsed Gauss rule
 * (regular) and the centroid split (singular self term). */
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

#ifdef __cplusplus
}
#endif
#endif /* INTEGRAL_H */
