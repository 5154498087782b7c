/* translation.h -- the reference's translation interface (translation.h:128-335 of
 * ZiqiFrancisFan/FMBEM_GPU_C) as implemented by libfmmbem.so.
 *
 * The reference declares these with C++ linkage and includes GSL; this header declares
 * them extern "C" and needs no GSL, so the reference's main.c builds against it as C or
 * C++.  Routines that returned gsl_complex (rglBasis, sglBasis, gsl_sf_bessel_hl) are not
 * part of this interface.  Matrix generators run on the GPU in FP64 and return FP32
 * arrays in host memory, as the reference's do; the rotation coefficients come from the
 * stable Wigner-d recurrence instead of the reference's recurrence in m.
 */
#ifndef NUMERICAL_H
#define NUMERICAL_H

#include <cuda_runtime.h>
#include <cuComplex.h>
#include <stdio.h>
#include <stdlib.h>
#include "structs.h"

#ifdef __cplusplus
extern "C" {
#endif

#ifndef TRUNCERR
#define TRUNCERR (0.05f)
#endif
#ifndef NM2IDX0
#define NM2IDX0(n, m) ((n) * (n) + (m) + (n))
#endif
#ifndef HOST_CALL
#define HOST_CALL(x) do { if ((x) != EXIT_SUCCESS) { printf("Error at %s:%d\n", __FILE__, __LINE__); return EXIT_FAILURE; } } while (0)
#endif
#ifndef CUDA_CALL
#define CUDA_CALL(x) do { if ((x) != cudaSuccess) { printf("Error at %s:%d\n", __FILE__, __LINE__); return EXIT_FAILURE; } } while (0)
#endif

int sparseRotSize(const int p);                                       /* translation.cu:12 */
int sparseCoaxTransSize(const int p);                                 /* translation.cu:17 */
void reduceSparseRotMat(const cuFloatComplex *rot1, cuFloatComplex *rot2, const int p2); /* translation.cu:22 */
void reduceSparseCoaxTransMat(const cuFloatComplex *coaxMat1, const int p1, cuFloatComplex *coaxMat2,
                              const int p2);                          /* translation.cu:34 */
void printMat_cuFloatComplex(const cuFloatComplex *A, const int numRow, const int numCol, const int lda); /* :58 */
cuFloatComplex cplxExp(const float theta);                            /* translation.cu:111 */
double factorial(const int n);                                        /* translation.cu:129 */
float aCoeff(const int n, const int m);                               /* translation.cu:189 */
float bCoeff(const int n, const int m);                               /* translation.cu:199 */

/* sparse rotation matrices for numRot angles at order p (translation.cu:1297) */
int genSparseRotMats(const rotAng *rotAngle, const int numRot, const int p, cuFloatComplex *sparseMat);
/* sparse coaxial matrices for numVec translation lengths (translation.cu:822, 912, 982) */
int genRRSparseCoaxTransMat(const float wavNum, const float *vec, const int numVec, const int p, cuFloatComplex *sparseMat);
int genSSSparseCoaxTransMat(const float wavNum, const float *vec, const int numVec, const int p, cuFloatComplex *sparseMat);
int genSRSparseCoaxTransMat(const float wavNum, const float *vec, const int numVec, const int p, cuFloatComplex *sparseMat);
/* block products (translation.cu:1552, 1593) */
void cuSparseRotVecMul(const cuFloatComplex *mat, const cuFloatComplex *vec, const int p, cuFloatComplex *prod);
void cuSparseCoaxTransMatVecMul(const cuFloatComplex *mat, const cuFloatComplex *vec, const int p, cuFloatComplex *prod);

/* translation geometry tables (translation.cu:2479-2969) */
void genSRCoaxTransVecsRotAngles(const int l, const double d, const cartCoord_d pt_min, float **pVec, int *pNumVec,
                                 rotAng **pRotAngle, int *pNumRotAng);
void genSSCoaxTransVecsRotAngles(const int l, const double d, const cartCoord_d pt_min, float **pVec, int *pNumVec,
                                 rotAng **pRotAngle, int *pNumRotAng);
void genRRCoaxTransVecsRotAngles(const int l, const double d, const cartCoord_d pt_min, float **pVec, int *pNumVec,
                                 rotAng **pRotAngle, int *pNumRotAng);
void genSSIdxArrs(int **fmmLevelSet, const int lmax, const cartCoord_d pt_min, const double d,
                  const float *rrCoaxTransVec, const int numRRTransVec, const rotAng *ang, const int numRot,
                  transIdx **ssTransIdxLevelSet, int **ssTransDestArr);
void genSRIdxArrs(int **fmmLevelSet, int **SRNumLevelArr, const int lmax, const cartCoord_d pt_min, const double d,
                  const float *srCoaxTransVec, const int numSRTransVec, const rotAng *ang, const int numRot,
                  transIdx **srTransIdxLevelArr, int **srTransOriginArr, int **srTransDestArr);
void genRRIdxArrs(int **fmmLevelSet, const int lmax, const cartCoord_d pt_min, const double d,
                  const float *rrCoaxTransVec, const int numRRTransVec, const rotAng *ang, const int numRot,
                  transIdx **rrTransIdxLevelSet, int **rrTransOriginArr);

/* octree lifecycle (translation.cu:2971, 3007, 3350) */
void initOctree(octree *oct);
int genOctree(const char *filename, const float wavNum, const int s, octree *oct);
void destroyOctree(octree *oct);

/* the single-layer operator: prod = L q at the element centroids (translation.cu:3412).
 * The reference stops after the downward pass; this computes the complete operator (near
 * field with the singular self term, M2L/M2M/L2L, and L2P) with the FP64 GPU matvec. */
int OprL(const float wavNum, const octree *oct, const float *intPt, const float *intWgt, const cuFloatComplex *q,
         cuFloatComplex *prod);

#ifdef __cplusplus
}
#endif
#endif /* NUMERICAL_H */
