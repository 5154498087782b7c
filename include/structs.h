/* structs.h -- geometry and octree types of the reference's C interface.
 *
 * Reference: structs.h:29-198 (ZiqiFrancisFan/FMBEM_GPU_C).  The struct layouts are kept
 * field for field so that code written against the reference (its main.c) compiles and
 * links against libfmmbem.so unchanged; the functions are this library's implementations.
 */
#ifndef STRUCTS_H
#define STRUCTS_H

#include <cuComplex.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef PI
#define PI 3.1415926535897932f
#endif

#ifndef IDXC0
#define IDXC0(row, column, stride) ((column) * (stride) + (row))
#endif

/* triangular element: node indices and Robin coefficients alpha p + beta dp/dn = gamma */
struct triElem {
    int node[3];
    cuFloatComplex alpha;
    cuFloatComplex beta;
    cuFloatComplex gamma;
};
struct cartCoord { float x; float y; float z; };
struct cartCoord_double { double x; double y; double z; };
struct sphCoord { float r; float theta; float phi; };
struct sphCoord_double { double r; double theta; double phi; };
struct rotAng { float alpha; float beta; float gamma; };
/* index of the coaxial translation and of the rotation angle of one translation */
struct transIdx { int coaxIdx; int rotIdx; };

typedef struct triElem triElem;
typedef struct cartCoord cartCoord;
typedef struct cartCoord_double cartCoord_d;
typedef struct sphCoord sphCoord;
typedef struct sphCoord_double sphCoord_d;
typedef struct rotAng rotAng;
typedef struct transIdx transIdx;

/* the octree of genOctree (translation.cu:3007-3348); arrays are host memory owned by the
 * struct and released by destroyOctree */
struct octree {
    cartCoord *pt;
    triElem *elem;
    int numPt;
    int numElem;
    int **fmmLevelSet;            /* per level l-2: count-prefixed Morton box numbers */
    int lmax;
    int lmin;
    double d;
    cartCoord_d pt_min;
    cuFloatComplex *rotMat1;      /* sparse rotation matrices (alpha, beta, 0) at pmax */
    cuFloatComplex *rotMat2;      /* sparse rotation matrices (0, beta, alpha) at pmax */
    cuFloatComplex *srCoaxMat;    /* sparse (S|R) coaxial matrices at pmax_coax */
    cuFloatComplex *rrCoaxMat;    /* sparse (R|R) coaxial matrices at pmax_coax */
    float *srCoaxTransVec;
    int numSRCoaxTransVec;
    float *rrCoaxTransVec;
    int numRRCoaxTransVec;
    rotAng *ang;
    int numRotAng;
    float eps;
    float maxWavNum;
    int pmax;
    int pmax_coax;
    int *btmLvlElemIdx;
    transIdx **ssTransIdx;
    transIdx **srTransIdx;
    transIdx **rrTransIdx;
    int **ssTransDestArr;
    int **srNumLevelArr;
    int **srTransOriginArr;
    int **srTransDestArr;
    int **rrTransOriginArr;
};
typedef struct octree octree;

float dotProd(const cartCoord u, const cartCoord v);
cartCoord scalarMul(const float lambda, const cartCoord v);
cartCoord crossProd(const cartCoord u, const cartCoord v);
cartCoord cartCoordAdd(const cartCoord u, const cartCoord v);
cartCoord cartCoordSub(const cartCoord u, const cartCoord v);
float cartNorm(const cartCoord x);
float cartDist(const cartCoord x, const cartCoord y);
cartCoord normalize(const cartCoord x);
sphCoord cart2sph(const cartCoord s);
sphCoord_d cart_d2sph_d(const cartCoord_d s);
sphCoord sphCoord_d2sphCoord(const sphCoord_d s);
cartCoord sph2cart(const sphCoord s);
cartCoord_d cartCoordSub_d(const cartCoord_d u, const cartCoord_d v);
cartCoord_d triCentroid_d(const cartCoord_d nod[3]);
cartCoord cartCoord_d2cartCoord(const cartCoord_d s);
cartCoord_d cartCoord2cartCoord_d(const cartCoord s);
void printCartCoordArray_d(const cartCoord_d *arr, const int num);
void printCartCoordArray(const cartCoord *arr, const int num);
void printSphCoordArray(const sphCoord *arr, const int num);
void printFloatArray(const float *arr, const int num);
void printIntArray(const int *arr, const int num);
void printRotAngArray(const rotAng *angle, const int numAng);
bool equalRotArrays(const rotAng *ang1, const rotAng *ang2, const int numAng);
void bubbleSort(float *arr, const int n);
void sortRotArray(rotAng *ang, const int numRot, const float eps);

#ifdef __cplusplus
}
#endif
#endif /* STRUCTS_H */
