/* octree.h -- the reference's octree interface (octree.h:30-150 of ZiqiFrancisFan/FMBEM_GPU_C),
 * implemented by libfmmbem.so with the same results: Morton box numbers with digit 4x+2y+z,
 * count-prefixed sets in first-occurrence order, I2/I4 in the reference's enumeration order.
 * Unlike the reference, set routines have no MAX = 100000 stack limit. */
#ifndef OCTREE_H
#define OCTREE_H

#include "structs.h"
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef MAX
#define MAX 100000
#endif

void findNum(const char *filename, int *pV, int *pE);                 /* octree.c:563 */
int readOBJ(const char *filename, cartCoord_d *p, triElem *e);        /* octree.c:586 */
void printSet(const int *set);                                        /* octree.c:31 */
bool arrEqual(const int *a, const int *b, const int num);             /* octree.c:18 */
int parent(int num);                                                  /* octree.c:44 */
int child(int num, int cld);                                          /* octree.c:49 */
void children(const int num, int *cldrn);                             /* octree.c:54 */
cartCoord_d scale(const cartCoord_d x, const cartCoord_d x_min, const double d);    /* octree.c:62 */
cartCoord_d descale(const cartCoord_d x_s, const cartCoord_d x_min, const double d); /* octree.c:71 */
double descale_1d(const double a, const double D, const double v_min);              /* octree.c:812 */
void scalePnts(const cartCoord_d *pnt, const int numPnts, const cartCoord_d pnt_min, const double d,
               cartCoord_d *pnt_scaled);                              /* octree.c:80 */
void dec2bin_frac(double s, int l, int *h);                           /* octree.c:88 */
void bitIntleave(const int *x, const int *y, const int *z, const int l, int *result); /* octree.c:127 */
int indArr2num(const int *ind, const int l, const int d);             /* octree.c:136 */
int pnt2boxnum(const cartCoord_d pnt, const int l);                   /* octree.c:158 */
cartCoord_d boxCenter(const int num, const int l);                    /* octree.c:185 */
int neighbors(const int num, const int l, int *numNeighbors, int *nbr); /* octree.c:237 */
void createSet(const int *elems, const int numElems, int *set);       /* octree.c:393 */
bool isMember(const int t, const int *set);                           /* octree.c:412 */
bool isEmpty(const int *set);                                         /* octree.c:424 */
void intersection(const int *set1, const int *set2, int *set3);       /* octree.c:433 */
void Union(const int *set1, const int *set2, int *set3);              /* octree.c:445 */
void difference(const int *set1, const int *set2, int *set3);         /* octree.c:459 */
void pnts2numSet(const cartCoord_d *pnts, const int numPnts, const int l, int *set); /* octree.c:471 */
void I2(const int num, const int l, int *set);                        /* octree.c:497 */
void I4(const int num, const int l, int *set);                        /* octree.c:517 */
void orderArray(const int *a, const int num, int *ind);               /* octree.c:546 */
int deterLmax(const cartCoord_d *pnts, const int numPnts, const int s); /* octree.c:635 */
void findBoundingCube(const cartCoord_d *pnts, const int numPnts, const double eps, cartCoord_d *pnts_b,
                      double *d);                                     /* octree.c:681 */
void srcBoxes(const cartCoord_d *pnts, const triElem *elems, const int numElems, const int s, int *srcBoxSet,
              int *lmax, double *D, cartCoord_d *pnt_min);            /* octree.c:749 */
int truncNum(const double k, const double eps, const double sigma, const double a);   /* octree.c:777 */
int truncNum_2(const double wavNum, const double eps, const double sigma, const double a); /* octree.c:798 */
void prntLevelSet(const int *X, const int l, int *X_n);               /* octree.c:816 */
void FMMLevelSet(const int *btmLvl, const int lmax, int **pSet);      /* octree.c:890 */
int findSetInd(const int *X, const int num);                          /* octree.c:833 */
void sortSet(int *set);                                               /* octree.c:1034 */
void FMMLevelSetNumSR(int **pSet, const int lmax, int **numSet);      /* octree.c:908 */
void printFMMLevelSet(int **pSet, const int lmax);                    /* octree.c:932 */

#ifdef __cplusplus
}
#endif
#endif /* OCTREE_H */
