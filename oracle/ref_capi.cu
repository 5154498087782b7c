/* C entry points over the reference's own sources, for building golden fixtures.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file together with the
 * reference's octree.c, structs.cu, translation.cu and integral.cu (read in place, never
 * copied) and the project-written GSL shim into oracle/_ref/libfmmref.so.  Only
 * tests/golden/make_golden.py loads it.
 *
 * The reference's translation.h / integral.h declarations have C++ linkage, so these
 * wrappers give ctypes stable names.  ref_octree_build() runs the host steps of
 * genOctree (translation.cu:3007-3342) in the same order, with the GPU matrix generation
 * left out (it needs a device), so that the level sets, interaction lists, element-to-box
 * indices and translation index arrays come from the reference's own code.
 * ref_near_lists() gives the leaf near lists I2 ∩ leaf set of that tree, and
 * ref_octree_stage_times() times the reference's CPU octree stages on a mesh file, the work
 * that oracle/octree_port.c restates for machines without the reference's sources.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "translation.h"
#include "octree.h"
#include "integral.h"

struct RefTree {
    octree oct;
    int numElem;
};

static RefTree g_tree;
static int g_have = 0;

static void srcBoxesDepth(const cartCoord_d *pnts, const triElem *elems, const int numElems,
                          const int depth, int *srcBoxSet, int *lmax, double *D, cartCoord_d *pnt_min)
{
    /* srcBoxes (octree.c:749-768) with deterLmax replaced by a fixed depth */
    cartCoord_d *ctr = (cartCoord_d *)malloc(numElems * sizeof(cartCoord_d));
    cartCoord_d bnd[8];
    cartCoord_d *scaled = (cartCoord_d *)malloc(numElems * sizeof(cartCoord_d));
    cartCoord_d nod[3];
    for (int i = 0; i < numElems; i++) {
        nod[0] = pnts[elems[i].node[0]];
        nod[1] = pnts[elems[i].node[1]];
        nod[2] = pnts[elems[i].node[2]];
        ctr[i] = triCentroid_d(nod);
    }
    findBoundingCube(ctr, numElems, 0.01, bnd, D);
    *pnt_min = bnd[0];
    scalePnts(ctr, numElems, bnd[0], *D, scaled);
    *lmax = depth;
    pnts2numSet(scaled, numElems, depth, srcBoxSet);
    free(ctr);
    free(scaled);
}

extern "C" int ref_octree_build(const char *filename, int s, int depth)
{
    octree *oct = &g_tree.oct;
    memset(oct, 0, sizeof(*oct));
    initOctree(oct);
    int numPt, numElem;
    findNum(filename, &numPt, &numElem);
    cartCoord_d *pt = (cartCoord_d *)malloc(numPt * sizeof(cartCoord_d));
    triElem *elem = (triElem *)malloc(numElem * sizeof(triElem));
    readOBJ(filename, pt, elem);
    oct->pt = (cartCoord *)malloc(numPt * sizeof(cartCoord));
    oct->elem = (triElem *)malloc(numElem * sizeof(triElem));
    oct->numPt = numPt;
    oct->numElem = numElem;
    for (int i = 0; i < numPt; i++) oct->pt[i] = cartCoord_d2cartCoord(pt[i]);
    for (int i = 0; i < numElem; i++) oct->elem[i] = elem[i];
    int *srcBoxSet = (int *)malloc((numElem + 1) * sizeof(int));
    if (depth > 0)
        srcBoxesDepth(pt, elem, numElem, depth, srcBoxSet, &oct->lmax, &oct->d, &oct->pt_min);
    else
        srcBoxes(pt, elem, numElem, s, srcBoxSet, &oct->lmax, &oct->d, &oct->pt_min);
    oct->fmmLevelSet = (int **)malloc((oct->lmax - oct->lmin + 1) * sizeof(int *));
    FMMLevelSet(srcBoxSet, oct->lmax, oct->fmmLevelSet);
    free(pt); free(elem); free(srcBoxSet);

    oct->srNumLevelArr = (int **)malloc((oct->lmax - oct->lmin + 1) * sizeof(int *));
    FMMLevelSetNumSR(oct->fmmLevelSet, oct->lmax, oct->srNumLevelArr);

    /* element -> leaf index, translation.cu:3062-3076 */
    oct->btmLvlElemIdx = (int *)malloc(oct->numElem * sizeof(int));
    for (int i = 0; i < oct->numElem; i++) {
        cartCoord nod[3], ctr;
        for (int j = 0; j < 3; j++) nod[j] = oct->pt[oct->elem[i].node[j]];
        ctr = triCentroid(nod);
        ctr = cartCoord_d2cartCoord(scale(cartCoord2cartCoord_d(ctr), oct->pt_min, oct->d));
        int num = pnt2boxnum(cartCoord2cartCoord_d(ctr), oct->lmax);
        oct->btmLvlElemIdx[i] = findSetInd(oct->fmmLevelSet[oct->lmax - oct->lmin], num);
    }

    /* angle and distance tables, translation.cu:3078-3158 and 3188-3292 */
    oct->pmax = truncNum(oct->maxWavNum, oct->eps, 1.5, pow(2, -oct->lmin) * oct->d);
    float epsilon = 0.000000001 * oct->d;
    rotAng *ang = NULL;
    float *vec = NULL;
    int numRot, numVec;
    for (int l = oct->lmin; l <= oct->lmax; l++) {
        genSRCoaxTransVecsRotAngles(l, oct->d, oct->pt_min, &vec, &numVec, &ang, &numRot);
        if (oct->numRotAng == 0) {
            oct->ang = (rotAng *)malloc(numRot * sizeof(rotAng));
            memcpy(oct->ang, ang, numRot * sizeof(rotAng));
            oct->numRotAng = numRot;
        }
        if (oct->numSRCoaxTransVec == 0) {
            oct->srCoaxTransVec = (float *)malloc(numVec * sizeof(float));
            memcpy(oct->srCoaxTransVec, vec, numVec * sizeof(float));
            oct->numSRCoaxTransVec = numVec;
        } else {
            float *tmp = (float *)malloc((oct->numSRCoaxTransVec + numVec) * sizeof(float));
            memcpy(tmp, oct->srCoaxTransVec, oct->numSRCoaxTransVec * sizeof(float));
            free(oct->srCoaxTransVec);
            for (int i = 0; i < numVec; i++) {
                bool found = false;
                for (int j = 0; j < oct->numSRCoaxTransVec; j++)
                    if (abs(vec[i] - tmp[j]) < epsilon) { found = true; break; }
                if (!found) tmp[oct->numSRCoaxTransVec++] = vec[i];
            }
            oct->srCoaxTransVec = tmp;
        }
        free(vec); free(ang);
    }
    sortRotArray(oct->ang, oct->numRotAng, oct->eps);
    bubbleSort(oct->srCoaxTransVec, oct->numSRCoaxTransVec);

    for (int pass = 0; pass < 2; pass++) {
        int lbeg = pass == 0 ? oct->lmax : oct->lmin + 1;
        int lend = pass == 0 ? oct->lmin + 1 : oct->lmax;
        int step = pass == 0 ? -1 : 1;
        for (int l = lbeg; pass == 0 ? l >= lend : l <= lend; l += step) {
            if (pass == 0)
                genSSCoaxTransVecsRotAngles(l, oct->d, oct->pt_min, &vec, &numVec, &ang, &numRot);
            else
                genRRCoaxTransVecsRotAngles(l, oct->d, oct->pt_min, &vec, &numVec, &ang, &numRot);
            if (oct->numRRCoaxTransVec == 0) {
                oct->rrCoaxTransVec = (float *)malloc(numVec * sizeof(float));
                memcpy(oct->rrCoaxTransVec, vec, numVec * sizeof(float));
                oct->numRRCoaxTransVec = numVec;
            } else {
                float *tmp = (float *)malloc((oct->numRRCoaxTransVec + numVec) * sizeof(float));
                memcpy(tmp, oct->rrCoaxTransVec, oct->numRRCoaxTransVec * sizeof(float));
                free(oct->rrCoaxTransVec);
                for (int i = 0; i < numVec; i++) {
                    bool found = false;
                    for (int j = 0; j < oct->numRRCoaxTransVec; j++)
                        if (abs(vec[i] - tmp[j]) < epsilon) { found = true; break; }
                    if (!found) tmp[oct->numRRCoaxTransVec++] = vec[i];
                }
                oct->rrCoaxTransVec = tmp;
            }
            free(vec); free(ang);
        }
    }
    bubbleSort(oct->rrCoaxTransVec, oct->numRRCoaxTransVec);

    int nl = oct->lmax - oct->lmin;
    oct->ssTransDestArr = (int **)calloc(nl > 0 ? nl : 1, sizeof(int *));
    oct->ssTransIdx = (transIdx **)calloc(nl > 0 ? nl : 1, sizeof(transIdx *));
    oct->srTransOriginArr = (int **)calloc(nl + 1, sizeof(int *));
    oct->srTransDestArr = (int **)calloc(nl + 1, sizeof(int *));
    oct->srTransIdx = (transIdx **)calloc(nl + 1, sizeof(transIdx *));
    oct->rrTransOriginArr = (int **)calloc(nl > 0 ? nl : 1, sizeof(int *));
    oct->rrTransIdx = (transIdx **)calloc(nl > 0 ? nl : 1, sizeof(transIdx *));
    genSSIdxArrs(oct->fmmLevelSet, oct->lmax, oct->pt_min, oct->d, oct->rrCoaxTransVec, oct->numRRCoaxTransVec,
                 oct->ang, oct->numRotAng, oct->ssTransIdx, oct->ssTransDestArr);
    genSRIdxArrs(oct->fmmLevelSet, oct->srNumLevelArr, oct->lmax, oct->pt_min, oct->d, oct->srCoaxTransVec,
                 oct->numSRCoaxTransVec, oct->ang, oct->numRotAng, oct->srTransIdx, oct->srTransOriginArr,
                 oct->srTransDestArr);
    genRRIdxArrs(oct->fmmLevelSet, oct->lmax, oct->pt_min, oct->d, oct->rrCoaxTransVec, oct->numRRCoaxTransVec,
                 oct->ang, oct->numRotAng, oct->rrTransIdx, oct->rrTransOriginArr);
    g_tree.numElem = numElem;
    g_have = 1;
    return 0;
}

/* scalar getters */
extern "C" int ref_lmax(void) { return g_tree.oct.lmax; }
extern "C" double ref_d(void) { return g_tree.oct.d; }
extern "C" void ref_pt_min(double *out) { out[0] = g_tree.oct.pt_min.x; out[1] = g_tree.oct.pt_min.y; out[2] = g_tree.oct.pt_min.z; }
extern "C" int ref_num_elem(void) { return g_tree.numElem; }
extern "C" int ref_level_count(int l) { return g_tree.oct.fmmLevelSet[l - 2][0]; }
extern "C" void ref_level_set(int l, int *out)
{
    int n = g_tree.oct.fmmLevelSet[l - 2][0];
    memcpy(out, g_tree.oct.fmmLevelSet[l - 2] + 1, n * sizeof(int));
}
extern "C" void ref_sr_num(int l, int *out)
{
    int n = g_tree.oct.fmmLevelSet[l - 2][0];
    memcpy(out, g_tree.oct.srNumLevelArr[l - 2], n * sizeof(int));
}
extern "C" int ref_sr_total(int l)
{
    int n = g_tree.oct.fmmLevelSet[l - 2][0], t = 0;
    for (int i = 0; i < n; i++) t += g_tree.oct.srNumLevelArr[l - 2][i];
    return t;
}
extern "C" void ref_sr_arrays(int l, int *origin, int *dest, int *coax, int *rot)
{
    int t = ref_sr_total(l);
    for (int i = 0; i < t; i++) {
        origin[i] = g_tree.oct.srTransOriginArr[l - 2][i];
        dest[i] = g_tree.oct.srTransDestArr[l - 2][i];
        coax[i] = g_tree.oct.srTransIdx[l - 2][i].coaxIdx;
        rot[i] = g_tree.oct.srTransIdx[l - 2][i].rotIdx;
    }
}
extern "C" void ref_ss_arrays(int l, int *dest, int *coax, int *rot)
{
    int n = g_tree.oct.fmmLevelSet[l - 2][0];
    for (int i = 0; i < n; i++) {
        dest[i] = g_tree.oct.ssTransDestArr[l - 3][i];
        coax[i] = g_tree.oct.ssTransIdx[l - 3][i].coaxIdx;
        rot[i] = g_tree.oct.ssTransIdx[l - 3][i].rotIdx;
    }
}
extern "C" void ref_rr_arrays(int l, int *origin, int *coax, int *rot)
{
    int n = g_tree.oct.fmmLevelSet[l - 2][0];
    for (int i = 0; i < n; i++) {
        origin[i] = g_tree.oct.rrTransOriginArr[l - 3][i];
        coax[i] = g_tree.oct.rrTransIdx[l - 3][i].coaxIdx;
        rot[i] = g_tree.oct.rrTransIdx[l - 3][i].rotIdx;
    }
}
extern "C" void ref_btm_idx(int *out) { memcpy(out, g_tree.oct.btmLvlElemIdx, g_tree.numElem * sizeof(int)); }
extern "C" int ref_num_ang(void) { return g_tree.oct.numRotAng; }
extern "C" void ref_angles(float *out)
{
    for (int i = 0; i < g_tree.oct.numRotAng; i++) {
        out[3 * i] = g_tree.oct.ang[i].alpha;
        out[3 * i + 1] = g_tree.oct.ang[i].beta;
        out[3 * i + 2] = g_tree.oct.ang[i].gamma;
    }
}
extern "C" int ref_num_sr_vec(void) { return g_tree.oct.numSRCoaxTransVec; }
extern "C" void ref_sr_vec(float *out) { memcpy(out, g_tree.oct.srCoaxTransVec, g_tree.oct.numSRCoaxTransVec * sizeof(float)); }
extern "C" int ref_num_rr_vec(void) { return g_tree.oct.numRRCoaxTransVec; }
extern "C" void ref_rr_vec(float *out) { memcpy(out, g_tree.oct.rrCoaxTransVec, g_tree.oct.numRRCoaxTransVec * sizeof(float)); }
extern "C" int ref_pmax(void) { return g_tree.oct.pmax; }

/* ---- translation tables and products (host-callable reference functions) ---- */
extern "C" void ref_sparse_rot(float alpha, float beta, float gamma, int p, float *out /* complex */)
{
    rotAng a; a.alpha = alpha; a.beta = beta; a.gamma = gamma;
    size_t sz = (size_t)(2 * p - 1) * (2 * p - 1);
    float *H = (float *)malloc(sz * sz * sizeof(float));
    rotMatsInit(&a, 1, p, H);
    sparseRotMatGen(a, p, H, (cuFloatComplex *)out);
    free(H);
}
extern "C" void ref_sparse_coax(float k, float t, int p, int sr, float *out /* complex */)
{
    size_t sz = (size_t)(2 * p - 1) * (2 * p - 1);
    cuFloatComplex *E = (cuFloatComplex *)malloc(sz * sz * sizeof(cuFloatComplex));
    if (sr) srCoaxTransMatsInit(k, &t, 1, p, E);
    else rrCoaxTransMatsInit(k, &t, 1, p, E);
    sparseCoaxTransMatGen(E, p, (cuFloatComplex *)out);
    free(E);
}
extern "C" void ref_rot_vec(const float *mat, const float *vec, int p, float *out)
{
    cuSparseRotVecMul((const cuFloatComplex *)mat, (const cuFloatComplex *)vec, p, (cuFloatComplex *)out);
}
extern "C" void ref_coax_vec(const float *mat, const float *vec, int p, float *out)
{
    cuSparseCoaxTransMatVecMul((const cuFloatComplex *)mat, (const cuFloatComplex *)vec, p, (cuFloatComplex *)out);
}
extern "C" int ref_truncnum(double k, double eps, double sigma, double a) { return truncNum(k, eps, sigma, a); }
extern "C" int ref_gauss(int n, float *pt, float *wgt) { return genGaussParams(n, pt, wgt); }
extern "C" void ref_elem_G(float k, const float *nod9, const float *y3, int sgl, float *out)
{
    float pt[INTORDER], wgt[INTORDER];
    genGaussParams(INTORDER, pt, wgt);
    cartCoord nod[3] = {{nod9[0], nod9[1], nod9[2]}, {nod9[3], nod9[4], nod9[5]}, {nod9[6], nod9[7], nod9[8]}};
    cartCoord y = {y3[0], y3[1], y3[2]};
    cuFloatComplex z = sgl ? triElemIntegral_G_sgl(k, nod, pt, wgt) : triElemIntegral_G_nsgl(k, nod, y, pt, wgt);
    out[0] = cuCrealf(z); out[1] = cuCimagf(z);
}
extern "C" void ref_elem_dGdn(float k, const float *nod9, const float *y3, int sgl, float *out)
{
    float pt[INTORDER], wgt[INTORDER];
    genGaussParams(INTORDER, pt, wgt);
    cartCoord nod[3] = {{nod9[0], nod9[1], nod9[2]}, {nod9[3], nod9[4], nod9[5]}, {nod9[6], nod9[7], nod9[8]}};
    cartCoord y = {y3[0], y3[1], y3[2]};
    cuFloatComplex z = sgl ? triElemIntegral_pGp1n_sgl(k, nod, pt, wgt) : triElemIntegral_pGp1n_nsgl(k, nod, y, pt, wgt);
    out[0] = cuCrealf(z); out[1] = cuCimagf(z);
}
extern "C" void ref_elem_R(float k, const float *nod9, int n, int m, const float *c3, int deriv, float *out)
{
    float pt[INTORDER], wgt[INTORDER];
    genGaussParams(INTORDER, pt, wgt);
    cartCoord nod[3] = {{nod9[0], nod9[1], nod9[2]}, {nod9[3], nod9[4], nod9[5]}, {nod9[6], nod9[7], nod9[8]}};
    cartCoord c = {c3[0], c3[1], c3[2]};
    cuFloatComplex z = deriv ? triElemIntegral_pRpn(k, nod, n, m, c, pt, wgt) : triElemIntegral_R(k, nod, n, m, c, pt, wgt);
    out[0] = cuCrealf(z); out[1] = cuCimagf(z);
}
/* directional derivative of R_n^m along nrml at x (dirDev_R, integral.cu:284-331) */
extern "C" void ref_dirdev_R(float k, int n, int m, const float *nrml3, const float *x3, float *out)
{
    cartCoord nr = {nrml3[0], nrml3[1], nrml3[2]}, x = {x3[0], x3[1], x3[2]};
    cuFloatComplex z = dirDev_R(k, n, m, nr, x);
    out[0] = cuCrealf(z); out[1] = cuCimagf(z);
}
/* element integrals of dG/dn_y (triElemIntegral_pGp2n_nsgl / _sgl, integral.cu:509-601) and of
 * d2G/dn_x dn_y (triElemIntegral_p2Gp1np2n_nsgl / _sgl, integral.cu:624-660, 738-751) */
extern "C" void ref_elem_dGdny(float k, const float *nod9, const float *nrml3, const float *y3, int sgl, float *out)
{
    float pt[INTORDER], wgt[INTORDER];
    genGaussParams(INTORDER, pt, wgt);
    cartCoord nod[3] = {{nod9[0], nod9[1], nod9[2]}, {nod9[3], nod9[4], nod9[5]}, {nod9[6], nod9[7], nod9[8]}};
    cartCoord nr = {nrml3[0], nrml3[1], nrml3[2]}, y = {y3[0], y3[1], y3[2]};
    cuFloatComplex z = sgl ? triElemIntegral_pGp2n_sgl(k, nod, pt, wgt) : triElemIntegral_pGp2n_nsgl(k, nod, nr, y, pt, wgt);
    out[0] = cuCrealf(z); out[1] = cuCimagf(z);
}
extern "C" void ref_elem_hyper(float k, const float *nod9, const float *nrml3, const float *y3, int sgl, float *out)
{
    float pt[INTORDER], wgt[INTORDER];
    genGaussParams(INTORDER, pt, wgt);
    cartCoord nod[3] = {{nod9[0], nod9[1], nod9[2]}, {nod9[3], nod9[4], nod9[5]}, {nod9[6], nod9[7], nod9[8]}};
    cartCoord nr = {nrml3[0], nrml3[1], nrml3[2]}, y = {y3[0], y3[1], y3[2]};
    cuFloatComplex z = sgl ? triElemIntegral_p2Gp1np2n_sgl(k, nod, pt, wgt)
                           : triElemIntegral_p2Gp1np2n_nsgl(k, nod, nr, y, pt, wgt);
    out[0] = cuCrealf(z); out[1] = cuCimagf(z);
}

/* Leaf near lists of the last ref_octree_build: for each leaf box (leaf-set order) the boxes
 * of I2(box) (its neighbours in x-y-z order, then itself; octree.c:497-505) that are in the
 * leaf set, in that order (intersection, octree.c:425-437), as leaf-set indices (findSetInd).
 * beg[B+1] and idx may be NULL to get the total only. */
extern "C" long long ref_near_lists(int *beg, int *idx)
{
    int l = g_tree.oct.lmax;
    const int *leaf = g_tree.oct.fmmLevelSet[l - g_tree.oct.lmin];
    int set1[28], set2[28];
    long long pos = 0;
    if (beg) beg[0] = 0;
    for (int i = 0; i < leaf[0]; i++) {
        I2(leaf[i + 1], l, set1);
        intersection(set1, leaf, set2);
        for (int j = 0; j < set2[0]; j++) {
            if (idx) idx[pos] = findSetInd(leaf, set2[j + 1]);
            pos++;
        }
        if (beg) beg[i + 1] = (int)pos;
    }
    return pos;
}

static double ref_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* Seconds of the reference's CPU octree stages on an OBJ file: times[0] srcBoxes (or, with
 * depth > 0, its fixed-depth variant), times[1] FMMLevelSet, times[2] FMMLevelSetNumSR.
 * Returns lmax. */
extern "C" int ref_octree_stage_times(const char *filename, int s, int depth, double *times)
{
    int numPt, numElem, lmax = 0;
    double d;
    cartCoord_d pt_min;
    findNum(filename, &numPt, &numElem);
    cartCoord_d *pt = (cartCoord_d *)malloc(numPt * sizeof(cartCoord_d));
    triElem *elem = (triElem *)malloc(numElem * sizeof(triElem));
    readOBJ(filename, pt, elem);
    int *srcBoxSet = (int *)malloc((numElem + 1) * sizeof(int));
    double t0 = ref_now();
    if (depth > 0)
        srcBoxesDepth(pt, elem, numElem, depth, srcBoxSet, &lmax, &d, &pt_min);
    else
        srcBoxes(pt, elem, numElem, s, srcBoxSet, &lmax, &d, &pt_min);
    double t1 = ref_now();
    int **sets = (int **)malloc((lmax - 1) * sizeof(int *));
    FMMLevelSet(srcBoxSet, lmax, sets);
    double t2 = ref_now();
    int **num = (int **)malloc((lmax - 1) * sizeof(int *));
    FMMLevelSetNumSR(sets, lmax, num);
    double t3 = ref_now();
    times[0] = t1 - t0;
    times[1] = t2 - t1;
    times[2] = t3 - t2;
    for (int l = 0; l < lmax - 1; l++) { free(sets[l]); free(num[l]); }
    free(sets); free(num); free(srcBoxSet); free(pt); free(elem);
    return lmax;
}
