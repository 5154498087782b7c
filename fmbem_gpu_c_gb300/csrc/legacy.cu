// The reference's C entry points (structs.h, octree.h, translation.h, integral.h of
// ZiqiFrancisFan/FMBEM_GPU_C) implemented over this library, so that code written against
// the reference (its main.c) links unchanged.
//
// * Octree routines return exactly what octree.c returns (same Morton numbers, same
//   first-occurrence set order, same I2/I4 enumeration order), computed from integer box
//   coordinates instead of bit arrays, and without the MAX = 100000 stack arrays.
// * genOctree fills every field of struct octree like translation.cu:3007-3348.  The angle
//   and distance tables and the SS/SR/RR index arrays repeat the reference's float
//   arithmetic (cart2sph in float, tolerance matching) so they come out identical; the
//   rotation and coaxial matrices are generated on the GPU in FP64 (Wigner-d rotation
//   coefficients) and stored as the FP32 sparse matrices the reference stores.
// * OprL returns the complete single-layer operator L q (near field with the singular self
//   term, far field by FMM, L2P), which the reference's driver does not reach.
// Host code of this file is compiled with -ffp-contract=off.
#include "plan.h"
#include "../../include/octree.h"
#include "../../include/translation.h"
#include "../../include/integral.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

using namespace fmm;

// ============================================================================ structs.h
extern "C" float dotProd(const cartCoord u, const cartCoord v) { return u.x * v.x + u.y * v.y + u.z * v.z; }
extern "C" cartCoord crossProd(const cartCoord u, const cartCoord v)
{
    cartCoord r;
    r.x = u.y * v.z - u.z * v.y;
    r.y = u.z * v.x - u.x * v.z;
    r.z = u.x * v.y - u.y * v.x;
    return r;
}
extern "C" cartCoord cartCoordAdd(const cartCoord u, const cartCoord v) { return {u.x + v.x, u.y + v.y, u.z + v.z}; }
extern "C" cartCoord cartCoordSub(const cartCoord u, const cartCoord v) { return {u.x - v.x, u.y - v.y, u.z - v.z}; }
extern "C" cartCoord scalarMul(const float lambda, const cartCoord v) { return {lambda * v.x, lambda * v.y, lambda * v.z}; }
extern "C" float cartNorm(const cartCoord x) { return sqrtf(x.x * x.x + x.y * x.y + x.z * x.z); }
extern "C" float cartDist(const cartCoord x, const cartCoord y) { return cartNorm(cartCoordSub(x, y)); }
extern "C" cartCoord normalize(const cartCoord x) { return scalarMul(1.0f / cartNorm(x), x); }
extern "C" sphCoord cart2sph(const cartCoord s)
{
    // structs.cu:48-55 in float
    sphCoord t;
    t.r = sqrtf(powf(s.x, 2.0f) + powf(s.y, 2.0f) + powf(s.z, 2.0f));
    t.theta = acosf(s.z / t.r);
    t.phi = atan2f(s.y, s.x);
    return t;
}
extern "C" sphCoord_d cart_d2sph_d(const cartCoord_d s)
{
    sphCoord_d t;
    t.r = sqrt(pow(s.x, 2) + pow(s.y, 2) + pow(s.z, 2));
    t.theta = acos(s.z / t.r);
    t.phi = atan2(s.y, s.x);
    return t;
}
extern "C" sphCoord sphCoord_d2sphCoord(const sphCoord_d s) { return {(float)s.r, (float)s.theta, (float)s.phi}; }
extern "C" cartCoord sph2cart(const sphCoord s)
{
    return {s.r * sinf(s.theta) * cosf(s.phi), s.r * sinf(s.theta) * sinf(s.phi), s.r * cosf(s.theta)};
}
extern "C" cartCoord_d cartCoordSub_d(const cartCoord_d u, const cartCoord_d v) { return {u.x - v.x, u.y - v.y, u.z - v.z}; }
extern "C" cartCoord_d triCentroid_d(const cartCoord_d nod[3])
{
    double a[3] = {nod[0].x, nod[0].y, nod[0].z}, b[3] = {nod[1].x, nod[1].y, nod[1].z}, c[3] = {nod[2].x, nod[2].y, nod[2].z};
    double r[3];
    centroid(a, b, c, r);
    return {r[0], r[1], r[2]};
}
extern "C" cartCoord cartCoord_d2cartCoord(const cartCoord_d s) { return {(float)s.x, (float)s.y, (float)s.z}; }
extern "C" cartCoord_d cartCoord2cartCoord_d(const cartCoord s) { return {s.x, s.y, s.z}; }
extern "C" void printCartCoordArray_d(const cartCoord_d *arr, const int num)
{
    for (int i = 0; i < num; i++) printf("(%f,%f,%f)\n", arr[i].x, arr[i].y, arr[i].z);
}
extern "C" void printCartCoordArray(const cartCoord *arr, const int num)
{
    for (int i = 0; i < num; i++) printf("(%f,%f,%f)\n", arr[i].x, arr[i].y, arr[i].z);
}
extern "C" void printSphCoordArray(const sphCoord *arr, const int num)
{
    for (int i = 0; i < num; i++) printf("(%f,%f,%f)\n", arr[i].r, arr[i].theta, arr[i].phi);
}
extern "C" void printFloatArray(const float *arr, const int num)
{
    for (int i = 0; i < num; i++) printf("%f\n", arr[i]);
}
extern "C" void printIntArray(const int *arr, const int num)
{
    for (int i = 0; i < num; i++) printf("%d ", arr[i]);
    printf("\n");
}
extern "C" void printRotAngArray(const rotAng *a, const int n)
{
    for (int i = 0; i < n; i++) printf("(%f,%f,%f)\n", a[i].alpha, a[i].beta, a[i].gamma);
}
extern "C" bool equalRotArrays(const rotAng *a1, const rotAng *a2, const int n)
{
    for (int i = 0; i < n; i++) {
        bool found = false;
        for (int j = 0; j < n; j++)
            if (a1[i].alpha == a2[j].alpha && a1[i].beta == a2[j].beta && a1[i].gamma == a2[j].gamma) { found = true; break; }
        if (!found) return false;
    }
    return true;
}
extern "C" void bubbleSort(float *arr, const int n)
{
    // structs.cu:229-240: adjacent exchanges, strict comparison
    for (int i = 0; i < n - 1; i++)
        for (int j = 0; j < n - i - 1; j++)
            if (arr[j] > arr[j + 1]) std::swap(arr[j], arr[j + 1]);
}
extern "C" void sortRotArray(rotAng *ang, const int numRot, const float eps)
{
    // structs.cu:242-287: bubble sort by alpha, then by beta within runs of alpha equal to
    // within eps of the run's first alpha
    for (int i = 0; i < numRot; i++)
        for (int j = 0; j < numRot - i - 1; j++)
            if (ang[j].alpha > ang[j + 1].alpha) std::swap(ang[j], ang[j + 1]);
    if (numRot == 0) return;
    int idx = 0, num = 0;
    float alpha = ang[0].alpha;
    auto sort_beta = [&](int start, int cnt) {
        for (int i = 0; i < cnt; i++)
            for (int j = start; j < start + cnt - i - 1; j++)
                if (ang[j].beta > ang[j + 1].beta) std::swap(ang[j], ang[j + 1]);
    };
    while (idx + num < numRot) {
        if (fabsf(ang[idx + num].alpha - alpha) < eps) {
            num++;
        } else {
            sort_beta(idx, num);
            alpha = ang[idx + num].alpha;
            idx += num;
            num = 0;
        }
    }
    sort_beta(idx, num);
}

// ============================================================================ octree.h
static void fgets_chunks_count(const char *filename, int *pV, int *pE)
{
    std::vector<double> V;
    std::vector<int> F;
    read_obj(filename, V, F);
    *pV = (int)(V.size() / 3);
    *pE = (int)(F.size() / 3);
}

extern "C" void findNum(const char *filename, int *pV, int *pE)
{
    FILE *fp = fopen(filename, "r");
    if (!fp) {
        printf("Failed to open file.\n");
        exit(EXIT_FAILURE);
    }
    fclose(fp);
    fgets_chunks_count(filename, pV, pE);
}

extern "C" int readOBJ(const char *filename, cartCoord_d *p, triElem *e)
{
    std::vector<double> V;
    std::vector<int> F;
    if (read_obj(filename, V, F) != 0) {
        printf("Failed to open file.\n");
        exit(EXIT_FAILURE);
    }
    for (size_t i = 0; i < V.size() / 3; i++) p[i] = {V[3 * i], V[3 * i + 1], V[3 * i + 2]};
    for (size_t j = 0; j < F.size() / 3; j++) {
        e[j].node[0] = F[3 * j];
        e[j].node[1] = F[3 * j + 1];
        e[j].node[2] = F[3 * j + 2];
        e[j].alpha = make_cuFloatComplex(0, 0);
        e[j].beta = make_cuFloatComplex(0, 0);
        e[j].gamma = make_cuFloatComplex(0, 0);
    }
    return EXIT_SUCCESS;
}

extern "C" void printSet(const int *set)
{
    if (set[0] == 0) printf("Empty set.");
    else
        for (int i = 1; i <= set[0]; i++) printf("%d ", set[i]);
    printf("\n");
}
extern "C" bool arrEqual(const int *a, const int *b, const int num)
{
    for (int i = 0; i < num; i++)
        if (a[i] != b[i]) return false;
    return true;
}
extern "C" int parent(int num) { return num / 8; }
extern "C" int child(int num, int cld) { return 8 * num + cld; }
extern "C" void children(const int num, int *c)
{
    for (int i = 0; i < 8; i++) c[i] = 8 * num + i;
}
extern "C" cartCoord_d scale(const cartCoord_d x, const cartCoord_d x_min, const double d)
{
    return {(x.x - x_min.x) / d, (x.y - x_min.y) / d, (x.z - x_min.z) / d};
}
extern "C" cartCoord_d descale(const cartCoord_d x_s, const cartCoord_d x_min, const double d)
{
    return {d * x_s.x + x_min.x, d * x_s.y + x_min.y, d * x_s.z + x_min.z};
}
extern "C" double descale_1d(const double a, const double D, const double v_min) { return D * a + v_min; }
extern "C" void scalePnts(const cartCoord_d *pnt, const int n, const cartCoord_d pnt_min, const double d, cartCoord_d *out)
{
    for (int i = 0; i < n; i++) out[i] = scale(pnt[i], pnt_min, d);
}
extern "C" void dec2bin_frac(double s, int l, int *h)
{
    for (int i = 1; i <= l; i++) {
        s *= 2;
        double t = floor(s);
        h[i - 1] = (int)t;
        s -= t;
    }
}
extern "C" void bitIntleave(const int *x, const int *y, const int *z, const int l, int *result)
{
    for (int i = 0; i < l; i++) result[i] = 4 * x[i] + 2 * y[i] + z[i];
}
extern "C" int indArr2num(const int *ind, const int l, const int d)
{
    long long result = 0, base = 1LL << d;
    for (int i = 0; i < l; i++) result = result * base + ind[i];
    return (int)result;
}
extern "C" int pnt2boxnum(const cartCoord_d pnt, const int l)
{
    double s[3] = {pnt.x, pnt.y, pnt.z};
    return (int)morton_key(s, l);
}
extern "C" cartCoord_d boxCenter(const int num, const int l)
{
    if (num < 0 || num > pow(pow(2, 3), l) - 1) {
        printf("Illegal input.\n");
        cartCoord_d t = {nan("1"), nan("2"), nan("3")};
        return t;
    }
    int x, y, z;
    box_xyz(num, l, &x, &y, &z);
    double h = pow(2, -l), h2 = pow(2, -l - 1);
    return {h * x + h2, h * y + h2, h * z + h2};
}

// neighbours of (num, l) in the reference order (x outer, z inner), self excluded
static int nbr_list(int num, int l, int *out)
{
    int x, y, z, top = (1 << l) - 1, n = 0;
    box_xyz(num, l, &x, &y, &z);
    int xl = x > 0 ? x - 1 : 0, xh = x < top ? x + 1 : top;
    int yl = y > 0 ? y - 1 : 0, yh = y < top ? y + 1 : top;
    int zl = z > 0 ? z - 1 : 0, zh = z < top ? z + 1 : top;
    for (int a = xl; a <= xh; a++)
        for (int b = yl; b <= yh; b++)
            for (int c = zl; c <= zh; c++) {
                int t = (int)box_num(a, b, c, l);
                if (t != num) out[n++] = t;
            }
    return n;
}

extern "C" int neighbors(const int num, const int l, int *numNeighbors, int *nbr)
{
    *numNeighbors = nbr_list(num, l, nbr);
    return EXIT_SUCCESS;
}
extern "C" void createSet(const int *elems, const int numElems, int *set)
{
    std::vector<long long> v(elems, elems + numElems);
    std::vector<long long> u = first_occurrence(v);
    set[0] = (int)u.size();
    for (size_t i = 0; i < u.size(); i++) set[i + 1] = (int)u[i];
}
extern "C" bool isMember(const int t, const int *set)
{
    for (int i = 1; i <= set[0]; i++)
        if (set[i] == t) return true;
    return false;
}
extern "C" bool isEmpty(const int *set) { return set[0] == 0; }
extern "C" void intersection(const int *set1, const int *set2, int *set3)
{
    std::vector<int> s2(set2 + 1, set2 + 1 + set2[0]);
    std::sort(s2.begin(), s2.end());
    int n = 0, m = set1[0];
    for (int i = 1; i <= m; i++)
        if (std::binary_search(s2.begin(), s2.end(), set1[i])) set3[++n] = set1[i];
    set3[0] = n;
}
extern "C" void Union(const int *set1, const int *set2, int *set3)
{
    std::vector<int> s1(set1 + 1, set1 + 1 + set1[0]);
    std::sort(s1.begin(), s1.end());
    int n2 = set2[0];
    for (int i = 0; i <= set1[0]; i++) set3[i] = set1[i];
    for (int i = 1; i <= n2; i++)
        if (!std::binary_search(s1.begin(), s1.end(), set2[i])) set3[++set3[0]] = set2[i];
}
extern "C" void difference(const int *set1, const int *set2, int *set3)
{
    std::vector<int> s2(set2 + 1, set2 + 1 + set2[0]);
    std::sort(s2.begin(), s2.end());
    int n = 0, m = set1[0];
    for (int i = 1; i <= m; i++)
        if (!std::binary_search(s2.begin(), s2.end(), set1[i])) set3[++n] = set1[i];
    set3[0] = n;
}
extern "C" void pnts2numSet(const cartCoord_d *pnts, const int numPnts, const int l, int *set)
{
    std::vector<int> v(numPnts);
    for (int i = 0; i < numPnts; i++) v[i] = pnt2boxnum(pnts[i], l);
    createSet(v.data(), numPnts, set);
}
extern "C" void I2(const int num, const int l, int *set)
{
    int nbr[27];
    int t = nbr_list(num, l, nbr);
    nbr[t] = num;
    set[0] = t + 1;
    for (int i = 0; i <= t; i++) set[i + 1] = nbr[i];
}
extern "C" void I4(const int num, const int l, int *set)
{
    // children of the parent's neighbours (reference order), then of the parent, minus the
    // box's own neighbourhood
    int x, y, z;
    box_xyz(num, l, &x, &y, &z);
    int pn[27];
    int np = nbr_list(num / 8, l - 1, pn);
    pn[np++] = num / 8;
    int n = 0;
    for (int i = 0; i < np; i++)
        for (int c = 0; c < 8; c++) {
            int ch = 8 * pn[i] + c, cx, cy, cz;
            box_xyz(ch, l, &cx, &cy, &cz);
            if (std::abs(cx - x) <= 1 && std::abs(cy - y) <= 1 && std::abs(cz - z) <= 1) continue;
            set[++n] = ch;
        }
    set[0] = n;
}
extern "C" void orderArray(const int *a, const int num, int *ind)
{
    // same multiset order as the reference's exchange sort (ties broken by position)
    for (int i = 0; i < num; i++) ind[i] = i;
    std::stable_sort(ind, ind + num, [&](int p, int q) { return a[p] < a[q]; });
}
extern "C" int deterLmax(const cartCoord_d *pnts, const int numPnts, const int s)
{
    std::vector<double> S(3 * (size_t)numPnts);
    for (int i = 0; i < numPnts; i++) { S[3 * i] = pnts[i].x; S[3 * i + 1] = pnts[i].y; S[3 * i + 2] = pnts[i].z; }
    return deter_lmax(S, s);
}
extern "C" void findBoundingCube(const cartCoord_d *pnts, const int numPnts, const double eps, cartCoord_d *pnts_b, double *d)
{
    std::vector<double> P(3 * (size_t)numPnts);
    for (int i = 0; i < numPnts; i++) { P[3 * i] = pnts[i].x; P[3 * i + 1] = pnts[i].y; P[3 * i + 2] = pnts[i].z; }
    double mn[3];
    bounding_cube(P, eps, mn, d);
    double mx[3] = {mn[0] + *d, mn[1] + *d, mn[2] + *d};
    for (int c = 0; c < 8; c++)
        pnts_b[c] = {(c & 4) ? mx[0] : mn[0], (c & 2) ? mx[1] : mn[1], (c & 1) ? mx[2] : mn[2]};
}
extern "C" void srcBoxes(const cartCoord_d *pnts, const triElem *elems, const int numElems, const int s, int *srcBoxSet,
                         int *lmax, double *D, cartCoord_d *pnt_min)
{
    std::vector<double> V;
    std::vector<int> F(3 * (size_t)numElems);
    int nv = 0;
    for (int e = 0; e < numElems; e++)
        for (int t = 0; t < 3; t++) { F[3 * e + t] = elems[e].node[t]; nv = std::max(nv, elems[e].node[t] + 1); }
    V.resize(3 * (size_t)nv);
    for (int i = 0; i < nv; i++) { V[3 * i] = pnts[i].x; V[3 * i + 1] = pnts[i].y; V[3 * i + 2] = pnts[i].z; }
    HostTree T;
    build_tree(V, F, s, 0, T);
    *lmax = T.lmax;
    *D = T.d;
    *pnt_min = {T.pt_min[0], T.pt_min[1], T.pt_min[2]};
    const std::vector<long long> &leaf = T.sets[T.lmax];
    srcBoxSet[0] = (int)leaf.size();
    for (size_t i = 0; i < leaf.size(); i++) srcBoxSet[i + 1] = (int)leaf[i];
}
extern "C" int truncNum(const double k, const double eps, const double sigma, const double a)
{
    double p_lo = 1 - log(eps * pow(1 - 1.0 / sigma, 1.5)) / log(sigma);
    double t0 = k * a, t1 = pow(3 * log(1.0 / eps), 1.5) / 2;
    double p_hi = t0 + t1 * pow(t0, 1.0 / 3);
    return (int)ceil(pow(pow(p_lo, 4) + pow(p_hi, 4), 0.25));
}
extern "C" int truncNum_2(const double wavNum, const double eps, const double sigma, const double a)
{
    double ka_s = 3.0 / (pow(2, 1.5) * pow(sigma - 1, 1.5)) * log(1.0 / (eps * sigma));
    double p_s = 3.0 * sigma / (pow(2, 1.5) * pow(sigma - 1, 1.5)) * log(1.0 / (eps * sigma));
    double p = (wavNum * a <= ka_s) ? p_s : wavNum * a + 0.5 * pow(3 * log(1.0 / (eps * sigma)), 2.0 / 3) * pow(wavNum * a, 1.0 / 3);
    return (int)ceil(p);
}
extern "C" void prntLevelSet(const int *X, const int l, int *X_n)
{
    if (l == 0) return;
    std::vector<int> t(X[0]);
    for (int i = 0; i < X[0]; i++) {
        if (X[i + 1] >= pow(8, l)) {
            printf("Error in box number: %d.\n", X[i + 1]);
            return;
        }
        t[i] = X[i + 1] / 8;
    }
    createSet(t.data(), X[0], X_n);
}
extern "C" void FMMLevelSet(const int *btmLvl, const int lmax, int **pSet)
{
    pSet[lmax - 2] = (int *)malloc((btmLvl[0] + 1) * sizeof(int));
    memcpy(pSet[lmax - 2], btmLvl, (btmLvl[0] + 1) * sizeof(int));
    for (int l = lmax - 1; l >= 2; l--) {
        std::vector<int> tmp(pSet[l + 1 - 2][0] + 1);
        prntLevelSet(pSet[l + 1 - 2], l + 1, tmp.data());
        pSet[l - 2] = (int *)malloc((tmp[0] + 1) * sizeof(int));
        memcpy(pSet[l - 2], tmp.data(), (tmp[0] + 1) * sizeof(int));
    }
}
extern "C" int findSetInd(const int *X, const int num)
{
    if (X[0] == 0) {
        printf("Empty set.\n");
        return -1;
    }
    for (int i = 1; i <= X[0]; i++)
        if (X[i] == num) return i - 1;
    printf("Not in the set.\n");
    return -1;
}
extern "C" void sortSet(int *set) { std::sort(set + 1, set + 1 + set[0]); }
extern "C" void FMMLevelSetNumSR(int **pSet, const int lmax, int **numSet)
{
    for (int l = 2; l <= lmax; l++) {
        const int *S = pSet[l - 2];
        std::vector<int> sorted(S + 1, S + 1 + S[0]);
        std::sort(sorted.begin(), sorted.end());
        numSet[l - 2] = (int *)malloc(std::max(1, S[0]) * sizeof(int));
        int set[8 * 27 + 1];
        for (int i = 0; i < S[0]; i++) {
            I4(S[i + 1], l, set);
            int c = 0;
            for (int j = 1; j <= set[0]; j++) c += std::binary_search(sorted.begin(), sorted.end(), set[j]);
            numSet[l - 2][i] = c;
        }
    }
}
extern "C" void printFMMLevelSet(int **pSet, const int lmax)
{
    printf("FMM level set: \n");
    for (int l = 2; l <= lmax; l++) {
        printf("Level %d, number of boxes: %d\n", l, pSet[l - 2][0]);
        printSet(pSet[l - 2]);
    }
}

// ============================================================================ translation.h
extern "C" int sparseRotSize(const int p) { return rot_size(p); }
extern "C" int sparseCoaxTransSize(const int p) { return coax_size(p); }
extern "C" void reduceSparseRotMat(const cuFloatComplex *rot1, cuFloatComplex *rot2, const int p2)
{
    memcpy(rot2, rot1, rot_size(p2) * sizeof(cuFloatComplex));
}
extern "C" void reduceSparseCoaxTransMat(const cuFloatComplex *m1, const int p1, cuFloatComplex *m2, const int p2)
{
    for (int m = 0; m < p2; m++) {
        int o1 = coax_off(p1, m), o2 = coax_off(p2, m);
        for (int np = m; np < p2; np++)
            for (int n = m; n < p2; n++) m2[o2 + IDXC0(np - m, n - m, p2 - m)] = m1[o1 + IDXC0(np - m, n - m, p1 - m)];
    }
}
extern "C" void printMat_cuFloatComplex(const cuFloatComplex *A, const int numRow, const int numCol, const int lda)
{
    for (int i = 0; i < numRow; i++) {
        for (int j = 0; j < numCol; j++) printf("(%.6f,%.6f)", cuCrealf(A[IDXC0(i, j, lda)]), cuCimagf(A[IDXC0(i, j, lda)]));
        printf("\n");
    }
}
extern "C" cuFloatComplex cplxExp(const float theta) { return make_cuFloatComplex(cos(theta), sin(theta)); }
extern "C" double factorial(const int n)
{
    double r = 1;
    for (int i = 2; i <= n; i++) r *= (double)i;
    return r;
}
extern "C" float aCoeff(const int n, const int m) { return (float)coefA(n, m); }
extern "C" float bCoeff(const int n, const int m) { return (float)coefB(n, m); }

extern "C" int genSparseRotMats(const rotAng *rotAngle, const int numRot, const int p, cuFloatComplex *sparseMat)
{
    if (numRot <= 0) return EXIT_SUCCESS;
    if (p < 1 || p > 64) return EXIT_FAILURE;
    std::vector<double> a(numRot), b(numRot), g(numRot);
    for (int i = 0; i < numRot; i++) { a[i] = rotAngle[i].alpha; b[i] = rotAngle[i].beta; g[i] = rotAngle[i].gamma; }
    return gen_rotation_matrices_f32(a.data(), b.data(), g.data(), numRot, p, (float2 *)sparseMat) == FMM_OK ? EXIT_SUCCESS
                                                                                                             : EXIT_FAILURE;
}
static int gen_coax_legacy(float k, const float *vec, int n, int p, int sr, cuFloatComplex *out)
{
    if (n <= 0) return EXIT_SUCCESS;
    if (p < 1 || p > 64) return EXIT_FAILURE;
    std::vector<double> t(vec, vec + n);
    return gen_coax_matrices_f32(k, t.data(), n, p, sr, (float2 *)out) == FMM_OK ? EXIT_SUCCESS : EXIT_FAILURE;
}
extern "C" int genRRSparseCoaxTransMat(const float k, const float *vec, const int n, const int p, cuFloatComplex *m)
{
    return gen_coax_legacy(k, vec, n, p, 0, m);
}
extern "C" int genSSSparseCoaxTransMat(const float k, const float *vec, const int n, const int p, cuFloatComplex *m)
{
    return gen_coax_legacy(k, vec, n, p, 0, m);
}
extern "C" int genSRSparseCoaxTransMat(const float k, const float *vec, const int n, const int p, cuFloatComplex *m)
{
    return gen_coax_legacy(k, vec, n, p, 1, m);
}
extern "C" void cuSparseRotVecMul(const cuFloatComplex *mat, const cuFloatComplex *vec, const int p, cuFloatComplex *prod)
{
    for (int n = 0; n < p; n++) {
        int w = 2 * n + 1, off = rot_off(n);
        for (int mp = -n; mp <= n; mp++) {
            cuFloatComplex acc = make_cuFloatComplex(0, 0);
            for (int m = -n; m <= n; m++) acc = cuCaddf(acc, cuCmulf(mat[off + IDXC0(mp + n, m + n, w)], vec[NM2IDX0(n, m)]));
            prod[NM2IDX0(n, mp)] = acc;
        }
    }
}
extern "C" void cuSparseCoaxTransMatVecMul(const cuFloatComplex *mat, const cuFloatComplex *vec, const int p,
                                           cuFloatComplex *prod)
{
    for (int m = -(p - 1); m <= p - 1; m++) {
        int am = std::abs(m), sz = p - am, off = coax_off(p, am);
        for (int np = am; np < p; np++) {
            cuFloatComplex acc = make_cuFloatComplex(0, 0);
            for (int n = am; n < p; n++) acc = cuCaddf(acc, cuCmulf(mat[off + IDXC0(np - am, n - am, sz)], vec[NM2IDX0(n, m)]));
            prod[NM2IDX0(np, m)] = acc;
        }
    }
}

// --------------------------------------------------------------- translation geometry tables
// box centre at level l in physical coordinates: descale(boxCenter(num, l))
static cartCoord_d ctr_phys(int num, int l, const cartCoord_d pt_min, double d) { return descale(boxCenter(num, l), pt_min, d); }

// angle and length of the vector from box a to box b as the reference computes them
static void vec_angles(cartCoord_d from, cartCoord_d to, rotAng *ang, float *t)
{
    cartCoord_d v = cartCoordSub_d(to, from);
    sphCoord s = cart2sph(cartCoord_d2cartCoord(v));
    ang->alpha = s.phi;
    ang->beta = s.theta;
    ang->gamma = 0;
    *t = s.r;
}

static void push_unique(std::vector<float> &vecs, std::vector<rotAng> &angs, rotAng a, float t, float eps)
{
    bool f = false;
    for (float v : vecs)
        if (fabsf(v - t) < eps) { f = true; break; }
    if (!f) vecs.push_back(t);
    f = false;
    for (const rotAng &b : angs)
        if (fabsf(a.alpha - b.alpha) < eps && fabsf(a.beta - b.beta) < eps) { f = true; break; }
    if (!f) angs.push_back(a);
}

static void emit(std::vector<float> &vecs, std::vector<rotAng> &angs, float **pVec, int *pNumVec, rotAng **pAng, int *pNumAng)
{
    *pNumVec = (int)vecs.size();
    *pNumAng = (int)angs.size();
    *pVec = (float *)malloc(std::max<size_t>(1, vecs.size()) * sizeof(float));
    *pAng = (rotAng *)malloc(std::max<size_t>(1, angs.size()) * sizeof(rotAng));
    std::copy(vecs.begin(), vecs.end(), *pVec);
    std::copy(angs.begin(), angs.end(), *pAng);
}

extern "C" void genSRCoaxTransVecsRotAngles(const int l, const double d, const cartCoord_d pt_min, float **pVec, int *pNumVec,
                                            rotAng **pRotAngle, int *pNumRotAng)
{
    // translation.cu:2479-2642
    std::vector<float> vecs;
    std::vector<rotAng> angs;
    float eps = 0.00001 * d;
    int set[8 * 27 + 1];
    auto process = [&](int idx) {
        cartCoord_d c1 = ctr_phys(idx, l, pt_min, d);
        I4(idx, l, set);
        for (int i = 0; i < set[0]; i++) {
            rotAng a;
            float t;
            vec_angles(ctr_phys(set[i + 1], l, pt_min, d), c1, &a, &t);
            push_unique(vecs, angs, a, t, eps);
        }
    };
    if (l == 2) {
        for (int idx = 0; idx < 64; idx++) process(idx);
    } else {
        int idx = 0, total = (int)pow(8, l);
        for (idx = 0; idx < total; idx++) {
            I4(idx, l, set);
            if (set[0] == 189) break;
        }
        int prnt = idx / 8;
        for (int c = 0; c < 8; c++) process(8 * prnt + c);
    }
    emit(vecs, angs, pVec, pNumVec, pRotAngle, pNumRotAng);
}

static void gen_parent_child(int l, double d, cartCoord_d pt_min, float epsf, bool to_parent, float **pVec, int *pNumVec,
                             rotAng **pAng, int *pNumAng)
{
    std::vector<float> vecs;
    std::vector<rotAng> angs;
    cartCoord_d pc = ctr_phys(0, l - 1, pt_min, d);
    for (int c = 0; c < 8; c++) {
        cartCoord_d cc = ctr_phys(c, l, pt_min, d);
        rotAng a;
        float t;
        if (to_parent) vec_angles(cc, pc, &a, &t);
        else vec_angles(pc, cc, &a, &t);
        push_unique(vecs, angs, a, t, epsf);
    }
    emit(vecs, angs, pVec, pNumVec, pAng, pNumAng);
}

extern "C" void genSSCoaxTransVecsRotAngles(const int l, const double d, const cartCoord_d pt_min, float **pVec, int *pNumVec,
                                            rotAng **pRotAngle, int *pNumRotAng)
{
    gen_parent_child(l, d, pt_min, (float)(0.000001 * d), true, pVec, pNumVec, pRotAngle, pNumRotAng); // :2644-2718
}
extern "C" void genRRCoaxTransVecsRotAngles(const int l, const double d, const cartCoord_d pt_min, float **pVec, int *pNumVec,
                                            rotAng **pRotAngle, int *pNumRotAng)
{
    gen_parent_child(l, d, pt_min, (float)(0.00001 * d), false, pVec, pNumVec, pRotAngle, pNumRotAng); // :2720-2795
}

static void match(float t, rotAng a, const float *vec, int nvec, const rotAng *ang, int nang, float eps, transIdx *out)
{
    out->coaxIdx = -1;
    out->rotIdx = -1;
    for (int j = 0; j < nvec; j++)
        if (fabsf(t - vec[j]) < eps) { out->coaxIdx = j; break; }
    for (int j = 0; j < nang; j++)
        if (fabsf(a.alpha - ang[j].alpha) < eps && fabsf(a.beta - ang[j].beta) < eps) { out->rotIdx = j; break; }
}

extern "C" void genSSIdxArrs(int **fmmLevelSet, const int lmax, const cartCoord_d pt_min, const double d,
                             const float *rrVec, const int nrr, const rotAng *ang, const int numRot, transIdx **ssIdx,
                             int **ssDest)
{
    float eps = 0.000001 * d;
    for (int l = lmax; l > 2; l--) {
        const int *S = fmmLevelSet[l - 2];
        ssIdx[l - 3] = (transIdx *)malloc(std::max(1, S[0]) * sizeof(transIdx));
        ssDest[l - 3] = (int *)malloc(std::max(1, S[0]) * sizeof(int));
        std::unordered_map<int, int> pos;
        const int *PS = fmmLevelSet[l - 3];
        for (int i = 0; i < PS[0]; i++) pos.emplace(PS[i + 1], i);
        for (int i = 0; i < S[0]; i++) {
            int b = S[i + 1];
            auto it = pos.find(b / 8);
            ssDest[l - 3][i] = it == pos.end() ? -1 : it->second;
            rotAng a;
            float t;
            vec_angles(ctr_phys(b, l, pt_min, d), ctr_phys(b / 8, l - 1, pt_min, d), &a, &t);
            match(t, a, rrVec, nrr, ang, numRot, eps, &ssIdx[l - 3][i]);
        }
    }
}

extern "C" void genSRIdxArrs(int **fmmLevelSet, int **SRNumLevelArr, const int lmax, const cartCoord_d pt_min, const double d,
                             const float *srVec, const int nsr, const rotAng *ang, const int numRot, transIdx **srIdx,
                             int **srOrigin, int **srDest)
{
    float eps = 0.000001 * d;
    int set[8 * 27 + 1];
    for (int l = 2; l <= lmax; l++) {
        const int *S = fmmLevelSet[l - 2];
        long long total = 0;
        for (int i = 0; i < S[0]; i++) total += SRNumLevelArr[l - 2][i];
        srIdx[l - 2] = (transIdx *)malloc(std::max<long long>(1, total) * sizeof(transIdx));
        srOrigin[l - 2] = (int *)malloc(std::max<long long>(1, total) * sizeof(int));
        srDest[l - 2] = (int *)malloc(std::max<long long>(1, total) * sizeof(int));
        std::unordered_map<int, int> pos;
        for (int i = 0; i < S[0]; i++) pos.emplace(S[i + 1], i);
        long long k = 0;
        for (int i = 0; i < S[0]; i++) {
            int b = S[i + 1];
            cartCoord_d c1 = ctr_phys(b, l, pt_min, d);
            I4(b, l, set);
            for (int j = 1; j <= set[0]; j++) {
                auto it = pos.find(set[j]);
                if (it == pos.end()) continue;
                srOrigin[l - 2][k] = it->second;
                srDest[l - 2][k] = b;
                rotAng a;
                float t;
                vec_angles(ctr_phys(set[j], l, pt_min, d), c1, &a, &t);
                match(t, a, srVec, nsr, ang, numRot, eps, &srIdx[l - 2][k]);
                k++;
            }
        }
    }
}

extern "C" void genRRIdxArrs(int **fmmLevelSet, const int lmax, const cartCoord_d pt_min, const double d,
                             const float *rrVec, const int nrr, const rotAng *ang, const int numRot, transIdx **rrIdx,
                             int **rrOrigin)
{
    float eps = 0.000001 * d;
    for (int l = 3; l <= lmax; l++) {
        const int *S = fmmLevelSet[l - 2];
        rrIdx[l - 3] = (transIdx *)malloc(std::max(1, S[0]) * sizeof(transIdx));
        rrOrigin[l - 3] = (int *)malloc(std::max(1, S[0]) * sizeof(int));
        std::unordered_map<int, int> pos;
        const int *PS = fmmLevelSet[l - 3];
        for (int i = 0; i < PS[0]; i++) pos.emplace(PS[i + 1], i);
        for (int i = 0; i < S[0]; i++) {
            int b = S[i + 1];
            auto it = pos.find(b / 8);
            rrOrigin[l - 3][i] = it == pos.end() ? -1 : it->second;
            rotAng a;
            float t;
            vec_angles(ctr_phys(b / 8, l - 1, pt_min, d), ctr_phys(b, l, pt_min, d), &a, &t);
            match(t, a, rrVec, nrr, ang, numRot, eps, &rrIdx[l - 3][i]);
        }
    }
}

// --------------------------------------------------------------------------- octree lifecycle
static std::mutex g_oprl_mu;
static std::map<const octree *, std::pair<float, fmm_plan *>> g_oprl_plans;

extern "C" void initOctree(octree *oct)
{
    memset(oct, 0, sizeof(*oct));
    oct->lmin = 2;
    oct->eps = 0.05f;
    oct->maxWavNum = 2 * PI * 20000 / 343.0f;
}

static void merge_vecs(float *&dst, int &n, const float *src, int m, float epsilon)
{
    std::vector<float> tmp(dst, dst + n);
    for (int i = 0; i < m; i++) {
        bool f = false;
        for (int j = 0; j < n; j++)
            if (fabsf(src[i] - tmp[j]) < epsilon) { f = true; break; }
        if (!f) { tmp.push_back(src[i]); n++; }
    }
    free(dst);
    dst = (float *)malloc(std::max<size_t>(1, tmp.size()) * sizeof(float));
    std::copy(tmp.begin(), tmp.end(), dst);
}

extern "C" int genOctree(const char *filename, const float wavNum, const int s, octree *oct)
{
    if (oct->fmmLevelSet == NULL) {
        std::vector<double> V;
        std::vector<int> F;
        if (read_obj(filename, V, F) != 0) {
            printf("Failed to open file.\n");
            return EXIT_FAILURE;
        }
        int nv = (int)(V.size() / 3), nf = (int)(F.size() / 3);
        oct->pt = (cartCoord *)malloc(std::max(1, nv) * sizeof(cartCoord));
        oct->elem = (triElem *)malloc(std::max(1, nf) * sizeof(triElem));
        oct->numPt = nv;
        oct->numElem = nf;
        for (int i = 0; i < nv; i++) oct->pt[i] = {(float)V[3 * i], (float)V[3 * i + 1], (float)V[3 * i + 2]};
        for (int e = 0; e < nf; e++) {
            for (int t = 0; t < 3; t++) oct->elem[e].node[t] = F[3 * e + t];
            oct->elem[e].alpha = oct->elem[e].beta = oct->elem[e].gamma = make_cuFloatComplex(0, 0);
        }
        HostTree T;
        if (build_tree(V, F, s, 0, T) != 0) return EXIT_FAILURE;
        oct->lmax = T.lmax;
        oct->d = T.d;
        oct->pt_min = {T.pt_min[0], T.pt_min[1], T.pt_min[2]};
        oct->fmmLevelSet = (int **)malloc((oct->lmax - oct->lmin + 1) * sizeof(int *));
        for (int l = oct->lmin; l <= oct->lmax; l++) {
            const std::vector<long long> &st = T.sets[l];
            int *a = (int *)malloc((st.size() + 1) * sizeof(int));
            a[0] = (int)st.size();
            for (size_t i = 0; i < st.size(); i++) a[i + 1] = (int)st[i];
            oct->fmmLevelSet[l - oct->lmin] = a;
        }
    }
    if (oct->srNumLevelArr == NULL) {
        oct->srNumLevelArr = (int **)malloc((oct->lmax - oct->lmin + 1) * sizeof(int *));
        FMMLevelSetNumSR(oct->fmmLevelSet, oct->lmax, oct->srNumLevelArr);
    }
    if (oct->btmLvlElemIdx == NULL) {
        // translation.cu:3062-3076: float centroid (integral.cu:659-664), double scaling
        oct->btmLvlElemIdx = (int *)malloc(std::max(1, oct->numElem) * sizeof(int));
        const int *leaf = oct->fmmLevelSet[oct->lmax - oct->lmin];
        std::unordered_map<int, int> pos;
        for (int i = 0; i < leaf[0]; i++) pos.emplace(leaf[i + 1], i);
        for (int i = 0; i < oct->numElem; i++) {
            cartCoord n0 = oct->pt[oct->elem[i].node[0]], n1 = oct->pt[oct->elem[i].node[1]], n2 = oct->pt[oct->elem[i].node[2]];
            cartCoord c23 = scalarMul(0.5, cartCoordAdd(n1, n2));
            cartCoord ctr = cartCoordAdd(n0, scalarMul(2.0 / 3.0, cartCoordSub(c23, n0)));
            ctr = cartCoord_d2cartCoord(scale(cartCoord2cartCoord_d(ctr), oct->pt_min, oct->d));
            int num = pnt2boxnum(cartCoord2cartCoord_d(ctr), oct->lmax);
            auto it = pos.find(num);
            oct->btmLvlElemIdx[i] = it == pos.end() ? -1 : it->second;
        }
    }
    oct->pmax = truncNum(oct->maxWavNum, oct->eps, 1.5, pow(2, -oct->lmin) * oct->d);
    float epsilon = 0.000000001 * oct->d;
    float *vec = NULL;
    rotAng *ang = NULL;
    int numVec, numRot;
    for (int l = oct->lmin; l <= oct->lmax; l++) {
        genSRCoaxTransVecsRotAngles(l, oct->d, oct->pt_min, &vec, &numVec, &ang, &numRot);
        if (oct->numRotAng == 0) {
            oct->ang = (rotAng *)malloc(std::max(1, numRot) * sizeof(rotAng));
            memcpy(oct->ang, ang, numRot * sizeof(rotAng));
            oct->numRotAng = numRot;
        }
        merge_vecs(oct->srCoaxTransVec, oct->numSRCoaxTransVec, vec, numVec, epsilon);
        free(vec);
        free(ang);
    }
    sortRotArray(oct->ang, oct->numRotAng, oct->eps);
    bubbleSort(oct->srCoaxTransVec, oct->numSRCoaxTransVec);
    if (oct->rotMat1 == NULL) {
        int rs = rot_size(oct->pmax);
        oct->rotMat1 = (cuFloatComplex *)malloc((size_t)oct->numRotAng * rs * sizeof(cuFloatComplex));
        oct->rotMat2 = (cuFloatComplex *)malloc((size_t)oct->numRotAng * rs * sizeof(cuFloatComplex));
        std::vector<rotAng> swapped(oct->numRotAng);
        for (int i = 0; i < oct->numRotAng; i++) swapped[i] = {oct->ang[i].gamma, oct->ang[i].beta, oct->ang[i].alpha};
        HOST_CALL(genSparseRotMats(oct->ang, oct->numRotAng, oct->pmax, oct->rotMat1));
        HOST_CALL(genSparseRotMats(swapped.data(), oct->numRotAng, oct->pmax, oct->rotMat2));
    }
    int pc = truncNum(wavNum, oct->eps, 1.5, pow(2, -oct->lmin) * oct->d);
    oct->pmax_coax = pc;
    free(oct->srCoaxMat);
    oct->srCoaxMat = (cuFloatComplex *)malloc((size_t)std::max(1, oct->numSRCoaxTransVec) * coax_size(pc) * sizeof(cuFloatComplex));
    HOST_CALL(genSRSparseCoaxTransMat(wavNum, oct->srCoaxTransVec, oct->numSRCoaxTransVec, pc, oct->srCoaxMat));
    for (int pass = 0; pass < 2; pass++) {
        for (int i = 0; i < oct->lmax - oct->lmin; i++) {
            int l = pass == 0 ? oct->lmax - i : oct->lmin + 1 + i;
            if (pass == 0) genSSCoaxTransVecsRotAngles(l, oct->d, oct->pt_min, &vec, &numVec, &ang, &numRot);
            else genRRCoaxTransVecsRotAngles(l, oct->d, oct->pt_min, &vec, &numVec, &ang, &numRot);
            merge_vecs(oct->rrCoaxTransVec, oct->numRRCoaxTransVec, vec, numVec, epsilon);
            free(vec);
            free(ang);
        }
    }
    bubbleSort(oct->rrCoaxTransVec, oct->numRRCoaxTransVec);
    free(oct->rrCoaxMat);
    oct->rrCoaxMat = (cuFloatComplex *)malloc((size_t)std::max(1, oct->numRRCoaxTransVec) * coax_size(pc) * sizeof(cuFloatComplex));
    HOST_CALL(genRRSparseCoaxTransMat(wavNum, oct->rrCoaxTransVec, oct->numRRCoaxTransVec, pc, oct->rrCoaxMat));
    int nl = oct->lmax - oct->lmin;
    if (!oct->ssTransDestArr) oct->ssTransDestArr = (int **)calloc(std::max(1, nl), sizeof(int *));
    if (!oct->ssTransIdx) oct->ssTransIdx = (transIdx **)calloc(std::max(1, nl), sizeof(transIdx *));
    if (!oct->srTransOriginArr) oct->srTransOriginArr = (int **)calloc(nl + 1, sizeof(int *));
    if (!oct->srTransDestArr) oct->srTransDestArr = (int **)calloc(nl + 1, sizeof(int *));
    if (!oct->srTransIdx) oct->srTransIdx = (transIdx **)calloc(nl + 1, sizeof(transIdx *));
    if (!oct->rrTransOriginArr) oct->rrTransOriginArr = (int **)calloc(std::max(1, nl), sizeof(int *));
    if (!oct->rrTransIdx) oct->rrTransIdx = (transIdx **)calloc(std::max(1, nl), sizeof(transIdx *));
    genSSIdxArrs(oct->fmmLevelSet, oct->lmax, oct->pt_min, oct->d, oct->rrCoaxTransVec, oct->numRRCoaxTransVec, oct->ang,
                 oct->numRotAng, oct->ssTransIdx, oct->ssTransDestArr);
    genSRIdxArrs(oct->fmmLevelSet, oct->srNumLevelArr, oct->lmax, oct->pt_min, oct->d, oct->srCoaxTransVec,
                 oct->numSRCoaxTransVec, oct->ang, oct->numRotAng, oct->srTransIdx, oct->srTransOriginArr, oct->srTransDestArr);
    genRRIdxArrs(oct->fmmLevelSet, oct->lmax, oct->pt_min, oct->d, oct->rrCoaxTransVec, oct->numRRCoaxTransVec, oct->ang,
                 oct->numRotAng, oct->rrTransIdx, oct->rrTransOriginArr);
    return EXIT_SUCCESS;
}

extern "C" void destroyOctree(octree *oct)
{
    {
        std::lock_guard<std::mutex> g(g_oprl_mu);
        auto it = g_oprl_plans.find(oct);
        if (it != g_oprl_plans.end()) {
            fmm_plan_destroy(it->second.second);
            g_oprl_plans.erase(it);
        }
    }
    free(oct->pt);
    free(oct->elem);
    if (oct->fmmLevelSet) {
        for (int l = oct->lmin; l <= oct->lmax; l++) {
            int i = l - oct->lmin;
            free(oct->fmmLevelSet[i]);
            if (oct->srNumLevelArr) free(oct->srNumLevelArr[i]);
            if (oct->srTransIdx) free(oct->srTransIdx[i]);
            if (oct->srTransOriginArr) free(oct->srTransOriginArr[i]);
            if (oct->srTransDestArr) free(oct->srTransDestArr[i]);
            if (l > oct->lmin) {
                if (oct->ssTransIdx) free(oct->ssTransIdx[i - 1]);
                if (oct->ssTransDestArr) free(oct->ssTransDestArr[i - 1]);
                if (oct->rrTransIdx) free(oct->rrTransIdx[i - 1]);
                if (oct->rrTransOriginArr) free(oct->rrTransOriginArr[i - 1]);
            }
        }
    }
    free(oct->fmmLevelSet); free(oct->srNumLevelArr); free(oct->srTransIdx); free(oct->ssTransIdx);
    free(oct->rrTransIdx); free(oct->ssTransDestArr); free(oct->srTransOriginArr); free(oct->srTransDestArr);
    free(oct->rrTransOriginArr); free(oct->ang); free(oct->rotMat1); free(oct->rotMat2);
    free(oct->srCoaxTransVec); free(oct->srCoaxMat); free(oct->rrCoaxTransVec); free(oct->rrCoaxMat);
    free(oct->btmLvlElemIdx);
    int lmin = oct->lmin;
    memset(oct, 0, sizeof(*oct));
    oct->lmin = lmin;
}

extern "C" int OprL(const float wavNum, const octree *oct, const float *intPt, const float *intWgt, const cuFloatComplex *q,
                    cuFloatComplex *prod)
{
    (void)intPt;
    (void)intWgt; // the plan uses the same 3x3 collapsed Gauss rule (INTORDER = 3)
    if (!oct || !oct->pt || !oct->elem || !q || !prod) return EXIT_FAILURE;
    fmm_plan *plan = nullptr;
    {
        std::lock_guard<std::mutex> g(g_oprl_mu);
        auto it = g_oprl_plans.find(oct);
        if (it != g_oprl_plans.end() && it->second.first == wavNum) plan = it->second.second;
        if (!plan) {
            if (it != g_oprl_plans.end()) {
                fmm_plan_destroy(it->second.second);
                g_oprl_plans.erase(it);
            }
            std::vector<double> V(3 * (size_t)oct->numPt);
            std::vector<int> F(3 * (size_t)oct->numElem);
            for (int i = 0; i < oct->numPt; i++) { V[3 * i] = oct->pt[i].x; V[3 * i + 1] = oct->pt[i].y; V[3 * i + 2] = oct->pt[i].z; }
            for (int e = 0; e < oct->numElem; e++)
                for (int t = 0; t < 3; t++) F[3 * e + t] = oct->elem[e].node[t];
            fmm_options o;
            fmm_default_options(&o);
            o.k = wavNum;
            o.depth = oct->lmax;
            o.eps = TRUNCERR;
            o.a_re = 0.0; o.b_re = 1.0; o.c_re = 0.0;
            o.build_mixed = 0;
            if (fmm_plan_create(V.data(), oct->numPt, F.data(), oct->numElem, &o, &plan) != FMM_OK) return EXIT_FAILURE;
            g_oprl_plans[oct] = {wavNum, plan};
        }
    }
    std::vector<cuDoubleComplex> x(oct->numElem), y(oct->numElem);
    for (int i = 0; i < oct->numElem; i++) x[i] = make_cuDoubleComplex(cuCrealf(q[i]), cuCimagf(q[i]));
    if (fmm_matvec(plan, x.data(), y.data(), 1, FMM_FP64) != FMM_OK) return EXIT_FAILURE;
    for (int i = 0; i < oct->numElem; i++) prod[i] = make_cuFloatComplex((float)cuCreal(y[i]), (float)cuCimag(y[i]));
    return EXIT_SUCCESS;
}

// ============================================================================ integral.h
float INTPT_h[INTORDER];
float INTWGT_h[INTORDER];

extern "C" int genGaussParams(const int n, float *pt, float *wgt)
{
    // Gauss-Legendre nodes and weights (the reference solves the Golub-Welsch eigenproblem,
    // integral.cu:23-63; Newton on P_n gives the same rule)
    if (n < 1 || n > 64) return EXIT_FAILURE;
    for (int i = 0; i < n; i++) {
        double z = cos(FMM_PI * (i + 0.75) / (n + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= n; j++) {
                double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-16) break;
        }
        pt[n - 1 - i] = (float)z;
        wgt[n - 1 - i] = (float)(2.0 / ((1.0 - z * z) * pp * pp));
    }
    return EXIT_SUCCESS;
}
extern "C" int gaussPtsToDevice(const float *pt, const float *wgt)
{
    // the GPU kernels carry their own rule tables; keep the host copies the reference exposes
    for (int i = 0; i < INTORDER; i++) { INTPT_h[i] = pt[i]; INTWGT_h[i] = wgt[i]; }
    return EXIT_SUCCESS;
}
extern "C" cuFloatComplex green(const float k, const cartCoord x, const cartCoord y)
{
    float r = cartDist(x, y);
    cuFloatComplex e = cplxExp(k * r);
    float den = 4 * PI * r;
    return make_cuFloatComplex(cuCrealf(e) / den, cuCimagf(e) / den);
}
static cuFloatComplex pgp1n(const float k, const cartCoord x, const cartCoord y, const cartCoord n)
{
    float dist = cartDist(x, y);
    cuFloatComplex g = cuCmulf(green(k, x, y), make_cuFloatComplex(-1.0f / dist, k));
    float f = ((x.x - y.x) * n.x + (x.y - y.y) * n.y + (x.z - y.z) * n.z) / dist;
    return make_cuFloatComplex(cuCrealf(g) * f, cuCimagf(g) * f);
}
// collapsed rule over a triangle whose singular vertex (if any) is nod[2]
static cuFloatComplex collapsed(const float k, const cartCoord nod[3], const cartCoord y, const float *pt, const float *wgt,
                                int kern)
{
    cartCoord nrml = crossProd(cartCoordSub(nod[0], nod[2]), cartCoordSub(nod[1], nod[2]));
    cartCoord nh = normalize(nrml);
    float J = cartNorm(nrml);
    cuFloatComplex acc = make_cuFloatComplex(0, 0);
    for (int n = 0; n < INTORDER; n++) {
        float theta = 0.5f + 0.5f * pt[n], wn = wgt[n];
        for (int m = 0; m < INTORDER; m++) {
            float rho = 0.5f + 0.5f * pt[m], wm = wgt[m];
            float w = 0.25f * wn * wm * rho * J;
            float xi1 = rho * (1 - theta), xi2 = rho - xi1, xi3 = 1 - xi1 - xi2;
            cartCoord x = {nod[0].x * xi1 + nod[1].x * xi2 + nod[2].x * xi3, nod[0].y * xi1 + nod[1].y * xi2 + nod[2].y * xi3,
                           nod[0].z * xi1 + nod[1].z * xi2 + nod[2].z * xi3};
            cuFloatComplex g = kern ? pgp1n(k, x, y, nh) : green(k, x, y);
            acc = cuCaddf(acc, make_cuFloatComplex(w * cuCrealf(g), w * cuCimagf(g)));
        }
    }
    return acc;
}
static cuFloatComplex split_sgl(const float k, const cartCoord nod[3], const float *pt, const float *wgt, int kern)
{
    cartCoord c23 = scalarMul(0.5, cartCoordAdd(nod[1], nod[2]));
    cartCoord y = cartCoordAdd(nod[0], scalarMul(2.0f / 3.0f, cartCoordSub(c23, nod[0])));
    cuFloatComplex r = make_cuFloatComplex(0, 0);
    for (int s = 0; s < 3; s++) {
        cartCoord sub[3] = {nod[s], nod[(s + 1) % 3], y};
        r = cuCaddf(r, collapsed(k, sub, y, pt, wgt, kern));
    }
    return r;
}
extern "C" cuFloatComplex triElemIntegral_G_nsgl(const float k, const cartCoord nod[3], const cartCoord y, const float *pt,
                                                  const float *wgt)
{
    return collapsed(k, nod, y, pt, wgt, 0);
}
extern "C" cuFloatComplex triElemIntegral_G_sgl(const float k, const cartCoord nod[3], const float *pt, const float *wgt)
{
    return split_sgl(k, nod, pt, wgt, 0);
}
extern "C" cuFloatComplex triElemIntegral_pGp1n_nsgl(const float k, const cartCoord nod[3], const cartCoord y, const float *pt,
                                                      const float *wgt)
{
    return collapsed(k, nod, y, pt, wgt, 1);
}
extern "C" cuFloatComplex triElemIntegral_pGp1n_sgl(const float k, const cartCoord nod[3], const float *pt, const float *wgt)
{
    return split_sgl(k, nod, pt, wgt, 1);
}

// ------------------------------------------------- integral.h: regular-basis moments, dG/dn_y,
// d2G/dn_x dn_y, derivative coefficients.  Host routines like the reference's; arithmetic in
// FP64 from the FP32 arguments, results rounded to FP32 once.
namespace {

inline double2 z2(double re, double im) { return make_double2(re, im); }
inline double2 zscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
inline cuFloatComplex to_f(double2 a) { return make_cuFloatComplex((float)a.x, (float)a.y); }

// R_n^m(v) = j_n(k |v|) Q_n^{|m|}(cos theta) e^{i m phi}, n < P, index n^2 + n + m: the regular
// basis of rglBasis (translation.cu:171-178) with the reference's spherical harmonics
void regular_basis(int P, double k, const double v[3], std::vector<double2> &R)
{
    R.assign((size_t)P * P, z2(0.0, 0.0));
    if (P <= 0) return;
    double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (r == 0.0) {
        R[0].x = 0.28209479177387814;
        return;
    }
    std::vector<double> jn(P), Q((size_t)P * (P + 1) / 2);
    sph_jn_array(P, k * r, jn.data());
    legendre_Q(P, v[2] / r, Q.data());
    double phi = atan2(v[1], v[0]);
    for (int n = 0; n < P; n++)
        for (int m = 0; m <= n; m++) {
            double a = jn[n] * Q[n * (n + 1) / 2 + m], c = cos(m * phi), s = sin(m * phi);
            R[nm_idx(n, m)] = z2(a * c, a * s);
            R[nm_idx(n, -m)] = z2(a * c, -a * s);
        }
}

inline double2 basis_at(const std::vector<double2> &R, int n, int m)
{
    if (n < 0 || m > n || -m > n) return z2(0.0, 0.0);
    return R[nm_idx(n, m)];
}

// d R_n^m / dn from the basis of orders up to n+1 (G&D differentiation relations):
//   k/2 (n_x - i n_y) [b_{n+1}^{-m-1} R_{n+1}^{m+1} - b_n^m R_{n-1}^{m+1}]
// + k/2 (n_x + i n_y) [b_{n+1}^{m-1} R_{n+1}^{m-1} - b_n^{-m} R_{n-1}^{m-1}]
// + k n_z [a_{n-1}^m R_{n-1}^m - a_n^m R_{n+1}^m]
double2 dirdev(double k, int n, int m, const double nr[3], const std::vector<double2> &R)
{
    double2 t0 = csub(zscale(basis_at(R, n + 1, m + 1), coefB(n + 1, -m - 1)), zscale(basis_at(R, n - 1, m + 1), coefB(n, m)));
    double2 t1 = csub(zscale(basis_at(R, n + 1, m - 1), coefB(n + 1, m - 1)), zscale(basis_at(R, n - 1, m - 1), coefB(n, -m)));
    double2 t2 = csub(zscale(basis_at(R, n - 1, m), coefA(n - 1, m)), zscale(basis_at(R, n + 1, m), coefA(n, m)));
    double2 r = cmul(z2(0.5 * k * nr[0], -0.5 * k * nr[1]), t0);
    r = cadd(r, cmul(z2(0.5 * k * nr[0], 0.5 * k * nr[1]), t1));
    return cadd(r, zscale(t2, k * nr[2]));
}

struct Tri {
    double v[3][3];   // nodes
    double nrml[3];   // (v0 - v2) x (v1 - v2)
    double J, nh[3];  // |nrml| and the unit normal
    explicit Tri(const cartCoord nod[3])
    {
        for (int i = 0; i < 3; i++) { v[i][0] = nod[i].x; v[i][1] = nod[i].y; v[i][2] = nod[i].z; }
        init();
    }
    Tri(const double a[3], const double b[3], const double c[3])
    {
        for (int t = 0; t < 3; t++) { v[0][t] = a[t]; v[1][t] = b[t]; v[2][t] = c[t]; }
        init();
    }
    void init()
    {
        double e0[3], e1[3];
        for (int t = 0; t < 3; t++) { e0[t] = v[0][t] - v[2][t]; e1[t] = v[1][t] - v[2][t]; }
        nrml[0] = e0[1] * e1[2] - e0[2] * e1[1];
        nrml[1] = e0[2] * e1[0] - e0[0] * e1[2];
        nrml[2] = e0[0] * e1[1] - e0[1] * e1[0];
        J = sqrt(nrml[0] * nrml[0] + nrml[1] * nrml[1] + nrml[2] * nrml[2]);
        for (int t = 0; t < 3; t++) nh[t] = nrml[t] / J;
    }
    void centroid(double c[3]) const
    {
        for (int t = 0; t < 3; t++) c[t] = v[0][t] + (2.0 / 3.0) * (0.5 * (v[1][t] + v[2][t]) - v[0][t]);
    }
};

// The collapsed Gauss rule of integral.cu:80-109 over a triangle whose singular vertex (if any)
// is v2: theta = (1 + pt_i)/2, rho = (1 + pt_j)/2, x = rho(1-theta) v0 + rho theta v1 + (1-rho) v2,
// weight wgt_i wgt_j rho J / 4.  visit(x, w) is called for every point.
template <class F> void collapsed_points(const Tri &T, const float *pt, const float *wgt, F visit)
{
    for (int i = 0; i < INTORDER; i++) {
        double theta = 0.5 + 0.5 * (double)pt[i];
        for (int j = 0; j < INTORDER; j++) {
            double rho = 0.5 + 0.5 * (double)pt[j], w = 0.25 * (double)wgt[i] * (double)wgt[j] * rho * T.J;
            double xi1 = rho * (1.0 - theta), xi2 = rho * theta, xi3 = 1.0 - rho, x[3];
            for (int t = 0; t < 3; t++) x[t] = xi1 * T.v[0][t] + xi2 * T.v[1][t] + xi3 * T.v[2][t];
            visit(x, w);
        }
    }
}

template <class K> double2 collapsed_d(const Tri &T, const float *pt, const float *wgt, K kern)
{
    double2 acc = z2(0.0, 0.0);
    collapsed_points(T, pt, wgt, [&](const double *x, double w) { acc = cadd(acc, zscale(kern(x), w)); });
    return acc;
}

// dG(x, y)/dn_y = G (ik - 1/r) (y - x).n / r   (pGp2n, integral.cu:400-413)
double2 dgreen_dny(double k, const double x[3], const double y[3], const double n[3])
{
    double d[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double s = 1.0 / (4.0 * FMM_PI * r), dn = (d[0] * n[0] + d[1] * n[1] + d[2] * n[2]) / r;
    double2 g = z2(cos(k * r) * s, sin(k * r) * s);
    return zscale(cmul(g, z2(-1.0 / r, k)), dn);
}

// d2G(x, y)/dn_x dn_y = e^{ikr}/(4 pi r^3) [(3 - 3ikr - k^2 r^2) ((x-y).n1/r) ((y-x).n2/r)
//                                          + (1 - ikr) n1.n2]      (p2Gp1np2n, integral.cu:603-622)
double2 d2green(double k, const double n1[3], const double n2[3], const double x[3], const double y[3])
{
    double d[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
    double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    double a1 = (d[0] * n1[0] + d[1] * n1[1] + d[2] * n1[2]) / r;
    double a2 = -(d[0] * n2[0] + d[1] * n2[1] + d[2] * n2[2]) / r;
    double n12 = n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2];
    double s = 1.0 / (4.0 * FMM_PI * r * r * r), kr = k * r;
    double2 e = z2(cos(kr) * s, sin(kr) * s);
    double2 br = cadd(zscale(z2(3.0 - kr * kr, -3.0 * kr), a1 * a2), zscale(z2(1.0, -kr), n12));
    return cmul(e, br);
}

// Distance from the centroid to the triangle's boundary along the in-plane direction at angle
// theta (theta2rho, integral.cu:668-736).  The frame is the reference's: node 0 on the polar
// axis, node 1 at the angle 0c1 (in [0, pi]), node 2 at 0c1 + 1c2, all from the side lengths;
// below 0c1 the ray meets edge 01, below 0c1 + 1c2 edge 12, else edge 20.
double centroid_ray(const Tri &T, double theta)
{
    double c[3], dc[3], de[3];
    T.centroid(c);
    auto dist = [](const double *a, const double *b) {
        return sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    };
    for (int i = 0; i < 3; i++) { dc[i] = dist(T.v[i], c); de[i] = dist(T.v[i], T.v[(i + 1) % 3]); }
    double a01 = acos((dc[0] * dc[0] + dc[1] * dc[1] - de[0] * de[0]) / (2.0 * dc[0] * dc[1]));
    double a02 = a01 + acos((dc[1] * dc[1] + dc[2] * dc[2] - de[1] * de[1]) / (2.0 * dc[1] * dc[2]));
    double P[3][2] = {{dc[0], 0.0}, {dc[1] * cos(a01), dc[1] * sin(a01)}, {dc[2] * cos(a02), dc[2] * sin(a02)}};
    int e = theta < a01 ? 0 : (theta < a02 ? 1 : 2);
    const double *A = P[e], *B = P[(e + 1) % 3];
    double u0 = cos(theta), u1 = sin(theta), v0 = B[0] - A[0], v1 = B[1] - A[1];
    // the ray t u meets the edge A + s (B - A) at t = (A x (B - A)) / (u x (B - A))
    return fabs((A[0] * v1 - A[1] * v0) / (u0 * v1 - u1 * v0));
}

} // namespace

extern "C" cuFloatComplex triElemIntegral_R(const float wavNum, const cartCoord nod[3], const int n, const int m,
                                             const cartCoord x_lp, const float *pt, const float *wgt)
{
    Tri T(nod);
    const double c[3] = {x_lp.x, x_lp.y, x_lp.z};
    std::vector<double2> R;
    if (n < 0) return make_cuFloatComplex(0.0f, 0.0f);
    return to_f(collapsed_d(T, pt, wgt, [&](const double *x) {
        double v[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
        regular_basis(n + 1, wavNum, v, R);
        return basis_at(R, n, m);
    }));
}

extern "C" cuFloatComplex dirDev_R(const float wavNum, const int n, const int m, const cartCoord nrml, const cartCoord x)
{
    if (n < 0) return make_cuFloatComplex(0.0f, 0.0f);
    const double v[3] = {x.x, x.y, x.z}, nr[3] = {nrml.x, nrml.y, nrml.z};
    std::vector<double2> R;
    regular_basis(n + 2, wavNum, v, R);
    return to_f(dirdev(wavNum, n, m, nr, R));
}

extern "C" cuFloatComplex triElemIntegral_pRpn(const float wavNum, const cartCoord nod[3], const int n, const int m,
                                                const cartCoord x_lp, const float *pt, const float *wgt)
{
    Tri T(nod);
    const double c[3] = {x_lp.x, x_lp.y, x_lp.z};
    std::vector<double2> R;
    if (n < 0) return make_cuFloatComplex(0.0f, 0.0f);
    return to_f(collapsed_d(T, pt, wgt, [&](const double *x) {
        double v[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
        regular_basis(n + 2, wavNum, v, R);
        return dirdev(wavNum, n, m, T.nh, R);
    }));
}

extern "C" cuFloatComplex triElemIntegral_pGp2n_nsgl(const float wavNum, const cartCoord nod[3], const cartCoord nrml,
                                                      const cartCoord y, const float *pt, const float *wgt)
{
    Tri T(nod);
    const double yy[3] = {y.x, y.y, y.z}, nr[3] = {nrml.x, nrml.y, nrml.z};
    return to_f(collapsed_d(T, pt, wgt, [&](const double *x) { return dgreen_dny(wavNum, x, yy, nr); }));
}

extern "C" cuFloatComplex triElemIntegral_pGp2n_sgl(const float wavNum, const cartCoord nod[3], const float *pt, const float *wgt)
{
    // centroid split (integral.cu:539-601): three sub-triangles with the centroid as the
    // singular vertex, each integrated with its own unit normal at y = centroid
    Tri T(nod);
    double c[3];
    T.centroid(c);
    double2 acc = z2(0.0, 0.0);
    for (int s = 0; s < 3; s++) {
        Tri S(T.v[s], T.v[(s + 1) % 3], c);
        acc = cadd(acc, collapsed_d(S, pt, wgt, [&](const double *x) { return dgreen_dny(wavNum, x, c, S.nh); }));
    }
    return to_f(acc);
}

extern "C" cuFloatComplex triElemIntegral_p2Gp1np2n_nsgl(const float wavNum, const cartCoord nod[3], const cartCoord nrml_y,
                                                          const cartCoord y, const float *pt, const float *wgt)
{
    Tri T(nod);
    const double yy[3] = {y.x, y.y, y.z}, nr[3] = {nrml_y.x, nrml_y.y, nrml_y.z};
    return to_f(collapsed_d(T, pt, wgt, [&](const double *x) { return d2green(wavNum, T.nh, nr, x, yy); }));
}

extern "C" cuFloatComplex triElemIntegral_p2Gp1np2n_sgl(const float wavNum, const cartCoord nod[3], const float *pt, const float *wgt)
{
    // Hadamard finite part of int_T d2G/dn_x dn_y at the centroid of the flat element
    // (integral.cu:738-751): the kernel is e^{ikr}(1 - ikr)/(4 pi r^3) = d/dr[-e^{ikr}/r]/(4 pi r),
    // so in polar coordinates about the centroid
    //   FP = -1/(4 pi) [ int_0^{2 pi} e^{ik rho(theta)}/rho(theta) dtheta - 2 pi i k ],
    // the angle integral by the caller's Gauss rule mapped to theta = pi s + pi.
    Tri T(nod);
    double2 sum = z2(0.0, 0.0);
    for (int i = 0; i < INTORDER; i++) {
        double rho = centroid_ray(T, FMM_PI * (double)pt[i] + FMM_PI), w = (double)wgt[i] / rho;
        sum = cadd(sum, z2(w * cos(wavNum * rho), w * sin(wavNum * rho)));
    }
    sum = csub(zscale(sum, FMM_PI), z2(0.0, 2.0 * FMM_PI * wavNum));
    return to_f(zscale(sum, -1.0 / (4.0 * FMM_PI)));
}

extern "C" void cmptDiffCoeff(const float wavNum, const cuFloatComplex *coeff, const int p, const cartCoord nrml,
                              cuFloatComplex *coeff_n)
{
    // coefficients of d/dn sum_{n<=p} c_n^m R_n^m on R_n^m, n < p: the relations of dirDev_R
    // collected by output index (integral.cu:753-823, whose temporaries 3-5 are never
    // assigned; this is the sum that code sets out to form).  coeff holds (p+1)^2 entries.
    const double k = wavNum, nr[3] = {nrml.x, nrml.y, nrml.z};
    auto c = [&](int n, int m) {
        if (n < 0 || m > n || -m > n) return z2(0.0, 0.0);
        cuFloatComplex v = coeff[nm_idx(n, m)];
        return z2(cuCrealf(v), cuCimagf(v));
    };
    for (int n = 0; n < p; n++)
        for (int m = -n; m <= n; m++) {
            double2 t0 = csub(zscale(c(n - 1, m - 1), coefB(n, -m)), zscale(c(n + 1, m - 1), coefB(n + 1, m - 1)));
            double2 t1 = csub(zscale(c(n - 1, m + 1), coefB(n, m)), zscale(c(n + 1, m + 1), coefB(n + 1, -m - 1)));
            double2 t2 = csub(zscale(c(n + 1, m), coefA(n, m)), zscale(c(n - 1, m), coefA(n - 1, m)));
            double2 r = cmul(z2(0.5 * k * nr[0], -0.5 * k * nr[1]), t0);
            r = cadd(r, cmul(z2(0.5 * k * nr[0], 0.5 * k * nr[1]), t1));
            coeff_n[nm_idx(n, m)] = to_f(cadd(r, zscale(t2, k * nr[2])));
        }
}

extern "C" void bottomLevelCoeff_L(const float wavNum, const triElem elem, const cuFloatComplex q, const cartCoord *pt,
                                   const cartCoord x_lp, const float *intPt, const float *intWgt, cuFloatComplex *coeff,
                                   const int p)
{
    // multipole coefficients of the single layer of density q on one element about x_lp:
    // coeff[n, m] = i k q int R_n^{-m}(x - x_lp) dS, n < p (integral.cu:825-840, whose inner
    // loop tests n <= n; this is the loop over m = -n..n it stands for)
    cartCoord nod[3] = {pt[elem.node[0]], pt[elem.node[1]], pt[elem.node[2]]};
    Tri T(nod);
    const double c[3] = {x_lp.x, x_lp.y, x_lp.z};
    std::vector<double2> acc((size_t)p * p, z2(0.0, 0.0)), R;
    collapsed_points(T, intPt, intWgt, [&](const double *x, double w) {
        double v[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
        regular_basis(p, wavNum, v, R);
        for (int n = 0; n < p; n++)
            for (int m = -n; m <= n; m++) acc[nm_idx(n, m)] = cadd(acc[nm_idx(n, m)], zscale(R[nm_idx(n, -m)], w));
    });
    const double2 ikq = cmul(z2(0.0, (double)wavNum), z2(cuCrealf(q), cuCimagf(q)));
    for (int i = 0; i < p * p; i++) coeff[i] = to_f(cmul(ikq, acc[i]));
}
