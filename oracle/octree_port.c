/* octree_port.c -- the reference's CPU octree build, restated in C with the reference's own
 * algorithms and therefore their costs: the CPU baseline of the octree stage.
 *
 * TEST AND BASELINE INFRASTRUCTURE, like the rest of oracle/: bench.py's CPU-baseline leg
 * times it, and tests/test_octree_port.py pins its output against the fixtures that the
 * reference's own octree.c produced (tests/golden).  The product library never calls it.
 *
 * The reference's sources are compiled only where they are mounted (oracle/build_ref.sh);
 * a machine without them times this port instead.  Steps, with the reference routine each
 * one follows (paths within the reference project):
 *
 *   srcBoxes (octree.c:749-767)
 *     centroids            triCentroid_d, structs.cu:126-131: n0 + 2/3 ((n1+n2)/2 - n0)
 *     bounding cube        findBoundingCube, octree.c:681-747, z bounds seeded from y
 *     scaling              scalePnts, octree.c:62-86
 *     leaf level           deterLmax, octree.c:635-679, with orderArray's O(N^2) exchange
 *                          sort (octree.c:546-561); skipped when a depth is given
 *     leaf set             pnts2numSet, octree.c:471-479: Morton keys (pnt2boxnum,
 *                          octree.c:158-183) deduplicated by createSet's linear scan
 *                          (octree.c:393-410), first-occurrence order
 *   FMMLevelSet (octree.c:890-906)
 *                          parents by prntLevelSet (octree.c:816-831), createSet again
 *   FMMLevelSetNumSR (octree.c:908-919)
 *                          per box: I4 (octree.c:517-543) -- createSet of the children of
 *                          the parent's neighbourhood, createSet of the own neighbourhood,
 *                          their difference, neighbours in x-y-z order (neighbors,
 *                          octree.c:237-391) with the box itself last -- then intersection
 *                          with the level set by linear membership tests (intersection and
 *                          isMember, octree.c:412-437)
 *
 * The quadratic scans of the set algebra are kept as they are, since they are the cost.  The
 * per-call mallocs and binary digit arrays of neighbors/pnt2boxnum/boxCenter become integer
 * arithmetic, so this port is, if anything, faster than the reference.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double port_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ------------------------------------------------------------------ count-prefixed sets */
/* A set is an int array whose element 0 holds the count, as in octree.c. */

static int port_member(int v, const int *set)
{
    for (int i = 1; i <= set[0]; i++)
        if (set[i] == v) return 1;
    return 0;
}

/* first-occurrence dedupe by linear scan of what is kept so far */
static void port_make_set(const int *vals, int n, int *set)
{
    set[0] = 0;
    for (int i = 0; i < n; i++)
        if (!port_member(vals[i], set)) set[++set[0]] = vals[i];
}

/* elements of a (in a's order) that are (keep = 1) or are not (keep = 0) in b */
static void port_filter(const int *a, const int *b, int keep, int *out)
{
    out[0] = 0;
    for (int i = 1; i <= a[0]; i++)
        if (port_member(a[i], b) == keep) out[++out[0]] = a[i];
}

/* ------------------------------------------------------------------ Morton boxes */
static int port_key(double sx, double sy, double sz, int l)
{
    /* dec2bin_frac: digits by repeated doubling (exact in binary floating point) */
    int key = 0;
    for (int b = 0; b < l; b++) {
        sx *= 2.0; sy *= 2.0; sz *= 2.0;
        double fx = floor(sx), fy = floor(sy), fz = floor(sz);
        sx -= fx; sy -= fy; sz -= fz;
        key = 8 * key + 4 * (int)fx + 2 * (int)fy + (int)fz;
    }
    return key;
}

static void port_xyz(int num, int l, int *x, int *y, int *z)
{
    int xx = 0, yy = 0, zz = 0;
    for (int b = l - 1; b >= 0; b--) {
        int d = (num >> (3 * b)) & 7;
        xx = 2 * xx + ((d >> 2) & 1);
        yy = 2 * yy + ((d >> 1) & 1);
        zz = 2 * zz + (d & 1);
    }
    *x = xx; *y = yy; *z = zz;
}

static int port_num(int x, int y, int z, int l)
{
    int key = 0;
    for (int b = l - 1; b >= 0; b--) key = 8 * key + 4 * ((x >> b) & 1) + 2 * ((y >> b) & 1) + ((z >> b) & 1);
    return key;
}

/* neighbours of a box at level l (not the box itself), x outermost, then y, then z */
static int port_neighbours(int num, int l, int *out)
{
    int x, y, z, n = 0, top = (1 << l) - 1;
    port_xyz(num, l, &x, &y, &z);
    for (int a = (x > 0 ? x - 1 : 0); a <= (x < top ? x + 1 : top); a++)
        for (int b = (y > 0 ? y - 1 : 0); b <= (y < top ? y + 1 : top); b++)
            for (int c = (z > 0 ? z - 1 : 0); c <= (z < top ? z + 1 : top); c++) {
                int q = port_num(a, b, c, l);
                if (q != num) out[n++] = q;
            }
    return n;
}

/* I4: children of the parent's neighbourhood that are not in the box's own neighbourhood */
static void port_i4(int num, int l, int *out)
{
    int nb[28], nbp[28], cand[8 * 27], setp[8 * 27 + 1], setc[28];
    int t = port_neighbours(num, l, nb);
    nb[t++] = num;
    int tp = port_neighbours(num / 8, l - 1, nbp);
    nbp[tp++] = num / 8;
    for (int i = 0; i < tp; i++)
        for (int c = 0; c < 8; c++) cand[8 * i + c] = 8 * nbp[i] + c;
    port_make_set(cand, 8 * tp, setp);
    port_make_set(nb, t, setc);
    port_filter(setp, setc, 0, out);
}

/* ------------------------------------------------------------------ the build */
/* deterLmax: orderArray's exchange sort of the level-10 keys, then the deepest level at
 * which keys i and i+s share a box, plus one; 11 when two keys coincide at level 10 */
static int port_lmax(const double *S, int n, int s)
{
    int *key = (int *)malloc(sizeof(int) * (n > 0 ? n : 1)), *ord = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
    for (int i = 0; i < n; i++) {
        key[i] = port_key(S[3 * i], S[3 * i + 1], S[3 * i + 2], 10);
        ord[i] = i;
    }
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++)
            if (key[ord[i]] > key[ord[j]]) { int t = ord[i]; ord[i] = ord[j]; ord[j] = t; }
    int lmax = 0;
    for (int i = 0, j = s; j < n; i++, j++) {
        int a = key[ord[i]], b = key[ord[j]], l = 10;
        if (a == b) { lmax = 11; break; }
        while (a != b) { l--; a /= 8; b /= 8; }
        if (l + 1 > lmax) lmax = l + 1;
    }
    free(key);
    free(ord);
    return lmax;
}

/* Build the octree of a triangle mesh.  depth > 0 fixes the leaf level, else deterLmax with
 * leaf occupancy s decides it.  sr_sample > 0 runs FMMLevelSetNumSR only on every k-th box of
 * a level with more than sr_sample boxes (k = ceil(B / sr_sample)); times[3] then scales that
 * level's time by B / (boxes run).
 * Outputs: *lmax; counts[l] (l = 2..lmax) the boxes of level l; sets (capacity cap) the level
 * sets of levels 2..lmax one after another; srnum (same layout) the SR counts, -1 for boxes
 * the sample left out; times[0] srcBoxes, [1] FMMLevelSet, [2] FMMLevelSetNumSR as run,
 * [3] FMMLevelSetNumSR scaled to every box.  Returns 0, or -1 if cap is too small or the
 * leaf level is out of range. */
int orc_port_octree(const double *V, const int *F, int nf, int s, int depth, int sr_sample, int *lmax_out,
                    int *counts, int *sets, int *srnum, long long cap, double *times)
{
    double t0 = port_now();
    double *S = (double *)malloc(sizeof(double) * 3 * (nf > 0 ? nf : 1));
    for (int e = 0; e < nf; e++) {
        for (int a = 0; a < 3; a++) {
            double n0 = V[3 * F[3 * e] + a], n1 = V[3 * F[3 * e + 1] + a], n2 = V[3 * F[3 * e + 2] + a];
            double mid = 0.5 * (n1 + n2);
            S[3 * e + a] = n0 + (2.0 / 3.0) * (mid - n0);
        }
    }
    double lo[3], hi[3];
    lo[0] = hi[0] = S[0];
    lo[1] = hi[1] = S[1];
    lo[2] = hi[2] = S[1]; /* the reference seeds the z bounds with y */
    for (int e = 1; e < nf; e++)
        for (int a = 0; a < 3; a++) {
            if (S[3 * e + a] < lo[a]) lo[a] = S[3 * e + a];
            if (S[3 * e + a] > hi[a]) hi[a] = S[3 * e + a];
        }
    double pad = 0.000001 * fmin(fmin(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    pad = fmin(0.01, pad);
    double ext[3], d = 0.0;
    for (int a = 0; a < 3; a++) {
        hi[a] += pad;
        lo[a] -= pad;
        ext[a] = hi[a] - lo[a];
    }
    d = fmax(fmax(ext[0], ext[1]), ext[2]);
    for (int a = 0; a < 3; a++) lo[a] -= (d - ext[a]) / 2;
    for (int e = 0; e < nf; e++)
        for (int a = 0; a < 3; a++) S[3 * e + a] = (S[3 * e + a] - lo[a]) / d;
    int lmax = depth > 0 ? depth : port_lmax(S, nf, s);
    *lmax_out = lmax;
    if (lmax < 2 || lmax > 10) { free(S); return -1; }

    int **lev = (int **)calloc(lmax + 1, sizeof(int *));
    int *keys = (int *)malloc(sizeof(int) * (nf > 0 ? nf : 1));
    for (int e = 0; e < nf; e++) keys[e] = port_key(S[3 * e], S[3 * e + 1], S[3 * e + 2], lmax);
    lev[lmax] = (int *)malloc(sizeof(int) * (nf + 1));
    port_make_set(keys, nf, lev[lmax]);
    double t1 = port_now();
    for (int l = lmax - 1; l >= 2; l--) {
        int n = lev[l + 1][0];
        for (int i = 0; i < n; i++) keys[i] = lev[l + 1][i + 1] / 8;
        lev[l] = (int *)malloc(sizeof(int) * (n + 1));
        port_make_set(keys, n, lev[l]);
    }
    double t2 = port_now();
    long long total = 0;
    for (int l = 2; l <= lmax; l++) total += lev[l][0];
    int rc = total <= cap ? 0 : -1;
    double scaled = 0.0;
    long long pos = 0;
    for (int l = 2; l <= lmax && rc == 0; l++) {
        int B = lev[l][0], step = 1;
        if (sr_sample > 0 && B > sr_sample) step = (B + sr_sample - 1) / sr_sample;
        int set[8 * 27 + 1], hit[8 * 27 + 1], ran = 0;
        double a = port_now();
        for (int i = 0; i < B; i++) {
            sets[pos + i] = lev[l][i + 1];
            srnum[pos + i] = -1;
            if (i % step) continue;
            port_i4(lev[l][i + 1], l, set);
            port_filter(set, lev[l], 1, hit);
            srnum[pos + i] = hit[0];
            ran++;
        }
        double dt = port_now() - a;
        scaled += ran ? dt * (double)B / ran : 0.0;
        counts[l] = B;
        pos += B;
    }
    double t3 = port_now();
    times[0] = t1 - t0;
    times[1] = t2 - t1;
    times[2] = t3 - t2;
    times[3] = scaled;
    for (int l = 2; l <= lmax; l++) free(lev[l]);
    free(lev);
    free(keys);
    free(S);
    return rc;
}
