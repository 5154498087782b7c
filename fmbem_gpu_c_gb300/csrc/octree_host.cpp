// Level sets of the octree, bit-exact with octree.c.  The reference's quadratic steps
// (orderArray, createSet, FMMLevelSetNumSR) become sorts here and a GPU kernel for the
// interaction lists; the results, including the first-occurrence ordering of every set,
// are identical.  Compiled with -ffp-contract=off so the double arithmetic of the centroid,
// bounding cube and scaling rounds exactly as the reference's does.
#include "octree_host.h"
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace fmm {

int read_obj(const char *path, std::vector<double> &V, std::vector<int> &F)
{
    FILE *fp = fopen(path, "r");
    if (!fp) return -1;
    char line[50];
    V.clear();
    F.clear();
    while (fgets(line, 49, fp) != NULL) {
        if (line[0] == 'v') {
            char type[64];
            double x = 0, y = 0, z = 0;
            sscanf(line, "%63s %lf %lf %lf", type, &x, &y, &z);
            V.push_back(x); V.push_back(y); V.push_back(z);
        }
        if (line[0] == 'f') {
            char type[64];
            int a = 0, b = 0, c = 0;
            sscanf(line, "%63s %d %d %d", type, &a, &b, &c);
            F.push_back(a - 1); F.push_back(b - 1); F.push_back(c - 1);
        }
    }
    fclose(fp);
    return 0;
}

void centroid(const double *n0, const double *n1, const double *n2, double *c)
{
    for (int a = 0; a < 3; a++) {
        double c23 = 0.5 * (n1[a] + n2[a]);
        c[a] = n0[a] + (2.0 / 3.0) * (c23 - n0[a]);
    }
}

void bounding_cube(const std::vector<double> &P, double eps, double *pt_min, double *dout)
{
    size_t n = P.size() / 3;
    double x_min = P[0], x_max = P[0], y_min = P[1], y_max = P[1];
    double z_min = P[1], z_max = P[1]; // the reference seeds z from the first point's y
    for (size_t i = 1; i < n; i++) {
        const double *p = &P[3 * i];
        if (p[0] < x_min) x_min = p[0];
        if (p[0] > x_max) x_max = p[0];
        if (p[1] < y_min) y_min = p[1];
        if (p[1] > y_max) y_max = p[1];
        if (p[2] < z_min) z_min = p[2];
        if (p[2] > z_max) z_max = p[2];
    }
    double eps_d = 0.000001 * std::min(std::min(x_max - x_min, y_max - y_min), z_max - z_min);
    eps_d = std::min(eps, eps_d);
    x_max += eps_d; x_min -= eps_d;
    y_max += eps_d; y_min -= eps_d;
    z_max += eps_d; z_min -= eps_d;
    double d_x = x_max - x_min, d_y = y_max - y_min, d_z = z_max - z_min;
    double d_max = std::max(std::max(d_x, d_y), d_z);
    x_min -= (d_max - d_x) / 2;
    y_min -= (d_max - d_y) / 2;
    z_min -= (d_max - d_z) / 2;
    pt_min[0] = x_min; pt_min[1] = y_min; pt_min[2] = z_min;
    *dout = d_max;
}

long long morton_key(const double *s, int l)
{
    // repeated doubling in dec2bin_frac yields the binary digits of s, i.e. floor(s 2^l)
    long long ix = (long long)std::floor(s[0] * std::ldexp(1.0, l));
    long long iy = (long long)std::floor(s[1] * std::ldexp(1.0, l));
    long long iz = (long long)std::floor(s[2] * std::ldexp(1.0, l));
    long long key = 0;
    for (int b = l - 1; b >= 0; b--) key = key * 8 + 4 * ((ix >> b) & 1) + 2 * ((iy >> b) & 1) + ((iz >> b) & 1);
    return key;
}

int deter_lmax(const std::vector<double> &S, int s)
{
    size_t n = S.size() / 3;
    std::vector<long long> keys(n);
    for (size_t i = 0; i < n; i++) keys[i] = morton_key(&S[3 * i], 10);
    std::sort(keys.begin(), keys.end());
    int l_max = 0;
    for (size_t i = 0; i + (size_t)s < n; i++) {
        long long a = keys[i], b = keys[i + s];
        if (a == b) return 11; // "Integer type cannot accomodate the current accuracy."
        int l = 10;
        while (a != b) { l--; a /= 8; b /= 8; }
        l_max = std::max(l_max, l + 1);
    }
    return l_max;
}

std::vector<long long> first_occurrence(const std::vector<long long> &v)
{
    std::vector<std::pair<long long, int>> kv(v.size());
    for (size_t i = 0; i < v.size(); i++) kv[i] = {v[i], (int)i};
    std::sort(kv.begin(), kv.end());
    std::vector<std::pair<int, long long>> firsts;
    for (size_t i = 0; i < kv.size(); i++)
        if (i == 0 || kv[i].first != kv[i - 1].first) firsts.push_back({kv[i].second, kv[i].first});
    std::sort(firsts.begin(), firsts.end());
    std::vector<long long> out(firsts.size());
    for (size_t i = 0; i < firsts.size(); i++) out[i] = firsts[i].second;
    return out;
}

int build_tree(const std::vector<double> &V, const std::vector<int> &F, int s, int depth, HostTree &T)
{
    size_t nf = F.size() / 3;
    if (nf == 0) return -1;
    std::vector<double> C(3 * nf), S(3 * nf);
    for (size_t e = 0; e < nf; e++)
        centroid(&V[3 * F[3 * e]], &V[3 * F[3 * e + 1]], &V[3 * F[3 * e + 2]], &C[3 * e]);
    bounding_cube(C, 0.01, T.pt_min, &T.d);
    for (size_t e = 0; e < nf; e++)
        for (int a = 0; a < 3; a++) S[3 * e + a] = (C[3 * e + a] - T.pt_min[a]) / T.d;
    T.lmax = depth > 0 ? depth : deter_lmax(S, s);
    if (depth < 0) {
        // the reference's rule, capped where leaf boxes would get smaller than 1.5 times the
        // longest element edge: an element filed under its centroid's box reaches outside it,
        // and the expansions of boxes only one box apart lose their accuracy
        double emax = 0.0;
        for (size_t e = 0; e < nf; e++)
            for (int a = 0; a < 3; a++) {
                const double *p0 = &V[3 * F[3 * e + a]], *p1 = &V[3 * F[3 * e + (a + 1) % 3]];
                double dx = p0[0] - p1[0], dy = p0[1] - p1[1], dz = p0[2] - p1[2];
                emax = std::max(emax, sqrt(dx * dx + dy * dy + dz * dz));
            }
        int cap = T.lmin;
        while (cap < 30 && T.d * ldexp(1.0, -(cap + 1)) >= 1.5 * emax) cap++;
        T.lmax = std::max(T.lmin, std::min(T.lmax, cap));
    }
    if (T.lmax < T.lmin) return -2;
    T.elem_key.resize(nf);
    for (size_t e = 0; e < nf; e++) T.elem_key[e] = morton_key(&S[3 * e], T.lmax);
    T.sets.assign(T.lmax + 1, std::vector<long long>());
    T.sets[T.lmax] = first_occurrence(T.elem_key);
    for (int l = T.lmax - 1; l >= T.lmin; l--) {
        std::vector<long long> par(T.sets[l + 1].size());
        for (size_t i = 0; i < par.size(); i++) par[i] = T.sets[l + 1][i] / 8;
        T.sets[l] = first_occurrence(par);
    }
    // leaf index of every element, consistent with the leaf set
    std::vector<std::pair<long long, int>> kv(T.sets[T.lmax].size());
    for (size_t i = 0; i < kv.size(); i++) kv[i] = {T.sets[T.lmax][i], (int)i};
    std::sort(kv.begin(), kv.end());
    T.elem_leaf.resize(nf);
    for (size_t e = 0; e < nf; e++) {
        auto it = std::lower_bound(kv.begin(), kv.end(), std::make_pair(T.elem_key[e], -1));
        T.elem_leaf[e] = it->second;
    }
    return 0;
}

void box_xyz(long long num, int l, int *x, int *y, int *z)
{
    int xx = 0, yy = 0, zz = 0;
    for (int b = 0; b < l; b++) {
        int digit = (int)((num >> (3 * (l - 1 - b))) & 7);
        xx = (xx << 1) | ((digit >> 2) & 1);
        yy = (yy << 1) | ((digit >> 1) & 1);
        zz = (zz << 1) | (digit & 1);
    }
    *x = xx; *y = yy; *z = zz;
}

long long box_num(int x, int y, int z, int l)
{
    long long key = 0;
    for (int b = l - 1; b >= 0; b--) key = key * 8 + 4 * ((x >> b) & 1) + 2 * ((y >> b) & 1) + ((z >> b) & 1);
    return key;
}

} // namespace fmm
