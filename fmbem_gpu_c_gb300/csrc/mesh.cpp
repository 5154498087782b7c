// Mesh front end: generators for the synthetic bodies (geodesic sphere of any frequency,
// ellipsoid with seeded spherical-harmonic bumps, box).  The reference reads meshes from OBJ
// files only (octree.c:563-619); these produce the same vertex/triangle arrays directly.
// All meshes are closed, triangles counter-clockwise seen from outside (outward normal
// (v0 - v2) x (v1 - v2)), shared vertices merged, coordinates rounded to 9 significant
// digits like the OBJ files this library writes.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/fmmbem.h"

void fmm_set_error(const char *fmt, ...);

namespace {

double round9(double v)
{
    char buf[64];
    snprintf(buf, sizeof(buf), "%.9g", v);
    return strtod(buf, nullptr);
}

// Deduplicates points that coincide up to 1e-9 of the unit scale.
struct PointSet {
    std::vector<double> V;
    std::map<std::tuple<long long, long long, long long>, int> index;
    int add(const double *p)
    {
        auto key = std::make_tuple(llround(p[0] * 1e9), llround(p[1] * 1e9), llround(p[2] * 1e9));
        auto it = index.find(key);
        if (it != index.end()) return it->second;
        int id = (int)(V.size() / 3);
        V.push_back(p[0]);
        V.push_back(p[1]);
        V.push_back(p[2]);
        index.emplace(key, id);
        return id;
    }
};

const double ICO_T = 1.6180339887498948482;
const double ICO_V[12][3] = {{-1, ICO_T, 0}, {1, ICO_T, 0}, {-1, -ICO_T, 0}, {1, -ICO_T, 0}, {0, -1, ICO_T}, {0, 1, ICO_T},
                             {0, -1, -ICO_T}, {0, 1, -ICO_T}, {ICO_T, 0, -1}, {ICO_T, 0, 1}, {-ICO_T, 0, -1}, {-ICO_T, 0, 1}};
const int ICO_F[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                          {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                          {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};

// Unit-sphere geodesic mesh: every icosahedron face divided into freq^2 triangles, points
// projected radially.
void geodesic(int freq, std::vector<double> &V, std::vector<int> &F)
{
    PointSet ps;
    F.clear();
    for (int f = 0; f < 20; f++) {
        const double *A = ICO_V[ICO_F[f][0]], *B = ICO_V[ICO_F[f][1]], *C = ICO_V[ICO_F[f][2]];
        std::vector<int> id((freq + 1) * (freq + 2) / 2);
        auto at = [&](int i, int j) -> int & { return id[i * (2 * freq + 3 - i) / 2 + j]; };
        for (int i = 0; i <= freq; i++)
            for (int j = 0; i + j <= freq; j++) {
                double p[3], nn = 0.0;
                for (int a = 0; a < 3; a++) {
                    p[a] = A[a] + (B[a] - A[a]) * i / freq + (C[a] - A[a]) * j / freq;
                    nn += p[a] * p[a];
                }
                nn = sqrt(nn);
                for (int a = 0; a < 3; a++) p[a] /= nn;
                at(i, j) = ps.add(p);
            }
        for (int i = 0; i < freq; i++)
            for (int j = 0; i + j < freq; j++) {
                F.push_back(at(i, j));
                F.push_back(at(i + 1, j));
                F.push_back(at(i, j + 1));
                if (i + j + 1 < freq) {
                    F.push_back(at(i + 1, j));
                    F.push_back(at(i + 1, j + 1));
                    F.push_back(at(i, j + 1));
                }
            }
    }
    V = ps.V;
}

// SplitMix64 and Box-Muller: the seeded N(0, 1) stream of the bump coefficients
struct Rng {
    unsigned long long s;
    unsigned long long next()
    {
        unsigned long long z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal()
    {
        double u1 = uniform(), u2 = uniform();
        return sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2);
    }
};

// real orthonormal spherical harmonics up to degree L at the unit vector u, index l^2+l+m:
// Q_l^|m|(cos theta) times sqrt(2) cos(m phi) (m > 0), sqrt(2) sin(|m| phi) (m < 0), 1 (m = 0)
void real_sh(int L, const double *u, std::vector<double> &Y)
{
    int P = L + 1;
    std::vector<double> Q(P * (P + 1) / 2);
    double ct = u[2], st = sqrt(std::max(0.0, 1.0 - ct * ct)), phi = atan2(u[1], u[0]);
    Q[0] = 0.28209479177387814;
    for (int m = 1; m < P; m++) Q[m * (m + 1) / 2 + m] = sqrt((2.0 * m + 1.0) / (2.0 * m)) * st * Q[(m - 1) * m / 2 + (m - 1)];
    for (int m = 0; m < P; m++) {
        if (m + 1 < P) Q[(m + 1) * (m + 2) / 2 + m] = sqrt(2.0 * m + 3.0) * ct * Q[m * (m + 1) / 2 + m];
        for (int n = m + 2; n < P; n++) {
            double a = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
            double b = sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) / (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
            Q[n * (n + 1) / 2 + m] = a * (ct * Q[(n - 1) * n / 2 + m] - b * Q[(n - 2) * (n - 1) / 2 + m]);
        }
    }
    Y.assign(P * P, 0.0);
    for (int l = 0; l <= L; l++) {
        Y[l * l + l] = Q[l * (l + 1) / 2];
        for (int m = 1; m <= l; m++) {
            double q = sqrt(2.0) * Q[l * (l + 1) / 2 + m];
            Y[l * l + l + m] = q * cos(m * phi);
            Y[l * l + l - m] = q * sin(m * phi);
        }
    }
}

int emit(const std::vector<double> &V, const std::vector<int> &F, double *Vout, int *nv, int *Fout, int *nf)
{
    *nv = (int)(V.size() / 3);
    *nf = (int)(F.size() / 3);
    if (Vout)
        for (size_t i = 0; i < V.size(); i++) Vout[i] = round9(V[i]);
    if (Fout) memcpy(Fout, F.data(), sizeof(int) * F.size());
    return FMM_OK;
}

} // namespace

extern "C" int fmm_mesh_geodesic(int freq, double radius, double *V, int *nv, int *F, int *nf)
{
    if (freq < 1 || freq > 1000 || !(radius > 0) || !nv || !nf) { fmm_set_error("fmm_mesh_geodesic: invalid argument"); return FMM_ERR_ARG; }
    std::vector<double> Vs;
    std::vector<int> Fs;
    geodesic(freq, Vs, Fs);
    for (auto &v : Vs) v *= radius;
    return emit(Vs, Fs, V, nv, F, nf);
}

extern "C" int fmm_mesh_ellipsoid(int freq, double ax, double ay, double az, int lmax, double sigma,
                                  unsigned long long seed, double *V, int *nv, int *F, int *nf)
{
    if (freq < 1 || freq > 1000 || !(ax > 0) || !(ay > 0) || !(az > 0) || lmax < -1 || lmax > 30 || !(sigma >= 0) || !nv || !nf) {
        fmm_set_error("fmm_mesh_ellipsoid: invalid argument");
        return FMM_ERR_ARG;
    }
    std::vector<double> Vs;
    std::vector<int> Fs;
    geodesic(freq, Vs, Fs);
    std::vector<double> c;
    if (lmax >= 0) {
        Rng rng{seed};
        c.resize((lmax + 1) * (lmax + 1));
        for (auto &v : c) v = sigma * rng.normal();
    }
    std::vector<double> Y;
    for (size_t i = 0; i < Vs.size(); i += 3) {
        double *u = &Vs[i];
        double e[3] = {ax * u[0], ay * u[1], az * u[2]};
        double r = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]), bump = 0.0;
        if (lmax >= 0) {
            real_sh(lmax, u, Y);
            for (size_t q = 0; q < c.size(); q++) bump += c[q] * Y[q];
        }
        double s = (r + bump) / r;
        if (!(s > 0.05)) { fmm_set_error("fmm_mesh_ellipsoid: bumps deeper than the body"); return FMM_ERR_ARG; }
        for (int a = 0; a < 3; a++) u[a] = e[a] * s;
    }
    return emit(Vs, Fs, V, nv, F, nf);
}

extern "C" int fmm_mesh_box(int n, double lx, double ly, double lz, double *V, int *nv, int *F, int *nf)
{
    if (n < 1 || n > 2000 || !(lx > 0) || !(ly > 0) || !(lz > 0) || !nv || !nf) { fmm_set_error("fmm_mesh_box: invalid argument"); return FMM_ERR_ARG; }
    PointSet ps;
    std::vector<int> Fs;
    double L[3] = {lx, ly, lz};
    // face with outward axis a and sign s: (u, v) spans the other two axes, ordered so that
    // (du x dv) points along s e_a
    for (int a = 0; a < 3; a++)
        for (int s = -1; s <= 1; s += 2) {
            int b = (a + 1) % 3, c = (a + 2) % 3;
            if (s < 0) std::swap(b, c);
            std::vector<int> id((n + 1) * (n + 1));
            for (int i = 0; i <= n; i++)
                for (int j = 0; j <= n; j++) {
                    double p[3];
                    p[a] = 0.5 * s * L[a];
                    p[b] = L[b] * ((double)i / n - 0.5);
                    p[c] = L[c] * ((double)j / n - 0.5);
                    id[i * (n + 1) + j] = ps.add(p);
                }
            for (int i = 0; i < n; i++)
                for (int j = 0; j < n; j++) {
                    int v00 = id[i * (n + 1) + j], v10 = id[(i + 1) * (n + 1) + j], v01 = id[i * (n + 1) + j + 1],
                        v11 = id[(i + 1) * (n + 1) + j + 1];
                    Fs.insert(Fs.end(), {v00, v10, v01, v10, v11, v01});
                }
        }
    return emit(ps.V, Fs, V, nv, F, nf);
}
