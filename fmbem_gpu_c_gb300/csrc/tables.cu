// Setup kernels: rotation and coaxial translation tables, element moment tables for
// P2M/L2P, the near-field matrix by quadrature, far-field evaluation.  All in FP64; the
// mixed-precision path receives FP32 copies.
#include "plan.h"
#include "coax_recurrence.cuh"
#include <cstdio>
#include <math.h>
#include <vector>
#include <algorithm>

namespace fmm {

// ----------------------------------------------------------------------------- quadrature
// Regular rules: barycentric points and weights with  int_T f dS = J * sum_q w_q f(x_q),
// J = |(n0-n2) x (n1-n2)|.  Rule 0 is the collapsed 3x3 Gauss rule of integral.cu:80-109
// (weights 0.25 w_n w_m rho, points in the reference's loop order); rule 1 is Dunavant's
// 7-point degree-5 rule (area = J/2).  CRULE holds the collapsed rule that also serves the
// singular centroid split (integral.cu:202-249).
__constant__ double c_rule_bary[2][16 * 3];
__constant__ double c_rule_w[2][16];
__constant__ int c_rule_n[2];
// Gauss-Legendre rule on [-1, 1] for the edge integrals of the Burton-Miller terms
#define LINE_PTS 8
__constant__ double c_line_x[LINE_PTS], c_line_w[LINE_PTS];

static void gauss_legendre(int n, double *x, double *w)
{
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
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

// Gauss-Legendre nodes and weights on [-1, 1]
void line_rule(int n, double *x, double *w) { gauss_legendre(n, x, w); }

// The two regular rules as host tables (barycentric points, weights in units of J, counts).
void rule_tables(double bary[2][48], double w[2][16], int n[2])
{
    for (int r = 0; r < 2; r++)
        for (int i = 0; i < 48; i++) bary[r][i] = 0.0;
    for (int r = 0; r < 2; r++)
        for (int i = 0; i < 16; i++) w[r][i] = 0.0;
    double x[3], wt[3];
    gauss_legendre(3, x, wt);
    int q = 0;
    for (int i = 0; i < 3; i++) {
        double theta = 0.5 + 0.5 * x[i];
        for (int j = 0; j < 3; j++) {
            double rho = 0.5 + 0.5 * x[j];
            double xi1 = rho * (1 - theta), xi2 = rho - xi1, xi3 = 1 - xi1 - xi2;
            bary[0][3 * q] = xi1; bary[0][3 * q + 1] = xi2; bary[0][3 * q + 2] = xi3;
            w[0][q] = 0.25 * wt[i] * wt[j] * rho;
            q++;
        }
    }
    n[0] = q;
    double s15 = sqrt(15.0);
    double b1 = (6.0 - s15) / 21.0, a1 = 1.0 - 2.0 * b1, w1 = (155.0 - s15) / 1200.0;
    double b2 = (6.0 + s15) / 21.0, a2 = 1.0 - 2.0 * b2, w2 = (155.0 + s15) / 1200.0;
    double pts[7][3] = {{1.0 / 3, 1.0 / 3, 1.0 / 3}, {a1, b1, b1}, {b1, a1, b1}, {b1, b1, a1},
                        {a2, b2, b2}, {b2, a2, b2}, {b2, b2, a2}};
    double ww[7] = {9.0 / 40, w1, w1, w1, w2, w2, w2};
    for (int t = 0; t < 7; t++) {
        for (int a = 0; a < 3; a++) bary[1][3 * t + a] = pts[t][a];
        w[1][t] = 0.5 * ww[t];
    }
    n[1] = 7;
}

static int upload_rules()
{
    double bary[2][48], w[2][16];
    int n[2];
    rule_tables(bary, w, n);
    FMM_CUDA_TRY(cudaMemcpyToSymbol(c_rule_bary, bary, sizeof(bary)));
    FMM_CUDA_TRY(cudaMemcpyToSymbol(c_rule_w, w, sizeof(w)));
    FMM_CUDA_TRY(cudaMemcpyToSymbol(c_rule_n, n, sizeof(n)));
    double lx[LINE_PTS], lw[LINE_PTS];
    gauss_legendre(LINE_PTS, lx, lw);
    FMM_CUDA_TRY(cudaMemcpyToSymbol(c_line_x, lx, sizeof(lx)));
    FMM_CUDA_TRY(cudaMemcpyToSymbol(c_line_w, lw, sizeof(lw)));
    return FMM_OK;
}

// ----------------------------------------------------------------------------- rotations
// H_n^{m'm}(beta) of the reference (rotMatsInit + sparseRotMatGen, translation.cu:1064-1237)
// evaluated from Wigner's d^n_{m'm}(beta) with the stable three-term recurrence in degree:
//   j sqrt(((j+1)^2-m^2)((j+1)^2-m'^2)) d^{j+1} = (2j+1)(j(j+1)cos b - m m') d^j
//                                               - (j+1) sqrt((j^2-m^2)(j^2-m'^2)) d^{j-1},
// started at j0 = max(|m|,|m'|) from the one-term Wigner sum, and
//   H = (-1)^{max(m',0)} (-1)^{max(-m,0)} d.
// The reference's recurrence over m loses orthogonality in FP64 beyond p ~ 15.
__device__ double wigner_start(int j, int mp, int m, double c, double s)
{
    int mu, sgn = 1;
    if (m == j) mu = mp;
    else if (mp == j) { mu = m; if ((m - j) & 1) sgn = -1; }
    else if (m == -j) { mu = -mp; if ((-mp - j) & 1) sgn = -1; }
    else mu = -m;
    double binom = 1.0;
    for (int i = 1; i <= j - mu; i++) binom = binom * (double)(j + mu + i) / (double)i;
    double v = sqrt(binom);
    for (int i = 0; i < j + mu; i++) v *= c;
    for (int i = 0; i < j - mu; i++) v *= s;
    return sgn * v;
}

__global__ void wigner_H_kernel(const double *betas, int p, double *H)
{
    int dir = blockIdx.y;
    double beta = betas[dir];
    double c = cos(0.5 * beta), s = sin(0.5 * beta), cb = cos(beta);
    int w = 2 * p - 1, npair = w * w, rs = rot_size(p);
    double *Hd = H + (size_t)dir * rs;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < npair; t += gridDim.x * blockDim.x) {
        int mp = t / w - (p - 1), m = t % w - (p - 1);
        int amp = mp < 0 ? -mp : mp, am = m < 0 ? -m : m;
        int j0 = amp > am ? amp : am;
        double sign = ((((mp > 0) ? mp : 0) + ((m < 0) ? -m : 0)) & 1) ? -1.0 : 1.0;
        double dprev = 0.0, dcur = wigner_start(j0, mp, m, c, s);
        Hd[rot_off(j0) + (mp + j0) + (m + j0) * (2 * j0 + 1)] = sign * dcur;
        for (int j = j0; j + 1 < p; j++) {
            double dn;
            if (j == 0) {
                dn = cb * dcur;
            } else {
                double a = j * sqrt(((j + 1.0) * (j + 1.0) - (double)m * m) * ((j + 1.0) * (j + 1.0) - (double)mp * mp));
                double b = (2.0 * j + 1.0) * (j * (j + 1.0) * cb - (double)m * mp);
                double cc = (j + 1.0) * sqrt(((double)j * j - (double)m * m) * ((double)j * j - (double)mp * mp));
                dn = (b * dcur - cc * dprev) / a;
            }
            dprev = dcur;
            dcur = dn;
            Hd[rot_off(j + 1) + (mp + j + 1) + (m + j + 1) * (2 * j + 3)] = sign * dcur;
        }
    }
}

__global__ void phase_kernel(const double *phis, int ndir, int p, double2 *PH)
{
    int w = 2 * p - 1;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ndir * w; t += gridDim.x * blockDim.x) {
        int dir = t / w, m = t % w - (p - 1);
        double s, c;
        sincos(m * phis[dir], &s, &c);
        PH[t] = make_double2(c, s);
    }
}

__global__ void to_float_kernel(const double *in, float *out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

// FP32 copy of an [rows][p^2] table with entry (n, m) times d[n]
__global__ void to_float_degree_kernel(const double2 *in, float2 *out, size_t n, int p, const double *d)
{
    const int pp = p * p;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        int nm = (int)(i % pp), q = (int)sqrtf((float)nm);
        while (q * q > nm) q--;
        while ((q + 1) * (q + 1) <= nm) q++;
        double2 v = in[i];
        out[i] = make_float2((float)(v.x * d[q]), (float)(v.y * d[q]));
    }
}

static void to_float(const double *in, float *out, size_t n, cudaStream_t s)
{
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    if (blocks < 1) blocks = 1;
    to_float_kernel<<<blocks, 256, 0, s>>>(in, out, n);
}

int gen_rotation_tables(Plan *P)
{
    int p = P->pmax, rs = rot_size(p), w = 2 * p - 1;
    std::vector<double> beta_sr(NDIR), phi_sr(NDIR), beta_ss(8), phi_ss(8), beta_rr(8), phi_rr(8);
    int idx = 0;
    std::vector<int> polar_key(NDIR);  // (dz, dx^2 + dy^2) of each direction
    for (int s = 0; s < 343; s++) {
        int dx = s / 49 - 3, dy = (s / 7) % 7 - 3, dz = s % 7 - 3;
        if (std::abs(dx) <= 1 && std::abs(dy) <= 1 && std::abs(dz) <= 1) { P->dir_slot[s] = -1; continue; }
        double r = sqrt((double)(dx * dx + dy * dy + dz * dz));
        beta_sr[idx] = acos(dz / r);
        phi_sr[idx] = atan2((double)dy, (double)dx);
        int s2 = dx * dx + dy * dy + dz * dz;
        static const int s2list[NDIST] = {4, 5, 6, 8, 9, 10, 11, 12, 13, 14, 17, 18, 19, 22, 27};
        int slot = -1;
        for (int q = 0; q < NDIST; q++) if (s2list[q] == s2) slot = q;
        P->dir_dist[idx] = slot;
        // directions of equal dz and dx^2 + dy^2 have the same polar angle, so bit-identical
        // rotation tables: all of them read the first one's, which keeps the tables in cache
        P->dir_hrep[idx] = idx;
        for (int q = 0; q < idx; q++)
            if (polar_key[q] == (dz + 8) * 100 + dx * dx + dy * dy) { P->dir_hrep[idx] = q; break; }
        polar_key[idx] = (dz + 8) * 100 + dx * dx + dy * dy;
        P->dir_slot[s] = idx++;
    }
    for (int o = 0; o < 8; o++) {
        double t[3] = {0.5 - ((o >> 2) & 1), 0.5 - ((o >> 1) & 1), 0.5 - (o & 1)};
        double r = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        beta_ss[o] = acos(t[2] / r);  // M2M: parent - child
        phi_ss[o] = atan2(t[1], t[0]);
        beta_rr[o] = acos(-t[2] / r); // L2L: child - parent
        phi_rr[o] = atan2(-t[1], -t[0]);
    }
    double *dtmp = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&dtmp, sizeof(double) * (NDIR + 16) * 2));
    std::vector<double> ball(NDIR + 16), pall(NDIR + 16);
    for (int i = 0; i < NDIR; i++) { ball[i] = beta_sr[i]; pall[i] = phi_sr[i]; }
    for (int o = 0; o < 8; o++) {
        ball[NDIR + o] = beta_ss[o]; pall[NDIR + o] = phi_ss[o];
        ball[NDIR + 8 + o] = beta_rr[o]; pall[NDIR + 8 + o] = phi_rr[o];
    }
    FMM_CUDA_TRY(cudaMemcpy(dtmp, ball.data(), sizeof(double) * (NDIR + 16), cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(dtmp + NDIR + 16, pall.data(), sizeof(double) * (NDIR + 16), cudaMemcpyHostToDevice));
    double *Hall = nullptr;
    double2 *PHall = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&Hall, sizeof(double) * (size_t)(NDIR + 16) * rs));
    FMM_CUDA_TRY(cudaMalloc(&PHall, sizeof(double2) * (size_t)(NDIR + 16) * w));
    dim3 grid((w * w + 255) / 256, NDIR + 16);
    wigner_H_kernel<<<grid, 256, 0, P->stream>>>(dtmp, p, Hall);
    phase_kernel<<<((NDIR + 16) * w + 255) / 256, 256, 0, P->stream>>>(dtmp + NDIR + 16, NDIR + 16, p, PHall);
    FMM_CUDA_TRY(cudaGetLastError());
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    // split into the three families (views into one allocation)
    P->Hsr64 = Hall;
    P->Hss64 = Hall + (size_t)NDIR * rs;
    P->Hrr64 = Hall + (size_t)(NDIR + 8) * rs;
    P->PHsr64 = PHall;
    P->PHss64 = PHall + (size_t)NDIR * w;
    P->PHrr64 = PHall + (size_t)(NDIR + 8) * w;
    P->device_bytes += sizeof(double) * (size_t)(NDIR + 16) * rs + sizeof(double2) * (size_t)(NDIR + 16) * w;
    if (P->opt.build_mixed) {
        float *H32 = nullptr;
        float2 *PH32 = nullptr;
        FMM_CUDA_TRY(cudaMalloc(&H32, sizeof(float) * (size_t)(NDIR + 16) * rs));
        FMM_CUDA_TRY(cudaMalloc(&PH32, sizeof(float2) * (size_t)(NDIR + 16) * w));
        to_float(Hall, H32, (size_t)(NDIR + 16) * rs, P->stream);
        to_float((const double *)PHall, (float *)PH32, (size_t)(NDIR + 16) * w * 2, P->stream);
        P->Hsr32 = H32;
        P->Hss32 = H32 + (size_t)NDIR * rs;
        P->Hrr32 = H32 + (size_t)(NDIR + 8) * rs;
        P->PHsr32 = PH32;
        P->PHss32 = PH32 + (size_t)NDIR * w;
        P->PHrr32 = PH32 + (size_t)(NDIR + 8) * w;
        P->device_bytes += sizeof(float) * (size_t)(NDIR + 16) * rs + sizeof(float2) * (size_t)(NDIR + 16) * w;
    }
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    cudaFree(dtmp);
    return FMM_OK;
}

// Complex rotation matrices e^{i m alpha} e^{-i m' gamma} H_n^{m'm}(beta) in FP32, the
// sparse layout of sparseRotMatGen (translation.cu:1221-1235).
__global__ void assemble_rot_kernel(const double *H, const double *alpha, const double *gamma, int p, float2 *out)
{
    int a = blockIdx.y, rs = rot_size(p);
    const double *Ha = H + (size_t)a * rs;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rs; i += gridDim.x * blockDim.x) {
        int n = 0;
        while (rot_off(n + 1) <= i) n++;
        int loc = i - rot_off(n), w = 2 * n + 1;
        int mp = loc % w - n, m = loc / w - n;
        double s, c;
        sincos(m * alpha[a] - mp * gamma[a], &s, &c);
        out[(size_t)a * rs + i] = make_float2((float)(c * Ha[i]), (float)(s * Ha[i]));
    }
}

int gen_rotation_matrices_f32(const double *alpha, const double *beta, const double *gamma, int n, int p, float2 *host_out)
{
    if (n <= 0) return FMM_OK;
    int rs = rot_size(p), w = 2 * p - 1;
    double *d = nullptr, *H = nullptr;
    float2 *o = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&d, sizeof(double) * 3 * n));
    FMM_CUDA_TRY(cudaMalloc(&H, sizeof(double) * (size_t)n * rs));
    FMM_CUDA_TRY(cudaMalloc(&o, sizeof(float2) * (size_t)n * rs));
    FMM_CUDA_TRY(cudaMemcpy(d, alpha, sizeof(double) * n, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(d + n, beta, sizeof(double) * n, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(d + 2 * n, gamma, sizeof(double) * n, cudaMemcpyHostToDevice));
    wigner_H_kernel<<<dim3((w * w + 255) / 256, n), 256>>>(d + n, p, H);
    assemble_rot_kernel<<<dim3((rs + 255) / 256, n), 256>>>(H, d, d + 2 * n, p, o);
    FMM_CUDA_TRY(cudaGetLastError());
    FMM_CUDA_TRY(cudaMemcpy(host_out, o, sizeof(float2) * (size_t)n * rs, cudaMemcpyDeviceToHost));
    cudaFree(d); cudaFree(H); cudaFree(o);
    return FMM_OK;
}

// ----------------------------------------------------------------------------- coaxial
// (S|R) or (R|R) coaxial blocks for translation length t along z (coax_recurrence.cuh:
// sparseCoaxTransMatGen, translation.cu:678-771, in FP64).  One CTA per matrix; the
// enlarged matrix E[m][n'][n] lives in a global scratch slice.
__global__ void coax_kernel(double k, const double *tvals, int p, int sr, double2 *scratch, double2 *out)
{
    int mat = blockIdx.x;
    extern __shared__ double sh[];
    coax_matrix_cta(k * tvals[mat], p, sr, scratch + (size_t)mat * p * (2 * p - 1) * p, out + (size_t)mat * coax_size(p),
                    sh, sh + 2 * p - 1);
}

// The mixed-precision path stores the coaxial blocks in FP32.  At high order and small k t
// the (S|R) entries grow like h_{2p-2}(k t) (and the multipole coefficients fall like
// (k r)^n / (2n+1)!!) beyond the float range.  Such plans keep their FP32 expansions scaled
// by degree: multipoles of level l as d_n M_n, locals as L_n / d_n, with d_n the square root
// of the largest diagonal (S|R) entry of degree n at that level.  The scaling commutes with
// the rotations (block-diagonal in n), so only the coaxial blocks (scaled (S|R):
// C / (d_n' d_n); M2M: d^{l-1}_n' C / d^l_n; L2L: d^{l-1}_n C / d^l_n') and the element
// tables (both times d^{lmax}_n) change; the kernels do not.  The scaled blocks are near
// one in size, the expansions of order one.  Plans whose largest unscaled entry stays below
// 1e20 keep the plain tables.
static const double SCALE_ABOVE = 1e20;

static double max_abs(const std::vector<double2> &h)
{
    double mx = 0.0;
    for (const double2 &v : h) {
        double a = std::max(fabs(v.x), fabs(v.y));
        if (!(a <= mx)) mx = a; // NaN propagates
    }
    return mx;
}

// FP32 copy of coaxial blocks of order p for nmat matrices: entry (n', n) of block m times
// row[n'] * col[n]
static std::vector<float2> scaled_coax(const std::vector<double2> &in, int p, int nmat, const std::vector<double> &row,
                                       const std::vector<double> &col, double *maxout)
{
    std::vector<float2> out(in.size());
    double mx = 0.0;
    const int cs = coax_size(p);
    for (int q = 0; q < nmat; q++)
        for (int m = 0; m < p; m++) {
            int sz = p - m, off = q * cs + coax_off(p, m);
            for (int i = 0; i < sz * sz; i++) {
                int a = i % sz, b = i / sz; // a = n' - m, b = n - m
                double f = row[m + a] * col[m + b];
                double2 v = in[off + i];
                double x = v.x * f, y = v.y * f;
                double av = std::max(fabs(x), fabs(y));
                if (!(av <= mx)) mx = av;
                out[off + i] = make_float2((float)x, (float)y);
            }
        }
    *maxout = mx;
    return out;
}

int gen_coax_tables(Plan *P)
{
    double k = P->opt.k;
    static const int s2list[NDIST] = {4, 5, 6, 8, 9, 10, 11, 12, 13, 14, 17, 18, 19, 22, 27};
    size_t maxScratch = 0;
    for (int l = P->lmin; l <= P->lmax; l++) {
        int p = P->lev[l].p;
        maxScratch = std::max(maxScratch, (size_t)NDIST * p * (2 * p - 1) * p);
        if (l > P->lmin) {
            int pp = P->lev[l - 1].p;
            maxScratch = std::max(maxScratch, (size_t)pp * (2 * pp - 1) * pp);
        }
    }
    double2 *scratch = nullptr;
    double *tdev = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&scratch, sizeof(double2) * maxScratch));
    FMM_CUDA_TRY(cudaMalloc(&tdev, sizeof(double) * NDIST));
    // FP64 blocks of every level (host copies kept for the FP32 conversion)
    std::vector<double2> hsr[FMM_MAX_LEVEL + 2], hrr[FMM_MAX_LEVEL + 2];
    double unscaled_max = 0.0;
    int worst_level = P->lmin;
    for (int l = P->lmin; l <= P->lmax; l++) {
        LevelDev &L = P->lev[l];
        int p = L.p;
        double size = P->tree.d * ldexp(1.0, -l);
        double tv[NDIST];
        for (int q = 0; q < NDIST; q++) tv[q] = sqrt((double)s2list[q]) * size;
        FMM_CUDA_TRY(cudaMemcpy(tdev, tv, sizeof(tv), cudaMemcpyHostToDevice));
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Csr64, sizeof(double2) * NDIST * coax_size(p)));
        coax_kernel<<<NDIST, 256, sizeof(double) * 2 * (2 * p - 1), P->stream>>>(k, tdev, p, 1, scratch, L.Csr64);
        FMM_CUDA_TRY(cudaGetLastError());
        FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
        if (P->opt.build_mixed) {
            hsr[l].resize((size_t)NDIST * coax_size(p));
            FMM_CUDA_TRY(cudaMemcpy(hsr[l].data(), L.Csr64, sizeof(double2) * hsr[l].size(), cudaMemcpyDeviceToHost));
            double mx = max_abs(hsr[l]);
            if (!(mx <= unscaled_max)) { unscaled_max = mx; worst_level = l; }
        }
        if (l > P->lmin) {
            int pp = P->lev[l - 1].p;
            double trr = 0.5 * sqrt(3.0) * size;
            FMM_CUDA_TRY(cudaMemcpy(tdev, &trr, sizeof(double), cudaMemcpyHostToDevice));
            FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Crr64, sizeof(double2) * coax_size(pp)));
            coax_kernel<<<1, 256, sizeof(double) * 2 * (2 * pp - 1), P->stream>>>(k, tdev, pp, 0, scratch, L.Crr64);
            FMM_CUDA_TRY(cudaGetLastError());
            FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
            if (P->opt.build_mixed) {
                hrr[l].resize(coax_size(pp));
                FMM_CUDA_TRY(cudaMemcpy(hrr[l].data(), L.Crr64, sizeof(double2) * hrr[l].size(), cudaMemcpyDeviceToHost));
                double mx = max_abs(hrr[l]);
                if (!(mx <= unscaled_max)) { unscaled_max = mx; worst_level = l; }
            }
        }
    }
    cudaFree(scratch);
    cudaFree(tdev);
    if (!P->opt.build_mixed) return FMM_OK;
    if (!std::isfinite(unscaled_max)) {
        P->opt.build_mixed = 0;
        snprintf(P->mixed_note, sizeof(P->mixed_note), "no mixed-precision tables: level %d coaxial entries are not finite",
                 worst_level);
        return FMM_OK;
    }
    P->scaled = unscaled_max >= SCALE_ABOVE;
    int pall = 0;
    for (int l = P->lmin; l <= P->lmax; l++) pall = std::max(pall, P->lev[l].p);
    // d^l_n for n < p_l (1 elsewhere, and for unscaled plans)
    for (int l = P->lmin; l <= P->lmax; l++) {
        int p = P->lev[l].p, cs = coax_size(p);
        P->dsc[l].assign(pall, 1.0);
        if (!P->scaled) continue;
        for (int n = 0; n < p; n++) {
            double mx = 0.0;
            for (int q = 0; q < NDIST; q++)
                for (int m = 0; m <= n; m++) {
                    int sz = p - m;
                    double2 v = hsr[l][(size_t)q * cs + coax_off(p, m) + (size_t)(n - m) * sz + (n - m)];
                    mx = std::max(mx, hypot(v.x, v.y));
                }
            P->dsc[l][n] = mx > 0.0 && std::isfinite(mx) ? sqrt(mx) : 1.0;
        }
    }
    double scaled_max = 0.0;
    std::vector<double> ones(pall, 1.0);
    for (int l = P->lmin; l <= P->lmax; l++) {
        LevelDev &L = P->lev[l];
        int p = L.p;
        std::vector<double> inv(pall, 1.0);
        for (int n = 0; n < pall; n++) inv[n] = 1.0 / P->dsc[l][n];
        double mx;
        std::vector<float2> f = scaled_coax(hsr[l], p, NDIST, inv, inv, &mx);
        scaled_max = std::max(scaled_max, mx);
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Csr32, sizeof(float2) * f.size()));
        FMM_CUDA_TRY(cudaMemcpy(L.Csr32, f.data(), sizeof(float2) * f.size(), cudaMemcpyHostToDevice));
        if (l > P->lmin) {
            int pp = P->lev[l - 1].p;
            // M2M: rows are parent degrees (times d^{l-1}), columns child degrees (over d^l; zero
            // beyond the child's order, whose sources are zero padding); L2L the other way round
            // (rows beyond the child's order are never read).  Unscaled plans share one plain table.
            std::vector<double> up_col(pall, P->scaled ? 0.0 : 1.0), down_row(pall, 0.0);
            for (int n = 0; n < p && n < pall; n++) up_col[n] = down_row[n] = inv[n];
            f = scaled_coax(hrr[l], pp, 1, P->dsc[l - 1], up_col, &mx);
            scaled_max = std::max(scaled_max, mx);
            FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Crr32, sizeof(float2) * f.size()));
            FMM_CUDA_TRY(cudaMemcpy(L.Crr32, f.data(), sizeof(float2) * f.size(), cudaMemcpyHostToDevice));
            if (P->scaled) {
                f = scaled_coax(hrr[l], pp, 1, down_row, P->dsc[l - 1], &mx);
                scaled_max = std::max(scaled_max, mx);
                FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Crr32L, sizeof(float2) * f.size()));
                FMM_CUDA_TRY(cudaMemcpy(L.Crr32L, f.data(), sizeof(float2) * f.size(), cudaMemcpyHostToDevice));
            }
        }
    }
    if (!(scaled_max < 1e37)) {
        P->opt.build_mixed = 0;
        snprintf(P->mixed_note, sizeof(P->mixed_note),
                 "no mixed-precision tables: coaxial entries reach %.3g%s, beyond FP32 range (lower p or use FMM_FP64)",
                 scaled_max, P->scaled ? " after scaling" : "");
    }
    return FMM_OK;
}

// FP32 sparse coaxial matrices for n translation lengths (the output of
// genRR/SRSparseCoaxTransMat, translation.cu:822-1062), generated in FP64.
int gen_coax_matrices_f32(double k, const double *t, int n, int p, int sr, float2 *host_out)
{
    if (n <= 0) return FMM_OK;
    int cs = coax_size(p);
    double2 *scratch = nullptr, *o = nullptr;
    double *td = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&scratch, sizeof(double2) * (size_t)n * p * (2 * p - 1) * p));
    FMM_CUDA_TRY(cudaMalloc(&o, sizeof(double2) * (size_t)n * cs));
    FMM_CUDA_TRY(cudaMalloc(&td, sizeof(double) * n));
    FMM_CUDA_TRY(cudaMemcpy(td, t, sizeof(double) * n, cudaMemcpyHostToDevice));
    coax_kernel<<<n, 256, sizeof(double) * 2 * (2 * p - 1)>>>(k, td, p, sr, scratch, o);
    FMM_CUDA_TRY(cudaGetLastError());
    std::vector<double2> h((size_t)n * cs);
    FMM_CUDA_TRY(cudaMemcpy(h.data(), o, sizeof(double2) * h.size(), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < h.size(); i++) host_out[i] = make_float2((float)h[i].x, (float)h[i].y);
    cudaFree(scratch); cudaFree(o); cudaFree(td);
    return FMM_OK;
}

// ----------------------------------------------------------------------------- geometry
__device__ __forceinline__ void load_tri(const double *V, const int *F, int e, double *nod)
{
    for (int t = 0; t < 3; t++) {
        int v = F[3 * e + t];
        nod[3 * t] = V[3 * v]; nod[3 * t + 1] = V[3 * v + 1]; nod[3 * t + 2] = V[3 * v + 2];
    }
}
__device__ __forceinline__ void tri_centroid(const double *nod, double *y)
{
    for (int a = 0; a < 3; a++) {
        double c23 = 0.5 * (nod[3 + a] + nod[6 + a]);
        y[a] = nod[a] + (2.0 / 3.0) * (c23 - nod[a]);
    }
}
__device__ __forceinline__ double tri_normal(const double *nod, double *nh)
{
    double u0 = nod[0] - nod[6], u1 = nod[1] - nod[7], u2 = nod[2] - nod[8];
    double v0 = nod[3] - nod[6], v1 = nod[4] - nod[7], v2 = nod[5] - nod[8];
    double n0 = u1 * v2 - u2 * v1, n1 = u2 * v0 - u0 * v2, n2 = u0 * v1 - u1 * v0;
    double J = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    nh[0] = n0 / J; nh[1] = n1 / J; nh[2] = n2 / J;
    return J;
}

// G = exp(ikr)/(4 pi r) (integral.cu:72-78) and dG/dn_x (integral.cu:391-402)
__device__ __forceinline__ double2 green_k(double k, const double *x, const double *y, const double *nh, int kern)
{
    double d0 = x[0] - y[0], d1 = x[1] - y[1], d2 = x[2] - y[2];
    double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    double s, c;
    sincos(k * r, &s, &c);
    double inv = 1.0 / (4.0 * FMM_PI * r);
    double gr = c * inv, gi = s * inv;
    if (!kern) return make_double2(gr, gi);
    double dn = (d0 * nh[0] + d1 * nh[1] + d2 * nh[2]) / r;
    // g * (-1/r + i k) * dn
    double ar = -1.0 / r, ai = k;
    return make_double2((gr * ar - gi * ai) * dn, (gr * ai + gi * ar) * dn);
}

__device__ double2 elem_integral(double k, const double *nod, const double *y, int rule, int kern)
{
    double nh[3];
    double J = tri_normal(nod, nh);
    double2 acc = make_double2(0.0, 0.0);
    int nq = c_rule_n[rule];
    for (int q = 0; q < nq; q++) {
        const double *b = &c_rule_bary[rule][3 * q];
        double x[3];
        for (int a = 0; a < 3; a++) x[a] = nod[a] * b[0] + nod[3 + a] * b[1] + nod[6 + a] * b[2];
        double2 g = green_k(k, x, y, nh, kern);
        double wq = c_rule_w[rule][q] * J;
        acc.x += wq * g.x; acc.y += wq * g.y;
    }
    return acc;
}

__device__ double2 elem_integral_sgl(double k, const double *nod, int kern)
{
    double y[3];
    tri_centroid(nod, y);
    double2 acc = make_double2(0.0, 0.0);
    for (int s = 0; s < 3; s++) {
        double sub[9];
        int a0 = 3 * s, b0 = 3 * ((s + 1) % 3);
        for (int t = 0; t < 3; t++) { sub[t] = nod[a0 + t]; sub[3 + t] = nod[b0 + t]; sub[6 + t] = y[t]; }
        double2 part = elem_integral(k, sub, y, 0, kern);
        acc.x += part.x; acc.y += part.y;
    }
    return acc;
}

// ----------------------------------------------------------------------------- Burton-Miller terms
// The combined operator adds alpha d/dn_y (b L + c M) at the collocation point y (unit normal
// ny): alpha (b K' + c N).  K' integrates dG/dn_y (pGp2n, integral.cu:400-413); N integrates
// d2G/dn_x dn_y (p2Gp1np2n, integral.cu:603-622), taken here in forms that stay accurate for
// the near pairs: the regularised (Maue) form off the element and the polar finite part on it.

// K' = int_T dG(x, y)/dn_y dS_x = int_T G (ik - 1/r) (y - x).ny / r (zero on the flat element
// itself) is taken with the other regular integrals in elem_integrals_fused.

// number of equal segments of an edge of length len seen from distance dist: no longer than
// dist, so that the 8-point rule converges like 4.2^-16 on the 1/r^2 and 1/r^3 integrands
__device__ __forceinline__ int edge_segments(double len, double dist)
{
    double m = ceil(len / fmax(dist, 1e-12 * len));
    return m > 64.0 ? 64 : (int)m;
}

// Hadamard finite part of int_T d2G/dn_x dn_y at the centroid c of the flat element T:
//   -1/(4 pi) [ int_0^{2 pi} e^{ik rho(theta)}/rho(theta) dtheta - 2 pi i k ]
// (integral.cu:738-751 with the angle integral taken accurately): along edge e, at distance
// h_e from c and of length L_e, dtheta = h_e L_e / rho^3 ds for s in [0, 1].
__device__ double2 elem_hyper_self(double k, const double *nod)
{
    double c[3];
    tri_centroid(nod, c);
    double sr = 0.0, si = 0.0;
    for (int e = 0; e < 3; e++) {
        const double *va = nod + 3 * e, *vb = nod + 3 * ((e + 1) % 3);
        double t[3] = {vb[0] - va[0], vb[1] - va[1], vb[2] - va[2]}, u[3] = {va[0] - c[0], va[1] - c[1], va[2] - c[2]};
        double c0 = u[1] * t[2] - u[2] * t[1], c1 = u[2] * t[0] - u[0] * t[2], c2 = u[0] * t[1] - u[1] * t[0];
        double hL = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
        double len = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        int nseg = edge_segments(len, hL / len);
        for (int g = 0; g < nseg; g++)
            for (int q = 0; q < LINE_PTS; q++) {
                double s = (g + 0.5 + 0.5 * c_line_x[q]) / nseg, w = 0.5 * c_line_w[q] / nseg;
                double d0 = u[0] + s * t[0], d1 = u[1] + s * t[1], d2 = u[2] + s * t[2];
                double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                double sn, cs;
                sincos(k * r, &sn, &cs);
                double f = w * hL / (r * r * r);
                sr += f * cs; si += f * sn;
            }
    }
    return make_double2(-sr / (4.0 * FMM_PI), (2.0 * FMM_PI * k - si) / (4.0 * FMM_PI));
}

// int_T d2G/dn_x dn_y dS_x at y off T (unit normal ny), regularised (Maue):
//   k^2 (ny.nT) int_T G dS  -  oint_{dT} (ny x grad_y G) . dl,
// the boundary traversed v0 -> v1 -> v2 (counter-clockwise about nT); grad_y G =
// G (ik - 1/r) (y - x)/r.  The edge integrals are regular for y off the element; this is the
// boundary term (the surface term uses int G from elem_integrals_fused).
__device__ double2 hyper_edges(double k, const double *nod, const double *y, const double *ny)
{
    double lr = 0.0, li = 0.0;
    for (int e = 0; e < 3; e++) {
        const double *va = nod + 3 * e, *vb = nod + 3 * ((e + 1) % 3);
        double t[3] = {vb[0] - va[0], vb[1] - va[1], vb[2] - va[2]}, a[3] = {y[0] - va[0], y[1] - va[1], y[2] - va[2]};
        double tt = t[0] * t[0] + t[1] * t[1] + t[2] * t[2], len = sqrt(tt);
        double sc = fmin(fmax((a[0] * t[0] + a[1] * t[1] + a[2] * t[2]) / tt, 0.0), 1.0);
        double e0 = a[0] - sc * t[0], e1 = a[1] - sc * t[1], e2 = a[2] - sc * t[2];
        int nseg = edge_segments(len, sqrt(e0 * e0 + e1 * e1 + e2 * e2));
        // (ny x d) . t = d . (t x ny), d = y - x
        double tn0 = t[1] * ny[2] - t[2] * ny[1], tn1 = t[2] * ny[0] - t[0] * ny[2], tn2 = t[0] * ny[1] - t[1] * ny[0];
        for (int g = 0; g < nseg; g++)
            for (int q = 0; q < LINE_PTS; q++) {
                double s = (g + 0.5 + 0.5 * c_line_x[q]) / nseg, w = 0.5 * c_line_w[q] / nseg;
                double d0 = a[0] - s * t[0], d1 = a[1] - s * t[1], d2 = a[2] - s * t[2];
                double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                double sn, cs;
                sincos(k * r, &sn, &cs);
                double f = w * (d0 * tn0 + d1 * tn1 + d2 * tn2) / (4.0 * FMM_PI * r * r);
                // G (ik - 1/r) = e^{ikr}/(4 pi r) (ik - 1/r); times f r = w (.)/(4 pi r)
                double gr = cs, gi = sn, ar = -1.0 / r, ai = k;
                lr += f * (gr * ar - gi * ai);
                li += f * (gr * ai + gi * ar);
            }
    }
    return make_double2(lr, li);
}

// The regular-rule integrals of one source element at an off-element collocation point y
// (unit normal ny) in one pass over the quadrature points, each with the arithmetic and
// summation order of its own routine: G -> int G (elem_integral kern 0), dGx -> int dG/dn_x
// (kern 1), dGy -> int dG/dn_y (elem_dGdny), each only where its flag is set; nT the
// element's unit normal.
__device__ void elem_integrals_fused(double k, const double *nod, const double *y, const double *ny, int rule,
                                     bool wG, bool wx, bool wy, double2 &G, double2 &dGx, double2 &dGy, double *nT)
{
    const double J = tri_normal(nod, nT);
    G = dGx = dGy = make_double2(0.0, 0.0);
    const int nq = c_rule_n[rule];
    for (int q = 0; q < nq; q++) {
        const double *b = &c_rule_bary[rule][3 * q];
        double x[3];
        for (int a = 0; a < 3; a++) x[a] = nod[a] * b[0] + nod[3 + a] * b[1] + nod[6 + a] * b[2];
        double d0 = x[0] - y[0], d1 = x[1] - y[1], d2 = x[2] - y[2];
        double r = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        double sn, cs;
        sincos(k * r, &sn, &cs);
        double inv = 1.0 / (4.0 * FMM_PI * r);
        double gr = cs * inv, gi = sn * inv, ar = -1.0 / r, ai = k;
        double wq = c_rule_w[rule][q] * J;
        if (wG) { G.x += wq * gr; G.y += wq * gi; }
        if (wx) {
            double dn = (d0 * nT[0] + d1 * nT[1] + d2 * nT[2]) / r;
            double2 g = make_double2((gr * ar - gi * ai) * dn, (gr * ai + gi * ar) * dn);
            dGx.x += wq * g.x; dGx.y += wq * g.y;
        }
        if (wy) {
            double dn = (d0 * ny[0] + d1 * ny[1] + d2 * ny[2]) / r;
            double2 g = make_double2((gr * ar - gi * ai) * dn, (gr * ai + gi * ar) * dn);
            dGy.x -= wq * g.x; dGy.y -= wq * g.y;
        }
    }
}

// ----------------------------------------------------------------------------- element tables
// U_e[n,m] = b int R_n^{-m}(x - c) dS + c int dR_n^{-m}/dn dS   (integral.cu:251-365, the P2M
// moments of bottomLevelCoeff_L with its loop corrected), Rv_e[n,m] = R_n^m(y_e - c) (L2P).
// One warp per element; the basis at each quadrature point is staged in shared memory.
struct BasisSh {
    double *jn, *Q;
    double2 *ph;
};

// Factors of the basis recurrences that depend only on (n, m), tabulated on the host with the
// same expressions (FP64 square roots and divisions are slow on this GPU; the results are the
// same to the bit): fac[i] = sqrt((2i+1)/(2i)), s3[m] = sqrt(2m+3), la/lb the three-term
// Legendre coefficients at n(n+1)/2 + m, and coefA(n, m) / coefB(n, m) at
// (n + 1) W + m + pb + 1 for n = -1..pb, |m| <= pb + 1 (W = 2 pb + 3).
struct BasisTab {
    const double *fac, *s3, *la, *lb, *cA, *cB;
    int W, pb;
};

__device__ __forceinline__ double tabA(const BasisTab &T, int n, int m) { return T.cA[(n + 1) * T.W + m + T.pb + 1]; }
__device__ __forceinline__ double tabB(const BasisTab &T, int n, int m) { return T.cB[(n + 1) * T.W + m + T.pb + 1]; }

__device__ __forceinline__ double2 basis_R(const BasisSh &B, int pb, int n, int m)
{
    // R_n^m = j_n Q_n^{|m|} e^{i m phi}; zero outside the valid range
    if (n < 0 || n >= pb) return make_double2(0.0, 0.0);
    int am = m < 0 ? -m : m;
    if (am > n) return make_double2(0.0, 0.0);
    double v = B.jn[n] * B.Q[n * (n + 1) / 2 + am];
    double2 e = B.ph[m + pb];
    return make_double2(v * e.x, v * e.y);
}

// The basis of order pb at v, spread over the warp: lane 0 runs the spherical Bessel
// recurrence, lane m (and m + 32) the Legendre column m (its diagonal entry as a product, then
// the same three-term recurrence in n as legendre_Q), every lane a few phases.
__device__ __forceinline__ void basis_prepare(const BasisSh &B, const BasisTab &T, int pb, double k, const double *v,
                                              int lane)
{
    double r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    double ct = 1.0, phi = 0.0;
    if (r > 0.0) { ct = v[2] / r; phi = atan2(v[1], v[0]); }
    if (lane == 0) sph_jn_array(pb, k * r, B.jn);
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    for (int m = lane; m < pb; m += 32) {
        double q = 0.28209479177387814; // 1/sqrt(4 pi)
        for (int i = 1; i <= m; i++) q = __ldg(T.fac + i) * st * q;
        B.Q[m * (m + 1) / 2 + m] = q;
        if (m + 1 < pb) {
            double q1 = __ldg(T.s3 + m) * ct * q, q0 = q;
            B.Q[(m + 1) * (m + 2) / 2 + m] = q1;
            for (int n = m + 2; n < pb; n++) {
                const int ix = n * (n + 1) / 2 + m;
                double a = __ldg(T.la + ix), b = __ldg(T.lb + ix);
                double q2 = a * (ct * q1 - b * q0);
                B.Q[n * (n + 1) / 2 + m] = q2;
                q0 = q1;
                q1 = q2;
            }
        }
    }
    for (int m = lane - pb; m <= pb; m += 32) {
        double s, c;
        sincos(m * phi, &s, &c);
        B.ph[m + pb] = make_double2(c, s);
    }
    __syncwarp();
}

// nh . grad R_n^m from the staged basis of orders up to n+1 (integral.cu:284-331)
__device__ __forceinline__ double2 basis_dirdev(const BasisSh &B, const BasisTab &T, int pb, double k, int n, int mm,
                                                const double *nh)
{
    double2 t0 = csub(cscale(basis_R(B, pb, n + 1, mm + 1), tabB(T, n + 1, -(mm + 1))),
                      cscale(basis_R(B, pb, n - 1, mm + 1), tabB(T, n, mm)));
    double2 t1 = csub(cscale(basis_R(B, pb, n + 1, mm - 1), tabB(T, n + 1, mm - 1)),
                      cscale(basis_R(B, pb, n - 1, mm - 1), tabB(T, n, -mm)));
    double2 t2 = csub(cscale(basis_R(B, pb, n - 1, mm), tabA(T, n - 1, mm)),
                      cscale(basis_R(B, pb, n + 1, mm), tabA(T, n, mm)));
    double2 f0 = make_double2(0.5 * k * nh[0], -0.5 * k * nh[1]);
    double2 f1 = make_double2(0.5 * k * nh[0], 0.5 * k * nh[1]);
    return cadd(cadd(cmul(f0, t0), cmul(f1, t1)), cscale(t2, k * nh[2]));
}

// per-warp shared memory (in doubles) of the element-table kernel: j_n and Q, padded to an
// even count so the double2 phases that follow stay 16-byte aligned, then 2pb+1 phases
__host__ __device__ __forceinline__ int basis_ph_offset(int pb) { return (pb + pb * (pb + 1) / 2 + 1) & ~1; }
__host__ __device__ __forceinline__ int basis_per_warp(int pb) { return basis_ph_offset(pb) + 2 * (2 * pb + 1); }

__global__ void element_tables_kernel(const double *V, const int *F, const int *elem_leaf, const double *box_ctr,
                                      int nf, int pl, double k, double2 bco, double2 cco, double2 alpha,
                                      int rule, BasisTab T, double2 *U, double2 *Rv)
{
    extern __shared__ double2 smem2[];
    double *smem = (double *)smem2;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int pb = pl + 1;
    double *base = smem + (size_t)warp * basis_per_warp(pb);
    BasisSh B;
    B.jn = base;
    B.Q = base + pb;
    B.ph = (double2 *)(base + basis_ph_offset(pb));
    int ppl = pl * pl;
    for (int e = blockIdx.x * nw + warp; e < nf; e += gridDim.x * nw) {
        double nod[9], nh[3], c[3], y[3];
        load_tri(V, F, e, nod);
        double J = tri_normal(nod, nh);
        int b = elem_leaf[e];
        c[0] = box_ctr[3 * b]; c[1] = box_ctr[3 * b + 1]; c[2] = box_ctr[3 * b + 2];
        double2 *Ue = U + (size_t)e * ppl;
        for (int i = lane; i < ppl; i += 32) Ue[i] = make_double2(0.0, 0.0);
        int nq = c_rule_n[rule];
        for (int q = 0; q < nq; q++) {
            const double *bb = &c_rule_bary[rule][3 * q];
            double v[3];
            for (int a = 0; a < 3; a++) v[a] = nod[a] * bb[0] + nod[3 + a] * bb[1] + nod[6 + a] * bb[2] - c[a];
            double wq = c_rule_w[rule][q] * J;
            __syncwarp();
            basis_prepare(B, T, pb, k, v, lane);
            for (int i = lane; i < ppl; i += 32) {
                int n = (int)sqrtf((float)i);
                while (n * n > i) n--;
                while ((n + 1) * (n + 1) <= i) n++;
                int m = i - n * n - n;
                int mm = -m; // moments use R_n^{-m}
                double2 acc = make_double2(0.0, 0.0);
                if (bco.x != 0.0 || bco.y != 0.0) {
                    double2 r = basis_R(B, pb, n, mm);
                    acc = cadd(acc, cmul(bco, r));
                }
                if (cco.x != 0.0 || cco.y != 0.0) {
                    // directional derivative along nh (integral.cu:284-331)
                    acc = cadd(acc, cmul(cco, basis_dirdev(B, T, pb, k, n, mm, nh)));
                }
                Ue[i] = cadd(Ue[i], cscale(acc, wq));
            }
            __syncwarp();
        }
        tri_centroid(nod, y);
        double v[3] = {y[0] - c[0], y[1] - c[1], y[2] - c[2]};
        basis_prepare(B, T, pb, k, v, lane);
        double2 *Re = Rv + (size_t)e * ppl;
        for (int i = lane; i < ppl; i += 32) {
            int n = (int)sqrtf((float)i);
            while (n * n > i) n--;
            while ((n + 1) * (n + 1) <= i) n++;
            int m = i - n * n - n;
            // L2P vector of R + alpha dR/dn at the centroid (Burton-Miller: the target-side
            // normal derivative of the far field)
            double2 r = basis_R(B, pb, n, m);
            if (alpha.x != 0.0 || alpha.y != 0.0) r = cadd(r, cmul(alpha, basis_dirdev(B, T, pb, k, n, m, nh)));
            Re[i] = r;
        }
        __syncwarp();
    }
}

// The element tables of the operator with source coefficients (bco, cco) into U and Rv
// (nf * pleaf^2 entries each), on the plan's stream, synchronised.
static int launch_element_tables(Plan *P, double2 bco, double2 cco, double2 *U, double2 *Rv)
{
    int st = upload_rules();
    if (st != FMM_OK) return st;
    int pl = P->pleaf;
    LevelDev &L = P->lev[P->lmax];
    // leaf box centres: descale(boxCenter) = d (2^-l x + 2^-(l+1)) + pt_min
    std::vector<double> ctr(3 * L.nb);
    double h = ldexp(1.0, -P->lmax), h2 = ldexp(1.0, -P->lmax - 1);
    for (int i = 0; i < L.nb; i++) {
        int x, y, z;
        box_xyz(P->tree.sets[P->lmax][i], P->lmax, &x, &y, &z);
        ctr[3 * i] = P->tree.d * (h * x + h2) + P->tree.pt_min[0];
        ctr[3 * i + 1] = P->tree.d * (h * y + h2) + P->tree.pt_min[1];
        ctr[3 * i + 2] = P->tree.d * (h * z + h2) + P->tree.pt_min[2];
    }
    double *ctr_dev = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&ctr_dev, sizeof(double) * ctr.size()));
    FMM_CUDA_TRY(cudaMemcpy(ctr_dev, ctr.data(), sizeof(double) * ctr.size(), cudaMemcpyHostToDevice));
    int pb = pl + 1;
    int warps = 4;
    size_t shm = (size_t)basis_per_warp(pb) * warps * sizeof(double);
    static size_t shm_set = 48 * 1024;
    if (shm > 48 * 1024) {
        int e = raise_smem_limit((const void *)element_tables_kernel, shm, &shm_set);
        if (e) return e;
    }
    int blocks = std::min((P->nf + warps - 1) / warps, 152 * 32);
    double2 alpha = make_double2(P->opt.alpha_re, P->opt.alpha_im);
    // the recurrence factors, with the expressions the device used to evaluate per point
    const int W = 2 * pb + 3, ntri = pb * (pb + 1) / 2;
    std::vector<double> tab((size_t)(pb + 1) + pb + 2 * ntri + 2 * (size_t)(pb + 2) * W, 0.0);
    double *fac = tab.data(), *s3 = fac + pb + 1, *la = s3 + pb, *lb = la + ntri, *cA = lb + ntri,
           *cB = cA + (size_t)(pb + 2) * W;
    for (int i = 1; i <= pb; i++) fac[i] = sqrt((2.0 * i + 1.0) / (2.0 * i));
    for (int m = 0; m < pb; m++) s3[m] = sqrt(2.0 * m + 3.0);
    for (int n = 2; n < pb; n++)
        for (int m = 0; m + 2 <= n; m++) {
            la[n * (n + 1) / 2 + m] = sqrt((4.0 * n * n - 1.0) / ((double)n * n - (double)m * m));
            lb[n * (n + 1) / 2 + m] = sqrt(((n - 1.0) * (n - 1.0) - (double)m * m) / (4.0 * (n - 1.0) * (n - 1.0) - 1.0));
        }
    for (int n = -1; n <= pb; n++)
        for (int m = -(pb + 1); m <= pb + 1; m++) {
            cA[(size_t)(n + 1) * W + m + pb + 1] = coefA(n, m);
            cB[(size_t)(n + 1) * W + m + pb + 1] = coefB(n, m);
        }
    double *tab_dev = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&tab_dev, sizeof(double) * tab.size()));
    FMM_CUDA_TRY(cudaMemcpy(tab_dev, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice));
    BasisTab T;
    T.fac = tab_dev;
    T.s3 = tab_dev + (s3 - fac);
    T.la = tab_dev + (la - fac);
    T.lb = tab_dev + (lb - fac);
    T.cA = tab_dev + (cA - fac);
    T.cB = tab_dev + (cB - fac);
    T.W = W;
    T.pb = pb;
    element_tables_kernel<<<blocks, 32 * warps, shm, P->stream>>>(P->V_dev, P->F_dev, P->elem_leaf, ctr_dev, P->nf, pl,
                                                                   P->opt.k, bco, cco, alpha, P->opt.rule, T, U, Rv);
    FMM_CUDA_TRY(cudaGetLastError());
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    cudaFree(tab_dev);
    cudaFree(ctr_dev);
    return FMM_OK;
}

int gen_element_tables(Plan *P)
{
    int pl = P->pleaf;
    size_t tbl = (size_t)P->nf * pl * pl;
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->U64, sizeof(double2) * tbl));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->Rv64, sizeof(double2) * tbl));
    double2 bco = make_double2(P->opt.b_re, P->opt.b_im), cco = make_double2(P->opt.c_re, P->opt.c_im);
    int st = launch_element_tables(P, bco, cco, P->U64, P->Rv64);
    if (st) return st;
    if (P->opt.build_mixed) {
        FMM_CUDA_TRY(dev_alloc(P, (void **)&P->U32, sizeof(float2) * tbl));
        FMM_CUDA_TRY(dev_alloc(P, (void **)&P->Rv32, sizeof(float2) * tbl));
        if (P->scaled) {
            // multipole and local of the leaf level scaled by d_n (see gen_coax_tables)
            double *dd = nullptr;
            FMM_CUDA_TRY(cudaMalloc(&dd, sizeof(double) * pl));
            FMM_CUDA_TRY(cudaMemcpy(dd, P->dsc[P->lmax].data(), sizeof(double) * pl, cudaMemcpyHostToDevice));
            int blocks = (int)std::min<size_t>((tbl + 255) / 256, 152 * 16);
            to_float_degree_kernel<<<blocks, 256, 0, P->stream>>>(P->U64, P->U32, tbl, pl, dd);
            to_float_degree_kernel<<<blocks, 256, 0, P->stream>>>(P->Rv64, P->Rv32, tbl, pl, dd);
            FMM_CUDA_TRY(cudaGetLastError());
            FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
            cudaFree(dd);
        } else {
            to_float((const double *)P->U64, (float *)P->U32, 2 * tbl, P->stream);
            to_float((const double *)P->Rv64, (float *)P->Rv32, 2 * tbl, P->stream);
        }
        FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    }
    return FMM_OK;
}

// ----------------------------------------------------------------------------- near field
// A_ij = b int_{T_j} G(x, y_i) dS + c int_{T_j} dG/dn_x(x, y_i) dS
//        + alpha (b int_{T_j} dG/dn_y dS + c int_{T_j} d2G/dn_x dn_y dS)
// for source elements j in the leaf boxes adjacent to (or equal to) the leaf box of target i;
// the self term uses the centroid split (and the polar finite part for the hypersingular
// term).  One warp per target element, one lane per source element.
__global__ void near_field_kernel(const double *V, const int *F, int nf, const int *near_beg, const int *near_col,
                                  double k, double2 bco, double2 cco, double2 alpha, int rule, double2 *out)
{
    int lane = threadIdx.x & 31, warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nwt = (gridDim.x * blockDim.x) >> 5;
    bool bm = alpha.x != 0.0 || alpha.y != 0.0;
    for (int i = warp; i < nf; i += nwt) {
        double nodi[9], y[3], ny[3];
        load_tri(V, F, i, nodi);
        tri_centroid(nodi, y);
        tri_normal(nodi, ny);
        for (int s = near_beg[i] + lane; s < near_beg[i + 1]; s += 32) {
            int j = near_col[s];
            double nod[9];
            load_tri(V, F, j, nod);
            double2 v = make_double2(0.0, 0.0);
            bool sgl = (i == j);
            bool hb = bco.x != 0.0 || bco.y != 0.0, hc = cco.x != 0.0 || cco.y != 0.0;
            if (sgl) {
                if (hb) v = cadd(v, cmul(bco, elem_integral_sgl(k, nod, 0)));
                if (hc) v = cadd(v, cmul(cco, elem_integral_sgl(k, nod, 1)));
                if (bm && hc) v = cadd(v, cmul(alpha, cmul(cco, elem_hyper_self(k, nod))));
            } else {
                // every regular-rule integral of the pair from one evaluation of G per point
                double2 G, dGx, dGy;
                double nT[3];
                elem_integrals_fused(k, nod, y, ny, rule, hb || (bm && hc), hc, bm && hb, G, dGx, dGy, nT);
                if (hb) v = cadd(v, cmul(bco, G));
                if (hc) v = cadd(v, cmul(cco, dGx));
                if (bm) {
                    double2 w = make_double2(0.0, 0.0);
                    if (hb) w = cadd(w, cmul(bco, dGy));
                    if (hc) {
                        // Maue form: k^2 (ny.nT) int G - boundary term
                        double dn = ny[0] * nT[0] + ny[1] * nT[1] + ny[2] * nT[2], kk = k * k * dn;
                        double2 l = hyper_edges(k, nod, y, ny);
                        w = cadd(w, cmul(cco, make_double2(kk * G.x - l.x, kk * G.y - l.y)));
                    }
                    v = cadd(v, cmul(alpha, w));
                }
            }
            out[s] = v;
        }
    }
}

// The FP64 element tables (P2M moments U) and near-field matrix of the operator part with
// source coefficients (bco, cco) -- the plan's own a, b, c set aside -- into caller buffers of
// nf * pleaf^2 and num_near entries (the adjoint path's derivatives in b and c).  The L2P
// vectors do not depend on b and c; Rv_tmp (nf * pleaf^2 entries) receives a copy.
int gen_operator_part(Plan *P, double2 bco, double2 cco, double2 *U, double2 *Rv_tmp, double2 *nearv)
{
    int st = launch_element_tables(P, bco, cco, U, Rv_tmp);
    if (st) return st;
    int blocks = std::min((P->nf + 7) / 8, 152 * 16);
    double2 alpha = make_double2(P->opt.alpha_re, P->opt.alpha_im);
    near_field_kernel<<<blocks, 256, 0, P->stream>>>(P->V_dev, P->F_dev, P->nf, P->near_beg, P->near_col, P->opt.k,
                                                      bco, cco, alpha, P->opt.rule, nearv);
    FMM_CUDA_TRY(cudaGetLastError());
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    return FMM_OK;
}

int gen_near_field(Plan *P)
{
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->near64, sizeof(double2) * (P->num_near + 1)));
    double2 bco = make_double2(P->opt.b_re, P->opt.b_im), cco = make_double2(P->opt.c_re, P->opt.c_im);
    int blocks = std::min((P->nf + 7) / 8, 152 * 16);
    double2 alpha = make_double2(P->opt.alpha_re, P->opt.alpha_im);
    near_field_kernel<<<blocks, 256, 0, P->stream>>>(P->V_dev, P->F_dev, P->nf, P->near_beg, P->near_col, P->opt.k,
                                                      bco, cco, alpha, P->opt.rule, P->near64);
    FMM_CUDA_TRY(cudaGetLastError());
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    if (P->opt.build_mixed) {
        FMM_CUDA_TRY(dev_alloc(P, (void **)&P->near32, sizeof(float2) * (P->num_near + 1)));
        to_float((const double *)P->near64, (float *)P->near32, 2 * (size_t)P->num_near, P->stream);
        FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    }
    return FMM_OK;
}

// ----------------------------------------------------------------------------- far field
// -(b L + c M) p at exterior points: the scattered pressure p_s = M p - L dp/dn of the exterior
// problem written as c = -1, b = (dp/dn)/p (rigid body: b = 0, p_s = M p).  One block per point.
__global__ void far_field_kernel(const double *V, const int *F, int nf, double k, double2 bco, double2 cco, int rule,
                                 const double2 *p, const double *pts, double2 *out)
{
    int t = blockIdx.x;
    double y[3] = {pts[3 * t], pts[3 * t + 1], pts[3 * t + 2]};
    bool hb = bco.x != 0.0 || bco.y != 0.0, hc = cco.x != 0.0 || cco.y != 0.0;
    double2 acc = make_double2(0.0, 0.0);
    for (int j = threadIdx.x; j < nf; j += blockDim.x) {
        double nod[9];
        load_tri(V, F, j, nod);
        double2 v = make_double2(0.0, 0.0);
        if (hb) v = cadd(v, cmul(bco, elem_integral(k, nod, y, rule, 0)));
        if (hc) v = cadd(v, cmul(cco, elem_integral(k, nod, y, rule, 1)));
        acc = csub(acc, cmul(p[j], v));
    }
    __shared__ double2 red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[t] = red[0];
}

int launch_far_field(Plan *P, const double2 *p, const double *pts, int npts, double2 *out)
{
    if (npts <= 0) return FMM_OK;
    double2 bco = make_double2(P->opt.b_re, P->opt.b_im), cco = make_double2(P->opt.c_re, P->opt.c_im);
    far_field_kernel<<<npts, 256, 0, P->stream>>>(P->V_dev, P->F_dev, P->nf, P->opt.k, bco, cco, P->opt.rule, p, pts,
                                                   out);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

// p_inc + alpha dp_inc/dn = e^{ik d.y} (1 + alpha i k d.n) at the centroids (alpha = 0: p_inc)
__global__ void plane_wave_kernel(const double *V, const int *F, int nf, double k, double dx, double dy, double dz,
                                  double2 alpha, double2 *rhs)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nf; e += gridDim.x * blockDim.x) {
        double nod[9], y[3];
        load_tri(V, F, e, nod);
        tri_centroid(nod, y);
        double s, c;
        sincos(k * (dx * y[0] + dy * y[1] + dz * y[2]), &s, &c);
        double2 v = make_double2(c, s);
        if (alpha.x != 0.0 || alpha.y != 0.0) {
            double nh[3];
            tri_normal(nod, nh);
            double kd = k * (dx * nh[0] + dy * nh[1] + dz * nh[2]);
            v = cmul(v, make_double2(1.0 - alpha.y * kd, alpha.x * kd));
        }
        rhs[e] = v;
    }
}

int launch_plane_wave(Plan *P, const double *dir, double2 *rhs)
{
    plane_wave_kernel<<<(P->nf + 255) / 256, 256, 0, P->stream>>>(P->V_dev, P->F_dev, P->nf, P->opt.k, dir[0], dir[1],
                                                                   dir[2], make_double2(P->opt.alpha_re, P->opt.alpha_im),
                                                                   rhs);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

} // namespace fmm
