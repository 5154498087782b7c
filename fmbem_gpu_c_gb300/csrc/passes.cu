// The FMM matvec: P2M, M2M, M2L (+ fused L2L), L2P + near field.  Templated on the
// arithmetic type: double for the plain path, float for the mixed-precision path, float-float
// (ff.cuh) for the M2L of the FMM_FLOAT2 path.
//
// Every translation is rotation - coaxial - rotation (RCR) as in the reference
// (transMatsVecsMul_SR_rcr, translation.cu:1864-1961): rotate by (phi, theta, 0), apply the
// coaxial blocks for |t|, rotate back by (0, theta, phi).  The rotation matrix is
// e^{i m alpha} e^{-i m' gamma} H_n^{m'm}(beta) (translation.cu:1221-1235), so one real
// table H per direction serves both rotations and the phases are applied elementwise.
// The FP64 path is owner-computes: each destination box is owned by one CTA that accumulates
// all its translations in shared memory and writes once (no atomics, bit-reproducible); on
// levels with few boxes a box's sources are split over several CTAs whose partial sums are
// added in a fixed order.
// The mixed path runs the batched direction-grouped tiles of batched.cu, which add into the
// expansions with FP32 atomics, so mixed results vary in the last bits from run to run.
#include "plan.h"
#include "ff.cuh"
#include <algorithm>
#include <vector>
#include <type_traits>

namespace fmm {

__constant__ int c_dir_dist[NDIR];
__constant__ int c_dir_hrep[NDIR]; // direction -> the direction whose (identical) rotation table it reads

template <typename T> struct Cx;
template <> struct Cx<double> { typedef double2 t; };
template <> struct Cx<float> { typedef float2 t; };
template <> struct Cx<ff> { typedef ff2 t; };

__device__ __forceinline__ void decode_nm(int i, int &n, int &m)
{
    int q = (int)sqrtf((float)i);
    while (q * q > i) q--;
    while ((q + 1) * (q + 1) <= i) q++;
    n = q;
    m = i - q * q - q;
}

__device__ __forceinline__ float2 to_c(double2 v, float) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ double2 to_c(double2 v, double) { return v; }
__device__ __forceinline__ double2 to_d(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 to_d(double2 v) { return v; }

// acc += a b: as written for FP32 and FP64 (contracted to an FMA), the fused float-float
// multiply-add for ff
template <typename T>
__device__ __forceinline__ void mac(T &acc, T a, T b)
{
    if constexpr (std::is_same<T, ff>::value)
        acc = ff_fma(a, b, acc);
    else
        acc += a * b;
}

// One RCR translation by a whole CTA.  x has pin^2 entries (zero padded to p); the result
// for n < pout is accumulated into sY.  H and ph are the direction's real rotation table
// (stride rot_size(pmax), prefix order p) and phases e^{i m phi} indexed m + pmax - 1.
template <typename T>
__device__ void rcr_block(int p, int pmax, const T *__restrict__ H, const typename Cx<T>::t *__restrict__ ph,
                          const typename Cx<T>::t *__restrict__ Cc, const typename Cx<T>::t *__restrict__ xin, int pin,
                          typename Cx<T>::t *sX, typename Cx<T>::t *sW1, typename Cx<T>::t *sW2,
                          typename Cx<T>::t *sY, int pout)
{
    typedef typename Cx<T>::t C;
    const int pp = p * p, pin2 = pin * pin, tid = threadIdx.x, nt = blockDim.x, off = pmax - 1;
    for (int i = tid; i < pp; i += nt) {
        int n, m;
        decode_nm(i, n, m);
        C v = (i < pin2) ? xin[i] : mk2((T)0, (T)0);
        sX[i] = cmul(v, ph[m + off]);
    }
    __syncthreads();
    for (int i = tid; i < pp; i += nt) {
        int n, mp;
        decode_nm(i, n, mp);
        const T *col = H + rot_off(n) + (mp + n);
        const int w = 2 * n + 1, base = n * n;
        T ar = 0, ai = 0;
        for (int m = 0; m < w; m++) {
            T h = col[m * w];
            C v = sX[base + m];
            mac(ar, h, v.x);
            mac(ai, h, v.y);
        }
        sW1[i] = mk2(ar, ai);
    }
    __syncthreads();
    for (int i = tid; i < pp; i += nt) {
        int np, m;
        decode_nm(i, np, m);
        int am = m < 0 ? -m : m, sz = p - am;
        const C *col = Cc + coax_off(p, am) + (np - am);
        T ar = 0, ai = 0;
        for (int n = am; n < p; n++) {
            C c = col[(n - am) * sz];
            C v = sW1[n * n + n + m];
            if constexpr (std::is_same<T, ff>::value) {
                ar = ff_fma(c.x, v.x, ar);
                ar = ff_fma(-c.y, v.y, ar);
                ai = ff_fma(c.x, v.y, ai);
                ai = ff_fma(c.y, v.x, ai);
            } else {
                ar += c.x * v.x - c.y * v.y;
                ai += c.x * v.y + c.y * v.x;
            }
        }
        sW2[i] = mk2(ar, ai);
    }
    __syncthreads();
    const int po2 = pout * pout;
    for (int i = tid; i < po2; i += nt) {
        int n, mp;
        decode_nm(i, n, mp);
        const T *col = H + rot_off(n) + (mp + n);
        const int w = 2 * n + 1, base = n * n;
        T ar = 0, ai = 0;
        for (int m = 0; m < w; m++) {
            T h = col[m * w];
            C v = sW2[base + m];
            mac(ar, h, v.x);
            mac(ai, h, v.y);
        }
        C e = ph[mp + off];
        // conj(e) * (ar + i ai)
        C y = sY[i];
        y.x += e.x * ar + e.y * ai;
        y.y += e.x * ai - e.y * ar;
        sY[i] = y;
    }
    __syncthreads();
}

// flip = 0: C_b[n,m] = ik sum_e x_e U_e[n,m] (element moments of R_n^{-m}).
// flip = 1 (transposed operator): the same with the table read at (n,-m); with U = Rv this
// is the multipole expansion ik sum_i y_i R_n^{-m}(y_i - c) of point sources at centroids.
// P2M of one leaf box (CTA) for a group of up to G right-hand sides (blockIdx.y): thread i takes
// coefficient i; the box's elements and their i k x_e are staged in shared memory once, so that
// the loads of U depend on shared memory only and can all be in flight together, and each U
// entry serves the whole group.  Each column's sum runs in the same order whatever the group.
// With x32 given, the CTA also writes its elements' x in FP32 there (every element lies in one
// leaf), for the gathers of the L2P + near-field pass: GB300 converts FP64 to FP32 at its FP64
// rate, and the near field would otherwise convert each x once per near pair.
template <typename T, int G>
__global__ void p2m_kernel(int pl, const int *__restrict__ leaf_beg, const int *__restrict__ leaf_elem,
                           const typename Cx<T>::t *__restrict__ U, const double2 *__restrict__ x, double k,
                           typename Cx<T>::t *__restrict__ Cm, int flip, int nf, int nb, int nrhs,
                           float2 *__restrict__ x32)
{
    typedef typename Cx<T>::t C;
    constexpr int MAXE = 64;
    __shared__ int s_e[MAXE];
    __shared__ C s_x[MAXE][G];
    const int b = blockIdx.x, ppl = pl * pl, r0 = blockIdx.y * G, ng = min(G, nrhs - r0);
    const int s0 = leaf_beg[b], ne = leaf_beg[b + 1] - s0;
    for (int j = threadIdx.x; j < ne; j += blockDim.x) {
        const int e = leaf_elem[s0 + j];
        if (j < MAXE) s_e[j] = e;
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (g >= ng) break;
            const size_t k_e = (size_t)(r0 + g) * nf + e;
            const double2 xe = x[k_e];
            if (j < MAXE) s_x[j][g] = mk2((T)(-k * xe.y), (T)(k * xe.x));  // i k x_e
            if (x32) x32[k_e] = make_float2((float)xe.x, (float)xe.y);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ppl; i += blockDim.x) {
        int q = i;
        if (flip) {
            int n, m;
            decode_nm(i, n, m);
            q = n * n + n - m;
        }
        T ar[G], ai[G];
#pragma unroll
        for (int g = 0; g < G; g++) ar[g] = ai[g] = 0;
#pragma unroll 4
        for (int j = 0; j < ne && j < MAXE; j++) {
            const C u = U[(size_t)s_e[j] * ppl + q];
#pragma unroll
            for (int g = 0; g < G; g++) {
                if (g >= ng) break;
                const C xe = s_x[j][g];
                ar[g] += xe.x * u.x - xe.y * u.y;
                ai[g] += xe.x * u.y + xe.y * u.x;
            }
        }
        // boxes with more than MAXE elements (none at the usual leaf occupancy): the rest directly
        for (int j = MAXE; j < ne; j++) {
            const int e = leaf_elem[s0 + j];
            const C u = U[(size_t)e * ppl + q];
#pragma unroll
            for (int g = 0; g < G; g++) {
                if (g >= ng) break;
                const double2 xd = x[(size_t)(r0 + g) * nf + e];
                const T xr = (T)(-k * xd.y), xi = (T)(k * xd.x);
                ar[g] += xr * u.x - xi * u.y;
                ai[g] += xr * u.y + xi * u.x;
            }
        }
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (g >= ng) break;
            Cm[((size_t)b * nrhs + r0 + g) * ppl + i] = mk2(ar[g], ai[g]); // [box][rhs][p^2]
        }
    }
}

template <typename T>
__global__ void m2m_kernel(int pp, int pc, int pmax, const int *__restrict__ child_beg, const int *__restrict__ child_list,
                           const unsigned char *__restrict__ octant, const T *__restrict__ Hss,
                           const typename Cx<T>::t *__restrict__ PHss, const typename Cx<T>::t *__restrict__ Crr,
                           const typename Cx<T>::t *__restrict__ Cchild, typename Cx<T>::t *__restrict__ Cpar)
{
    typedef typename Cx<T>::t C;
    extern __shared__ unsigned char smraw[];
    C *sX = (C *)smraw;
    int P2 = pp * pp;
    C *sW1 = sX + P2, *sW2 = sW1 + P2, *sY = sW2 + P2;
    int q = blockIdx.x, rs = rot_size(pmax), w = 2 * pmax - 1;
    for (int i = threadIdx.x; i < P2; i += blockDim.x) sY[i] = mk2((T)0, (T)0);
    __syncthreads();
    for (int s = child_beg[q]; s < child_beg[q + 1]; s++) {
        int ch = child_list[s], o = octant[ch];
        rcr_block<T>(pp, pmax, Hss + (size_t)o * rs, PHss + (size_t)o * w, Crr, Cchild + (size_t)ch * pc * pc, pc,
                     sX, sW1, sW2, sY, pp);
    }
    for (int i = threadIdx.x; i < P2; i += blockDim.x) Cpar[(size_t)q * P2 + i] = sY[i];
}

__global__ void to_float_kernel2(const double *in, float *out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

template <typename T>
__global__ void m2l_kernel(int p, int pmax, int pp, const int *__restrict__ sr_beg, const int *__restrict__ sr_src,
                           const short *__restrict__ sr_dir, const T *__restrict__ Hsr,
                           const typename Cx<T>::t *__restrict__ PHsr, const typename Cx<T>::t *__restrict__ Csr,
                           const typename Cx<T>::t *__restrict__ Cm, const int *__restrict__ parent,
                           const unsigned char *__restrict__ octant, const T *__restrict__ Hrr,
                           const typename Cx<T>::t *__restrict__ PHrr, const typename Cx<T>::t *__restrict__ Crr,
                           const typename Cx<T>::t *__restrict__ Dpar, typename Cx<T>::t *__restrict__ Dl,
                           typename Cx<T>::t *__restrict__ part)
{
    typedef typename Cx<T>::t C;
    extern __shared__ unsigned char smraw[];
    int pe = pp > p ? pp : p, E2 = pe * pe, P2 = p * p;
    C *sX = (C *)smraw;
    C *sW1 = sX + E2, *sW2 = sW1 + E2, *sY = sW2 + E2;
    int b = blockIdx.x, rs = rot_size(pmax), w = 2 * pmax - 1, cs = coax_size(p);
    // owner-computes: the L2L from the parent and every M2L source, accumulated in shared
    // memory and written once.  With gridDim.y = S > 1 (levels with few boxes), CTA (b, c)
    // takes the c-th of S runs of box b's sources (run 0 also the L2L) and writes its partial
    // sum to part[c][b]; m2l_reduce_kernel adds the runs in order.
    const int S = gridDim.y, c = blockIdx.y, s0 = sr_beg[b], ns = sr_beg[b + 1] - s0;
    const int sa = s0 + (int)((long long)ns * c / S), sb = s0 + (int)((long long)ns * (c + 1) / S);
    for (int i = threadIdx.x; i < P2; i += blockDim.x) sY[i] = mk2((T)0, (T)0);
    __syncthreads();
    if (pp > 0 && c == 0) {
        // L2L: parent local (order pp) translated to this box, truncated to p
        int o = octant[b];
        rcr_block<T>(pp, pmax, Hrr + (size_t)o * rs, PHrr + (size_t)o * w, Crr, Dpar + (size_t)parent[b] * pp * pp, pp,
                     sX, sW1, sW2, sY, p);
    }
    for (int s = sa; s < sb; s++) {
        int src = sr_src[s], dir = sr_dir[s];
        rcr_block<T>(p, pmax, Hsr + (size_t)c_dir_hrep[dir] * rs, PHsr + (size_t)dir * w, Csr + (size_t)c_dir_dist[dir] * cs,
                     Cm + (size_t)src * P2, p, sX, sW1, sW2, sY, p);
    }
    C *out = S > 1 ? part + ((size_t)c * gridDim.x + b) * P2 : Dl + (size_t)b * P2;
    for (int i = threadIdx.x; i < P2; i += blockDim.x) out[i] = sY[i];
}

// Dl[b] = sum over c of part[c][b], c in order (the result does not depend on the schedule)
template <typename T>
__global__ void m2l_reduce_kernel(int S, size_t n, const typename Cx<T>::t *__restrict__ part, typename Cx<T>::t *__restrict__ Dl)
{
    typedef typename Cx<T>::t C;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        C a = part[i];
        for (int c = 1; c < S; c++) {
            C v = part[(size_t)c * n + i];
            a.x += v.x;
            a.y += v.y;
        }
        Dl[i] = a;
    }
}


// L2P + near field + identity for element e (one warp) and a group of up to G right-hand sides
// (blockIdx.y): the near row and the element's basis are loaded once for the group, the x
// gathers and the local expansions per right-hand side.  Each column's sums run in the same
// order whatever the group, so a column's result does not depend on nrhs.  T = float gathers
// the near field's x from x32, the FP32 copy P2M wrote (the same values as converting x here).
template <typename T, int G>
__global__ void l2p_near_kernel(int nf, int pl, const int *__restrict__ elem_leaf, const typename Cx<T>::t *__restrict__ Dl,
                                const typename Cx<T>::t *__restrict__ Rv, const int *__restrict__ near_beg,
                                const int *__restrict__ near_col, const typename Cx<T>::t *__restrict__ nearv,
                                const double2 *__restrict__ x, const float2 *__restrict__ x32, double2 a,
                                double2 *__restrict__ y, int flip, int nb, int nrhs)
{
    typedef typename Cx<T>::t C;
    int lane = threadIdx.x & 31;
    int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (e >= nf) return;
    const int r0 = blockIdx.y * G, ng = min(G, nrhs - r0);
    int ppl = pl * pl;
    T ar[G], ai[G];
#pragma unroll
    for (int g = 0; g < G; g++) ar[g] = ai[g] = 0;
    for (int s = near_beg[e] + lane; s < near_beg[e + 1]; s += 32) {
        const C v = nearv[s];
        const int col = near_col[s];
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (g >= ng) break;
            T xr, xi;
            if constexpr (sizeof(T) == 4) {
                const float2 xf = x32[(size_t)(r0 + g) * nf + col];
                xr = xf.x;
                xi = xf.y;
            } else {
                const double2 xd = x[(size_t)(r0 + g) * nf + col];
                xr = xd.x;
                xi = xd.y;
            }
            ar[g] += v.x * xr - v.y * xi;
            ai[g] += v.x * xi + v.y * xr;
        }
    }
    const C *R = Rv + (size_t)e * ppl;
    const size_t db = (size_t)elem_leaf[e] * nrhs; // [box][rhs][p^2]
    for (int i = lane; i < ppl; i += 32) {
        int q = i;
        if (flip) {
            int n, m;
            decode_nm(i, n, m);
            q = n * n + n - m;
        }
        const C r = R[q];
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (g >= ng) break;
            const C d = Dl[(db + r0 + g) * ppl + i];
            ar[g] += d.x * r.x - d.y * r.y;
            ai[g] += d.x * r.y + d.y * r.x;
        }
    }
#pragma unroll
    for (int g = 0; g < G; g++) {
        if (g >= ng) break;
        T sr = ar[g], si = ai[g];
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (lane == 0) {
            const size_t k = (size_t)(r0 + g) * nf + e;
            const double2 xe = x[k];
            y[k] = make_double2(a.x * xe.x - a.y * xe.y + (double)sr, a.x * xe.y + a.y * xe.x + (double)si);
        }
    }
}

static inline int block_for(int p) { return p >= 16 ? 256 : 128; }

static void timer_begin(Plan *P, const char *name, cudaStream_t st = nullptr)
{
    if (P->profiling != 1 || P->ntimers >= MAX_TIMERS) return;
    Timer &t = P->timers[P->ntimers];
    t.name = name;
    cudaEventRecord(t.beg, st ? st : P->stream);
}
static void timer_end(Plan *P, cudaStream_t st = nullptr)
{
    if (P->profiling != 1 || P->ntimers >= MAX_TIMERS) return;
    cudaEventRecord(P->timers[P->ntimers].end, st ? st : P->stream);
    P->ntimers++;
}

// Raise the dynamic shared-memory limit of the owner-computes translation kernels to what
// order pmax needs (4 p^2 complex for the CTA-level RCR).
template <typename T>
static int set_smem_attrs(int pmax)
{
    typedef typename Cx<T>::t C;
    static size_t m2m_set = 0, m2l_set = 0;
    size_t smax = 4 * (size_t)pmax * pmax * sizeof(C);
    int st = raise_smem_limit((const void *)m2m_kernel<T>, smax, &m2m_set);
    if (st) return st;
    return raise_smem_limit((const void *)m2l_kernel<T>, smax, &m2l_set);
}

template <typename T>
static int launch_m2l_level(Plan *P, int l, const char *tname)
{
    typedef typename Cx<T>::t C;
    const bool f64 = sizeof(T) == 8;
    int lmin = P->lmin, pmax = P->pmax;
    cudaStream_t st = P->stream;
    LevelDev &L = P->lev[l];
    const T *Hsr = f64 ? (const T *)P->Hsr64 : (const T *)P->Hsr32;
    const T *Hrr = f64 ? (const T *)P->Hrr64 : (const T *)P->Hrr32;
    const C *PHsr = f64 ? (const C *)P->PHsr64 : (const C *)P->PHsr32;
    const C *PHrr = f64 ? (const C *)P->PHrr64 : (const C *)P->PHrr32;
    const C *Csr = f64 ? (const C *)L.Csr64 : (const C *)L.Csr32;
    // the fused L2L: FP64, or the FP32 table scaled for L2L (plans with scaled expansions)
    const C *Crr = l > lmin ? (f64 ? (const C *)L.Crr64 : (const C *)(L.Crr32L ? L.Crr32L : L.Crr32)) : nullptr;
    const C *Cm = f64 ? (const C *)L.Cm64 : (const C *)L.Cm32;
    C *Dl = f64 ? (C *)L.Dl64 : (C *)L.Dl32;
    const C *Dpar = l > lmin ? (f64 ? (const C *)P->lev[l - 1].Dl64 : (const C *)P->lev[l - 1].Dl32) : nullptr;
    int pp = l > lmin ? P->lev[l - 1].p : 0;
    int pe = pp > L.p ? pp : L.p;
    size_t sm = 4 * (size_t)pe * pe * sizeof(C);
    timer_begin(P, tname);
    // levels with few boxes split each box's sources over S CTAs (P->m2l_split, sized at plan
    // creation so that the level fills the GPU) and add the runs in a second pass
    const int S = std::max(1, L.m2l_split);
    C *part = S > 1 ? (C *)P->m2l_part64 : nullptr;
    m2l_kernel<T><<<dim3(L.nb, S), block_for(pe), sm, st>>>(L.p, pmax, pp, L.sr_beg, L.sr_src, L.sr_dir, Hsr, PHsr, Csr,
                                                              Cm, L.parent, L.octant, Hrr, PHrr, Crr, Dpar, Dl, part);
    if (S > 1) {
        size_t n = (size_t)L.nb * L.p * L.p;
        int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
        m2l_reduce_kernel<T><<<blocks, 256, 0, st>>>(S, n, part, Dl);
    }
    timer_end(P);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

// ---------------------------------------------------------------- float-float M2L (FMM_FLOAT2)
__global__ void ff_from_real_kernel(const double *__restrict__ in, float2 *__restrict__ out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const ff a = ff_from(in[i]);
        out[i] = make_float2(a.hi, a.lo);
    }
}
__global__ void ff_from_cplx_kernel(const double2 *__restrict__ in, float4 *__restrict__ out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const ff a = ff_from(in[i].x), b = ff_from(in[i].y);
        out[i] = make_float4(a.hi, a.lo, b.hi, b.lo);
    }
}
__global__ void ff_to_cplx_kernel(const float4 *__restrict__ in, double2 *__restrict__ out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float4 v = in[i];
        out[i] = make_double2(ff_to(ff(v.x, v.y)), ff_to(ff(v.z, v.w)));
    }
}
// the same for expansions [box][p^2] kept scaled by degree: entry i times ds[degree of i % ppl]
__global__ void ff_from_cplx_deg_kernel(const double2 *__restrict__ in, float4 *__restrict__ out, size_t n, int ppl,
                                        const double *__restrict__ ds)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        int deg, m;
        decode_nm((int)(i % ppl), deg, m);
        const double f = ds[deg];
        const ff a = ff_from(in[i].x * f), b = ff_from(in[i].y * f);
        out[i] = make_float4(a.hi, a.lo, b.hi, b.lo);
    }
}
__global__ void ff_to_cplx_deg_kernel(const float4 *__restrict__ in, double2 *__restrict__ out, size_t n, int ppl,
                                      const double *__restrict__ ds)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        int deg, m;
        decode_nm((int)(i % ppl), deg, m);
        const double f = ds[deg];
        const float4 v = in[i];
        out[i] = make_double2(ff_to(ff(v.x, v.y)) * f, ff_to(ff(v.z, v.w)) * f);
    }
}
static unsigned ew_grid(size_t n) { return (unsigned)std::min<size_t>((n + 255) / 256, 152 * 16); }

// nmat coaxial tables of order p (the layout of coax_off: block m, entry (n', n) at
// (n - m)(p - m) + n' - m) with rows times row[n'] and columns times col[n], in float-float
static std::vector<float4> ff_scaled_coax(const std::vector<double2> &in, int p, int nmat, const std::vector<double> &row,
                                          const std::vector<double> &col)
{
    std::vector<float4> out(in.size());
    const int cs = coax_size(p);
    for (int q = 0; q < nmat; q++)
        for (int m = 0; m < p; m++) {
            const int sz = p - m, off = q * cs + coax_off(p, m);
            for (int i = 0; i < sz * sz; i++) {
                const int a = i % sz, b = i / sz;
                const double f = row[m + a] * col[m + b], x = in[off + i].x * f, y = in[off + i].y * f;
                const float xh = (float)x, yh = (float)y;
                out[off + i] = make_float4(xh, (float)(x - (double)xh), yh, (float)(y - (double)yh));
            }
        }
    return out;
}

// The float-float copies of the translation tables (rotations, phases, coaxial blocks) and
// the expansions, made on first use.  Where the FP32 mixed tables are built, the FP32 exponent
// range holds them: plain, or scaled by degree as the FP32 ones (multipoles d_n M_n, locals
// L_n / d_n, the coaxial tables scaled to match, the leaf expansions scaled on the way in and
// out); elsewhere FMM_FLOAT2 runs FMM_FP64.
static int ensure_ff(Plan *P)
{
    if (P->ff_ready) return FMM_OK;
    if (!P->opt.build_mixed || !P->U32) {
        P->ff_ready = -1;
        return FMM_OK;
    }
    const int pmax = P->pmax, rs = rot_size(pmax), w = 2 * pmax - 1;
    const size_t nh = (size_t)(NDIR + 16) * rs, nph = (size_t)(NDIR + 16) * w;
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->Hall_ff, sizeof(float2) * nh));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->PHall_ff, sizeof(float4) * nph));
    ff_from_real_kernel<<<ew_grid(nh), 256, 0, P->stream>>>(P->Hsr64, P->Hall_ff, nh);
    ff_from_cplx_kernel<<<ew_grid(nph), 256, 0, P->stream>>>(P->PHsr64, P->PHall_ff, nph);
    for (int l = P->lmin; l <= P->lmax; l++) {
        LevelDev &L = P->lev[l];
        const size_t ncs = (size_t)NDIST * coax_size(L.p), ne = (size_t)L.nb * L.p * L.p;
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Csr_ff, sizeof(float4) * ncs));
        if (l > P->lmin) FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Crr_ff, sizeof(float4) * coax_size(P->lev[l - 1].p)));
        if (!P->scaled) {
            ff_from_cplx_kernel<<<ew_grid(ncs), 256, 0, P->stream>>>(L.Csr64, L.Csr_ff, ncs);
            if (l > P->lmin)
                ff_from_cplx_kernel<<<ew_grid(coax_size(P->lev[l - 1].p)), 256, 0, P->stream>>>(
                    L.Crr64, L.Crr_ff, coax_size(P->lev[l - 1].p));
        } else {
            // the scalings of the FP32 tables (gen_coax_tables): M2L 1/d^l both sides; M2M rows
            // d^{l-1}, columns 1/d^l below the child order (0 above); L2L rows 1/d^l below the
            // child order (0 above), columns d^{l-1}
            const int pall = (int)P->dsc[l].size();
            std::vector<double> inv(pall), up(pall, 0.0), down(pall, 0.0);
            for (int n = 0; n < pall; n++) inv[n] = 1.0 / P->dsc[l][n];
            for (int n = 0; n < L.p && n < pall; n++) up[n] = down[n] = inv[n];
            std::vector<double2> h(ncs);
            FMM_CUDA_TRY(cudaMemcpy(h.data(), L.Csr64, sizeof(double2) * ncs, cudaMemcpyDeviceToHost));
            std::vector<float4> f = ff_scaled_coax(h, L.p, NDIST, inv, inv);
            FMM_CUDA_TRY(cudaMemcpy(L.Csr_ff, f.data(), sizeof(float4) * ncs, cudaMemcpyHostToDevice));
            if (l > P->lmin) {
                const int pp = P->lev[l - 1].p;
                const size_t nrr = coax_size(pp);
                h.resize(nrr);
                FMM_CUDA_TRY(cudaMemcpy(h.data(), L.Crr64, sizeof(double2) * nrr, cudaMemcpyDeviceToHost));
                f = ff_scaled_coax(h, pp, 1, P->dsc[l - 1], up);
                FMM_CUDA_TRY(cudaMemcpy(L.Crr_ff, f.data(), sizeof(float4) * nrr, cudaMemcpyHostToDevice));
                f = ff_scaled_coax(h, pp, 1, down, P->dsc[l - 1]);
                FMM_CUDA_TRY(dev_alloc(P, (void **)&L.CrrL_ff, sizeof(float4) * nrr));
                FMM_CUDA_TRY(cudaMemcpy(L.CrrL_ff, f.data(), sizeof(float4) * nrr, cudaMemcpyHostToDevice));
            }
        }
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Cm_ff, sizeof(float4) * ne));
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Dl_ff, sizeof(float4) * ne));
    }
    if (P->scaled) {
        const std::vector<double> &d = P->dsc[P->lmax];
        FMM_CUDA_TRY(dev_alloc(P, (void **)&P->dsc_leaf_dev, sizeof(double) * d.size()));
        FMM_CUDA_TRY(cudaMemcpy(P->dsc_leaf_dev, d.data(), sizeof(double) * d.size(), cudaMemcpyHostToDevice));
    }
    FMM_CUDA_TRY(cudaGetLastError());
    P->ff_ready = 1;
    return FMM_OK;
}

// The M2M of level l into level l - 1 in float-float (the parent-owned m2m_kernel).
static int launch_m2m_level_ff(Plan *P, int l, const char *tname)
{
    static size_t m2m_set = 0;
    const int pmax = P->pmax, rs = rot_size(pmax), w = 2 * pmax - 1;
    int e = raise_smem_limit((const void *)m2m_kernel<ff>, 4 * (size_t)pmax * pmax * sizeof(ff2), &m2m_set);
    if (e) return e;
    LevelDev &L = P->lev[l], &PL = P->lev[l - 1];
    const ff *Hss = reinterpret_cast<const ff *>(P->Hall_ff) + (size_t)NDIR * rs;
    const ff2 *PHss = reinterpret_cast<const ff2 *>(P->PHall_ff) + (size_t)NDIR * w;
    const size_t sm = 4 * (size_t)PL.p * PL.p * sizeof(ff2);
    timer_begin(P, tname);
    m2m_kernel<ff><<<PL.nb, block_for(PL.p), sm, P->stream>>>(
        PL.p, L.p, pmax, PL.child_beg, PL.child_list, L.octant, Hss, PHss, reinterpret_cast<const ff2 *>(L.Crr_ff),
        reinterpret_cast<const ff2 *>(L.Cm_ff), reinterpret_cast<ff2 *>(PL.Cm_ff));
    timer_end(P);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

// The M2L (+ fused L2L) of level l in float-float: the owner-computes m2l_kernel on the
// float-float tables and expansions.
static int launch_m2l_level_ff(Plan *P, int l, const char *tname)
{
    static size_t m2l_set = 0;
    const int lmin = P->lmin, pmax = P->pmax, rs = rot_size(pmax), w = 2 * pmax - 1;
    int e = raise_smem_limit((const void *)m2l_kernel<ff>, 4 * (size_t)pmax * pmax * sizeof(ff2), &m2l_set);
    if (e) return e;
    cudaStream_t st = P->stream;
    LevelDev &L = P->lev[l];
    const ff *Hall = reinterpret_cast<const ff *>(P->Hall_ff);
    const ff2 *PHall = reinterpret_cast<const ff2 *>(P->PHall_ff);
    const ff *Hsr = Hall, *Hrr = Hall + (size_t)(NDIR + 8) * rs;
    const ff2 *PHsr = PHall, *PHrr = PHall + (size_t)(NDIR + 8) * w;
    const ff2 *Csr = reinterpret_cast<const ff2 *>(L.Csr_ff);
    const ff2 *Crr = l > lmin ? reinterpret_cast<const ff2 *>(L.CrrL_ff ? L.CrrL_ff : L.Crr_ff) : nullptr;
    const ff2 *Cm = reinterpret_cast<const ff2 *>(L.Cm_ff);
    ff2 *Dl = reinterpret_cast<ff2 *>(L.Dl_ff);
    const ff2 *Dpar = l > lmin ? reinterpret_cast<const ff2 *>(P->lev[l - 1].Dl_ff) : nullptr;
    const int pp = l > lmin ? P->lev[l - 1].p : 0, pe = pp > L.p ? pp : L.p;
    const size_t sm = 4 * (size_t)pe * pe * sizeof(ff2);
    timer_begin(P, tname);
    const int S = std::max(1, L.m2l_split);
    ff2 *part = S > 1 ? reinterpret_cast<ff2 *>(P->m2l_part64) : nullptr;
    m2l_kernel<ff><<<dim3(L.nb, S), block_for(pe), sm, st>>>(L.p, pmax, pp, L.sr_beg, L.sr_src, L.sr_dir, Hsr, PHsr, Csr,
                                                               Cm, L.parent, L.octant, Hrr, PHrr, Crr, Dpar, Dl, part);
    if (S > 1) {
        const size_t n = (size_t)L.nb * L.p * L.p;
        m2l_reduce_kernel<ff><<<(int)std::min<size_t>((n + 255) / 256, 152 * 8), 256, 0, st>>>(S, n, part, Dl);
    }
    timer_end(P);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

static RcrPass make_pass(int p, int pin, int pout, int atomic, const float *H, int hstride, const float2 *PH,
                         int phstride, int phoff, const float2 *Cc, const float2 *src, float2 *dst, int nrhs, int nsrc,
                         int ndst)
{
    RcrPass ps;
    ps.p = p;
    ps.pin = pin;
    ps.pout = pout;
    ps.atomic = atomic;
    ps.nrhs = nrhs;
    ps.nsrc = nsrc;
    ps.ndst = ndst;
    ps.hstride = hstride;
    ps.phstride = phstride;
    ps.phoff = phoff;
    ps.H = H;
    ps.PH = PH;
    ps.Cc = Cc;
    ps.src = src;
    ps.dst = dst;
    ps.items = nullptr;
    ps.g_src = ps.g_dst = nullptr;
    ps.hrep = nullptr;
    return ps;
}

// One batched FP32 pass of the mixed path for level l: PASS_M2M (level l into its parents),
// PASS_M2L (level l), PASS_L2L (parents into level l).
RcrList *pass32_desc(Plan *P, int l, int which, int nrhs, RcrPass &ps)
{
    const int pmax = P->pmax, rs = rot_size(pmax), w = 2 * pmax - 1;
    LevelDev &L = P->lev[l];
    if (which == PASS_M2L) {
        ps = make_pass(L.p, L.p, L.p, 1, P->Hsr32, rs, P->PHsr32, w, pmax - 1, L.Csr32, L.Cm32, L.Dl32, nrhs, L.nb, L.nb);
        ps.hrep = P->hrep_dev;
        return &L.m2l;
    }
    if (l <= P->lmin) return nullptr;
    LevelDev &PL = P->lev[l - 1];
    if (which == PASS_M2M) {
        ps = make_pass(PL.p, L.p, PL.p, 1, P->Hss32, rs, P->PHss32, w, pmax - 1, L.Crr32, L.Cm32, PL.Cm32, nrhs, L.nb,
                       PL.nb);
        return &L.m2m;
    }
    ps = make_pass(PL.p, PL.p, L.p, 0, P->Hrr32, rs, P->PHrr32, w, pmax - 1, L.Crr32L ? L.Crr32L : L.Crr32, PL.Dl32,
                   L.Dl32, nrhs, PL.nb, L.nb);
    return &L.l2l;
}

int launch_pass32(Plan *P, int l, int which, int nrhs, cudaStream_t st)
{
    RcrPass ps;
    RcrList *Lst = pass32_desc(P, l, which, nrhs, ps);
    if (Lst && Lst->t3.on) return launch_tc3_pass(P, l, which, nrhs, st);
    if (Lst && Lst->td.on) return launch_tc_dense(P, l, which, nrhs, st);
    return Lst ? launch_rcr_pass(*Lst, ps, st) : FMM_OK;
}

// The mixed path's translation passes for nrhs columns: zero the expansions, M2M up, the
// M2L of every level forked onto the side streams (one level's tail overlaps the next
// level's work), join, L2L down.  M2M and M2L add into zeroed expansions with atomics; L2L
// then adds the parents' locals top-down.
static int translate32_direct(Plan *P, int nrhs)
{
    const int lmin = P->lmin, lmax = P->lmax;
    cudaStream_t st = P->stream;
    if (P->profiling == 1) {
        cudaEventRecord(P->phase.beg, st);
        P->have_phase = 1;
    }
    static const char *m2m_names[] = {"m2m_l0", "m2m_l1", "m2m_l2", "m2m_l3", "m2m_l4", "m2m_l5", "m2m_l6",
                                      "m2m_l7", "m2m_l8", "m2m_l9", "m2m_l10", "m2m_l11", "m2m_l12", "m2m_l13"};
    static const char *m2l_names[] = {"m2l_l0", "m2l_l1", "m2l_l2", "m2l_l3", "m2l_l4", "m2l_l5", "m2l_l6",
                                      "m2l_l7", "m2l_l8", "m2l_l9", "m2l_l10", "m2l_l11", "m2l_l12", "m2l_l13"};
    static const char *l2l_names[] = {"l2l_l0", "l2l_l1", "l2l_l2", "l2l_l3", "l2l_l4", "l2l_l5", "l2l_l6",
                                      "l2l_l7", "l2l_l8", "l2l_l9", "l2l_l10", "l2l_l11", "l2l_l12", "l2l_l13"};
    for (int l = lmin; l <= lmax; l++) {
        size_t n = (size_t)P->lev[l].nb * P->lev[l].p * P->lev[l].p * sizeof(float2) * nrhs;
        if (l < lmax) FMM_CUDA_TRY(cudaMemsetAsync(P->lev[l].Cm32, 0, n, st));
        FMM_CUDA_TRY(cudaMemsetAsync(P->lev[l].Dl32, 0, n, st));
    }
    for (int l = lmax; l > lmin; l--) {
        timer_begin(P, m2m_names[l]);
        int e = launch_pass32(P, l, PASS_M2M, nrhs, st);
        if (e) return e;
        timer_end(P);
    }
    // every side stream waits on the fork, also one that gets no pass, so that all of them
    // join a graph capture
    FMM_CUDA_TRY(cudaEventRecord(P->fork_ev, st));
    for (int i = 0; i < P->nside; i++) FMM_CUDA_TRY(cudaStreamWaitEvent(P->side[i], P->fork_ev, 0));
    for (int l = lmin; l <= lmax; l++) {
        cudaStream_t sl = P->side[(l - lmin) % P->nside];
        timer_begin(P, m2l_names[l], sl);
        int e = launch_pass32(P, l, PASS_M2L, nrhs, sl);
        if (e) return e;
        timer_end(P, sl);
        FMM_CUDA_TRY(cudaEventRecord(P->m2l_ev[l], sl));
    }
    // L2L into level l adds the parents' locals once level l's M2L (and the L2L above it) is
    // complete, so the top of the downward pass overlaps the M2L of the deeper levels
    FMM_CUDA_TRY(cudaStreamWaitEvent(st, P->m2l_ev[lmin], 0));
    for (int l = lmin + 1; l <= lmax; l++) {
        FMM_CUDA_TRY(cudaStreamWaitEvent(st, P->m2l_ev[l], 0));
        timer_begin(P, l2l_names[l]);
        int e = launch_pass32(P, l, PASS_L2L, nrhs, st);
        if (e) return e;
        timer_end(P);
    }
    for (int i = 0; i < P->nside; i++) {
        FMM_CUDA_TRY(cudaEventRecord(P->join_ev[i], P->side[i]));
        FMM_CUDA_TRY(cudaStreamWaitEvent(st, P->join_ev[i], 0));
    }
    if (P->profiling == 1) cudaEventRecord(P->phase.end, st);
    return FMM_OK;
}

void drop_graph(Plan *P)
{
    if (P->graph_exec) cudaGraphExecDestroy(P->graph_exec);
    P->graph_exec = nullptr;
    P->graph_nrhs = 0;
    P->graph_seen = 0;
}

// Translation passes as a CUDA graph: the second call with the same number of columns
// captures them (the first has built the work items and set the kernels' attributes), later
// calls replay the graph, which saves the ~25 launches and memsets per matvec.  Per-pass
// profiling (mode 1) runs the passes directly so that each pass gets its own timer.
static int translate32(Plan *P, int nrhs)
{
    if (P->profiling == 1) return translate32_direct(P, nrhs);
    if (P->graph_exec && P->graph_nrhs == nrhs) {
        FMM_CUDA_TRY(cudaGraphLaunch(P->graph_exec, P->stream));
        return FMM_OK;
    }
    if (P->graph_seen != nrhs) {
        drop_graph(P);
        P->graph_seen = nrhs;
        return translate32_direct(P, nrhs);
    }
    cudaGraph_t g = nullptr;
    FMM_CUDA_TRY(cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal));
    int e = translate32_direct(P, nrhs);
    cudaError_t ce = cudaStreamEndCapture(P->stream, &g);
    if (e) {
        if (g) cudaGraphDestroy(g);
        return e;
    }
    if (ce != cudaSuccess) {
        fmm_set_error("capturing the translation passes: %s", cudaGetErrorString(ce));
        return FMM_ERR_CUDA;
    }
    ce = cudaGraphInstantiate(&P->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
        P->graph_exec = nullptr;
        fmm_set_error("instantiating the translation graph: %s", cudaGetErrorString(ce));
        return FMM_ERR_CUDA;
    }
    P->graph_nrhs = nrhs;
    FMM_CUDA_TRY(cudaGraphLaunch(P->graph_exec, P->stream));
    return FMM_OK;
}

// ffm2l (T = double only): the M2L and its fused L2L in float-float (FMM_FLOAT2)
template <typename T>
static int run_matvec_t(Plan *P, const double2 *x, double2 *y, int transpose, int nrhs, bool ffm2l = false)
{
    typedef typename Cx<T>::t C;
    const bool f64 = sizeof(T) == 8;
    // owner-computes translations: the FP64 path, and the mixed path of deterministic plans
    const bool owner = f64 || P->opt.deterministic;
    int lmin = P->lmin, lmax = P->lmax, pmax = P->pmax;
    cudaStream_t st = P->stream;
    {
        int st = set_smem_attrs<T>(pmax);
        if (st) return st;
    }
    P->ntimers = 0;
    P->have_total = 0;
    P->have_phase = 0;
    if (P->profiling) cudaEventRecord(P->total.beg, st);
    const T *Hsr = f64 ? (const T *)P->Hsr64 : (const T *)P->Hsr32;
    const T *Hss = f64 ? (const T *)P->Hss64 : (const T *)P->Hss32;
    const T *Hrr = f64 ? (const T *)P->Hrr64 : (const T *)P->Hrr32;
    const C *PHsr = f64 ? (const C *)P->PHsr64 : (const C *)P->PHsr32;
    const C *PHss = f64 ? (const C *)P->PHss64 : (const C *)P->PHss32;
    const C *PHrr = f64 ? (const C *)P->PHrr64 : (const C *)P->PHrr32;
    auto Cm = [&](int l) { return f64 ? (C *)P->lev[l].Cm64 : (C *)P->lev[l].Cm32; };
    auto Dl = [&](int l) { return f64 ? (C *)P->lev[l].Dl64 : (C *)P->lev[l].Dl32; };
    auto Csr = [&](int l) { return f64 ? (const C *)P->lev[l].Csr64 : (const C *)P->lev[l].Csr32; };
    auto Crr = [&](int l) { return f64 ? (const C *)P->lev[l].Crr64 : (const C *)P->lev[l].Crr32; };
    const C *U = f64 ? (const C *)P->U64 : (const C *)P->U32;
    const C *Rv = f64 ? (const C *)P->Rv64 : (const C *)P->Rv32;
    const C *nearv = f64 ? (const C *)P->near64 : (const C *)P->near32;
    LevelDev &LL = P->lev[lmax];
    float2 *x32 = f64 ? nullptr : P->x32;
    if (!f64 && (!x32 || P->x32_cap < nrhs)) {
        fmm_set_error("mixed matvec: FP32 input buffer missing");
        return FMM_ERR_CUDA;
    }

    static const char *m2m_names[] = {"m2m_l0", "m2m_l1", "m2m_l2", "m2m_l3", "m2m_l4", "m2m_l5", "m2m_l6",
                                      "m2m_l7", "m2m_l8", "m2m_l9", "m2m_l10", "m2m_l11", "m2m_l12", "m2m_l13"};
    static const char *m2l_names[] = {"m2l_l0", "m2l_l1", "m2l_l2", "m2l_l3", "m2l_l4", "m2l_l5", "m2l_l6",
                                      "m2l_l7", "m2l_l8", "m2l_l9", "m2l_l10", "m2l_l11", "m2l_l12", "m2l_l13"};
    timer_begin(P, "p2m");
    // the transposed operator swaps the roles of the element moments and the centroid basis
    // (index-flipped), keeps every translation, and uses the transposed near-field matrix
    if (nrhs == 1)
        p2m_kernel<T, 1><<<dim3(LL.nb, 1), 128, 0, st>>>(LL.p, P->leaf_beg, P->leaf_elem, transpose ? Rv : U, x, P->opt.k,
                                                      Cm(lmax), transpose, P->nf, LL.nb, 1, x32);
    else
        p2m_kernel<T, 8><<<dim3(LL.nb, (nrhs + 7) / 8), 128, 0, st>>>(LL.p, P->leaf_beg, P->leaf_elem, transpose ? Rv : U, x,
                                                                   P->opt.k, Cm(lmax), transpose, P->nf, LL.nb, nrhs, x32);
    timer_end(P);
    if (!owner) {
        int e = translate32(P, nrhs);
        if (e) return e;
    }
    for (int l = lmax; l > lmin && owner && !ffm2l; l--) {
        LevelDev &L = P->lev[l], &PL = P->lev[l - 1];
        size_t sm = 4 * (size_t)PL.p * PL.p * sizeof(C);
        timer_begin(P, m2m_names[l]);
        m2m_kernel<T><<<PL.nb, block_for(PL.p), sm, st>>>(PL.p, L.p, pmax, PL.child_beg, PL.child_list, L.octant, Hss,
                                                           PHss, Crr(l), Cm(l), Cm(l - 1));
        timer_end(P);
    }
    if (f64 && ffm2l) {
        // the leaf multipoles into float-float; M2M, M2L and L2L in float-float; the leaf locals
        // back to FP64 for L2P
        {
            const size_t n = (size_t)LL.nb * LL.p * LL.p;
            if (P->dsc_leaf_dev)
                ff_from_cplx_deg_kernel<<<ew_grid(n), 256, 0, st>>>(LL.Cm64, LL.Cm_ff, n, LL.p * LL.p, P->dsc_leaf_dev);
            else
                ff_from_cplx_kernel<<<ew_grid(n), 256, 0, st>>>(LL.Cm64, LL.Cm_ff, n);
        }
        for (int l = lmax; l > lmin; l--) {
            int st = launch_m2m_level_ff(P, l, m2m_names[l]);
            if (st) return st;
        }
        for (int l = lmin; l <= lmax; l++) {
            int st = launch_m2l_level_ff(P, l, m2l_names[l]);
            if (st) return st;
        }
        const size_t n = (size_t)LL.nb * LL.p * LL.p;
        if (P->dsc_leaf_dev)
            ff_to_cplx_deg_kernel<<<ew_grid(n), 256, 0, st>>>(LL.Dl_ff, LL.Dl64, n, LL.p * LL.p, P->dsc_leaf_dev);
        else
            ff_to_cplx_kernel<<<ew_grid(n), 256, 0, st>>>(LL.Dl_ff, LL.Dl64, n);
    }
    for (int l = lmin; l <= lmax && owner && !ffm2l; l++) {
        int st = launch_m2l_level<T>(P, l, m2l_names[l]);
        if (st) return st;
    }
    timer_begin(P, "l2p_near");
    double2 a = make_double2(P->opt.a_re, P->opt.a_im);
    const C *nearT = f64 ? (const C *)P->nearT64 : (const C *)P->nearT32;
    {
        const int *nb_ = transpose ? P->nearT_beg : P->near_beg, *nc_ = transpose ? P->nearT_col : P->near_col;
        const C *nv_ = transpose ? nearT : nearv, *rv_ = transpose ? U : Rv;
        const unsigned gx = (unsigned)((P->nf * 32 + 255) / 256);
        if (nrhs == 1)
            l2p_near_kernel<T, 1><<<dim3(gx, 1), 256, 0, st>>>(P->nf, LL.p, P->elem_leaf, Dl(lmax), rv_, nb_, nc_, nv_, x, x32,
                                                            a, y, transpose, LL.nb, 1);
        else
            l2p_near_kernel<T, 8><<<dim3(gx, (nrhs + 7) / 8), 256, 0, st>>>(P->nf, LL.p, P->elem_leaf, Dl(lmax), rv_, nb_,
                                                                         nc_, nv_, x, x32, a, y, transpose, LL.nb, nrhs);
    }
    timer_end(P);
    if (P->profiling) {
        cudaEventRecord(P->total.end, st);
        P->have_total = 1;
    }
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

// Dense operators for the tensor-core passes: T[c][i][j] (pout^2 x pin^2, FP64), the RCR
// translation of key keys[c] applied to the unit source e_j.  M2L (ph = null): direction
// keys[c] with its azimuthal phases left out (rotation by the polar angle, coaxial
// translation, rotation back); the translation of any direction d with the same polar angle
// and distance is then diag(e^{-i m' phi_d}) T diag(e^{i m phi_d}).  M2M / L2L: octant keys[c]
// with its phases.  One CTA per (operator, column).
__global__ void dense_rcr_kernel(int p, int pmax, int pin, int pout, const int *__restrict__ keys,
                                 const double *__restrict__ H, const double2 *__restrict__ PH,
                                 const double2 *__restrict__ Cc, int coax_per_dir, double2 *__restrict__ T)
{
    extern __shared__ unsigned char smraw[];
    const int P2 = p * p, c = blockIdx.x, d = keys[c], j = blockIdx.y, rs = rot_size(pmax), w = 2 * pmax - 1;
    const int pi2 = pin * pin, po2 = pout * pout;
    double2 *sE = (double2 *)smraw, *sX = sE + P2, *sW1 = sX + P2, *sW2 = sW1 + P2, *sY = sW2 + P2, *sOne = sY + P2;
    for (int i = threadIdx.x; i < P2; i += blockDim.x) {
        sE[i] = make_double2(i == j ? 1.0 : 0.0, 0.0);
        sY[i] = make_double2(0.0, 0.0);
    }
    for (int i = threadIdx.x; i < w; i += blockDim.x) sOne[i] = make_double2(1.0, 0.0);
    __syncthreads();
    const double2 *cb = Cc + (coax_per_dir ? (size_t)c_dir_dist[d] * coax_size(p) : 0);
    rcr_block<double>(p, pmax, H + (size_t)d * rs, PH ? PH + (size_t)d * w : sOne, cb, sE, pin, sX, sW1, sW2, sY, pout);
    for (int i = threadIdx.x; i < po2; i += blockDim.x) T[((size_t)c * po2 + i) * pi2 + j] = sY[i];
}

int gen_dense_rcr(Plan *P, int l, int which, const int *keys, int nkeys, double2 *T)
{
    const LevelDev &L = P->lev[l];
    int p, pin, pout;
    const double *H;
    const double2 *PH, *Cc;
    if (which == PASS_M2L) {
        p = pin = pout = L.p;
        H = P->Hsr64;
        PH = nullptr;
        Cc = L.Csr64;
    } else {
        const int pp = P->lev[l - 1].p;  // the RCR order of M2M / L2L is the parent's
        p = pp;
        pin = which == PASS_M2M ? L.p : pp;
        pout = which == PASS_M2M ? pp : L.p;
        H = which == PASS_M2M ? P->Hss64 : P->Hrr64;
        PH = which == PASS_M2M ? P->PHss64 : P->PHrr64;
        Cc = L.Crr64;
    }
    size_t sm = ((size_t)5 * p * p + 2 * P->pmax) * sizeof(double2);
    if (sm > 48 * 1024) FMM_CUDA_TRY(cudaFuncSetAttribute(dense_rcr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    dense_rcr_kernel<<<dim3(nkeys, pin * pin), 128, sm, P->stream>>>(p, P->pmax, pin, pout, keys, H, PH, Cc,
                                                                   which == PASS_M2L ? 1 : 0, T);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}

int set_dir_dist(const int *dd, const int *hrep)
{
    FMM_CUDA_TRY(cudaMemcpyToSymbol(c_dir_dist, dd, sizeof(int) * NDIR));
    FMM_CUDA_TRY(cudaMemcpyToSymbol(c_dir_hrep, hrep, sizeof(int) * NDIR));
    return FMM_OK;
}

// The FP32 expansions hold rhs_cap32 right-hand sides, level by level ([box][rhs][p^2]).
static int ensure_rhs32(Plan *P, int nrhs)
{
    if (nrhs > P->x32_cap) {
        cudaFree(P->x32);
        P->x32 = nullptr;
        P->device_bytes -= sizeof(float2) * (size_t)P->nf * P->x32_cap;
        P->x32_cap = 0;
        FMM_CUDA_TRY(dev_alloc(P, (void **)&P->x32, sizeof(float2) * (size_t)P->nf * nrhs));
        P->x32_cap = nrhs;
    }
    if (nrhs <= P->rhs_cap32) return FMM_OK;
    drop_graph(P); // the captured passes address the old expansions
    for (int l = P->lmin; l <= P->lmax; l++) {
        LevelDev &L = P->lev[l];
        size_t n = (size_t)L.nb * L.p * L.p;
        cudaFree(L.Cm32);
        cudaFree(L.Dl32);
        L.Cm32 = nullptr;
        L.Dl32 = nullptr;
        P->device_bytes -= 2 * sizeof(float2) * n * P->rhs_cap32;
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Cm32, sizeof(float2) * n * nrhs));
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.Dl32, sizeof(float2) * n * nrhs));
    }
    P->rhs_cap32 = nrhs;
    P->buf_gen++;
    return FMM_OK;
}

int run_matvec(Plan *P, const double2 *x, double2 *y, int precision, int transpose, int nrhs)
{
    if (transpose && !P->nearT_beg) {
        fmm_set_error("transposed near field not built");
        return FMM_ERR_ARG;
    }
    if (precision == FMM_MIXED) {
        if (!P->U32) {
            fmm_set_error("%s", P->mixed_note);
            return FMM_ERR_ARG;
        }
        int st = ensure_rhs32(P, nrhs);
        if (st) return st;
        if (!P->opt.deterministic) return run_matvec_t<float>(P, x, y, transpose, nrhs);
        // the owner-computes kernels take one right-hand side
        for (int r = 0; r < nrhs; r++) {
            st = run_matvec_t<float>(P, x + (size_t)r * P->nf, y + (size_t)r * P->nf, transpose, 1);
            if (st) return st;
        }
        return FMM_OK;
    }
    bool ffm2l = false;
    if (precision == FMM_FLOAT2) {
        int st = ensure_ff(P);
        if (st) return st;
        ffm2l = P->ff_ready > 0;
    }
    for (int r = 0; r < nrhs; r++) {
        int st = run_matvec_t<double>(P, x + (size_t)r * P->nf, y + (size_t)r * P->nf, transpose, 1, ffm2l);
        if (st) return st;
    }
    return FMM_OK;
}

__global__ void gather_kernel(const double2 *src, const long long *perm, long long n, double2 *dst)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[perm[i]];
}

__global__ void conj_kernel(const double2 *x, double2 *y, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        y[i] = make_double2(x[i].x, -x[i].y);
}

void launch_conj(Plan *P, const double2 *x, double2 *y, size_t n)
{
    conj_kernel<<<(unsigned)std::min<size_t>((n + 255) / 256, 152 * 8), 256, 0, P->stream>>>(x, y, n);
}

// Near-field matrix transposed (CSR by source element), built on first use of the
// transposed operator: (A^T y)_j collects A_ij y_i over the targets i near j.
// The transpose of the near-field pattern: row beginnings tb and columns tc by source
// element, and for each transposed entry the position of the same pair in the forward CSR.
static int near_transpose_pattern(Plan *P, std::vector<int> &tb, std::vector<int> &tc, std::vector<long long> &perm)
{
    long long nnz = P->num_near;
    std::vector<int> beg(P->nf + 1), col(nnz);
    FMM_CUDA_TRY(cudaMemcpy(beg.data(), P->near_beg, sizeof(int) * (P->nf + 1), cudaMemcpyDeviceToHost));
    FMM_CUDA_TRY(cudaMemcpy(col.data(), P->near_col, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    std::vector<int> fill(P->nf, 0);
    tb.assign(P->nf + 1, 0);
    tc.resize(nnz);
    perm.resize(nnz);
    for (long long s = 0; s < nnz; s++) tb[col[s] + 1]++;
    for (int j = 0; j < P->nf; j++) tb[j + 1] += tb[j];
    for (int i = 0; i < P->nf; i++)
        for (int s = beg[i]; s < beg[i + 1]; s++) {
            int j = col[s];
            long long pos = tb[j] + fill[j]++;
            tc[pos] = i;
            perm[pos] = s;
        }
    return FMM_OK;
}

// valsT = the near-field values `vals` (forward CSR order) in the transposed CSR order
int near_transpose_values(Plan *P, const double2 *vals, double2 *valsT)
{
    std::vector<int> tb, tc;
    std::vector<long long> perm;
    int st = near_transpose_pattern(P, tb, tc, perm);
    if (st) return st;
    long long nnz = P->num_near;
    long long *perm_dev = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&perm_dev, sizeof(long long) * std::max<long long>(1, nnz)));
    FMM_CUDA_TRY(cudaMemcpy(perm_dev, perm.data(), sizeof(long long) * nnz, cudaMemcpyHostToDevice));
    gather_kernel<<<152 * 8, 256, 0, P->stream>>>(vals, perm_dev, nnz, valsT);
    FMM_CUDA_TRY(cudaGetLastError());
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    cudaFree(perm_dev);
    return FMM_OK;
}

int build_transpose(Plan *P)
{
    if (P->nearT_beg) return FMM_OK;
    long long nnz = P->num_near;
    std::vector<int> tb, tc;
    std::vector<long long> perm;
    int st = near_transpose_pattern(P, tb, tc, perm);
    if (st) return st;
    long long *perm_dev = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&perm_dev, sizeof(long long) * std::max<long long>(1, nnz)));
    FMM_CUDA_TRY(cudaMemcpy(perm_dev, perm.data(), sizeof(long long) * nnz, cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->nearT_beg, sizeof(int) * (P->nf + 1)));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->nearT_col, sizeof(int) * std::max<long long>(1, nnz)));
    FMM_CUDA_TRY(dev_alloc(P, (void **)&P->nearT64, sizeof(double2) * std::max<long long>(1, nnz)));
    FMM_CUDA_TRY(cudaMemcpy(P->nearT_beg, tb.data(), sizeof(int) * (P->nf + 1), cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(P->nearT_col, tc.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice));
    gather_kernel<<<152 * 8, 256, 0, P->stream>>>(P->near64, perm_dev, nnz, P->nearT64);
    FMM_CUDA_TRY(cudaGetLastError());
    if (P->U32) {
        FMM_CUDA_TRY(dev_alloc(P, (void **)&P->nearT32, sizeof(float2) * std::max<long long>(1, nnz)));
        int blocks = 152 * 8;
        to_float_kernel2<<<blocks, 256, 0, P->stream>>>((const double *)P->nearT64, (float *)P->nearT32, 2 * (size_t)nnz);
        FMM_CUDA_TRY(cudaGetLastError());
    }
    FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
    cudaFree(perm_dev);
    return FMM_OK;
}


} // namespace fmm
