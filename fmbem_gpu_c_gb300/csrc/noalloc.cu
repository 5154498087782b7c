// fmm_coax_matrices_noalloc: the FP64 coaxial (R|R) / (S|R) matrix generator, without any
// device allocation.
//
// The plan builder and the reference-compatible generators (genRRSparseCoaxTransMat,
// genSRSparseCoaxTransMat) allocate a scratch buffer with cudaMalloc for the coaxial
// recurrence.  Some callers cannot allow that:
// - an application that gives all device memory to its own pool and forbids libraries to
//   allocate behind it;
// - a loop with timing limits, where cudaMalloc/cudaFree would synchronise the device;
// - a caller that only holds device buffers it was handed.
// This entry point works only on the caller's device buffers.  Its scratch is a fixed array
// in this file that every GPU using the library holds for the life of the process.
#include <atomic>

#include "fmm_common.cuh"
#include "../../include/fmmbem.h"

// Scratch of the recurrence: p (2p-1) p complex entries per matrix, at most 2^19 entries
// (8 MiB) for one call.
#define FMM_NOALLOC_SCRATCH_ENTRIES (1 << 19)
static __device__ __align__(256) double2 g_noalloc_scratch[FMM_NOALLOC_SCRATCH_ENTRIES];

// Device address of g_noalloc_scratch on each device.  The host-side symbol is only a
// handle; cudaGetSymbolAddress gives the address, once per device, with that device current.
static std::atomic<double2 *> g_noalloc_addr[128];

// Matrices whose k t falls outside (0, FMM_NOALLOC_MAX_KT] are written as NaN: the Bessel
// start index grows with k t, so an unchecked value could keep one thread busy for seconds.
#define FMM_NOALLOC_MAX_KT 1.0e5

// The coaxial recurrence of sparseCoaxTransMatGen (reference translation.cu:678-771) from the
// initial column of srCoaxTransMatsInit / rrCoaxTransMatsInit, one CTA of 256 threads per
// matrix, FP64 throughout: the same arithmetic as the plan builder's generator.  Every scratch
// entry the recurrence reads is written earlier in the same launch (the first column, then
// the diagonal columns m = n, then columns n > m in increasing n), so the scratch needs no
// clearing before a call.  Output: the sparse layout of sparseCoaxTransSize (one (p-m)^2
// column-major block per m).
__global__ void coax_noalloc_kernel(double k, const double *__restrict__ tvals, int p, int sr, double2 *scratch,
                                    double2 *out)
{
    int mat = blockIdx.x;
    double kt = k * tvals[mat];
    int R = 2 * p - 1;
    double2 *E = scratch + (size_t)mat * p * R * p;
    double2 *C = out + (size_t)mat * coax_size(p);
    if (!(kt > 0.0 && kt <= FMM_NOALLOC_MAX_KT)) { // uniform over the CTA
        for (int i = threadIdx.x; i < coax_size(p); i += blockDim.x) C[i] = make_double2(nan(""), nan(""));
        return;
    }
#define EE(m, np, n) E[((size_t)(m) * R + (np)) * p + (n)]
    extern __shared__ double bessel[];
    double *jn = bessel, *yn = bessel + R;
    if (threadIdx.x == 0) {
        sph_jn_array(R, kt, jn);
        if (sr) sph_yn_array(R, kt, yn);
    }
    __syncthreads();
    // column n = 0 of block m = 0: (-1)^n' sqrt(2n'+1) j_n'(kt)  [+ i y_n'(kt) for (S|R)]
    for (int np = threadIdx.x; np < R; np += blockDim.x) {
        double f = ((np & 1) ? -1.0 : 1.0) * sqrt(2.0 * np + 1.0);
        EE(0, np, 0) = make_double2(f * jn[np], sr ? f * yn[np] : 0.0);
    }
    __syncthreads();
    // diagonal columns n = m of block m+1 from block m (the b-coefficient relation)
    for (int m = 0; m + 1 <= p - 1; m++) {
        double den = coefB(m + 1, -m - 1);
        for (int np = m + 1 + threadIdx.x; np <= 2 * p - 2 - (m + 1); np += blockDim.x) {
            double c0 = coefB(np, -m - 1) / den, c1 = coefB(np + 1, m) / den;
            double2 lo = EE(m, np - 1, m), hi = EE(m, np + 1, m);
            EE(m + 1, np, m + 1) = make_double2(c0 * lo.x - c1 * hi.x, c0 * lo.y - c1 * hi.y);
        }
        __syncthreads();
    }
    // columns n+1 > m of block m from columns n and n-1 (the a-coefficient relation); one warp
    // owns a block, its lanes split n'
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int m = warp; m <= p - 2; m += nw) {
        for (int n = m; n + 1 <= p - 1; n++) {
            double den = coefA(n, m);
            for (int np = m + lane; np <= 2 * p - 2 - (n + 1); np += 32) {
                double c0 = coefA(np - 1, m) / den, c1 = coefA(np, m) / den, c2 = coefA(n - 1, m) / den;
                double2 e0 = (np - 1 >= m) ? EE(m, np - 1, n) : make_double2(0.0, 0.0);
                double2 e1 = EE(m, np + 1, n);
                double2 e2 = (n - 1 >= m) ? EE(m, np, n - 1) : make_double2(0.0, 0.0);
                EE(m, np, n + 1) = make_double2(c0 * e0.x - c1 * e1.x + c2 * e2.x, c0 * e0.y - c1 * e1.y + c2 * e2.y);
            }
            __syncwarp();
        }
    }
    __syncthreads();
    // (R|R) entries with n' < n from the exact symmetry (R|R)_{n'n} = (-1)^{n+n'} (R|R)_{nn'}:
    // the recurrence loses them to cancellation at small k t, as the plan builder's generator
    // describes
    for (int m = 0; m < p; m++) {
        int sz = p - m, off = coax_off(p, m);
        for (int i = threadIdx.x; i < sz * sz; i += blockDim.x) {
            int a = i % sz, b = i / sz;
            if (!sr && a < b) {
                double2 v = EE(m, m + b, m + a);
                double sg = ((a + b) & 1) ? -1.0 : 1.0;
                C[off + i] = make_double2(sg * v.x, sg * v.y);
            } else {
                C[off + i] = EE(m, m + a, m + b);
            }
        }
    }
#undef EE
}

static bool device_buffer_of(const void *ptr, int dev)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

extern "C" int fmm_coax_matrices_noalloc(double k, const double *t, int n, int p, int sr, cuDoubleComplex *out,
                                         cudaStream_t stream)
{
    if (!(k > 0.0) || n < 1 || p < 1 || p > 64 || !t || !out) {
        fmm_set_error("fmm_coax_matrices_noalloc: invalid argument (need k > 0, n >= 1, 1 <= p <= 64, "
                      "non-null t and out)");
        return FMM_ERR_ARG;
    }
    size_t need = (size_t)n * p * (2 * p - 1) * p;
    if (need > (size_t)FMM_NOALLOC_SCRATCH_ENTRIES) {
        fmm_set_error("fmm_coax_matrices_noalloc: n p (2p-1) p = %zu entries exceeds the fixed scratch of %d entries "
                      "(8 MiB); pass the distances in smaller batches",
                      need, FMM_NOALLOC_SCRATCH_ENTRIES);
        return FMM_ERR_ARG;
    }
    int dev = 0;
    FMM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) {
        fmm_set_error("fmm_coax_matrices_noalloc: device ordinal %d beyond the 128 this entry point supports", dev);
        return FMM_ERR_ARG;
    }
    if (!device_buffer_of(t, dev) || !device_buffer_of(out, dev)) {
        fmm_set_error("fmm_coax_matrices_noalloc: t and out must be device (or managed) memory of the current device");
        return FMM_ERR_ARG;
    }
    double2 *scratch = g_noalloc_addr[dev].load();
    if (!scratch) {
        FMM_CUDA_TRY(cudaGetSymbolAddress((void **)&scratch, g_noalloc_scratch));
        g_noalloc_addr[dev].store(scratch);
    }
    coax_noalloc_kernel<<<n, 256, sizeof(double) * 2 * (2 * p - 1), stream>>>(k, t, p, sr ? 1 : 0, scratch,
                                                                             (double2 *)out);
    FMM_CUDA_TRY(cudaGetLastError());
    return FMM_OK;
}
