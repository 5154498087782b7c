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

#include "coax_recurrence.cuh"
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

// One CTA of 256 threads per matrix, FP64 throughout: the plan builder's generator
// (coax_matrix_cta, coax_recurrence.cuh, after sparseCoaxTransMatGen, reference
// translation.cu:678-771) on a slice of the fixed scratch.  The recurrence writes every
// scratch entry before it reads it, so nothing has to be cleared between calls.  Output: the
// sparse layout of sparseCoaxTransSize (one (p-m)^2 column-major block per m).
__global__ void coax_noalloc_kernel(double k, const double *__restrict__ tvals, int p, int sr, double2 *scratch,
                                    double2 *out)
{
    int mat = blockIdx.x;
    double kt = k * tvals[mat];
    double2 *C = out + (size_t)mat * coax_size(p);
    if (!(kt > 0.0 && kt <= FMM_NOALLOC_MAX_KT)) { // uniform over the CTA
        for (int i = threadIdx.x; i < coax_size(p); i += blockDim.x) C[i] = make_double2(nan(""), nan(""));
        return;
    }
    extern __shared__ double bessel[];
    coax_matrix_cta(kt, p, sr, scratch + (size_t)mat * p * (2 * p - 1) * p, C, bessel, bessel + 2 * p - 1);
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
    // an error left pending by the caller's own earlier work is reported as such, not as a
    // failure of this launch
    cudaError_t prior = cudaPeekAtLastError();
    if (prior != cudaSuccess) {
        fmm_set_error("fmm_coax_matrices_noalloc: a CUDA error from earlier work is pending (%s); nothing was launched",
                      cudaGetErrorString(prior));
        return FMM_ERR_CUDA;
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
