// The FP64 coaxial translation matrix of one translation length, computed by one CTA.
//
// Shared by the plan builder's generator (coax_kernel, tables.cu) and the no-allocation
// entry point (coax_noalloc_kernel, noalloc.cu), so that both produce the same matrices from
// one piece of code.
//
// The recurrences are those of sparseCoaxTransMatGen (reference translation.cu:678-771),
// started from the initial column of srCoaxTransMatsInit / rrCoaxTransMatsInit
// (translation.cu:919-949, 555-585): column n = 0 of block m = 0 is
// (-1)^n' sqrt(2n'+1) j_n'(kt) [+ i y_n'(kt) for (S|R)]; the diagonal columns n = m of block
// m+1 follow from block m by the b-coefficient relation, and the columns n+1 > m of block m
// from columns n and n-1 by the a-coefficient relation.  Each matrix needs an "enlarged"
// scratch of p (2p-1) p entries (degrees n' up to 2p-2), here compact [m][n'][n].  Every
// scratch entry the recurrence reads is written earlier in the same call, so the scratch
// needs no clearing.  The result goes to C in the sparse layout of sparseCoaxTransSize (one
// (p-m)^2 column-major block per m, entry (n', n)).
#pragma once
#include "fmm_common.cuh"

// Called by every thread of the CTA (it synchronises the CTA).  E: this matrix's scratch of
// p (2p-1) p entries; C: its output of coax_size(p) entries; jn, yn: shared arrays of 2p-1
// doubles each (yn is used only for (S|R)).
__device__ __forceinline__ void coax_matrix_cta(double kt, int p, int sr, double2 *E, double2 *C, double *jn,
                                                double *yn)
{
    const int R = 2 * p - 1;
#define EE(m, np, n) E[((size_t)(m) * R + (np)) * p + (n)]
    if (threadIdx.x == 0) {
        sph_jn_array(R, kt, jn);
        if (sr) sph_yn_array(R, kt, yn);
    }
    __syncthreads();
    for (int np = threadIdx.x; np < R; np += blockDim.x) {
        double f = ((np & 1) ? -1.0 : 1.0) * sqrt(2.0 * np + 1.0);
        EE(0, np, 0) = make_double2(f * jn[np], sr ? f * yn[np] : 0.0);
    }
    __syncthreads();
    for (int m = 0; m + 1 <= p - 1; m++) {
        double den = coefB(m + 1, -m - 1);
        for (int np = m + 1 + threadIdx.x; np <= 2 * p - 2 - (m + 1); np += blockDim.x) {
            double c0 = coefB(np, -m - 1) / den, c1 = coefB(np + 1, m) / den;
            double2 lo = EE(m, np - 1, m), hi = EE(m, np + 1, m);
            EE(m + 1, np, m + 1) = make_double2(c0 * lo.x - c1 * hi.x, c0 * lo.y - c1 * hi.y);
        }
        __syncthreads();
    }
    // one warp owns block m; its lanes split n'
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
            // the next column reads what other lanes of this warp wrote to global memory
            __threadfence_block();
            __syncwarp();
        }
    }
    __syncthreads();
    // (R|R): the recurrence forms the entries with n' < n, which are tiny at small k t, by
    // cancellation and loses them (absolute error ~1e-16 against values down to (kt)^(n-n'));
    // an L2L multiplies them by the large high-degree local coefficients.  They are taken from
    // the exact coaxial symmetry (R|R)_{n'n} = (-1)^{n+n'} (R|R)_{nn'}, whose n' > n side the
    // recurrence forms to full relative accuracy.  (S|R) is accurate in both triangles.
    for (int m = 0; m < p; m++) {
        int sz = p - m, off = coax_off(p, m);
        for (int i = threadIdx.x; i < sz * sz; i += blockDim.x) {
            int a = i % sz, b = i / sz; // a = n'-m, b = n-m
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
