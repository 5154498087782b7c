// Interaction lists on the GPU.  The reference builds them by set algebra in O(B^2 * 189)
// (FMMLevelSetNumSR, octree.c:908-919; genSRIdxArrs, translation.cu:2848-2922); here one
// thread per box enumerates the I4 candidates in the reference's order (children of the
// parent's neighbours in x-y-z order, then of the parent, octree.c:517-543) and looks each
// up in the sorted level set, so counts and lists equal I4 ∩ level set element for element.
#include "plan.h"
#include <algorithm>
#include <numeric>

namespace fmm {

__device__ __forceinline__ void d_box_xyz(long long num, int l, int *x, int *y, int *z)
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

__device__ __forceinline__ long long d_box_num(int x, int y, int z, int l)
{
    long long key = 0;
    for (int b = l - 1; b >= 0; b--) key = key * 8 + 4 * ((x >> b) & 1) + 2 * ((y >> b) & 1) + ((z >> b) & 1);
    return key;
}

__device__ __forceinline__ int d_lookup(const long long *skey, const int *sidx, int n, long long key)
{
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        long long v = skey[mid];
        if (v == key) return sidx[mid];
        if (v < key) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

// pass 0 counts, pass 1 writes (sources and direction index)
__global__ void sr_lists_kernel(const long long *boxes, const long long *skey, const int *sidx, int nb, int l,
                                const int *dir_slot, int pass, int *count, const int *beg, int *src, short *dir)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    int x, y, z;
    d_box_xyz(boxes[i], l, &x, &y, &z);
    int X = x >> 1, Y = y >> 1, Z = z >> 1, ptop = (1 << (l - 1)) - 1;
    int xl = X > 0 ? X - 1 : 0, xh = X < ptop ? X + 1 : ptop;
    int yl = Y > 0 ? Y - 1 : 0, yh = Y < ptop ? Y + 1 : ptop;
    int zl = Z > 0 ? Z - 1 : 0, zh = Z < ptop ? Z + 1 : ptop;
    int cnt = 0, pos = pass ? beg[i] : 0;
    for (int stage = 0; stage < 2; stage++)
        for (int px = xl; px <= xh; px++)
            for (int py = yl; py <= yh; py++)
                for (int pz = zl; pz <= zh; pz++) {
                    bool self = (px == X && py == Y && pz == Z);
                    if ((stage == 0) == self) continue;
                    for (int c = 0; c < 8; c++) {
                        int cx = 2 * px + ((c >> 2) & 1), cy = 2 * py + ((c >> 1) & 1), cz = 2 * pz + (c & 1);
                        int ax = cx - x, ay = cy - y, az = cz - z;
                        if (ax >= -1 && ax <= 1 && ay >= -1 && ay <= 1 && az >= -1 && az <= 1) continue;
                        int s = d_lookup(skey, sidx, nb, d_box_num(cx, cy, cz, l));
                        if (s < 0) continue;
                        if (pass) {
                            src[pos + cnt] = s;
                            // translation vector = destination - source
                            dir[pos + cnt] = (short)dir_slot[(3 - ax) * 49 + (3 - ay) * 7 + (3 - az)];
                        }
                        cnt++;
                    }
                }
    if (!pass) count[i] = cnt;
}

// leaf near lists: I2 ∩ leaf set (octree.c:497-505, 425-437) in I2's order, up to 27
// boxes: the neighbours in x-y-z order, then the box itself (I2 appends it after neighbors)
__global__ void near_boxes_kernel(const long long *boxes, const long long *skey, const int *sidx, int nb, int l,
                                  int *nbr, int *nnb)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    int x, y, z;
    d_box_xyz(boxes[i], l, &x, &y, &z);
    int top = (1 << l) - 1, cnt = 0;
    int xl = x > 0 ? x - 1 : 0, xh = x < top ? x + 1 : top;
    int yl = y > 0 ? y - 1 : 0, yh = y < top ? y + 1 : top;
    int zl = z > 0 ? z - 1 : 0, zh = z < top ? z + 1 : top;
    for (int px = xl; px <= xh; px++)
        for (int py = yl; py <= yh; py++)
            for (int pz = zl; pz <= zh; pz++) {
                if (px == x && py == y && pz == z) continue;
                int s = d_lookup(skey, sidx, nb, d_box_num(px, py, pz, l));
                if (s >= 0) nbr[27 * i + cnt++] = s;
            }
    nbr[27 * i + cnt++] = i;
    nnb[i] = cnt;
}

__global__ void near_count_kernel(const int *elem_leaf, int nf, const int *nbr, const int *nnb, const int *leaf_beg,
                                  int *count)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nf) return;
    int b = elem_leaf[e], c = 0;
    for (int t = 0; t < nnb[b]; t++) {
        int q = nbr[27 * b + t];
        c += leaf_beg[q + 1] - leaf_beg[q];
    }
    count[e] = c;
}

__global__ void near_fill_kernel(const int *elem_leaf, int nf, const int *nbr, const int *nnb, const int *leaf_beg,
                                 const int *leaf_elem, const int *near_beg, int *near_col)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nf) return;
    int b = elem_leaf[e], pos = near_beg[e];
    for (int t = 0; t < nnb[b]; t++) {
        int q = nbr[27 * b + t];
        for (int s = leaf_beg[q]; s < leaf_beg[q + 1]; s++) near_col[pos++] = leaf_elem[s];
    }
}

static int sorted_lookup_arrays(const std::vector<long long> &set, long long **skey, int **sidx, long long **boxes)
{
    std::vector<std::pair<long long, int>> kv(set.size());
    for (size_t i = 0; i < set.size(); i++) kv[i] = {set[i], (int)i};
    std::sort(kv.begin(), kv.end());
    std::vector<long long> k(set.size());
    std::vector<int> ix(set.size());
    for (size_t i = 0; i < set.size(); i++) { k[i] = kv[i].first; ix[i] = kv[i].second; }
    FMM_CUDA_TRY(cudaMalloc(skey, sizeof(long long) * std::max<size_t>(1, set.size())));
    FMM_CUDA_TRY(cudaMalloc(sidx, sizeof(int) * std::max<size_t>(1, set.size())));
    FMM_CUDA_TRY(cudaMalloc(boxes, sizeof(long long) * std::max<size_t>(1, set.size())));
    FMM_CUDA_TRY(cudaMemcpy(*skey, k.data(), sizeof(long long) * set.size(), cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(*sidx, ix.data(), sizeof(int) * set.size(), cudaMemcpyHostToDevice));
    FMM_CUDA_TRY(cudaMemcpy(*boxes, set.data(), sizeof(long long) * set.size(), cudaMemcpyHostToDevice));
    return FMM_OK;
}

int build_lists(Plan *P)
{
    int *dir_slot_dev = nullptr;
    FMM_CUDA_TRY(cudaMalloc(&dir_slot_dev, sizeof(int) * 343));
    FMM_CUDA_TRY(cudaMemcpy(dir_slot_dev, P->dir_slot, sizeof(int) * 343, cudaMemcpyHostToDevice));
    for (int l = P->lmin; l <= P->lmax; l++) {
        LevelDev &L = P->lev[l];
        const std::vector<long long> &set = P->tree.sets[l];
        long long *skey, *boxes;
        int *sidx;
        int st = sorted_lookup_arrays(set, &skey, &sidx, &boxes);
        if (st) return st;
        int nb = L.nb, blocks = (nb + 127) / 128;
        int *count = nullptr;
        FMM_CUDA_TRY(cudaMalloc(&count, sizeof(int) * nb));
        sr_lists_kernel<<<blocks, 128, 0, P->stream>>>(boxes, skey, sidx, nb, l, dir_slot_dev, 0, count, nullptr, nullptr, nullptr);
        FMM_CUDA_TRY(cudaGetLastError());
        std::vector<int> hc(nb), hb(nb + 1, 0);
        FMM_CUDA_TRY(cudaMemcpyAsync(hc.data(), count, sizeof(int) * nb, cudaMemcpyDeviceToHost, P->stream));
        FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
        for (int i = 0; i < nb; i++) hb[i + 1] = hb[i] + hc[i];
        L.num_sr = hb[nb];
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.sr_beg, sizeof(int) * (nb + 1)));
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.sr_src, sizeof(int) * std::max<long long>(1, L.num_sr)));
        FMM_CUDA_TRY(dev_alloc(P, (void **)&L.sr_dir, sizeof(short) * std::max<long long>(1, L.num_sr)));
        FMM_CUDA_TRY(cudaMemcpy(L.sr_beg, hb.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice));
        sr_lists_kernel<<<blocks, 128, 0, P->stream>>>(boxes, skey, sidx, nb, l, dir_slot_dev, 1, nullptr, L.sr_beg, L.sr_src, L.sr_dir);
        FMM_CUDA_TRY(cudaGetLastError());
        // parents, octants and children from the key arithmetic (host, linear)
        if (l > P->lmin) {
            const std::vector<long long> &pset = P->tree.sets[l - 1];
            std::vector<std::pair<long long, int>> kv(pset.size());
            for (size_t i = 0; i < pset.size(); i++) kv[i] = {pset[i], (int)i};
            std::sort(kv.begin(), kv.end());
            std::vector<int> par(nb);
            std::vector<unsigned char> oct(nb);
            for (int i = 0; i < nb; i++) {
                auto it = std::lower_bound(kv.begin(), kv.end(), std::make_pair(set[i] / 8, -1));
                par[i] = it->second;
                oct[i] = (unsigned char)(set[i] & 7);
            }
            int np = (int)pset.size();
            std::vector<int> cb(np + 1, 0), cl(nb), fill(np, 0);
            for (int i = 0; i < nb; i++) cb[par[i] + 1]++;
            for (int i = 0; i < np; i++) cb[i + 1] += cb[i];
            for (int i = 0; i < nb; i++) cl[cb[par[i]] + fill[par[i]]++] = i;
            FMM_CUDA_TRY(dev_alloc(P, (void **)&L.parent, sizeof(int) * nb));
            FMM_CUDA_TRY(dev_alloc(P, (void **)&L.octant, nb));
            FMM_CUDA_TRY(cudaMemcpy(L.parent, par.data(), sizeof(int) * nb, cudaMemcpyHostToDevice));
            FMM_CUDA_TRY(cudaMemcpy(L.octant, oct.data(), nb, cudaMemcpyHostToDevice));
            LevelDev &PL = P->lev[l - 1];
            FMM_CUDA_TRY(dev_alloc(P, (void **)&PL.child_beg, sizeof(int) * (np + 1)));
            FMM_CUDA_TRY(dev_alloc(P, (void **)&PL.child_list, sizeof(int) * nb));
            FMM_CUDA_TRY(cudaMemcpy(PL.child_beg, cb.data(), sizeof(int) * (np + 1), cudaMemcpyHostToDevice));
            FMM_CUDA_TRY(cudaMemcpy(PL.child_list, cl.data(), sizeof(int) * nb, cudaMemcpyHostToDevice));
        }
        if (l == P->lmax) {
            // elements grouped by leaf box
            std::vector<int> lb(nb + 1, 0), le(P->nf), fill(nb, 0);
            for (int e = 0; e < P->nf; e++) lb[P->tree.elem_leaf[e] + 1]++;
            for (int i = 0; i < nb; i++) lb[i + 1] += lb[i];
            for (int e = 0; e < P->nf; e++) le[lb[P->tree.elem_leaf[e]] + fill[P->tree.elem_leaf[e]]++] = e;
            FMM_CUDA_TRY(dev_alloc(P, (void **)&P->leaf_beg, sizeof(int) * (nb + 1)));
            FMM_CUDA_TRY(dev_alloc(P, (void **)&P->leaf_elem, sizeof(int) * P->nf));
            FMM_CUDA_TRY(cudaMemcpy(P->leaf_beg, lb.data(), sizeof(int) * (nb + 1), cudaMemcpyHostToDevice));
            FMM_CUDA_TRY(cudaMemcpy(P->leaf_elem, le.data(), sizeof(int) * P->nf, cudaMemcpyHostToDevice));
            int *nbr = nullptr, *nnb = nullptr, *ncount = nullptr;
            FMM_CUDA_TRY(cudaMalloc(&nbr, sizeof(int) * 27 * nb));
            FMM_CUDA_TRY(cudaMalloc(&nnb, sizeof(int) * nb));
            FMM_CUDA_TRY(cudaMalloc(&ncount, sizeof(int) * P->nf));
            near_boxes_kernel<<<blocks, 128, 0, P->stream>>>(boxes, skey, sidx, nb, l, nbr, nnb);
            near_count_kernel<<<(P->nf + 255) / 256, 256, 0, P->stream>>>(P->elem_leaf, P->nf, nbr, nnb, P->leaf_beg, ncount);
            FMM_CUDA_TRY(cudaGetLastError());
            std::vector<int> nc(P->nf), nbeg(P->nf + 1, 0), hnbr((size_t)27 * nb), hnnb(nb);
            FMM_CUDA_TRY(cudaMemcpyAsync(nc.data(), ncount, sizeof(int) * P->nf, cudaMemcpyDeviceToHost, P->stream));
            FMM_CUDA_TRY(cudaMemcpyAsync(hnbr.data(), nbr, sizeof(int) * 27 * nb, cudaMemcpyDeviceToHost, P->stream));
            FMM_CUDA_TRY(cudaMemcpyAsync(hnnb.data(), nnb, sizeof(int) * nb, cudaMemcpyDeviceToHost, P->stream));
            FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
            // the box-level lists, kept on the host for fmm_plan_near_lists
            P->near_box_beg.assign(nb + 1, 0);
            P->near_box.clear();
            for (int i = 0; i < nb; i++) {
                P->near_box.insert(P->near_box.end(), hnbr.begin() + 27 * (size_t)i, hnbr.begin() + 27 * (size_t)i + hnnb[i]);
                P->near_box_beg[i + 1] = (int)P->near_box.size();
            }
            long long tot = 0;
            for (int e = 0; e < P->nf; e++) { tot += nc[e]; nbeg[e + 1] = (int)tot; }
            P->num_near = tot;
            FMM_CUDA_TRY(dev_alloc(P, (void **)&P->near_beg, sizeof(int) * (P->nf + 1)));
            FMM_CUDA_TRY(dev_alloc(P, (void **)&P->near_col, sizeof(int) * std::max<long long>(1, tot)));
            FMM_CUDA_TRY(cudaMemcpy(P->near_beg, nbeg.data(), sizeof(int) * (P->nf + 1), cudaMemcpyHostToDevice));
            near_fill_kernel<<<(P->nf + 255) / 256, 256, 0, P->stream>>>(P->elem_leaf, P->nf, nbr, nnb, P->leaf_beg,
                                                                          P->leaf_elem, P->near_beg, P->near_col);
            FMM_CUDA_TRY(cudaGetLastError());
            FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
            cudaFree(nbr); cudaFree(nnb); cudaFree(ncount);
        }
        FMM_CUDA_TRY(cudaStreamSynchronize(P->stream));
        cudaFree(count); cudaFree(skey); cudaFree(sidx); cudaFree(boxes);
    }
    cudaFree(dir_slot_dev);
    return FMM_OK;
}

} // namespace fmm
