// Host-only check of the work-item builder of the batched translation passes (build_items in
// batched.cu): a synthetic list of translations grouped by direction, each direction's
// translations sorted by the Morton rank of their destination, cut into items for several
// right-hand sides, with and without the destination ranges that a working set beyond the L2
// budget brings.  Prints the items as JSON for the test to check.  Nothing runs on a GPU.
#include "../../fmbem_gpu_c_gb300/csrc/batched.cu"
#include <cstdarg>
#include <cstdio>
#include <random>

// the three functions batched.cu takes from the rest of the library, unused here
namespace fmm {
int raise_smem_limit(const void *, size_t, size_t *) { return 0; }
cudaError_t dev_alloc(Plan *, void **, size_t) { return cudaErrorNotSupported; }
int launch_pass32(Plan *, int, int, int, cudaStream_t) { return 0; }
} // namespace fmm
void fmm_set_error(const char *, ...) {}

int main()
{
    std::mt19937 g(3);
    fmm::RcrList L;
    const int nkeys = 12, ndst = 200;
    L.key_beg.assign(1, 0);
    for (int d = 0; d < nkeys; d++) {
        int cnt = (int)(g() % 70);
        std::vector<int> r(cnt);
        for (int &v : r) v = (int)(g() % ndst);
        std::sort(r.begin(), r.end());
        L.dst_rank.insert(L.dst_rank.end(), r.begin(), r.end());
        L.key_beg.push_back(L.key_beg.back() + cnt);
        L.key_w.push_back(d % 5);
    }
    L.ndst_rank = ndst;
    printf("{\"key_beg\": [");
    for (size_t i = 0; i < L.key_beg.size(); i++) printf("%s%d", i ? ", " : "", L.key_beg[i]);
    printf("], \"dst_rank\": [");
    for (size_t i = 0; i < L.dst_rank.size(); i++) printf("%s%d", i ? ", " : "", L.dst_rank[i]);
    printf("], \"ndst\": %d, \"cases\": [", ndst);
    struct Case { int nrhs, width; size_t ws; };
    const Case cases[] = {{1, 8, 0}, {3, 16, 0}, {3, 16, (size_t)200 << 20}, {5, 128, (size_t)1 << 30}};
    for (int c = 0; c < 4; c++) {
        std::vector<int4> items;
        fmm::build_items(L, cases[c].nrhs, cases[c].width, cases[c].ws, c % 2 == 0, items);
        printf("%s{\"nrhs\": %d, \"width\": %d, \"ws\": %zu, \"coax_w\": %d, \"items\": [", c ? ", " : "", cases[c].nrhs,
               cases[c].width, cases[c].ws, c % 2 == 0 ? 1 : 0);
        for (size_t i = 0; i < items.size(); i++)
            printf("%s[%d, %d, %d, %d]", i ? ", " : "", items[i].x, items[i].y, items[i].z, items[i].w);
        printf("]}");
    }
    printf("], \"key_w\": [");
    for (int d = 0; d < nkeys; d++) printf("%s%d", d ? ", " : "", L.key_w[d]);
    printf("]}\n");
    return 0;
}
