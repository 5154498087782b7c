// Internal plan layout shared by the translation units of libfmmbem.
#pragma once
#include "fmm_common.cuh"
#include "octree_host.h"
#include "../../include/fmmbem.h"
#include <vector>

namespace fmm {

constexpr int NDIR = 316;      // M2L offsets (dx,dy,dz) in [-3,3]^3 with max |d| >= 2
constexpr int NDIST = 15;      // distinct squared lengths of those offsets
constexpr int MAX_TIMERS = 64;
constexpr int NSIDE = 8;      // side streams for the independent M2L passes (at most)

// Three-stage tensor-core form of one batched pass (tc_rcr3.cu): rotation blocks per
// polar-angle class and coaxial blocks per length class, split into TF32 hi/lo tiles; chunks,
// class orders and work items for items_nrhs right-hand sides; the W and Z scratch.
struct Tc3 {
    int on = 0, built = 0;
    int p = 0, pinr = 0, nq = 0, T = 0, nclsR = 0, nclsC = 0;
    std::vector<int> clsR_of_t, clsC_of_t;   // class of each translation (list order)
    std::vector<int4> hblkR, hblkC;          // per block: (table offset, K, Npad, valid N)
    long long strideR = 0, strideC = 0;      // floats per class
    float *opsR = nullptr, *opsC = nullptr;
    int4 *blkR = nullptr, *blkC = nullptr;
    int *t_dir = nullptr;                    // direction of each translation
    int items_nrhs = 0;
    std::vector<int> chunk_t0, it_beg;
    int4 *itR1 = nullptr, *itC = nullptr, *itR2 = nullptr;
    size_t capR1 = 0, capC = 0, capR2 = 0;
    int *listR = nullptr, *listC = nullptr;
    float2 *W = nullptr, *Z = nullptr;
    size_t scratch_cap = 0;
};

// A batched pass on the tensor cores as dense operators (tc_dense.cu).  M2L: one operator per
// class of the 316 directions with equal (dz, dx^2 + dy^2) -- equal polar angle and distance,
// so the class's directions differ only by their azimuthal phases, which the kernel applies
// to each row.  M2M / L2L: one operator per octant.  Real-embedded and split into TF32 hi/lo
// parts in the layout the MMA reads.
struct TcDense {
    int on = 0;                   // the pass runs on the tensor cores
    int pin = 0, pout = 0;        // source and destination orders
    int phased = 0;               // M2L: operators per class, phases per row
    int KC = 40, nch = 0, nhalf = 1, CH = 0, Nmma = 0;
    int res = 0;                  // the whole operator of a class stays in shared memory (small p)
    int ncls = 0;                 // operators
    std::vector<int> cls_of_dir;  // key (direction or octant) -> operator
    float *B = nullptr;           // [class][half][chunk][hi, lo][Nmma x KC core-matrix tile]
    size_t B_bytes = 0;
    int4 *items = nullptr;        // (class, first column, count, 0), 128 columns each
    size_t items_cap = 0;
    int *src = nullptr, *dst = nullptr, *dir = nullptr;  // the pass's translations in class order
    int n_items = 0, items_nrhs = 0;
};

// Work list of one batched translation pass: translations sorted by direction (src, dst,
// key_beg per direction, key_w = coaxial block per direction) and the device items
// (direction, first column, count, coaxial block) for items_nrhs right-hand sides, tc
// columns per item at most.
struct RcrList {
    int4 *items = nullptr;
    size_t items_cap = 0;
    int *src = nullptr, *dst = nullptr;
    std::vector<int> key_beg, key_w;
    std::vector<int> dst_rank;    // Morton rank of each translation's destination (list order)
    int ndst_rank = 0;            // boxes of the destination level
    int n_items = 0, items_nrhs = 0;
    int tc = 8, shc = 0;          // columns per item; rotation/coaxial blocks staged in shared memory
    int bal = 0;                  // balanced unit schedule (1, 2: two tile shapes; one-row units, boustrophedon order)
    Tc3 t3;                       // three-stage tensor-core form (used where t3.on)
    TcDense td;                   // dense tensor-core form (used where td.on)
};

// One batched FP32 translation pass as the tile kernels read it.
struct RcrPass {
    int p, pin, pout, atomic;        // RCR order, source order, destination order
    int nrhs, nsrc, ndst;            // right-hand sides; boxes per right-hand side in src and dst
    int hstride, phstride, phoff;    // per-direction strides of H and the phases; phase index m + phoff
    const int *hrep;                 // M2L: direction -> the direction whose H table it reads (null: its own)
    const float *H;
    const float2 *PH;
    const float2 *Cc;                // coaxial blocks, item.w selects one (stride coax_size(p))
    const float2 *src;               // [boxes][rhs][pin^2]
    float2 *dst;                     // [boxes][rhs][pout^2]
    const int4 *items;               // (direction, first, count, coaxial block) over columns e = t nrhs + r
    const int *g_src, *g_dst;        // source and destination box of translation t
};

struct LevelDev {
    int nb = 0, p = 0;
    int *parent = nullptr;        // [nb], index in level l-1 (l > lmin)
    unsigned char *octant = nullptr; // [nb], Morton digit of the box inside its parent
    int *child_beg = nullptr;     // [nb+1] CSR over level l+1
    int *child_list = nullptr;
    int *sr_beg = nullptr;        // [nb+1] CSR of M2L sources by destination
    int *sr_src = nullptr;        // source index in this level
    short *sr_dir = nullptr;      // direction index 0..315
    long long num_sr = 0;
    double2 *Cm64 = nullptr, *Dl64 = nullptr;
    // float-float M2L of the FP64 path (FMM_FLOAT2): coaxial tables and expansions, each
    // complex entry as (re hi, re lo, im hi, im lo)
    float4 *Csr_ff = nullptr, *Crr_ff = nullptr, *Cm_ff = nullptr, *Dl_ff = nullptr;
    float4 *CrrL_ff = nullptr;    // the L2L's float-float table where the expansions are scaled
    float2 *Cm32 = nullptr, *Dl32 = nullptr;
    double2 *Csr64 = nullptr;     // NDIST coaxial (S|R) blocks at order p
    float2 *Csr32 = nullptr;
    double2 *Crr64 = nullptr;     // coaxial (R|R) at order p_{l-1} for M2M into / L2L out of level l-1
    float2 *Crr32 = nullptr;      // FP32 (R|R) of the M2M (and of the L2L when not scaled)
    float2 *Crr32L = nullptr;     // FP32 (R|R) of the L2L in plans with scaled expansions
    // batched passes of the mixed path: M2L of this level, M2M (this level -> parents),
    // L2L (parents -> this level)
    RcrList m2l, m2m, l2l;
    int m2l_split = 1;            // FP64 M2L: CTAs per box (source runs), > 1 on levels with few boxes
};

struct Timer {
    const char *name;
    cudaEvent_t beg, end;
};

struct Plan {
    fmm_options opt;
    int nf = 0, nv = 0, lmin = 2, lmax = 0, pmax = 0, pleaf = 0;
    HostTree tree;
    std::vector<double> V;
    std::vector<int> F;
    LevelDev lev[FMM_MAX_LEVEL + 2];
    // direction tables
    int dir_slot[343];            // (dx+3)*49+(dy+3)*7+(dz+3) -> 0..315 or -1
    int dir_dist[NDIR];           // direction -> distance slot
    int dir_hrep[NDIR];           // direction -> the first direction of equal polar angle, whose
                                  // rotation table (bit-identical: the same acos(dz / |d|)) it reads
    int *hrep_dev = nullptr;      // dir_hrep on the device
    double *Hsr64 = nullptr, *Hss64 = nullptr, *Hrr64 = nullptr; // real rotation coefficients at pmax
    float *Hsr32 = nullptr, *Hss32 = nullptr, *Hrr32 = nullptr;
    double2 *PHsr64 = nullptr, *PHss64 = nullptr, *PHrr64 = nullptr; // e^{i m phi}, m = -(pmax-1)..pmax-1
    float2 *PHsr32 = nullptr, *PHss32 = nullptr, *PHrr32 = nullptr;
    // mesh and elements
    double *V_dev = nullptr;
    int *F_dev = nullptr;
    int *elem_leaf = nullptr;     // leaf index per element
    int *leaf_beg = nullptr, *leaf_elem = nullptr;
    double2 *U64 = nullptr, *Rv64 = nullptr;   // P2M / L2P element tables [nf * pleaf^2]
    float2 *U32 = nullptr, *Rv32 = nullptr;
    std::vector<int> near_box_beg, near_box; // leaf near boxes (I2 ∩ leaf set, I2 order) from near_boxes_kernel
    int *near_beg = nullptr, *near_col = nullptr;
    double2 *near64 = nullptr;
    float2 *near32 = nullptr;
    long long num_near = 0;
    int *nearT_beg = nullptr, *nearT_col = nullptr; // transposed near field, built on first use
    double2 *nearT64 = nullptr;
    float2 *nearT32 = nullptr;
    // work vectors
    double2 *xbuf = nullptr, *ybuf = nullptr;
    int nrhs_cap = 0;             // columns of xbuf / ybuf
    int rhs_cap32 = 1;            // right-hand sides the FP32 expansions (Cm32, Dl32) hold
    float2 *x32 = nullptr;        // the mixed matvec's input in FP32 ([rhs][element]), written by P2M
    int x32_cap = 0;              // columns of x32
    int buf_gen = 0;              // times Cm32 / Dl32 were reallocated (scenes hold their addresses)
    int scene_refs = 0;           // scenes built on this plan (it is not destroyed before them)
    cudaStream_t stream = nullptr;
    cudaStream_t side[NSIDE] = {};  // non-blocking side streams, forked from and joined to `stream`
    cudaEvent_t fork_ev = nullptr, join_ev[NSIDE] = {};
    cudaEvent_t m2l_ev[FMM_MAX_LEVEL + 2] = {}; // end of each level's M2L on its side stream
    int nside = 2;                // side streams in use (FMMBEM_M2L_STREAMS, 1..NSIDE)
    cudaGraphExec_t graph_exec = nullptr; // captured mixed translation passes for graph_nrhs columns
    int graph_nrhs = 0, graph_seen = 0;
    int *tc_err = nullptr;        // set by a tensor-core pass when one of its waits gives up
    float2 *tc_ones = nullptr;    // phases of the tensor-core passes without phases (all 1)
    float2 *Hall_ff = nullptr;    // float-float rotation tables (as the FP64 ones, (hi, lo) each)
    float4 *PHall_ff = nullptr;   // float-float phases
    int ff_ready = 0;             // 1 once the float-float tables exist, -1 where they cannot
    double *dsc_leaf_dev = nullptr; // degree scales d_n of the leaf level (plans with scaled expansions)
    double2 *m2l_part64 = nullptr; // FP64 M2L partial sums of split levels [run][box][p^2]
    size_t device_bytes = 0;
    char mixed_note[160] = "plan was created without build_mixed";
    // FP32 expansions scaled by degree (low k t): multipole d_n M_n, local L_n / d_n per level
    int scaled = 0;
    std::vector<double> dsc[FMM_MAX_LEVEL + 2];
    double setup_seconds = 0.0;
    // profiling
    int profiling = 0;
    Timer timers[MAX_TIMERS];
    Timer total;                  // whole matvec, recorded when profiling
    Timer phase;                  // the mixed translation passes as a whole (per-pass profiling)
    int have_total = 0, have_phase = 0;
    int ntimers = 0, timers_created = 0;
    // GMRES workspace
    double2 *gm_V = nullptr, *gm_w = nullptr, *gm_r = nullptr, *gm_x = nullptr, *gm_b = nullptr, *gm_d = nullptr;
    double2 *gm_dev_h = nullptr;
    double2 *gm_part = nullptr;    // per-block shares of the solver's dot products
    double *gm_alpha = nullptr;
    int gm_restart = 0, gm_cols = 0; // workspace for restart length and right-hand sides
};

// allocation tracking
cudaError_t dev_alloc(Plan *P, void **ptr, size_t bytes);
// raise func's dynamic shared-memory limit to at least bytes (thread-safe, never lowers it);
// *cache is the limit already set for func
int raise_smem_limit(const void *func, size_t bytes, size_t *cache);

// tables.cu
int gen_rotation_tables(Plan *P);
void rule_tables(double bary[2][48], double w[2][16], int n[2]);
void line_rule(int n, double *x, double *w);
int gen_coax_tables(Plan *P);
int gen_element_tables(Plan *P);
int gen_near_field(Plan *P);
int gen_operator_part(Plan *P, double2 bco, double2 cco, double2 *U, double2 *Rv_tmp, double2 *nearv);
int launch_far_field(Plan *P, const double2 *p, const double *pts, int npts, double2 *out);
int launch_plane_wave(Plan *P, const double *dir, double2 *rhs);
int gen_rotation_matrices_f32(const double *alpha, const double *beta, const double *gamma, int n, int p, float2 *host_out);
int gen_coax_matrices_f32(double k, const double *t, int n, int p, int sr, float2 *host_out);

// octree_gpu.cu
int build_lists(Plan *P);

// passes.cu
// y = A x (or A^T x) for nrhs columns of nf entries, device pointers
int run_matvec(Plan *P, const double2 *x, double2 *y, int precision, int transpose = 0, int nrhs = 1);
int build_transpose(Plan *P);
int near_transpose_values(Plan *P, const double2 *vals, double2 *valsT);
void launch_conj(Plan *P, const double2 *x, double2 *y, size_t n);
void drop_graph(Plan *P);

enum { PASS_M2M = 0, PASS_M2L = 1, PASS_L2L = 2 };
int launch_pass32(Plan *P, int l, int which, int nrhs, cudaStream_t st);
// the list and descriptor of a batched SIMT pass (items not set), or null where the level has none
RcrList *pass32_desc(Plan *P, int l, int which, int nrhs, RcrPass &ps);

// plan.cu: y = a x + b y over n entries
void launch_axpby(double a, const double2 *x, double b, double2 *y, size_t n, cudaStream_t st);

// tc_dense.cu
// Dense FP64 operators of a pass (passes.cu): T[c][i][j] (pout^2 x pin^2), the RCR translation
// of key keys[c] applied to the unit source e_j; M2L without its azimuthal phases.
int gen_dense_rcr(Plan *P, int l, int which, const int *keys, int nkeys, double2 *T);
// Classes of a pass's keys with one rotation: M2L directions of equal (dz, dx^2 + dy^2), M2M /
// L2L octants of equal z bit.  cls[key] = class, rep[class] = its first key.  (tc_rcr3.cu)
void direction_classes(const Plan *P, int which, int nkeys, std::vector<int> &cls, std::vector<int> &rep);
int tune_tc_dense(Plan *P);
int launch_tc_dense(Plan *P, int l, int which, int nrhs, cudaStream_t st);
int check_tc_error(Plan *P);

// tc_rcr3.cu
int build_tc3(Plan *P, int l, int which);
int launch_tc3_pass(Plan *P, int l, int which, int nrhs, cudaStream_t st);
int tune_tc3(Plan *P);

// batched.cu
int build_rcr_lists(Plan *P);
int tune_rcr_tiles(Plan *P);
size_t rcr_tile_smem(int p, int tc, int shc);
extern const size_t MAX_TILE_SMEM;
int launch_rcr_pass(RcrList &Lst, RcrPass ps, cudaStream_t st);
// work items (direction, first column, count, coaxial block) of a list for one right-hand side
void rcr_list_items(const RcrList &Lst, std::vector<int4> &out);
// items for nrhs columns in tiles of `width`, ordered by destination Morton ranges where the
// pass's expansions (ws_bytes) exceed L2
void build_items(const RcrList &Lst, int nrhs, int width, size_t ws_bytes, bool coax_w, std::vector<int4> &items);
// persistent work-queue launch over many passes of one tile shape (tc, shc, schedule bal as in
// RcrList); smem for the largest order among them; grid from rcr_queue_prepare (resident CTAs)
int rcr_queue_prepare(int tc, int shc, int bal, size_t smem, int nwork, int *grid);
// (*nwork: the number of items, read on the device)
int launch_rcr_queue(int tc, int shc, int bal, const RcrPass *passes, const int *work_pass, const int4 *work_item,
                     const int *nwork, int *head, size_t smem, int grid, cudaStream_t st);

} // namespace fmm
