/* fmmbem.h -- C ABI of the GB300 FMM-BEM Helmholtz solver (libfmmbem.so).
 *
 * One plan holds everything for one mesh and one wavenumber on one GPU: the octree
 * (bit-exact with the reference's octree.c), the rotation and coaxial translation tables,
 * the element moment tables for P2M/L2P, the near-field matrix, and device buffers for
 * the FP64 and mixed-precision matvecs.  The operator is
 *
 *     y = a x + (1 + alpha d/dn_y) (b L + c M) x,
 *         (L x)_i = sum_j int_{T_j} G(x, y_i) x_j dS,
 *         (M x)_i = sum_j int_{T_j} dG/dn_x(x, y_i) x_j dS,
 *
 * with collocation at triangle centroids y_i and one unknown per triangle (constant
 * elements), G = exp(ik r)/(4 pi r), d/dn_y the derivative along the unit normal at y_i.  The
 * reference's OprL (translation.cu:3412) computes the far part of L only; fmm_matvec replaces
 * it with the complete operator.  For a rigid (sound-hard) body the exterior Neumann problem
 * is a = 1/2, b = 0, c = -1 with right-hand side p_inc; a locally reacting surface
 * (dp/dn = i k beta p) has b = i k beta.  alpha != 0 is the Burton-Miller combination of that
 * equation with its normal derivative (the hypersingular kernels of integral.cu:603-751),
 * uniquely solvable at every wavenumber for Im(alpha) != 0 (alpha = i/k is usual); then
 * a = (1 + alpha b)/2 and the right-hand side is p_inc + alpha dp_inc/dn
 * (fmm_plane_wave_rhs adds the second term itself).
 *
 * Complex arrays are cuDoubleComplex (re, im interleaved doubles).  Every entry point
 * returns an fmm_status; FMM_OK is 0 (EXIT_SUCCESS).  Plans are not thread-safe: callers
 * serialise calls on one plan.  Pointers may be host or device memory (checked with
 * cudaPointerGetAttributes); host buffers are staged through the plan's pinned buffers.
 */
#ifndef FMMBEM_H
#define FMMBEM_H
#include <cuComplex.h>
#include <cuda_runtime_api.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FMM_OK = 0,
    FMM_ERR_ARG = 1,          /* invalid argument or size out of range */
    FMM_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    FMM_ERR_ALLOC = 3,        /* host or device allocation failed */
    FMM_ERR_IO = 4,           /* mesh file could not be read */
    FMM_ERR_BREAKDOWN = 5,    /* GMRES breakdown (zero Krylov vector, NaN) */
    FMM_ERR_NOT_CONVERGED = 6,/* GMRES hit maxit before tol */
    FMM_ERR_MESH = 7          /* degenerate mesh (zero-area element, bad index) */
} fmm_status;

/* FMM_FLOAT2: the FP64 matvec with its M2L translations (the bulk of its work) in float-float
 * arithmetic on the FP32 pipes (about 48 bits; GB300's FP64 rate is a 64th of its FP32 rate),
 * degree-scaled where the plan's mixed tables are; plans without mixed tables run FMM_FP64.  The mixed solvers'
 * residuals use it; fmm_gmres / fmm_solve_batched / fmm_scene_solve with FMM_FLOAT2 run plain
 * GMRES on it. */
typedef enum { FMM_FP64 = 0, FMM_MIXED = 1, FMM_FLOAT2 = 2 } fmm_precision;
typedef enum { FMM_RULE_GAUSS3 = 0, FMM_RULE_DUNAVANT7 = 1 } fmm_rule;

#define FMM_MAX_LEVEL 12

typedef struct {
    double k;                 /* wavenumber */
    int depth;                /* leaf level; 0 = choose from s like deterLmax (octree.c:635-679);
                                 -1 = the same, capped so that leaf boxes stay at least 1.5 times
                                 the longest element edge (meshes whose elements are coarse against
                                 the centroid spacing, e.g. flat faces) */
    int s;                    /* leaf occupancy for the depth rule (reference: 5) */
    int p_level[FMM_MAX_LEVEL + 1]; /* truncation order per level l (index l); 0 = truncNum */
    double eps;               /* truncNum accuracy parameter (reference: 0.05) */
    int rule;                 /* regular quadrature rule (fmm_rule) */
    double a_re, a_im, b_re, b_im, c_re, c_im; /* operator a I + b L + c M */
    int build_mixed;          /* also build the FP32 tables for FMM_MIXED (skipped, with the reason in
                                 fmm_last_error of a mixed call, where orders exceed 60 or even the
                                 degree-scaled coaxial entries exceed the FP32 range) */
    int device;               /* CUDA device ordinal */
    double alpha_re, alpha_im;/* Burton-Miller coupling alpha (0: the conventional operator) */
    int deterministic;        /* FMM_MIXED without atomics: each destination box accumulates its
                                 FP32 translations in one CTA (owner-computes, as the FP64 path),
                                 one right-hand side after another, so that mixed results are
                                 reproducible bit for bit; slower than the batched tiles */
} fmm_options;

typedef struct {
    int num_elem, num_vert, lmin, lmax;
    double d, pt_min[3];
    int p_level[FMM_MAX_LEVEL + 1];
    int num_box[FMM_MAX_LEVEL + 1];
    long long num_m2l[FMM_MAX_LEVEL + 1];
    long long num_near;
    size_t device_bytes;
    double setup_seconds;
    int m2l_columns[FMM_MAX_LEVEL + 1];  /* mixed path: M2L translations per CTA tile (0 without mixed tables) */
    int m2l_tensor[FMM_MAX_LEVEL + 1];   /* mixed path: 1 where the level's M2L runs on the tensor cores
                                            (tcgen05, split TF32, dense operators per class of directions; levels with
                                            p <= 16 where plan-time timing found it faster, or all of them
                                            with FMMBEM_TENSOR_M2L=1; none with FMMBEM_TENSOR_M2L=0) */
    int expansions_scaled;               /* mixed path: 1 where the FP32 expansions are kept scaled by degree
                                            (low k t, where the plain coaxial entries would leave the FP32
                                            range): multipoles d_n M_n, locals L_n / d_n per level */
    int pass_tc3[FMM_MAX_LEVEL + 1];     /* mixed path: passes of level l run as three tensor-core stages
                                            (tcgen05, split TF32: rotation, coaxial, rotation GEMMs over the
                                            translations that share each operator) -- bit 0 the M2M from
                                            level l into l-1, bit 1 the M2L of level l, bit 2 the L2L from
                                            l-1 into l; chosen at plan creation by timing against the other
                                            forms (FMMBEM_TC3=0: never, 1: wherever the order allows) */
    int pass_dense[FMM_MAX_LEVEL + 1];   /* mixed path: passes of level l run as one dense tensor-core GEMM
                                            per operator (tcgen05, split TF32; source and destination
                                            orders <= 16), same bits as pass_tc3 (bit 1 = m2l_tensor);
                                            M2L chosen at plan creation by timing (FMMBEM_TENSOR_M2L=0:
                                            never, 1: wherever the orders allow); M2M and L2L only with
                                            FMMBEM_TENSOR_M2M=1 (about ten times the rounding error of
                                            the SIMT form) */
    int pass_balanced[FMM_MAX_LEVEL + 1]; /* mixed path: SIMT-tile passes of level l that run the balanced
                                            unit schedule (one-row units in boustrophedon order), same bits
                                            as pass_tc3; chosen at plan creation by timing */
} fmm_info;

typedef struct fmm_plan fmm_plan;

/* Fill opt with the reference's defaults: s = 5, eps = 0.05, 3x3 collapsed Gauss rule,
 * single-layer operator (a = 0, b = 1, c = 0) as in OprL, device 0. */
void fmm_default_options(fmm_options *opt);

/* Create a plan from vertices V[3*nv] (double) and triangles F[3*nf] (0-based).  The octree
 * follows srcBoxes/FMMLevelSet (octree.c:749-906); tables are generated on the GPU. */
int fmm_plan_create(const double *V, int nv, const int *F, int nf, const fmm_options *opt, fmm_plan **plan);

/* Same from an OBJ file parsed like readOBJ (octree.c:586-619). */
int fmm_plan_create_obj(const char *path, const fmm_options *opt, fmm_plan **plan);

int fmm_plan_destroy(fmm_plan *plan);
int fmm_plan_info(const fmm_plan *plan, fmm_info *info);

/* Copies of the interaction lists the plan's matvecs read, for checking them against the
 * reference's own.  Host buffers; any may be NULL; sizes from fmm_plan_info.
 * fmm_plan_lists, level l (lmin..lmax):
 *   boxes[num_box[l]]       Morton numbers of the level's boxes in the plan's order, which is
 *                           the reference's fmmLevelSet order (FMMLevelSet, octree.c:890-906)
 *   m2l_beg[num_box[l]+1]   M2L translations grouped by destination box: those of box i are
 *                           m2l_beg[i] .. m2l_beg[i+1]-1, in the order of I4 ∩ level set
 *                           (FMMLevelSetNumSR, octree.c:908-919), so m2l_beg[i+1]-m2l_beg[i] is
 *                           srNumLevelArr[l-2][i] and m2l_src is srTransOriginArr[l-2]
 *                           (genSRIdxArrs, translation.cu:2848-2922)
 *   m2l_src[num_m2l[l]]     source box (index into boxes) of each translation
 *   m2l_dir[num_m2l[l]]     its direction, 0..315 (fmm_plan_direction gives the box offset) */
int fmm_plan_lists(const fmm_plan *plan, int level, long long *boxes, int *m2l_beg, int *m2l_src, int *m2l_dir);
/* The integer box offset (destination minus source, in boxes of the level) of M2L
 * direction dir. */
int fmm_plan_direction(const fmm_plan *plan, int dir, int *offset);
/* Near lists of the leaf level.  box_beg[num_box[lmax]+1] / box_idx[*num_box_pairs]: for each
 * leaf box the leaf boxes of I2 ∩ leaf set in I2's order -- its neighbours in x-y-z order, then
 * itself (I2, octree.c:497-505; intersection, octree.c:425-437).  elem_beg[num_elem+1] /
 * elem_col[*num_elem_pairs]: for each element the elements of those boxes, box after box, each
 * box's elements in increasing order: the rows of the near-field matrix. */
int fmm_plan_near_lists(const fmm_plan *plan, int *box_beg, int *box_idx, long long *num_box_pairs, int *elem_beg,
                        int *elem_col, long long *num_elem_pairs);

/* y = A x for nrhs right-hand sides stored one after another (nf each).  precision is
 * FMM_FP64 (plain path, one column after another) or FMM_MIXED (FP32 translations and near
 * field, all columns in one batched pass).  x and y may be host or device pointers. */
int fmm_matvec(fmm_plan *plan, const cuDoubleComplex *x, cuDoubleComplex *y, int nrhs, int precision);

/* y = A^T x (conjugate = 0) or y = A^H x (conjugate = 1), the transposed / adjoint operator
 * of fmm_matvec for reverse-mode derivatives (vector-Jacobian products) and adjoint solves.
 * Same translation tables and lists; the near-field matrix is transposed on the first call
 * (one extra CSR copy on the device).  No counterpart in the reference, whose operator is
 * only applied forward. */
int fmm_matvec_adjoint(fmm_plan *plan, const cuDoubleComplex *x, cuDoubleComplex *y, int nrhs, int precision,
                       int conjugate);

/* Solve A x = b with restarted GMRES (FP64 Arnoldi).  FMM_FP64 runs plain GMRES on the FP64
 * matvec; FMM_MIXED runs iterative refinement: FP64 outer residual, inner GMRES on the
 * mixed-precision matvec.  x holds the initial guess on entry.  iters/relres may be NULL. */
int fmm_gmres(fmm_plan *plan, const cuDoubleComplex *b, cuDoubleComplex *x, double tol, int maxit,
              int restart, int precision, int *iters, double *relres);

/* Solve A X = B for nrhs right-hand sides at once (B and X hold nrhs columns of nf, one
 * after another; X holds the initial guesses).  The columns advance in lockstep: every Krylov
 * step applies the operator to all of them in one batched matvec (FMM_MIXED: one pass of the
 * translation tiles over all columns), with FMM_MIXED running FP64-residual iterative
 * refinement as fmm_gmres does.  iters[nrhs] and relres[nrhs] (may be NULL) receive each
 * column's Krylov iterations and final relative residual.  FMM_ERR_NOT_CONVERGED if any
 * column misses tol.  No counterpart in the reference, which solves nothing. */
int fmm_solve_batched(fmm_plan *plan, const cuDoubleComplex *B, cuDoubleComplex *X, int nrhs, double tol, int maxit,
                      int restart, int precision, int *iters, double *relres);

/* Solve n independent systems, one per plan (bodies of a scene, each with its own mesh,
 * wavenumber and right-hand side), concurrently: nthreads host threads take plans from a
 * shared queue and run fmm_gmres on them.  Every plan has its own streams, so the GPU
 * overlaps the kernels of different bodies, which matters for small bodies whose kernels
 * leave most of the GPU idle.  b[i] and x[i] (initial guess in, solution out) have the
 * plan's nf entries, host or device.  iters, relres and status (FMM status per plan) may be
 * NULL.  FMM_MIXED runs each plan in mixed precision where it has the mixed tables and in
 * FP64 where plan creation could not build them (fmm_info.m2l_columns all zero then).
 * Returns the first hard error, else FMM_ERR_NOT_CONVERGED if a system missed tol, else
 * FMM_OK.  A plan may appear only once.  No counterpart in the reference. */
int fmm_solve_many(fmm_plan *const *plans, int n, const cuDoubleComplex *const *b, cuDoubleComplex *const *x,
                   double tol, int maxit, int restart, int precision, int nthreads, int *iters, double *relres,
                   int *status);

/* A scene: n plans (bodies of their own meshes and wavenumbers, or one mesh at several
 * frequencies) solved in lockstep.  Their unknowns form one vector, plan i at offsets[i]
 * (offsets[n] = the total).  A mixed scene matvec applies every plan's operator with one set
 * of launches whatever n is: one P2M kernel over all leaf boxes, persistent work-queue
 * launches per octree level for the M2M and L2L passes and one for all M2L passes (longest
 * tiles first, one launch per tile shape), one fused L2P + near-field kernel, all replayed
 * as a CUDA graph; FMM_FP64 runs each plan's FP64 matvec concurrently on the plans' streams.
 * Every plan needs its mixed-precision tables and must be on one device; the scene uses
 * the plans' buffers, so a plan is not used elsewhere while a scene call runs, and is
 * destroyed only after its scenes (fmm_plan_destroy refuses while a scene uses the plan).  A mixed matvec of a plan with more right-hand sides than
 * before reallocates those buffers; the scene's mixed calls then fail (FMM_ERR_ARG) until it
 * is created again.  No counterpart in the reference. */
typedef struct fmm_scene fmm_scene;
int fmm_scene_create(fmm_plan *const *plans, int n, fmm_scene **scene);
int fmm_scene_destroy(fmm_scene *scene);
/* total unknowns; offsets (n + 1 entries) may be NULL */
int fmm_scene_unknowns(const fmm_scene *scene, long long *total, long long *offsets);
/* y = A x for all plans at once; x, y of `total` entries, host or device.  Plans switched off by
 * fmm_scene_set_active (on[i] = 0; on = NULL switches all on) are skipped and get y = 0. */
int fmm_scene_matvec(fmm_scene *scene, const cuDoubleComplex *x, cuDoubleComplex *y, int precision);
int fmm_scene_set_active(fmm_scene *scene, const int *on);
/* All plans' systems by one lockstep GMRES (FMM_MIXED: FP64-refined, as fmm_gmres): every
 * Krylov step is one scene matvec, and a body whose residual estimate is below tol stops
 * extending its basis while the others continue.  b and x (initial guess in, solution out)
 * have `total` entries, host or device; iters and relres (n entries each) may be NULL.
 * Returns FMM_ERR_NOT_CONVERGED if a body missed tol. */
int fmm_scene_solve(fmm_scene *scene, const cuDoubleComplex *b, cuDoubleComplex *x, double tol, int maxit,
                    int restart, int precision, int *iters, double *relres);
/* The last fmm_scene_solve: wall seconds, and the device time (ms) and count of its mixed and
 * FP64-quality scene matvecs (the refinement's residuals: FMM_FLOAT2 by default, FMM_FP64 with
 * FMMBEM_FF_RESIDUAL=0; CUDA events around each); the rest is the Krylov vector work and the
 * host.  Any pointer may be NULL. */
int fmm_scene_timings(const fmm_scene *scene, double *solve_s, double *mixed_ms, int *mixed_calls, double *fp64_ms,
                      int *fp64_calls);

/* Failure detection of the tensor-core M2L: its waits on shared-memory barriers give up after a
 * time limit, set the plan's error flag and return, and the next mixed call reports the error.
 * This runs one such wait on `device` on a barrier nothing completes, with a ~1 ms limit
 * (*gave_up = 1 when it gave up), then completes the barrier and waits again (*completed = 1).
 * No counterpart in the reference. */
int fmm_selftest_bounded_wait(int device, int *gave_up, int *completed);

/* Reverse-mode derivative of a far-field objective with respect to the vertex positions.
 * x solves A x = b, b the plane wave exp(i k dir.c) at the centroids (dir NULL: b does not
 * depend on the mesh); p = F x is the scattered field at the npts points pts (fmm_far_field).
 * Given pbar with dJ = 2 Re(pbar^H dp) (pbar = p for J = sum |p|^2), grad[3*nv] receives
 *     dJ/dV = 2 Re[ pbar^H (dF/dV) x + lambda^H (db/dV - (dA/dV) x) ],
 * lambda solving A^H lambda = F^H pbar by GMRES to tol at `precision`; lambda[nf] (may be
 * NULL) receives it.  dA/dV is the derivative of the operator fmm_matvec applies, with the
 * octree, truncation orders and box centres held fixed (with the Burton-Miller coupling,
 * also its hypersingular near terms, the target normal derivative of the far field and the
 * alpha dp_inc/dn of the right-hand side).  Host or device buffers.  Leaf orders up to 23.
 * No counterpart in the reference. */
int fmm_vjp(fmm_plan *plan, const cuDoubleComplex *x, const double *dir, const double *pts, int npts,
            const cuDoubleComplex *pbar, double tol, int precision, double *grad, cuDoubleComplex *lambda);

/* Derivative of the same objective with respect to the surface admittance, for a plan built
 * for a locally reacting surface dp/dn = i k beta p: b = i k beta and, with the Burton-Miller
 * coupling alpha, a = (1 + alpha b)/2.  With beta allowed to vary per element,
 *     dJ = 2 Re sum_j g_beta[j] dbeta_j,
 * and for one admittance on the whole surface dJ_dbeta[0] = dJ/dRe(beta), dJ_dbeta[1] =
 * dJ/dIm(beta).  x, pts, pbar as for fmm_vjp and lambda the adjoint solution fmm_vjp returned
 * for them (no second adjoint solve).  The derivative of the operator in b is its
 * single-layer part (1 + alpha d/dn_y) L, applied transposed by one FP64 FMM pass with element
 * tables and a near-field matrix regenerated for it (temporary device memory of about the
 * plan's FP64 element tables plus two near-field matrices).  g_beta[nf] or dJ_dbeta[2] may be
 * NULL; host or device buffers.  No counterpart in the reference, whose triElem.alpha/beta/gamma
 * (structs.h:75-81) are never used. */
int fmm_vjp_admittance(fmm_plan *plan, const cuDoubleComplex *x, const double *pts, int npts,
                       const cuDoubleComplex *pbar, const cuDoubleComplex *lambda, cuDoubleComplex *g_beta,
                       double *dJ_dbeta);

/* Scattered pressure at npts exterior points y from the surface pressure p:
 * -sum_j p_j int_{T_j} (b G + c dG/dn_x)(x, y) dS(x) with the plan's b and c and regular rule,
 * i.e. M p - L dp/dn for the exterior problem (c = -1, b = (dp/dn)/p; rigid body: M p). */
int fmm_far_field(fmm_plan *plan, const cuDoubleComplex *p, const double *pts, int npts, cuDoubleComplex *out);

/* Right-hand side for a unit plane wave exp(i k d.x) at the element centroids, plus
 * alpha d/dn of it when the plan has a Burton-Miller coupling alpha. */
int fmm_plane_wave_rhs(fmm_plan *plan, const double *dir, cuDoubleComplex *rhs);

/* Mesh generators (front end for the synthetic configurations).  Return counts through
 * nv/nf; with V or F NULL only the counts are returned.  Vertex coordinates are rounded to
 * 9 significant digits, the precision an OBJ writer of this library emits. */
int fmm_mesh_icosphere(int subdiv, double radius, double *V, int *nv, int *F, int *nf);
/* Geodesic sphere: every face of the icosahedron divided into freq^2 triangles (20 freq^2 in
 * all, e.g. freq = 100 gives 200,000), vertices on the sphere of the given radius. */
int fmm_mesh_geodesic(int freq, double radius, double *V, int *nv, int *F, int *nf);
/* Ellipsoid with semi-axes (ax, ay, az) on the geodesic mesh of frequency freq, displaced
 * radially by sum_{l <= lmax} c_lm Y_lm (real orthonormal spherical harmonics, c_lm ~
 * N(0, sigma^2) from a SplitMix64/Box-Muller stream seeded by seed; lmax = -1: no bumps). */
int fmm_mesh_ellipsoid(int freq, double ax, double ay, double az, int lmax, double sigma, unsigned long long seed,
                       double *V, int *nv, int *F, int *nf);
/* Box with edges (lx, ly, lz) centred at the origin, each face an n x n grid of squares cut
 * into two triangles (12 n^2 triangles). */
int fmm_mesh_box(int n, double lx, double ly, double lz, double *V, int *nv, int *F, int *nf);

/* Coaxial translation matrices in FP64, without any device allocation.  This entry point has
 * no counterpart in the reference.  It is meant for callers that must not let a library
 * allocate device memory: an application that owns all device memory through its own pool,
 * a loop with timing limits where cudaMalloc/cudaFree would synchronise the device, or code
 * that only holds buffers it was handed.
 *   Input: t[n] translation lengths (device memory of the current device), wavenumber k,
 *   order p (1..64), sr = 1 for (S|R) and 0 for (R|R).
 *   Output: out[n * sparseCoaxTransSize(p)] on the current device, with matrix i at
 *   i * sparseCoaxTransSize(p), in the sparse layout of genSRSparseCoaxTransMat.
 * The kernel runs on `stream` and nothing is synchronised.  Its scratch is a fixed 8 MiB
 * array that the library holds on every device it is used on; a call needs
 * n * p * (2p-1) * p <= 2^19 complex entries and is rejected with FMM_ERR_ARG above that
 * (e.g. p = 30: n <= 9).  Nothing has to be zeroed first.  A matrix whose k*t is not in
 * (0, 1e5] comes out as NaN.
 * The first call on each device looks up the scratch address (cudaGetSymbolAddress), which
 * loads the library's device code on that device if it is not loaded yet.  Make that first
 * call before any stream capture.  The address is kept for the life of the process, so
 * cudaDeviceReset of a device after its first call is not supported (the module can reload
 * elsewhere).  Calls share one scratch per device: two calls whose kernels overlap
 * (different streams or host threads without ordering) race and corrupt each other's
 * results, so order them on one stream or with events.  A CUDA error already pending from
 * the caller's earlier work is reported (FMM_ERR_CUDA) and nothing is launched. */
int fmm_coax_matrices_noalloc(double k, const double *t, int n, int p, int sr, cuDoubleComplex *out,
                              cudaStream_t stream);

/* Last error message of the calling thread (static storage). */
const char *fmm_last_error(void);

/* Timing of the last matvec on the plan's stream (milliseconds).  fmm_set_profiling(plan,
 * mode): 0 off; 1 one entry per kernel or pass (the mixed translation passes then run as
 * direct launches) plus the whole matvec; 2 the whole matvec only (the mixed translation
 * passes keep running as a replayed CUDA graph).  names[i] are static strings; the last
 * entry, "matvec", spans the whole matvec (kernels, memsets and the gaps between them); in
 * mode 1 the mixed path adds "translations", the M2M/M2L/L2L phase as a whole (its M2L
 * passes overlap on side streams, so their own timers overlap too). */
int fmm_set_profiling(fmm_plan *plan, int on);
int fmm_last_timings(const fmm_plan *plan, const char **names, double *ms, int *count);

#ifdef __cplusplus
}
#endif
#endif
