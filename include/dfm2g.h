/*
 * dfm2g.h — C ABI of the GB300-native (sm_103a, one GPU) drop-in for DelFEM2's
 * implicit-FEM linear-solve path: block-CSR assembly (CMatrixSparse /
 * Merge), ILU(k) (CPreconditionerILU) and preconditioned Krylov solvers
 * (Solve_PCG, Solve_PBiCGStab).
 *
 * Conventions
 *  - Every entry point returns an int status (DFM2G_OK == 0). A failing call
 *    leaves a message for dfm2g_last_error() (per host thread). No C++
 *    exception leaves the library: a host-side failure inside a call (out of
 *    host memory, a host thread that could not start) returns
 *    DFM2G_ERR_HOST.
 *  - Index arrays are uint32 ("unsigned int" in the reference). Following
 *    CMatrixSparse, `row_start` is what the reference calls col_ind_ (row
 *    offsets, nblk+1 entries) and `col` is its row_ptr_ (column id of each
 *    off-diagonal block). Diagonal blocks are stored separately. Blocks are
 *    row-major ndim x ndim, vectors ndim entries per block row.
 *  - Vector arguments live in host or device memory as the per-call `mem`
 *    flag says (DFM2G_MEM_HOST / DFM2G_MEM_DEVICE). Device pointers must be on
 *    the library's current device; host pointers are copied in/out.
 *  - All work is queued on the library stream (dfm2g_set_stream); calls that
 *    return host data synchronise it. The library keeps one device context
 *    and one stream: call it from one host thread at a time (the error
 *    message is per thread; handles and cached kernel settings are shared
 *    and not locked).
 *  - Block sizes 1x1, 2x2 and 3x3 (ndim 1, 2, 3). The 3x3 path is the tuned
 *    one (TMA-staged SpMV, every sweep schedule); 1x1 and 2x2 matrices run
 *    warp-per-row kernels with the sync-free and level sweep schedules.
 *    Entry points written for one block size (the linear-tet elasticity and
 *    cloth assemblers: 3x3; Poisson: 1x1; the 2-D solid: 2x2) return
 *    DFM2G_ERR_UNSUPPORTED for another.
 */
#ifndef DFM2G_H
#define DFM2G_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DFM2G_API __attribute__((visibility("default")))

/* ---- status codes ------------------------------------------------------ */
enum dfm2g_status {
  DFM2G_OK = 0,
  DFM2G_ERR_ARG = 1,             /* bad argument / size mismatch           */
  DFM2G_ERR_CUDA = 2,            /* a CUDA runtime call failed             */
  DFM2G_ERR_MISSING_SLOT = 3,    /* Merge target block not in the pattern  */
  DFM2G_ERR_SINGULAR_PIVOT = 4,  /* more than 10 pivots with |det|<=1e-30  */
  DFM2G_ERR_NOT_CONVERGED = 5,   /* iteration limit hit (solution valid)   */
  DFM2G_ERR_WAIT_TIMEOUT = 6,    /* a bounded device-side wait gave up     */
  DFM2G_ERR_PATTERN = 7,         /* invalid sparsity pattern               */
  DFM2G_ERR_UNSUPPORTED = 8,     /* block size or mode not supported       */
  DFM2G_ERR_STATE = 9,           /* call order violated (e.g. no pattern)  */
  DFM2G_ERR_NONFINITE = 10,      /* NaN/Inf met in a solve                 */
  DFM2G_ERR_HOST = 11            /* host-side failure (host memory, thread) */
};

enum dfm2g_mem { DFM2G_MEM_HOST = 0, DFM2G_MEM_DEVICE = 1 };
enum dfm2g_prec { DFM2G_F64 = 0, DFM2G_F32 = 1 };

/* Triangular-sweep schedule (dfm2g_ilu_set_sweep_mode). */
enum dfm2g_sweep {
  DFM2G_SWEEP_SYNCFREE = 0, /* one persistent launch, per-row readiness     */
  DFM2G_SWEEP_LEVELS = 1,   /* one launch per level set                     */
  DFM2G_SWEEP_GROUPS = 2,   /* FP32: rows in compact blobs, one CTA per blob
                               (shared-memory dependencies inside a blob);
                               FP64 sweeps use the sync-free schedule        */
  DFM2G_SWEEP_BLOCK = 3,    /* one CTA walks the levels over a TMA-streamed,
                               level-ordered copy of the factors, one barrier
                               per level, recent results in a shared-memory
                               ring (for patterns with few rows per level)   */
  DFM2G_SWEEP_PARTS = 4,    /* sync-free over contiguous row ranges, one CTA
                               per range: dependencies inside a range are
                               polled in shared memory, only cross-range ones
                               in global memory (when a range's results fit
                               in shared memory)                            */
  DFM2G_SWEEP_CHAINS = 5,   /* sync-free over chains of consecutive rows in
                               which each row depends on the one before: one
                               warp per chain hands that dependency over in
                               registers and polls only the others; the
                               chain's factor blocks are TMA-streamed into
                               shared memory ahead of the warp               */
  DFM2G_SWEEP_TILES = 6,    /* 3x3: rows in tiles of up to 49
                               segments of dependency chains (7 x 7 columns
                               of grid lines on voxel meshes), one CTA per
                               tile walking the tile's local levels with
                               shared-memory hand-offs inside the tile and
                               copies or polls only across tiles; records
                               TMA-streamed per level. Patterns whose rows
                               have more than 16 blocks in a triangle use
                               the chain schedule                           */
  DFM2G_SWEEP_CLUSTER = 8,  /* 3x3 systems whose solution vector fits in
                               shared memory (9,400 block rows FP64, 18,900
                               FP32): one thread-block cluster of 8 CTAs
                               walks the levels, every CTA holding the whole
                               vector, results broadcast through distributed
                               shared memory, one cluster barrier per level;
                               larger systems use the AUTO choice. Slower than
                               the chains on the systems measured except the
                               smallest (a cluster barrier and broadcast cost
                               about 1.3 us per level in FP32, 2.9 in FP64)  */
  DFM2G_SWEEP_AUTO = 7      /* the default: DFM2G_SWEEP_TILES where the tiles'
                               steps hold 20 rows or more on average, rows
                               have at most 8 dependency blocks per
                               triangle and, for FP64, there are at least
                               half as many tiles as SMs (the FP64 steps are
                               bound by the SM's FP64 rate);
                               DFM2G_SWEEP_CHAINS otherwise (2-D meshes,
                               fill-in patterns, small grids)                */
};

typedef struct dfm2g_bsr_s *dfm2g_bsr;       /* CMatrixSparse<double>       */
typedef struct dfm2g_ilu_s *dfm2g_ilu;       /* CPreconditionerILU<double>  */
typedef struct dfm2g_tetmesh_s *dfm2g_tetmesh; /* linear-tet assembler      */
typedef struct dfm2g_trimesh2_s *dfm2g_trimesh2; /* 2-D linear-triangle assembler */
typedef struct dfm2g_hexmesh_s *dfm2g_hexmesh; /* trilinear-hex (Q1) assembler */

/* Per-solve record filled by the solvers (any pointer may be NULL). */
typedef struct dfm2g_solve_stats {
  unsigned iterations;     /* total (inner) PCG iterations                  */
  unsigned outer;          /* refinement steps (1 for plain solves)          */
  double rel_residual;     /* |b - K x| / |b| in FP64 at exit               */
  double ms;               /* device time of the solve (CUDA events)         */
} dfm2g_solve_stats;

/* ---- library ------------------------------------------------------------ */
DFM2G_API int dfm2g_version(void);
DFM2G_API const char *dfm2g_status_string(int status);
DFM2G_API const char *dfm2g_last_error(void);
/* Queue all further work on `stream` (a cudaStream_t; NULL = CUDA's legacy
 * default stream). Until the first call the library uses a non-blocking
 * stream of its own. */
DFM2G_API int dfm2g_set_stream(void *stream);
DFM2G_API int dfm2g_synchronize(void);

/* ---- host-side mesh and pattern helpers --------------------------------- */
/* MeshTet3D_VoxelGrid, include/delfem2/gridvoxel.cpp:194-271, every voxel
 * active, coordinates multiplied by `scale`. xyz: 3*(nx+1)(ny+1)(nz+1),
 * tet: 4*6*nx*ny*nz. */
DFM2G_API int dfm2g_mesh_tet_voxel_grid(unsigned nx, unsigned ny, unsigned nz, double scale,
                                        double *xyz, unsigned *tet);
/* JArray_PSuP_MeshElem + JArray_Sort, include/delfem2/msh_topology_uniform.cpp:301-316
 * and include/delfem2/jagarray.cpp:72-92. Call _count first (fills psup_ind,
 * np+1 entries, and *npsup), then _fill with a psup buffer of *npsup entries. */
DFM2G_API int dfm2g_psup_count(const unsigned *elem, size_t nelem, unsigned nnoel, size_t np,
                               unsigned *psup_ind, size_t *npsup);
DFM2G_API int dfm2g_psup_fill(const unsigned *elem, size_t nelem, unsigned nnoel, size_t np,
                              const unsigned *psup_ind, unsigned *psup);

/* ---- CMatrixSparse (include/delfem2/ls_block_sparse.h:24-204) ------------- */
/* Initialize(nblk, ndim, is_dia=true), ls_block_sparse.h:45-55; ndim 1, 2 or 3. */
DFM2G_API int dfm2g_bsr_create(dfm2g_bsr *out, unsigned nblk, unsigned ndim);
DFM2G_API int dfm2g_bsr_ndim(dfm2g_bsr m, unsigned *ndim);
DFM2G_API int dfm2g_bsr_destroy(dfm2g_bsr m);
/* SetPattern(colind, ncolind, rowptr, nrowptr), ls_block_sparse.h:72-85.
 * Host arrays. Values become zero. */
DFM2G_API int dfm2g_bsr_set_pattern(dfm2g_bsr m, const unsigned *row_start, size_t n_row_start,
                                    const unsigned *col, size_t ncol);
DFM2G_API int dfm2g_bsr_info(dfm2g_bsr m, unsigned *nblk, size_t *nnz);
/* setZero, ls_block_sparse.h:92-105. */
DFM2G_API int dfm2g_bsr_set_zero(dfm2g_bsr m);
/* Direct access to val_crs_ (ndim^2*nnz) and val_dia_ (ndim^2*nblk); either may be NULL. */
DFM2G_API int dfm2g_bsr_set_values(dfm2g_bsr m, const double *vcrs, const double *vdia, int mem);
DFM2G_API int dfm2g_bsr_get_values(dfm2g_bsr m, double *vcrs, double *vdia, int mem);
/* SetFixedBC = SetFixedBC_Dia(1)+Row+Col, ls_block_sparse.h:147-151,
 * ls_block_sparse.cpp:397-472. bc: ndim*nblk ints, nonzero = fixed. */
DFM2G_API int dfm2g_bsr_set_fixed_bc(dfm2g_bsr m, const int *bc, int mem);
/* AddDia(eps), ls_block_sparse.h:153-164. */
DFM2G_API int dfm2g_bsr_add_dia(dfm2g_bsr m, double eps);
/* MatVec: y = alpha*K*x + beta*y, ls_block_sparse.cpp:213-273 (y is scaled by
 * beta first, so a NaN in y survives beta == 0; the 1x1 / 2x2 / 3x3 loops of
 * 59-133). prec DFM2G_F32 uses the FP32
 * mirror of the values (refreshed by dfm2g_bsr_update_f32) and float vectors. */
DFM2G_API int dfm2g_bsr_matvec(dfm2g_bsr m, int prec, void *y, double alpha, const void *x,
                               double beta, int mem);
/* Refresh the FP32 mirror of the values from the FP64 values. */
DFM2G_API int dfm2g_bsr_update_f32(dfm2g_bsr m);
/* Merge / Mearge for a batch of elements, ls_block_sparse.h:209-358:
 * elem: nelem*nnoel node ids; emat: nelem*(nnoel*nnoel*ndim*ndim) row-major
 * [irow][jcol][ndim][ndim]. As in the reference, a pair (irow, jcol) whose
 * nodes are the same block adds the [irow][irow] block to the diagonal (this
 * differs from [irow][jcol] only for an element that repeats a node). The
 * batch is colour-scheduled (no two elements of one colour share a node), so
 * the scatter is atomic-free and deterministic. Returns
 * DFM2G_ERR_MISSING_SLOT (and adds nothing) if a block is absent. */
DFM2G_API int dfm2g_bsr_merge(dfm2g_bsr m, unsigned nelem, unsigned nnoel, const unsigned *elem,
                              const double *emat, int mem);

/* setRHS_Zero(b, bc, 0), include/delfem2/vecxitrsol.cpp:286-296 (FP64 vector of ndof). */
DFM2G_API int dfm2g_vec_zero_bc(double *b, const int *bc, size_t ndof, int mem);

/* ---- CPreconditionerILU (include/delfem2/ls_ilu_block_sparse.h:21-60) ----- */
DFM2G_API int dfm2g_ilu_create(dfm2g_ilu *out);
DFM2G_API int dfm2g_ilu_destroy(dfm2g_ilu p);
/* SetPattern0 / Initialize_ILUk(m, 0), ls_ilu_block_sparse.cpp:1057-1090 and
 * 854-857: pattern copied and row-sorted on the device, dia_ind found, and the
 * forward/backward level sets computed on the device. */
DFM2G_API int dfm2g_ilu_set_pattern0(dfm2g_ilu p, dfm2g_bsr m);
/* Initialize_ILUk(m, fill_level), ls_ilu_block_sparse.cpp:849-999: the
 * level-of-fill pattern of ILU(k) (fill_level 0: SetPattern0; -1: every fill),
 * computed on the host from the matrix pattern; the numeric phases
 * (CopyValue, Decompose, sweeps) then run on that pattern. */
DFM2G_API int dfm2g_ilu_set_pattern_k(dfm2g_ilu p, dfm2g_bsr m, int fill_level);
/* CopyValue, ls_ilu_block_sparse.cpp:1009-1047. */
DFM2G_API int dfm2g_ilu_copy_value(dfm2g_ilu p, dfm2g_bsr m);
/* Decompose, ls_ilu_block_sparse.cpp:152-356 (1x1, 2x2 and 3x3 branches),
 * level-scheduled on the device in FP64 (1x1 and 2x2 in the reference's own
 * rounding, so the factors equal the reference's); the FP32 copy of the factors
 * is refreshed when an FP32 solve first needs it.
 * More than 10 pivots with |det| <= 1e-30 -> DFM2G_ERR_SINGULAR_PIVOT.
 * *n_singular (may be NULL) receives the count of such pivots. */
DFM2G_API int dfm2g_ilu_decompose(dfm2g_ilu p, int *n_singular);
/* ForwardSubstitution / BackwardSubstitution / SolvePrecond (in place),
 * ls_ilu_block_sparse.cpp:500-573, 678-749, ls_ilu_block_sparse.h:38-41. */
DFM2G_API int dfm2g_ilu_forward(dfm2g_ilu p, int prec, void *vec, int mem);
DFM2G_API int dfm2g_ilu_backward(dfm2g_ilu p, int prec, void *vec, int mem);
DFM2G_API int dfm2g_ilu_solve_precond(dfm2g_ilu p, int prec, void *vec, int mem);
/* SolvePrecond that allocates nothing (no counterpart in the reference).
 * For callers that cannot allocate device memory while they solve: an
 * application that reserves all GPU memory up front, or a frame loop that must
 * not pay for cudaMalloc/cudaFree (cudaFree synchronises the whole device).
 * `vec` must be in device memory (in/out). The intermediate vector between
 * the two sweeps lives in one fixed array inside the library (8 MiB), which
 * every GPU that loads the library keeps until the process exits; so
 * ndim*nblk may not exceed 1,048,576 (DFM2G_ERR_ARG otherwise). The first call on
 * a device looks up that array's device address. All calls share the array:
 * calls that overlap on the GPU (other streams, other threads) race. FP32 needs
 * FP32 factors made earlier by a DFM2G_F32 dfm2g_ilu_solve_precond call.
 * The device current at the call must be the library's device
 * (DFM2G_ERR_STATE otherwise). Schedules whose data is built on first use
 * fall back to the sync-free schedule until an ordinary sweep of the same
 * precision has built that data: DFM2G_SWEEP_TILES (tile records),
 * DFM2G_SWEEP_CHAINS (chain records) and DFM2G_SWEEP_BLOCK (the level-ordered
 * stream and its input buffer). The other schedules (sync-free, levels,
 * groups, parts) need nothing built. */
DFM2G_API int dfm2g_ilu_solve_precond_noalloc(dfm2g_ilu p, int prec, void *vec);
/* 1x1 and 2x2 patterns take DFM2G_SWEEP_SYNCFREE, DFM2G_SWEEP_LEVELS, DFM2G_SWEEP_CHAINS and
 * DFM2G_SWEEP_AUTO (the chains). */
DFM2G_API int dfm2g_ilu_set_sweep_mode(dfm2g_ilu p, int mode);
/* Current schedule (a new pattern starts with DFM2G_SWEEP_AUTO). */
DFM2G_API int dfm2g_ilu_get_sweep_mode(dfm2g_ilu p, int *mode);
/* Schedule the last forward (backward = 0) or backward (backward = 1) sweep of
 * precision `prec` ran: one of the DFM2G_SWEEP_* schedules other than
 * DFM2G_SWEEP_AUTO (which picks among them), or -1 before the first sweep.
 * Shows which schedule the automatic choice, or a fallback of an explicit
 * mode, took. Host only: reads a value the host recorded at launch. */
DFM2G_API int dfm2g_ilu_last_schedule(dfm2g_ilu p, int prec, int backward, int *mode);
/* Inspection (host outputs): sorted pattern (col: nnz, dia_ind: nblk), factor
 * values, level sets (level: nblk, order: nblk, level_start: nlevels+1 with
 * room for nblk+1). */
/* Size of the ILU pattern (nnz differs from the matrix's after fill-in) and its
 * row offsets (nblk+1, host). */
DFM2G_API int dfm2g_ilu_info(dfm2g_ilu p, unsigned *nblk, size_t *nnz);
DFM2G_API int dfm2g_ilu_get_row_start(dfm2g_ilu p, unsigned *row_start);
DFM2G_API int dfm2g_ilu_get_pattern(dfm2g_ilu p, unsigned *col, unsigned *dia_ind);
DFM2G_API int dfm2g_ilu_get_values(dfm2g_ilu p, double *vcrs, double *vdia, int mem);
DFM2G_API int dfm2g_ilu_get_levels(dfm2g_ilu p, int backward, unsigned *level, unsigned *order,
                                   unsigned *level_start, unsigned *nlevels);
/* Diagnostic, host only (no counterpart in the reference): the chain partition
 * DFM2G_SWEEP_CHAINS uses, from a sorted ILU pattern (row offsets, columns,
 * dia_ind) and the sweep's level order (dfm2g_ilu_get_levels). chain_of[i] is
 * row i's chain (numbered in the level order of their first rows); *max_cross
 * the longest list of a row's dependencies outside its chain. */
DFM2G_API int dfm2g_chain_partition(unsigned n, const unsigned *row_start, const unsigned *col,
                                    const unsigned *dia_ind, const unsigned *order, int backward,
                                    unsigned *chain_of, unsigned *nchain, unsigned *max_cross);
/* Diagnostic, host only (no counterpart in the reference): the tile partition
 * DFM2G_SWEEP_TILES uses, from a sorted ILU pattern (row offsets, columns,
 * dia_ind) and the sweep's level order (dfm2g_ilu_get_levels). tile_of[i] is
 * row i's tile (numbered in dependency order), level[i] its local level inside
 * the tile; tiles hold at most max_width strand segments of at most
 * max_rows / max_width rows each (so at most max_width rows per local level);
 * the sweep uses max_rows 3185 (FP32) or 1617 (FP64), max_width 49.
 * *max_deps the most blocks of a
 * row's triangle (forward: strictly lower, backward: strictly upper). */
DFM2G_API int dfm2g_tile_partition(unsigned n, const unsigned *row_start, const unsigned *col,
                                   const unsigned *dia_ind, const unsigned *order, int backward,
                                   unsigned max_rows, unsigned max_width, unsigned *tile_of,
                                   unsigned *level, unsigned *ntiles, unsigned *max_deps);

/* ---- Krylov solvers -------------------------------------------------------- */
/* Solve_PCG, include/delfem2/lsitrsol.h:80-148, in FP64: x starts at 0; r is
 * overwritten with the final residual; hist receives the ABSOLUTE residual
 * norms [|r0|, |r1|, ...] (up to hist_cap entries; *n_hist is the full
 * length); stops when sqrt(|r|^2/|r0|^2) < tol; one extra final entry when
 * max_iter is exhausted (status DFM2G_ERR_NOT_CONVERGED, x still valid). */
DFM2G_API int dfm2g_solve_pcg(dfm2g_bsr m, dfm2g_ilu p, double *r, double *x, double tol,
                              unsigned max_iter, double *hist, unsigned hist_cap,
                              unsigned *n_hist, int mem, dfm2g_solve_stats *stats);
/* Solve_CG, include/delfem2/lsitrsol.h:35-74, FP64; hist receives the
 * RELATIVE ratios (the reference's convention for Solve_CG). */
DFM2G_API int dfm2g_solve_cg(dfm2g_bsr m, double *r, double *x, double tol, unsigned max_iter,
                             double *hist, unsigned hist_cap, unsigned *n_hist, int mem,
                             dfm2g_solve_stats *stats);
/* Mixed precision: FP32 K + FP32 ILU factors + FP32 inner PCG (relative tol
 * inner_tol per refinement step, FP64 alpha/beta reductions) inside an FP64
 * iterative-refinement loop (r = b - K x from the FP64 values, x accumulated in
 * FP64) until |b - K x|/|b| < tol. b is not modified. */
DFM2G_API int dfm2g_solve_pcg_mixed(dfm2g_bsr m, dfm2g_ilu p, const double *b, double *x,
                                    double tol, double inner_tol, unsigned max_iter,
                                    unsigned max_outer, int mem, dfm2g_solve_stats *stats);

/* Mixed precision with reliable updates: one FP32 PCG iteration (FP32 K and
 * factors, FP64 alpha/beta reductions) whose FP32 iterate is flushed into the
 * FP64 solution, and whose residual is replaced by the FP64 residual
 * b - K x (FP64 values), each time the FP32 residual has dropped by `delta`
 * since the last refresh; the search direction is kept across refreshes, so
 * the iteration count stays close to the FP64 solve's. Stops when the FP64
 * residual satisfies |b - K x|/|b| < tol. stats->outer = number of refreshes. */
DFM2G_API int dfm2g_solve_pcg_mixed_reliable(dfm2g_bsr m, dfm2g_ilu p, const double *b, double *x,
                                             double tol, double delta, unsigned max_iter, int mem,
                                             dfm2g_solve_stats *stats);

/* Solve_PBiCGStab, include/delfem2/vecxitrsol.h:350-437, FP64, for
 * non-symmetric K: x = 0, r overwritten with the final residual; hist receives
 * the RELATIVE residual after each iteration (iterations 1 .. max_iter-1, the
 * reference's loop); |r0|^2 < 1e-60 returns [|r0|]. Not converging returns
 * DFM2G_ERR_NOT_CONVERGED with x valid; a NaN/Inf residual stops with
 * DFM2G_ERR_NONFINITE. */
DFM2G_API int dfm2g_solve_pbicgstab(dfm2g_bsr m, dfm2g_ilu p, double *r, double *x, double tol,
                                    unsigned max_iter, double *hist, unsigned hist_cap,
                                    unsigned *n_hist, int mem, dfm2g_solve_stats *stats);

/* ---- linear-tet elasticity ------------------------------------------------- */
/* Builds, for mesh (xyz: 3*np, tet: 4*ntet, host arrays) against the pattern
 * of K: the element->slot map (device) and a greedy element colouring (no two
 * tets of one colour share a node). */
DFM2G_API int dfm2g_tetmesh_create(dfm2g_tetmesh *out, dfm2g_bsr m, const double *xyz, size_t np,
                                   const unsigned *tet, size_t ntet);
DFM2G_API int dfm2g_tetmesh_destroy(dfm2g_tetmesh t);
DFM2G_API int dfm2g_tetmesh_info(dfm2g_tetmesh t, unsigned *ncolor, size_t *ntet);
/* Per-tet-E assembly (adds): the loop of MergeLinSys_SolidLinear_Static_MeshTet3D,
 * include/delfem2/fem_solidlinear.h:192-237, with EMat_SolidLinear_Static_Tet
 * (fem_solidlinear.cpp:409-435) per element and (lambda, myu) from (E_e, nu).
 * b += rho*g*vol/4 - K_e u_e per node; K += K_e. young: ntet; g: 3 host
 * doubles; disp may be NULL (zero). */
DFM2G_API int dfm2g_tetmesh_assemble_linear(dfm2g_tetmesh t, dfm2g_bsr m, const double *young,
                                            double nu, double rho, const double *g,
                                            const double *disp, double *b, int mem);
/* Adjoint element term dL/dE_e = -lam_e^T (dK_e/dE_e) u_e (no reference
 * counterpart; K_e is linear in E). young is unused except for shape checks. */
DFM2G_API int dfm2g_tetmesh_dLdE(dfm2g_tetmesh t, const double *young, double nu,
                                 const double *u, const double *lam, double *dLdE, int mem);
/* Backward-Euler linear solid (adds; 3x3 blocks): MergeLinSys_SolidLinear_BEuler_MeshTet3D,
 * include/delfem2/fem_solidlinear.h:381-443, or, with rot (9*np row-major
 * rotations, else NULL), MergeLinSys_SolidStiffwarp_BEuler_MeshTet3D (445-530).
 * K += K_e + rho vol/(4 dt^2) I on the diagonal blocks, b += r_e/dt. disp,
 * velo: 3*np; g: 3 host doubles. */
DFM2G_API int dfm2g_tetmesh_assemble_beuler(dfm2g_tetmesh t, dfm2g_bsr m, double myu, double lambda, double rho,
                                            const double *g, double dt, const double *disp, const double *velo,
                                            const double *rot, double *b, int mem);
/* Newmark-beta linear solid (adds; 3x3 blocks): MergeLinSys_SolidLinear_NewmarkBeta_MeshTet3D,
 * fem_solidlinear.h:331-379, with the first-iteration element matrix of
 * EMat_SolidLinear_NewmarkBeta_MeshTet3D (fem_solidlinear.cpp:437-488):
 * K += M_e + beta dt^2 K_e (consistent mass), b += r_e. gamma is unused there. */
DFM2G_API int dfm2g_tetmesh_assemble_newmark(dfm2g_tetmesh t, dfm2g_bsr m, double myu, double lambda, double rho,
                                             const double *g, double dt, double gamma, double beta,
                                             const double *disp, const double *velo, const double *acc, double *b,
                                             int mem);
/* Scalar Poisson (adds; the matrix has 1x1 blocks): the loop of
 * MergeLinSys_Poission_MeshTet3D, include/delfem2/fem_poisson.h:128-162, with
 * EMat_Poisson_Tet3D (fem_poisson.cpp:163-194): K_e[a][b] = alpha vol
 * (dN_a . dN_b), b += source vol/4 - K_e val_e per node. val: np nodal values
 * (the fixed values lifted into b), or NULL for zero. */
DFM2G_API int dfm2g_tetmesh_assemble_poisson(dfm2g_tetmesh t, dfm2g_bsr m, double alpha, double source,
                                             const double *val, double *b, int mem);

/* ---- trilinear hexahedra (Q1) ------------------------------------------------- */
/* Builds, for mesh (xyz: 3*np, hex: 8*nhex in ShapeFunc_Hex8's corner order,
 * host arrays) against the pattern of a 3x3-block matrix: the element->slot map
 * and a greedy colouring. A hex that repeats a node is refused (DFM2G_ERR_ARG). */
DFM2G_API int dfm2g_hexmesh_create(dfm2g_hexmesh *out, dfm2g_bsr m, const double *xyz, size_t np,
                                   const unsigned *hex, size_t nhex);
DFM2G_API int dfm2g_hexmesh_destroy(dfm2g_hexmesh t);
/* Static linear solid (adds): the element loop of MergeLinSys_LinearSolid3D_Static_Q1,
 * include/delfem2/fem_solidlinear.h:239-276, with
 * elemMatRes_LinearSolidGravity3_Static_Q1 (fem_solidlinear.cpp:238-281, the
 * reference's three-point Gauss rule per direction): K += K_e,
 * b += int(rho g N) - K_e u_e. g: 3 host doubles; disp: 3*np or NULL. */
DFM2G_API int dfm2g_hexmesh_assemble_linear(dfm2g_hexmesh t, dfm2g_bsr m, double myu, double lambda, double rho,
                                            const double *g, const double *disp, double *b, int mem);

/* ---- 2-D linear triangles ---------------------------------------------------- */
/* Builds, for mesh (xy: 2*np, tri: 3*ntri, host arrays) against the pattern of
 * a 1x1- or 2x2-block matrix: the element->slot map and a greedy colouring. */
DFM2G_API int dfm2g_trimesh2_create(dfm2g_trimesh2 *out, dfm2g_bsr m, const double *xy, size_t np,
                                    const unsigned *tri, size_t ntri);
DFM2G_API int dfm2g_trimesh2_destroy(dfm2g_trimesh2 t);
/* Scalar Poisson (adds; 1x1 blocks): MergeLinSys_Poission_MeshTri2D,
 * include/delfem2/fem_poisson.h:92-127, with EMat_Poisson_Tri2D
 * (fem_poisson.cpp:15-46). val: np values or NULL. */
DFM2G_API int dfm2g_trimesh2_assemble_poisson(dfm2g_trimesh2 t, dfm2g_bsr m, double alpha, double source,
                                              const double *val, double *b, int mem);
/* Static linear solid (adds; 2x2 blocks): MergeLinSys_SolidLinear_Static_MeshTri2D,
 * include/delfem2/fem_solidlinear.h:155-187, with EMat_SolidStaticLinear_Tri2D
 * (fem_solidlinear.cpp:89-124). disp: 2*np or NULL; b: 2*np. */
DFM2G_API int dfm2g_trimesh2_assemble_solid_linear(dfm2g_trimesh2 t, dfm2g_bsr m, double myu, double lambda,
                                                   double rho, double gx, double gy, const double *disp,
                                                   double *b, int mem);

/* ---- implicit cloth (include/delfem2/femcloth.h, cloth_internal.h) --------- */
/* Triangle sheet with StVK CST membrane + quadratic bending over the quads of
 * adjacent triangle pairs. Built from host arrays (xyz0: 3*np rest positions,
 * tri: 3*ntri, quad: 4*nquad in WdWddW_Bend's order) against the pattern of K
 * (which must contain every tri and quad block): element->slot maps, greedy
 * colourings, per-element rest constants. */
typedef struct dfm2g_cloth_s *dfm2g_cloth;
DFM2G_API int dfm2g_cloth_create(dfm2g_cloth *out, dfm2g_bsr m, const double *xyz0, size_t np,
                                 const unsigned *tri, size_t ntri, const unsigned *quad, size_t nquad);
DFM2G_API int dfm2g_cloth_destroy(dfm2g_cloth c);
DFM2G_API int dfm2g_cloth_info(dfm2g_cloth c, unsigned *ncolor_tri, unsigned *ncolor_quad);
/* MergeLinSys_Cloth, femcloth.h:48-114, with per-triangle moduli: adds the
 * PD-projected CST Hessians (WdWddW_CST, fem_stvk.cpp:267-374) and the bending
 * Hessians (WdWddW_Bend, fem_quadratic_bending.cpp:49-107) into K and their
 * gradients into dW (3*np); *W (host, may be NULL) receives the energy.
 * young_tri: ntri; (lambda, myu) = (E nu/((1+nu)(1-2nu)), E/(2(1+nu))). */
DFM2G_API int dfm2g_cloth_merge(dfm2g_cloth c, dfm2g_bsr m, const double *xyz, const double *young_tri,
                                double nu, double stiff_bend, double *dW, double *W, int mem);
/* Linear solver inside the cloth step. */
enum dfm2g_cloth_solver {
  DFM2G_CLOTH_PCG_F64 = 0,      /* Solve_PCG in FP64 (the reference's solver)  */
  DFM2G_CLOTH_PCG_MIXED = 1     /* FP32 PCG with FP64 reliable updates         */
};
/* StepTime_InternalDynamicsILU, cloth_internal.h:179-269 (no contact): one
 * backward-Euler step with one Newton linearisation,
 *   A = M/dt^2 + ddW(x), b = -(dW(x) - M g) + M v/dt, clamped at bc,
 *   ILU(0)-PCG(tol, max_iter), free DOFs: x += dx, v = dx/dt.
 * g: 3 host doubles; mass: per vertex. Not reaching tol is not an error (the
 * reference continues with the last iterate); stats tells the iterations. */
DFM2G_API int dfm2g_cloth_step(dfm2g_cloth c, dfm2g_bsr m, dfm2g_ilu p, double *xyz, double *uvw,
                               const int *bc, const double *young_tri, double nu, double stiff_bend,
                               const double *g, double mass, double dt, double tol, unsigned max_iter,
                               int solver, dfm2g_solve_stats *stats, int mem);
/* Adjoint element terms of one step (no reference counterpart): with mu the
 * adjoint solve and dx the step's increment,
 *   xbar += -H(x) mu - grad_x( mu^T A(x) dx )   (H: unprojected Hessian),
 *   Ebar_t += -( mu_t . dW_t + mu_t^T A_t dx_t ) / E_t. */
DFM2G_API int dfm2g_cloth_adjoint_terms(dfm2g_cloth c, const double *xyz, const double *young_tri,
                                        double nu, double stiff_bend, const double *mu, const double *dx,
                                        double *xbar, double *Ebar, int mem);
/* Runs nsteps steps (as dfm2g_cloth_step) from (xyz, uvw), keeping on the
 * device the state every ckpt_every steps (0: no checkpoints) and the step
 * settings for dfm2g_cloth_rollout_adjoint. stats sums over the steps. */
DFM2G_API int dfm2g_cloth_rollout(dfm2g_cloth c, dfm2g_bsr m, dfm2g_ilu p, double *xyz, double *uvw,
                                  const int *bc, const double *young_tri, double nu, double stiff_bend,
                                  const double *g, double mass, double dt, double tol, unsigned max_iter,
                                  int solver, unsigned nsteps, unsigned ckpt_every,
                                  dfm2g_solve_stats *stats, int mem);
/* Reverse pass of the last rollout (checkpoint-and-recompute): from
 * xbar = dL/dx_N, vbar = dL/dv_N to dL/dx_0, dL/dv_0 in place, and
 * dLdE = dL/dE_t (ntri, overwritten). Re-runs each checkpoint segment forward,
 * then per step re-assembles and re-factorises A, solves A mu = P(xbar + vbar/dt)
 * and applies dfm2g_cloth_adjoint_terms. Needs ckpt_every > 0. */
DFM2G_API int dfm2g_cloth_rollout_adjoint(dfm2g_cloth c, dfm2g_bsr m, dfm2g_ilu p, double *xbar,
                                          double *vbar, double *dLdE, dfm2g_solve_stats *stats, int mem);

/* ---- device vectors (the compatibility path of dfm2g.hpp) ---------------- */
/* For callers without CUDA of their own: device memory and copies. */
enum dfm2g_copy_kind { DFM2G_COPY_H2D = 0, DFM2G_COPY_D2H = 1, DFM2G_COPY_D2D = 2 };
DFM2G_API int dfm2g_dev_alloc(void **p, size_t bytes);
DFM2G_API int dfm2g_dev_free(void *p);
DFM2G_API int dfm2g_dev_copy(void *dst, const void *src, size_t bytes, int kind);
/* The vector primitives Solve_PCG calls through ADL (view_vectorx.h:61-109),
 * FP64: Dot (deterministic reduction, result to the host), AddScaledVec
 * (y += alpha x), ScaleAndAddVec (y = beta y + x), setZero. */
DFM2G_API int dfm2g_vec_dot(const double *x, const double *y, size_t n, double *out, int mem);
DFM2G_API int dfm2g_vec_axpy(double *y, double alpha, const double *x, size_t n, int mem);
DFM2G_API int dfm2g_vec_scale_add(double *y, double beta, const double *x, size_t n, int mem);
DFM2G_API int dfm2g_vec_set_zero(double *x, size_t n, int mem);

/* ---- instrumentation ------------------------------------------------------- */
/* Kernel classes timed when profiling is on (CUDA events around every launch
 * of the solver loops; adds a little overhead, so off by default). */
enum dfm2g_prof_kind {
  DFM2G_PROF_SPMV = 0,     /* Ap = K p fused with p.Ap (3x3 patterns with
                              SpMV tiles: and the update, in one launch)       */
  DFM2G_PROF_UPDATE = 1,   /* r -= a Ap, x += a p, |r|^2, and the pending-
                              marker fill of the sweep outputs                 */
  DFM2G_PROF_FILL = 2,     /* (unused: the fill is part of the update)        */
  DFM2G_PROF_FWD = 3,      /* forward sweep                                    */
  DFM2G_PROF_BWD = 4,      /* backward sweep                                   */
  DFM2G_PROF_DOT = 5,      /* (r, z) and beta (3x3 patterns with SpMV tiles:
                              and p = z + beta p, in one launch)              */
  DFM2G_PROF_PUPDATE = 6,  /* p = z + beta p                                   */
  DFM2G_PROF_OUTER = 7,    /* FP64 residual / refinement kernels               */
  DFM2G_PROF_NKIND = 8
};
DFM2G_API int dfm2g_profile_enable(int on);
DFM2G_API int dfm2g_profile_reset(void);
DFM2G_API int dfm2g_profile_read(int kind, unsigned *launches, double *total_ms);
/* Number of kernels this library has launched since load (all kinds). */
DFM2G_API int dfm2g_launch_count(unsigned long long *count);
/* Number of device allocations (cudaMalloc) this library has made since load
 * (no counterpart in the reference; instrumentation). */
DFM2G_API int dfm2g_alloc_count(unsigned long long *count);

/* ---- test support ---------------------------------------------------------- */
/* Launches one tiny kernel that waits on a value nothing ever writes, bounded
 * by `timeout_ms`; must return DFM2G_ERR_WAIT_TIMEOUT with the context usable. */
DFM2G_API int dfm2g_debug_wait_timeout(unsigned timeout_ms);
/* Two rounds of the solver kernels' bounded grid barrier over 4 cooperative
 * CTAs: DFM2G_OK when every CTA arrives; with one_block_absent one CTA returns
 * without arriving and the call must return DFM2G_ERR_WAIT_TIMEOUT after about
 * `timeout_ms`, with the context usable. */
DFM2G_API int dfm2g_debug_grid_barrier(unsigned timeout_ms, int one_block_absent);
/* Host only: raises a C++ exception inside the call (kind 0: out of host
 * memory, 1: a standard exception, 2: anything else); must return
 * DFM2G_ERR_HOST with a message for dfm2g_last_error(). */
DFM2G_API int dfm2g_debug_host_failure(int kind);

#ifdef __cplusplus
}
#endif
#endif /* DFM2G_H */
