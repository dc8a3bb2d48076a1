/*
 * mpk_gb300: GB300 matrix powers kernel, status-returning C ABI.
 *
 * Computes vv = [x, Ax, A^2x, ..., A^k x] (level-major: vv[l*n + i]) for a
 * CSR matrix A with int32 indices and FP64 values, or for the reference's
 * row-normalised adjacency operator (A_ij = 1/deg(i) for every stored
 * column j of row i) when no values are given.
 *
 * Every function returns 0 on success or a negative MPKG_E* code; the
 * text of the last error on the calling thread is mpkg_last_error().
 * No function exits the process.  Plans are not thread-safe: use one plan
 * per thread, or serialise calls on a plan.  Device pointers and streams
 * must belong to the plan's device.
 *
 * Reference interfaces replaced (vatai/mpk):
 *   - task-list execution exec_mpk / exec_mpk_xd / vexec_mpk
 *     (mpk2/mpkexec.c:41-130, mpk2/mpkvexec.c:41-55) -> mpkg_plan_tasks +
 *     mpkg_exec_*;
 *   - PA1 diamond execution over part + skirt sets (mpk2/mpkprep.c:185-233
 *     consumed by mpk2/mpkexec.c:10-39) -> mpkg_plan_pa1 (tiles);
 *   - k chained SpMVs spmv_exec_seq/par and the verify_val gold chain
 *     (mpk2/spmvexec.c:8-50, mpk2/verify_val.c:44-75) ->
 *     mpkg_spmv_chain_device / mpkg_plan_spmv;
 *   - the prep tools comp (levels, weights; mpk2/comp.c:25-106) and skirt
 *     (mpk2/skirt.c:10-74) -> mpkg_levels, mpkg_level_weights,
 *     mpkg_skirt_write.
 * The legacy mpk2 names themselves are exported too (mpk2_compat.h).
 */
#ifndef MPK_GB300_H
#define MPK_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPKG_OK 0
#define MPKG_EINVAL -1   /* bad argument */
#define MPKG_EIO -2      /* file could not be opened/read/written */
#define MPKG_EFORMAT -3  /* malformed file */
#define MPKG_ESTRUCT -4  /* dependency/structure check failed */
#define MPKG_ECUDA -5    /* CUDA runtime error, or no GPU */
#define MPKG_ETIMEOUT -6 /* a bounded device-side wait gave up */
#define MPKG_ENOMEM -7   /* host or device allocation failed */
#define MPKG_ERANGE -8   /* index or size out of the supported range */

/* Arithmetic of the FP64 row sums, s over the stored columns in CSR order. */
#define MPKG_ARITH_FMA 0      /* s = fma(a, x, s): one rounding per term */
#define MPKG_ARITH_SEPARATE 1 /* s = s + a*x: two roundings per term (the
                                 reference compiled without contraction) */
#define MPKG_ARITH_DF64 2     /* double-float (FP32 pair) arithmetic on the
                                 FP32 pipes, FP64 storage; about 2^-46
                                 relative error per operation */
#define MPKG_ARITH_FIXED 3    /* 64-bit fixed point (1/deg operator, wavefront
                                 and k-SpMV executors): exact integer row sums at one
                                 scale 2^S per call, S = 62 - ceil(log2(longest
                                 row)) - e with max|x| < 2^e; error about 2^-S
                                 relative to max|x| per level; FP64 storage */

/* Executors. */
#define MPKG_EXEC_TASKS 0 /* reference task lists, one CTA per (phase,part) */
#define MPKG_EXEC_TILES 1 /* PA1: one CTA per part + k-deep skirt, levels
                             computed in shared memory */
#define MPKG_EXEC_PIPE 2  /* zero-redundancy level pipeline: chunks of rows
                             advance level by level behind their
                             neighbours, matrix chunk kept in shared memory */
#define MPKG_EXEC_SPMV 3  /* k separate SpMV launches (baseline) */
#define MPKG_EXEC_BUFS 4  /* MPI-2 rank buffers of all ranks on one GPU */
#define MPKG_EXEC_MIXED 5 /* mixed-precision pipeline (FP32/BF16 values) */
#define MPKG_EXEC_PDMPK 6 /* pdmpk buffers of all ranks on one GPU */
#define MPKG_EXEC_WAVE 7  /* wavefront: one persistent launch, each CTA owns
                             a row range at every level and waits only for
                             the CTAs owning its columns */
#define MPKG_EXEC_BATCH 8 /* batched block-vector form (FP32), many matrices */

/* Partition providers of the pdmpk prep (mpkg_pdmpk_prep). */
#define MPKG_PD_PART_BLOCKSHIFT 0 /* contiguous blocks, shifted by half a
                                     block per call */
#define MPKG_PD_PART_BFS 1        /* breadth-first recursive bisection */
#define MPKG_PD_PART_METIS 2      /* METIS_PartGraphKway with the reference's
                                     arguments (pdmpk/pdmpk_buffers.cc:
                                     183-202): the matrix pattern as is,
                                     default options; edge weights on the
                                     re-partitioning calls */

/* Value storage of the mixed-precision form. */
#define MPKG_VALUE_F32 0
#define MPKG_VALUE_BF16 1

typedef struct mpkg_plan mpkg_plan;

typedef struct {
  int n, nlevel, nphase, npart;
  int exec, arith, valued;
  long nnz;
  long rows_computed;   /* row evaluations per execution, redundancy included */
  long device_bytes;    /* device memory held by the plan */
  int launches;         /* kernels launched per execution */
  int tiles_in_smem;    /* TILES: 1 if the levels fit in shared memory */
  int max_tile_slots;   /* TILES: largest part + skirt */
  int pipe_chunk;       /* PIPE: rows per chunk */
  int pipe_reach;       /* PIPE: dependency reach in chunks */
  int pipe_grid;        /* PIPE: resident CTAs launched */
  int tile_regs;        /* MIXED on tiles: 1 when every tile's rows are held in
                           registers (register-resident tile kernel) */
  int tune_candidates;  /* mpkg_plan_mixed_tiles_tuned: part sizes timed */
  double tune_ms;       /* mpkg_plan_mixed_tiles_tuned: time spent choosing */
} mpkg_plan_info_t;

/* Plan over task lists in the reference layout: list t = phase*npart+part
 * holds entries level*n+vertex in idx[off[t]..off[t+1]), level-major
 * (mpk2/lib.h:78-99 task_t/mpk_t, filled by prep_mpk mpk2/mpkprep.c:7-258).
 * val == NULL selects the 1/deg operator.  ptr/col/val/off/idx are host
 * arrays, copied. */
int mpkg_plan_tasks(int n, const int *ptr, const int *col, const double *val,
                    int npart, int nlevel, int nphase, const long *off,
                    const long *idx, int arith, mpkg_plan **out);

/* PA1 plan straight from a partition (no dense skirt array): exec is
 * MPKG_EXEC_TILES or MPKG_EXEC_TASKS (reference task lists built from the
 * bounded skirts). */
int mpkg_plan_pa1(int n, const int *ptr, const int *col, const double *val,
                  const int *part, int npart, int nlevel, int exec, int arith,
                  mpkg_plan **out);

/* Zero-redundancy pipeline plan (chunk <= 0 picks a default). */
int mpkg_plan_pipe(int n, const int *ptr, const int *col, const double *val,
                   int nlevel, int chunk, int arith, mpkg_plan **out);

/* k chained SpMV launches (baseline; also the GPU spmv_exec_*).  arith
 * FMA/SEPARATE: FP64 rows (the reference's bits); DF64 and FIXED: the
 * wavefront's double-float and fixed-point rows with the levels in a
 * device ring, so the baseline runs the same arithmetic as the form it is
 * compared with (same bits as mpkg_plan_wave in that arith). */
int mpkg_plan_spmv(int n, const int *ptr, const int *col, const double *val,
                   int nlevel, int arith, mpkg_plan **out);

/* Wavefront executor (no counterpart in the reference: the GB300 form of
 * exec_mpk for a matrix whose slices stay in L2).  One cooperative launch
 * per call; CTA b computes its contiguous rows (equal nonzeros) at level l
 * once the CTAs owning the columns of those rows have published level
 * l-1 (bounded waits: MPKG_ETIMEOUT instead of a hang).  Computes every
 * row once per level.  arith MPKG_ARITH_DF64 runs the rows in
 * double-float on the FP32 pipes (1/deg operator: row sum then one
 * scaling; valued: multiply-add per entry) and writes the FP64 rounding of
 * each level. */
int mpkg_plan_wave(int n, const int *ptr, const int *col, const double *val, int nlevel, int arith,
                   mpkg_plan **out);
/* The same with at most ctas_per_sm resident CTAs per SM (fewer, larger row
 * ranges; the default is the kernel's occupancy). */
int mpkg_plan_wave_ctas(int n, const int *ptr, const int *col, const double *val, int nlevel, int arith,
                        int ctas_per_sm, mpkg_plan **out);

/* Batched block-vector form (no counterpart in the reference; the
 * batching pattern of the task): nmat independent matrices (host CSR
 * arrays, FP32 values), nrhs right-hand sides each (a power of two <=
 * 128), nlevel powers, all in ONE persistent cooperative launch that the
 * plan replays as a CUDA graph.  Vectors: one float buffer of
 * (nlevel+1) * N * nrhs, N = sum of n[m]; level l of matrix m starts at
 * (l*N + row0[m]) * nrhs, row0[m] = n[0] + ... + n[m-1], each row's nrhs
 * values contiguous; level 0 is the input.  Entries are accumulated with
 * FP32 FMA in CSR order.  tune = MPKG_BATCH_TUNE times every kernel
 * configuration (lanes per row x vector width, L2 group size, CTAs per SM,
 * and for nrhs a multiple of 4 the kernel that stages each CTA's window of
 * the previous level in shared memory) on these matrices at plan time and
 * keeps the fastest; MPKG_BATCH_DEFAULT takes the first configuration
 * untimed, MPKG_BATCH_STAGED / MPKG_BATCH_STAGED2 / MPKG_BATCH_STAGED4 the
 * staged kernel at one, two or four CTAs per SM untimed (EINVAL when nrhs
 * is not a multiple of 4).  All configurations give the same bits. */
enum {
  MPKG_BATCH_DEFAULT = 0,
  MPKG_BATCH_TUNE = 1,
  MPKG_BATCH_STAGED = 2,
  MPKG_BATCH_STAGED2 = 3,
  MPKG_BATCH_STAGED4 = 4
};
int mpkg_plan_batch(int nmat, const int *n, const int *const *ptr, const int *const *col, const float *const *val,
                    int nrhs, int nlevel, int tune, mpkg_plan **out);
typedef struct {
  int nmat, nrhs, nlevel;
  long rows, nnz;
  int lanes_per_row, vector_width; /* chosen kernel: lanes x floats = nrhs */
  long group_bytes;                /* L2 budget of a group of matrices */
  int ngroup, grid;                /* groups, CTAs of the persistent launch */
  int graph;                       /* 1: replayed as a CUDA graph */
  int candidates;                  /* configurations timed by the autotuner */
  double tune_ms;                  /* autotuning time at plan creation */
  long device_bytes;
  int staged;                      /* 1: previous level windowed in shared memory */
  int threads;                     /* CTA size */
  long window_bytes;               /* staged: shared-memory window per CTA */
} mpkg_batch_info_t;
int mpkg_batch_info(const mpkg_plan *p, mpkg_batch_info_t *info);
/* d_vb: device buffer as above (16-byte aligned), level 0 filled. */
int mpkg_exec_batch_device(mpkg_plan *p, float *d_vb, void *stream);
/* vb: host buffer as above; copies level 0 in and levels 1..nlevel out. */
int mpkg_exec_batch_host(mpkg_plan *p, float *vb);

/* ---- s-step CG and its basis shifts (no counterpart in the reference) ----
 * The consumer of the MPK basis.  Precision: FP32 matrix values and
 * basis vectors, FP64 Gram matrix Y^T Y and coefficient-space iteration on
 * the GPU, FP64 x and true residual (recomputed every outer iteration). */
typedef struct {
  int iterations;   /* outer iterations (s-step) or CG iterations */
  int mpk_steps;    /* inner CG steps taken (s per outer iteration) */
  int converged;    /* relres <= tol */
  int breakdowns;   /* inner loops stopped early (non-positive curvature) */
  double relres;    /* final true relative residual |b - A x| / |b| */
  double basis_cond;/* largest condition number of the s+1 vectors
                       p, rho_1(A) p, ..., rho_s(A) p over the outer iterations */
  double ms;        /* wall time of the call */
  double loop_ms;   /* wall time of the iterations alone (no upload or setup) */
  int loop_launches;/* graph launches of the s-step outer loop: 1 with the
                       device-side loop, one per outer iteration on the host */
} mpkg_cg_info_t;

/* Standard FP64 conjugate gradients on the GPU (the reference iteration
 * count).  x: initial guess in, solution out. */
int mpkg_cg(int n, const int *ptr, const int *col, const double *val, const double *b, double *x, double tol,
            int max_iter, mpkg_cg_info_t *info);
/* Accumulation of the s-step Gram matrix for the calling thread's later
 * mpkg_sstep_cg calls: MPKG_GRAM_FP64 (default; FP64 FMAs over the exact
 * FP64 products of the FP32 basis) or MPKG_GRAM_DF64 (the same products
 * split exactly and summed in double-float on the FP32 pipes, about
 * 2^-46 relative to the sum of |products|; faster on GB300). */
#define MPKG_GRAM_FP64 0
#define MPKG_GRAM_DF64 1
int mpkg_sstep_gram(int mode);
/* Where the calling thread's later mpkg_sstep_cg calls run their outer
 * loop: MPKG_SSTEP_DEVICE_LOOP (default; the whole solve is one CUDA graph
 * launch, a conditional WHILE node deciding on the device after each
 * iteration; falls back to the host loop where the runtime lacks it) or
 * MPKG_SSTEP_HOST_LOOP (one graph launch and one host synchronisation per
 * outer iteration).  Both give the same bits. */
#define MPKG_SSTEP_DEVICE_LOOP 0
#define MPKG_SSTEP_HOST_LOOP 1
int mpkg_sstep_loop(int mode);

/* How the calling thread's later mpkg_sstep_cg calls build the basis:
 * MPKG_SSTEP_BASIS_STEPS (default; one SpMV launch per basis step, both
 * blocks per launch) or MPKG_SSTEP_BASIS_MPK (the whole basis of both
 * blocks as ONE matrix powers launch, the wavefront form: each CTA owns a
 * row range at every level and waits only for the CTAs owning its columns,
 * bounded waits).  Both give the same bits.  Steps are the default
 * because, for a matrix that stays in L2 between steps, the matrix powers
 * launch saves no HBM traffic and its per-level waits cost more than the
 * launches they replace (96^3 diffusion, s = 8: 28.2 against 32.5 ms). */
#define MPKG_SSTEP_BASIS_MPK 0
#define MPKG_SSTEP_BASIS_STEPS 1
int mpkg_sstep_basis(int mode);
/* Test hook for failure detection: the calling thread's later matrix
 * powers bases wait for extra_levels levels more than exist, so their
 * bounded waits give up (about a second) and mpkg_sstep_cg returns
 * MPKG_ETIMEOUT with the context usable; 0 restores normal waits. */
int mpkg_sstep_debug_stall(int extra_levels);

/* s-step CG (s <= 10): Newton basis rho_(j+1) = (A - shifts[j]) rho_j /
 * scale (shifts NULL: monomial basis), 2s+1 FP32 basis vectors per outer
 * iteration, FP64 Gram + coefficient solve, FP64 residual replacement. */
int mpkg_sstep_cg(int n, const int *ptr, const int *col, const double *val, const double *b, double *x, int s,
                  const double *shifts, double scale, double tol, int max_outer, mpkg_cg_info_t *info);
/* m steps of Lanczos (FP64, GPU) from a seeded uniform start vector: the m
 * Ritz values ascending (and the tridiagonal when alpha/beta are given). */
int mpkg_lanczos(int n, const int *ptr, const int *col, const double *val, int m, uint64_t seed, double *ritz,
                 double *alpha, double *beta);
/* Eigenvalues of a symmetric tridiagonal matrix (bisection), ascending. */
void mpkg_tridiag_eigs(int m, const double *alpha, const double *beta, double *out);
/* Leja ordering of k points (in place): largest modulus first, then each
 * next point maximises the product of distances to those chosen. */
void mpkg_leja_order(int k, double *x);

/* Cheap matrix features (GPU): Gershgorin bounds, diagonal, off-diagonal
 * and row-norm statistics, degrees, diagonal dominance; normalised by the
 * Gershgorin upper bound.  glo/ghi receive the bounds. */
#define MPKG_NFEAT 12
int mpkg_features(int n, const int *ptr, const int *col, const double *val, float *feat, double *glo, double *ghi);

/* MLP nin -> width -> width -> nout (ReLU, linear output, MSE), FP32,
 * trained and evaluated by the library's own GPU kernels. */
typedef struct mpkg_mlp mpkg_mlp;
int mpkg_mlp_create(int nin, int width, int nout, uint64_t seed, mpkg_mlp **out);
void mpkg_mlp_destroy(mpkg_mlp *m);
int mpkg_mlp_nparams(const mpkg_mlp *m);
/* parameters flat: W1 (width x nin), b1, W2 (width x width), b2,
 * W3 (nout x width), b3; row-major */
int mpkg_mlp_get_params(const mpkg_mlp *m, float *params);
int mpkg_mlp_set_params(mpkg_mlp *m, const float *params);
int mpkg_mlp_forward(mpkg_mlp *m, int nsamples, const float *X, float *Y);
/* gradient of the mean squared error over the samples (and the loss) */
int mpkg_mlp_gradient(mpkg_mlp *m, int nsamples, const float *X, const float *T, float *grad, float *loss);
/* Adam over shuffled minibatches (seeded); loss_curve: mean loss per epoch */
int mpkg_mlp_train(mpkg_mlp *m, int nsamples, const float *X, const float *T, int epochs, int batch, float lr,
                   uint64_t seed, float *loss_curve);

/* MPI-2 rank buffers rank0.bufs .. rank{npart-1}.bufs in `dir` (the files
 * mpi2_mpkwrtbufs writes, mpk2/buffers.c:588-631; values required) run on
 * one GPU: each phase's per-rank computation (mpk2/mpi2_mpkexecbufs_val.c:
 * 13-30) is one launch over all ranks, each phase's MPI_Alltoallv
 * (mpi2_mpkexecbufs_val.c:32-48) one device gather.  Execution places x
 * from vv[0..n) into every rank's phase-0 receive buffer and collects every
 * rank's values into vv (collect_results, mpk2/mpi2_mpkexec.c:122-146). */
int mpkg_plan_bufs(const char *dir, int npart, int arith, mpkg_plan **out);

/* pdmpk buffers (the buf.bin / results.bin pair of every rank that
 * pdmpk's prep writes, pdmpk/buffers.cc:194-224, pdmpk/results.cc:36-46)
 * run on one GPU; replaces loading them rank by rank and running
 * Buffers::AsyncExec under MPI (apps/exec.cc, pdmpk/buffers.cc:120-191).
 * Every batch is one device gather (the batch's MPI_Ialltoallv) and one
 * launch over all ranks' rows (Buffers::DoComp with the init_idcs
 * partial-sum seeds).  Execution loads x from vv[0..n) into every rank's
 * mbuf (Buffers::LoadInput with the buffers' original_idcs) and writes
 * A^nlevel x to vv[nlevel*n ..) (Results::FillResults); levels 1 ..
 * nlevel-1 of vv are left untouched.  n and nlevel come from the buffers
 * (plan info).  arith: MPKG_ARITH_SEPARATE is bit-identical to the
 * reference's exec built without FMA contraction, MPKG_ARITH_FMA to one
 * built with it. */
int mpkg_plan_pdmpk(int npart, const char *const *buf_paths, const char *const *results_paths, int arith,
                    mpkg_plan **out);

/* The pdmpk prep of every rank (CommCompPatterns, pdmpk/
 * comm_comp_patterns.cc:26-768, as apps/prep.cc runs it), written as
 * buf_paths[r] / results_paths[r].  mirror_method 0..5 and
 * weight_update_method 0..3 as the reference's --mirror / --weight;
 * partitioner MPKG_PD_PART_* stands in for METIS_PartGraphKway.
 * MPKG_ESTRUCT when the mirror method cannot finish (the reference exits
 * there).  Files are byte-identical to the reference prep's when both use
 * the same partitions. */
/* Loads and validates pdmpk buffers on the host (no GPU needed): the
 * matrix size, the level count, the number of batches and of computed
 * rows (all ranks).  Any pointer may be null. */
int mpkg_pdmpk_info(int npart, const char *const *buf_paths, const char *const *results_paths, int *n,
                    int *nlevel, int *nbatch, long *rows);

int mpkg_pdmpk_prep(int n, const int *ptr, const int *col, const double *val, int npart, int nlevel,
                    int mirror_method, int weight_update_method, int partitioner, const char *const *buf_paths,
                    const char *const *results_paths);

/* Mixed-precision form (no counterpart in the reference's code; the
 * precision pattern of the task): matrix values stored as FP32 or BF16
 * (value_type), basis vectors FP32, FP32 accumulation in CSR order, every
 * level scaled by 2^-e with 2^e >= ||A||_inf so the monomial basis cannot
 * grow; the scaling is exact, A^l x = 2^(l*e) * v_l.  Same zero-redundancy
 * pipeline as MPKG_EXEC_PIPE (requires the resident grid to cover
 * (nlevel-1) x the matrix's dependency reach, else MPKG_ERANGE). */
int mpkg_plan_mixed(int n, const int *ptr, const int *col, const double *val, int nlevel, int value_type,
                    mpkg_plan **out);
/* The same mixed-precision form on PA1 tiles, for matrices larger than L2
 * (the PA1 diamond schedule of mpk2/mpkprep.c:186-233, temporal blocking):
 * every part plus the vertices within nlevel arcs of it is one tile; a
 * persistent CTA gathers the tile's level-0 halo into shared memory, loads
 * its rows' local columns and values once into registers, and computes all
 * nlevel levels on chip (skirt rows recomputed, no inter-CTA waits),
 * writing the part's own rows of each level.  The tile metadata is built on
 * the GPU (mpkg_tile_prep).  Same scaling, storage and bits as
 * mpkg_plan_mixed; executed with mpkg_exec_mixed_device.  MPKG_ERANGE when
 * a tile's two FP32 level vectors exceed shared memory (use more parts). */
int mpkg_plan_mixed_tiles(int n, const int *ptr, const int *col, const double *val, const int *part, int npart,
                          int nlevel, int value_type, mpkg_plan **out);
/* mpkg_plan_mixed_tiles with the part size chosen by measurement (no
 * counterpart in the reference, whose part count is an input): for part
 * sizes of 384, 512, 768, 1024 and 1536 rows it partitions the vertices by
 * recursive coordinate bisection of coords (n x dim ints), builds the
 * tile plan, times three executions on scratch vectors and keeps the
 * fastest plan (info: npart, tune_candidates, tune_ms).  Same bits as
 * mpkg_plan_mixed_tiles on that partition; MPKG_ERANGE when no size
 * gives a plan. */
int mpkg_plan_mixed_tiles_tuned(int n, const int *ptr, const int *col, const double *val, const int *coords, int dim,
                                int nlevel, int value_type, mpkg_plan **out);
/* e of the plan's scaling and the number of values the storage type
 * cannot represent exactly (0 means lossless, e.g. BF16 on stencils). */
int mpkg_mixed_scale(const mpkg_plan *p, int *exponent, long *inexact_values);
/* d_vv: (nlevel+1)*n floats on the device, x (pre-scaled as the caller
 * wishes) in d_vv[0..n); writes v_1..v_nlevel.  Asynchronous; mpkg_sync
 * reports device-side errors. */
int mpkg_exec_mixed_device(mpkg_plan *p, float *d_vv, void *stream);

int mpkg_plan_info(const mpkg_plan *p, mpkg_plan_info_t *info);

/* Execute with host memory: vv holds (nlevel+1)*n doubles, x in vv[0..n);
 * levels 1..nlevel are written back.  The host->device copy of x and the
 * device->host copy of the levels are part of the call.  When vv is
 * page-locked (cudaHostAlloc / cudaHostRegister) and the plan is a
 * wavefront plan in double-float or fixed point, the kernel reads x and
 * writes the levels through the host mapping while it computes. */
int mpkg_exec_host(mpkg_plan *p, double *vv);

/* Execute on device memory: d_vv as above, on `stream` (a cudaStream_t,
 * NULL = the plan's own stream).  Asynchronous: errors of the kernels
 * themselves are reported by mpkg_sync(). */
int mpkg_exec_device(mpkg_plan *p, double *d_vv, void *stream);

/* Wait for the plan's work on `stream` and report device-side errors
 * (MPKG_ETIMEOUT when a bounded wait gave up). */
int mpkg_sync(mpkg_plan *p, void *stream);

void mpkg_plan_destroy(mpkg_plan *p);

/* Test hook for failure detection: makes every later dependency wait of a
 * pipeline, wavefront, mixed-wavefront or batched plan wait for
 * `extra_levels` levels more than exist, so the
 * bounded waits give up (about a second) and mpkg_sync returns
 * MPKG_ETIMEOUT with the context still usable; 0 restores normal waits. */
int mpkg_debug_pipe_stall(mpkg_plan *p, int extra_levels);

/* Allocation-free pipeline (no counterpart in the reference).  For callers
 * that must not allocate device memory themselves, e.g. a solver plug-in
 * running inside an application whose memory pool owns the whole device, or
 * a time-stepping loop that cannot take cudaMalloc's implicit device
 * synchronisation.  Runs the FP64 (FMA) pipeline on caller-owned device
 * arrays: CSR d_ptr/d_col/d_val (values required) and d_vv with x in
 * d_vv[0..n); writes levels 1..nlevel.  Its bookkeeping lives in a
 * file-scope device array of about 1.2 MB that every GPU loading this
 * library holds until the process exits; limits: n <= 4096*1024 rows,
 * nlevel <= 16 (larger sizes return MPKG_ERANGE / MPKG_EINVAL).  The CSR is
 * checked on the device before anything is computed: a column outside
 * [0, n) returns MPKG_ERANGE, a ptr that decreases or does not start at 0
 * (or a matrix without entries) MPKG_EINVAL, and vv is then left as it was;
 * col and val must hold ptr[n] entries.  It calls no allocating routine.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls share the one array and
 * it keeps the last call's contents (each call clears what must start at
 * zero), so calls that overlap on the GPU race.  The call waits for its
 * kernels (stream may be NULL) and returns MPKG_ETIMEOUT if a bounded wait
 * gave up. */
int mpkg_pipe_noalloc(int n, const int *d_ptr, const int *d_col, const double *d_val,
                      int nlevel, double *d_vv, void *stream);

/* Measurement utility (no counterpart in the reference): the current
 * GPU's peak FP64 fused multiply-add rate in FMAs per second, from a
 * kernel of independent FMA chains timed with CUDA events (best of five
 * launches).  The plain FP64 forms are bound by it on GB300. */
int mpkg_fp64_fma_rate(double *fma_per_s);

/* Stand-alone k-SpMV on device arrays (no plan). */
int mpkg_spmv_chain_device(int n, const int *d_ptr, const int *d_col, const double *d_val,
                           int nlevel, double *d_vv, int arith, void *stream);

/* ---- host prep (bit-identical outputs to the reference prep tools) ---- */

/* Graph files. */
int mpkg_read_metis(const char *path, int *n, long *nnz, int **ptr, int **col);
/* Matrix Market file (coordinate, real or pattern, general or symmetric;
 * pattern => 1/deg values), the reader of pdmpk's Csr (pdmpk/csr.cc:9-122)
 * except that symmetric files give a consistent CSR.  ptr, col, val are
 * allocated (mpkg_free). */
int mpkg_read_mtx(const char *path, int *n, long *nnz, int **ptr, int **col, double **val);
int mpkg_read_values(const char *path, long nnz, double **val);
void mpkg_free(void *p);

/* comp_level (level_org == NULL) / update_level (mpk2/lib.c:330-412). */
int mpkg_levels(int n, const int *ptr, const int *col, const int *part, int npart,
                const int *level_org, int *level);
/* level2wcrs (mpk2/lib.c:504-537). */
int mpkg_level_weights(int n, const int *ptr, const int *col, const int *level,
                       int *wv, int *we);
/* The same two computed on the current GPU (host arrays in and out; the
 * same bytes as the host builds): every part's min-plus fixed point at
 * once by Jacobi sweeps, and the weights per entry. */
int mpkg_levels_gpu(int n, const int *ptr, const int *col, const int *part, int npart,
                    const int *level_org, int *level);
int mpkg_level_weights_gpu(int n, const int *ptr, const int *col, const int *level, int *wv, int *we);
/* `skirt` tool output file (mpk2/skirt.c + lib.c:584-654), computed with
 * bounded searches; lev == NULL for PA1. */
int mpkg_skirt_write(const char *path, int n, const int *ptr, const int *col,
                     const int *part, int npart, const int *lev, int nlevel);

/* Task lists of prep_mpk from files-free inputs: parts is max(nphase,1)*n,
 * levels nphase*n; the skirt comes from the bounded search on parts[0]
 * (and levels[nphase-1] when nphase > 0).  Returns the number of entries
 * through *count; off has (nphase+1)*npart+1 entries, idx is allocated
 * (mpkg_free).  check != 0 runs the reference's dependency checks. */
int mpkg_tasks(int n, const int *ptr, const int *col, int npart, int nlevel, int nphase,
               const int *parts, const int *levels, int check, long *off, long **idx,
               long *count);

/* PA1 tile metadata of mpkg_plan_pa1 (EXEC_TILES): for every part, the
 * vertices within nlevel arcs (the reference's skirt distance,
 * mpk2/lib.c:584-615, with radius nlevel so that the tile holds its level-0
 * halo) sorted by (distance, vertex), and the sliced-ELL local structure
 * of the rows computed at level 1.  on_gpu != 0 builds it on the current
 * GPU (one persistent CTA per SM, balls up to 32768 vertices; beyond that,
 * and for every error, the host build runs and built_on_gpu reports 0).
 * The arrays are malloc'd; release them with mpkg_tiles_free. */
typedef struct {
  int npart, nlevel, max_slots, built_on_gpu;
  long total_rows, nslots, nslices, nell;
  long *slot_off;         /* npart + 1: first slot of each tile */
  int *shell;             /* npart * (nlevel + 1): vertices within distance d */
  int *slot_vert;         /* nslots: vertex of each slot */
  long *slice_off;        /* npart + 1: first slice of each tile */
  long *ell_off;          /* nslices + 1: first entry of each slice */
  uint16_t *ell_col;      /* nell: local slot per entry, 32 rows per slice, 0xFFFF = padding */
  uint8_t *ell_width;     /* nslices */
} mpkg_tiles_t;
int mpkg_tile_prep(int n, const int *ptr, const int *col, const int *part, int npart, int nlevel,
                   int on_gpu, mpkg_tiles_t *out);
void mpkg_tiles_free(mpkg_tiles_t *t);

/* PA1 task lists (what mpkg_tasks returns for nphase = 0, without the
 * dependency checks): off has npart+1 entries, idx is allocated
 * (mpkg_free).  on_gpu != 0 builds the skirts and lists on the current GPU
 * (same fallback as mpkg_tile_prep; *built_on_gpu tells which ran). */
int mpkg_pa1_tasks(int n, const int *ptr, const int *col, const int *part, int npart, int nlevel,
                   int on_gpu, long *off, long **idx, long *count, int *built_on_gpu);

/* The MPI-2 prep of every rank at once (what mpi2_mpkwrtbufs does rank by
 * rank, mpk2/mpi2_mpkwrtbufs.c:41-60): reads `dir` (ghead_npart_nlevel_
 * nphase with loop.g0, g<ph>.part.<npart>, l<ph>, s<nphase>, and
 * <dir up to its first '_'>.loop.val) and writes dir/rank<r>.bufs for every
 * rank, byte-compatible with the reference's files. */
int mpkg_bufs_prepare(const char *dir);

/* The counts of the reference's work_count tool (mpk2/work_count.c:13-149)
 * for a prepared MPI-2 directory (ghead_npart_nlevel_nphase with loop.g0
 * and rank<r>.bufs): doubles communicated (received minus kept on the
 * rank), ops (row lengths of every rank's local CSR), minops (nlevel *
 * nnz), nvert (n * nlevel), and *redundant = the (rank, phase, index)
 * entries both received and computed on the rank (the reference prints
 * one line for each; 0 for a correct prep; may be NULL). */
int mpkg_work_count(const char *dir, long *comm, long *ops, long *minops, long *nvert, long *redundant);

/* The label assignment of the MPI-2 and pdmpk preps (mpk2/lapjv.c:366
 * lapjv(sums, npart, perm)): perm maximises sum_j sums[perm[j]*npart + j]
 * over permutations, with the reference's tie-breaking (Jonker-Volgenant
 * steps in the published order). */
int mpkg_lapjv(const int *sums, int npart, int *perm);

/* METIS k-way partition, as the reference's `gpmetis -ufactor=<ufactor>
 * graph npart` (mpk2/driver.c:63-66, mpk2/driver.sh:46,63) computes it: the
 * METIS library bundled with the CUDA toolkit, called on the graph without
 * its self loops, default options except the imbalance ufactor (<= 0
 * keeps METIS's default) and 0-based numbering.  vwgt (n) and adjwgt (one
 * per stored entry, as the weighted graphs level2wcrs writes) may be
 * NULL; edgecut may be NULL.  Returns MPKG_EINVAL when the library was
 * built without METIS (mpkg_have_metis() == 0). */
int mpkg_have_metis(void);
int mpkg_partition_metis(int n, const int *ptr, const int *col, const int *vwgt, const int *adjwgt, int npart,
                         int ufactor, int *part, long *edgecut);

/* Project partitioners: recursive coordinate bisection (coords: dim ints
 * per vertex) and breadth-first recursive bisection. */
int mpkg_partition_rcb(int n, const int *coords, int dim, int npart, int *part);
int mpkg_partition_bfs(int n, const int *ptr, const int *col, int npart, int *part);

/* Generators: the reference gen2 stencils (type m5p t5p m7p m9p cube) and
 * Laplacians on nx*ny*nz grids (coords optional, 3 ints per vertex). */
int mpkg_gen_stencil(const char *type, int size, int *n, long *nnz, int **ptr, int **col,
                     double **val);
int mpkg_gen_laplacian(int nx, int ny, int nz, double diag, double off, int *n, long *nnz,
                       int **ptr, int **col, double **val, int **coords);
/* Variable-coefficient diffusion with log-normal(0, sigma) edge
 * coefficients (symmetric, diagonal = (1+dominance) * sum |off-diagonal|):
 * nz <= 1 gives the 9-point operator on nx*ny with direction weights wx,
 * wy, wdiag; nz > 1 the 7-point operator on nx*ny*nz (weights ignored). */
/* Random banded operator (no counterpart in the reference; the batching
 * workload's "banded" half): row i has its diagonal and m-1 distinct
 * off-diagonals drawn from [i-bw, i+bw], m uniform in [nmin, nmax], values
 * N(0,1), diagonal N(0,1) + sum|off| + 1; columns ascending; seeded.
 * Arrays allocated (mpkg_free). */
int mpkg_gen_banded(long n, int bw, int nmin, int nmax, uint64_t seed, int *nout, long *nnz, int **ptr, int **col,
                    double **val);

int mpkg_gen_diffusion(int nx, int ny, int nz, double sigma, double wx, double wy, double wdiag,
                       double dominance, uint64_t seed, int *n, long *nnz, int **ptr, int **col, double **val);
void mpkg_uniform(uint64_t seed, long n, double *out);

const char *mpkg_last_error(void);
int mpkg_version(void);

#ifdef __cplusplus
}
#endif

#endif
