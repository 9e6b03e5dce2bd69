/*
 * perks.h — C ABI of the GB300 (sm_103a) PERKS stencil and CG library.
 *
 * Plain C types only: device or host pointers, sizes, small option structs.
 * Every entry point returns a status code and never exits the process; a
 * human-readable message for the last failure on the calling thread is
 * available from perks_last_error().
 *
 * Each entry point names the reference interface it replaces (paths inside
 * the neozhang307/PERKS project).
 */
#ifndef PERKS_GB300_H
#define PERKS_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define PERKS_API __attribute__((visibility("default")))
#else
#define PERKS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PERKS_ABI_VERSION 3

/* ------------------------------------------------------------------ codes */
typedef enum {
  PERKS_OK = 0,
  PERKS_ERR_INVALID_ARG = -10,  /* null pointer, bad size, unknown enum */
  PERKS_ERR_UNSUPPORTED = -11,  /* shape/dtype/size combination not built */
  PERKS_ERR_NO_DEVICE = -12,    /* no CUDA device / driver */
  PERKS_ERR_CUDA = -13,         /* a CUDA runtime call failed */
  PERKS_ERR_OOM = -14,          /* device allocation failed */
  PERKS_ERR_TIMEOUT = -15,      /* a device-side wait ran out its budget */
  PERKS_ERR_LAUNCH = -16,       /* cooperative grid does not fit the GPU */
  PERKS_ERR_BREAKDOWN = -17,    /* CG: p.Ap <= 0 or non-finite (matrix not SPD) */
  PERKS_ERR_NOT_CONVERGED = -18 /* CG: max_iter reached before the tolerance */
} perks_status;

/* Stencil shapes, one per reference executable
 * (stencil/2dstencil/<shape>/, stencil/3dstencil/<shape>/). */
typedef enum {
  PERKS_2D5PT = 0,   /* star, halo 1 */
  PERKS_2DS9PT = 1,  /* star, halo 2 */
  PERKS_2D13PT = 2,  /* star, halo 3 */
  PERKS_2D17PT = 3,  /* star, halo 4 */
  PERKS_2D21PT = 4,  /* star, halo 5 */
  PERKS_2DS25PT = 5, /* star, halo 6 */
  PERKS_2D9PT = 6,   /* box 3x3 */
  PERKS_2D25PT = 7,  /* box 5x5 */
  PERKS_3D7PT = 16,  /* star, halo 1 */
  PERKS_3D13PT = 17, /* star, halo 2 */
  PERKS_3D17PT = 18, /* corners + centre plane, halo 1 */
  PERKS_3D27PT = 19, /* box 3x3x3 */
  PERKS_POISSON = 20 /* 19-point, halo 1 */
} perks_shape;

typedef enum { PERKS_FP32 = 0, PERKS_FP64 = 1, PERKS_MIXED = 2 } perks_dtype;

typedef enum {
  PERKS_BOUNDARY_CLAMP = 0,    /* reference semantics: out-of-range neighbours clamp to the edge */
  PERKS_BOUNDARY_DIRICHLET = 1 /* the outer `halo` cells on each face stay fixed */
} perks_boundary;

typedef enum {
  PERKS_ORDER_REFERENCE = 0, /* bit-identical to the reference CPU gold code */
  PERKS_ORDER_FAST = 1       /* folded coefficients + FMA */
} perks_order;

typedef enum {
  PERKS_KERNEL_PERSISTENT = 0, /* one cooperative launch for all steps, rows/planes kept on chip */
  PERKS_KERNEL_PER_STEP = 1,   /* one launch per time step, nothing kept on chip (comparator) */
  PERKS_KERNEL_NAIVE = 2       /* 2D only: one launch per step, one thread per cell reading every
                                  neighbour from global memory (comparator: the reference's
                                  kernel2d_restrict, stencil/2dstencil/jacobi-naive.cu:7-106) */
} perks_kernel;

/* --------------------------------------------------------------- stencils */
typedef struct {
  int shape;       /* perks_shape */
  int dtype;       /* PERKS_FP32 or PERKS_FP64 (storage and arithmetic type) */
  int boundary;    /* perks_boundary */
  int order;       /* perks_order */
  int kernel;      /* perks_kernel */
  int cache_rows;  /* persistent kernel: rows (2D) / planes (3D) per CTA kept in shared memory;
                      -1 = as many as fit, 0 = none. Default: -1 for 2D, 0 for 3D (resident
                      planes are built and tested but measured slower on GB300) */
  int l2_sweep;    /* persistent kernel: alternate the sweep direction each step and drop dead
                      lines from L2, so the rows written last are read first from L2 (1 = on) */
  int tile_x;      /* columns per CTA tile; 0 = auto */
  int tile_y;      /* 3D only: rows per CTA tile; 0 = auto */
  int ctas;        /* CTAs in the persistent grid; 0 = one per SM */
  void* stream;    /* cudaStream_t; NULL = legacy default stream */
  int tma;         /* 2D persistent / per-step kernels: 1 = rows reach each warp's ring by TMA tensor
                      copies (one lane issues, an mbarrier per slot), 0 = per-lane cp.async (default).
                      The 3D kernels always use tensor copies; the naive kernel none. */
} perks_stencil_opts;

typedef struct {
  double ms;            /* device time of the stencil kernels (CUDA events), excludes layout copies */
  double gcells_per_s;  /* cells * steps / ms / 1e6 (reference formula, jacobi-2d.cu:822) */
  double cached_fraction; /* share of cells kept in shared memory across steps */
  int grid_x, grid_y, grid_z; /* tile grid */
  int tile_x, tile_y;
  int cached_rows;      /* rows (2D) / planes (3D) per CTA kept in shared memory */
  int launches;         /* kernels launched by the call */
} perks_stencil_stats;

/* Fill `opts` with defaults for a shape and dtype. */
PERKS_API void perks_stencil_default_opts(perks_stencil_opts* opts, int shape, int dtype);

/* 2D Jacobi time loop on device buffers.
 * d_in: width_y*width_x row-major, not modified. d_out: same size, written.
 * d_in and d_out must not overlap. `steps` >= 0 (0 copies d_in to d_out).
 * Replaces the device path of jacobi_iterative<REAL>
 * (stencil/2dstencil/jacobi-2d.cu:371-865). `stats` may be NULL. */
PERKS_API int perks_stencil2d(const perks_stencil_opts* opts, const void* d_in, void* d_out, int width_y,
                    int width_x, int steps, perks_stencil_stats* stats);

/* 3D Jacobi time loop on device buffers, layout [height][width_y][width_x].
 * Replaces the device path of j3d_iterative<REAL>
 * (stencil/3dstencil/j3d.cu:129-808). */
PERKS_API int perks_stencil3d(const perks_stencil_opts* opts, const void* d_in, void* d_out, int height,
                    int width_y, int width_x, int steps, perks_stencil_stats* stats);

/* perks_stencil2d for callers that cannot allocate device memory (programs
 * that fix their device-memory footprint at start-up, or run under another
 * framework's memory manager, and may not call cudaMalloc mid-run). No
 * counterpart in the reference. Same arguments and results as
 * perks_stencil2d (reference evaluation order only), but all scratch comes
 * from one 32 MiB static device array inside the library: fields needing more
 * (2 * width_y * padded width * sizeof(REAL) + 256 bytes) are rejected with
 * PERKS_ERR_INVALID_ARG. Every call looks up the array's address on the
 * current device (no allocation); the first call on a device may load the
 * library's device code and should come before any stream capture. Calls
 * share the array: calls whose GPU work overlaps race and must not be
 * issued. */
PERKS_API int perks_stencil2d_noalloc(const perks_stencil_opts* opts, const void* d_in, void* d_out,
                                      int width_y, int width_x, int steps, perks_stencil_stats* stats);

/* Host-buffer drop-ins with the reference's argument list. The stencil shape
 * is the first argument (the reference fixes it per executable with -D
 * macros). bdimx/blkpsm/async/useSM/isDoubleTile keep their meaning where
 * it carries over: useSM=0 disables shared-memory row caching; the others are
 * accepted and ignored. usewarmup runs `warmupiteration` (or `iteration`
 * when <=0) untimed steps first. Returns 0 on success, the reference's code 1
 * (jacobi-2d.cu:600) never, and a negative perks_status on failure.
 * Replaces jacobi_iterative<float/double> (stencil/2dstencil/common/jacobi_cuda.cuh:6-10). */
PERKS_API int perks_jacobi_iterative_f32(int shape, const float* h_in, int width_y, int width_x, float* h_out,
                               int bdimx, int blkpsm, int iteration, int async, int useSM,
                               int usewarmup, int warmupiteration, int isDoubleTile);
PERKS_API int perks_jacobi_iterative_f64(int shape, const double* h_in, int width_y, int width_x,
                               double* h_out, int bdimx, int blkpsm, int iteration, int async,
                               int useSM, int usewarmup, int warmupiteration, int isDoubleTile);
/* Replaces j3d_iterative<float/double> (stencil/3dstencil/common/jacobi_cuda.cuh:6-10).
 * Reference return codes kept: -2 unsupported widths, -4 height too small.
 * getminHeight=1 returns the minimum-domain height without running (h_in and
 * h_out may be NULL): perks_stencil3d_min_domain for this shape and dtype
 * (useSM=0: 0, the reference's answer for a run without a plane cache,
 * j3d.driver.cpp:102-108). */
PERKS_API int perks_j3d_iterative_f32(int shape, const float* h_in, int height, int width_y, int width_x,
                            float* h_out, int bdimx, int blkpsm, int iteration, int useSM,
                            int usewarmup, int warmupiteration, int isDoubleTile, int getminHeight);
PERKS_API int perks_j3d_iterative_f64(int shape, const double* h_in, int height, int width_y, int width_x,
                            double* h_out, int bdimx, int blkpsm, int iteration, int useSM,
                            int usewarmup, int warmupiteration, int isDoubleTile, int getminHeight);

/* Minimum-domain mode (the reference's --small: jacobi.driver.cpp:84-109
 * with getMinWidthY, stencil/2dstencil/jacobi-2d.cu:79-136). Writes to
 * *width_y the largest height of a width_x-wide field at which the persistent
 * 2D kernel keeps, between time steps, every row in shared memory except the
 * H rows at each end of each row band (those are the halo the neighbouring
 * bands read from the field). Depends on shape, dtype, cache_rows and ctas of
 * `opts`; 0 when the options cache nothing (per-step kernel, cache_rows=0). */
PERKS_API int perks_stencil2d_min_domain(const perks_stencil_opts* opts, int width_x, int* width_y);
/* The 3D counterpart (the reference's getminHeight, j3d.driver.cpp:62-144):
 * writes to *height the largest height of a width_y x width_x field at which
 * the persistent 3D kernel keeps, between time steps, every plane tile of
 * every CTA's z-runs in shared memory except the H planes at each end of a
 * run (those are the halo the neighbouring runs read from the field).
 * Depends on shape, dtype, order, cache_rows (planes per CTA) and ctas of
 * `opts`; 0 when no plane tile fits next to the kernel's copy ring or
 * cache_rows = 0. */
PERKS_API int perks_stencil3d_min_domain(const perks_stencil_opts* opts, int width_y, int width_x, int* height);
/* getMinWidthY<REAL>(width_x, bdimx, registers, useSM, blkpsm, isDoubleTile)
 * (stencil/2dstencil/common/jacobi_cuda.cuh:14) with the shape and dtype
 * first: returns that width_y (>= 0) or a negative perks_status. bdimx,
 * registers, blkpsm and isDoubleTile are accepted and ignored. */
PERKS_API int perks_get_min_width_y(int shape, int dtype, int width_x, int bdimx, int registers, int useSM,
                                    int blkpsm, int isDoubleTile);

/* --------------------------------------------------------------------- CG */
typedef enum {
  PERKS_STOP_ABS_RR = 0, /* reference: stop when r.r < tol*tol (cg_kernels.cuh:834) */
  PERKS_STOP_REL = 1     /* stop when ||r|| / ||b|| < tol */
} perks_cg_stop;

typedef enum {
  PERKS_CG_PLAIN = 0,            /* the reference's iteration (cg_cpu.cpp:40-81): p, A p, alpha, x, r, beta */
  PERKS_CG_SINGLE_REDUCTION = 1  /* Chronopoulos & Gear (1989): A p and A r carried by recurrences, one row
                                    pass, one barrier and one fused reduction of r.r and (A r).r per
                                    iteration; the same iterates in exact arithmetic, other rounding.
                                    Persistent kernel, FP64 or FP32, no checkpoint. */
} perks_cg_algorithm;

/* CG checkpoint: the iteration state between two iterations, so that a
 * solve can stop and later resume exactly where it stopped (the resumed run
 * gives bit-identical x and r to one uninterrupted run with the same options).
 * The caller owns d_r and d_p (n elements of the working type: FP64 for
 * PERKS_FP64, FP32 for PERKS_FP32 and PERKS_MIXED) and, for PERKS_MIXED, d_xs
 * (n floats); the solution itself is the caller's x. A mixed-precision solve
 * given a checkpoint keeps the increment that its last iterations built in
 * d_xs instead of adding it to x when it stops at max_iter, so that the
 * resumed solve continues exactly as an uninterrupted one: x + d_xs is then
 * the iterate. */
typedef struct {
  void* d_r;        /* device: residual r (PERKS_MIXED: the FP32 recursive residual) */
  void* d_p;        /* device: the last search direction p */
  void* d_xs;       /* device, PERKS_MIXED only: the FP32 solution increment not yet added to x */
  double rr;        /* r.r as the iteration holds it (in the working precision) */
  double rr_prev;   /* r.r one iteration earlier (for beta) */
  double bb;        /* b.b (relative stop) */
  double maxrr;     /* PERKS_MIXED: r.r at the last reliable update */
  int outer;        /* PERKS_MIXED: reliable updates done */
  int since;        /* PERKS_MIXED: iterations since the last reliable update */
  int k;            /* iterations completed; 0 = no state yet (start from x) */
  int kernel;       /* perks_kernel that wrote the state; resuming needs the same */
  int dtype;        /* perks_dtype that wrote the state; resuming needs the same */
  int n;            /* rows of the solve that wrote it; resuming needs the same */
} perks_cg_state;

typedef struct {
  int dtype;          /* PERKS_FP64, PERKS_FP32 (reference float build), PERKS_MIXED
                         (FP32 inner CG, FP64 x, true residual and refinement) */
  int stop;           /* perks_cg_stop */
  double tol;
  int max_iter;       /* iteration cap (inner iterations for PERKS_MIXED) */
  int static_iter;    /* 1 = run exactly max_iter iterations (reference --staticiter) */
  int kernel;         /* PERKS_KERNEL_PERSISTENT (one cooperative launch) or PERKS_KERNEL_PER_STEP */
  int replace_every;  /* PERKS_MIXED: recompute r = b - A x in FP64 every this many inner iterations
                         (0 = auto) */
  int ctas;           /* CTAs in the persistent grid; 0 = auto */
  void* stream;       /* cudaStream_t */
  perks_cg_state* checkpoint; /* NULL = none. Otherwise the solve resumes from *checkpoint when
                                 checkpoint->k > 0 (x must hold the iterate saved with it) and
                                 writes its final state back, also when it returns
                                 PERKS_ERR_NOT_CONVERGED. max_iter counts all iterations,
                                 including those before the checkpoint. */
  int cache_vectors;  /* persistent kernel: KB of shared memory per CTA in which each CTA keeps its
                         rows of the vectors that only it touches (r unless the SpMV gathers it, x
                         or the mixed increment, Ap) for the whole solve; the rest streams.
                         0 = none, -1 = the library's default: 160 KB for the DIA and ELL layouts,
                         none for CSR and SELL (the shared memory is taken from the L1 cache that
                         the SpMV gathers use: more than about 160 KB cost more than it saved) */
  int cluster;        /* persistent kernel: CTAs per thread-block cluster (1 = none, default; 2, 4,
                         8, 16): the CTAs of a cluster combine their dot-product partials over
                         distributed shared memory and only one CTA per cluster takes part in the
                         grid barrier; the grid is then as many whole clusters as fit at once */
  int algorithm;      /* perks_cg_algorithm (default PERKS_CG_PLAIN) */
} perks_cg_opts;

typedef struct {
  int iterations;        /* CG iterations executed (inner iterations summed for PERKS_MIXED) */
  int outer;             /* PERKS_MIXED: residual replacements / refinement restarts */
  double rr;             /* last recursive r.r */
  double true_rel_res;   /* ||b - A x|| / ||b|| recomputed in FP64 on the device after the solve */
  double ms;             /* device time of the solve */
  int launches;
  int layout;            /* matrix layout the iteration ran on: 0 CSR as given (lane groups per row),
                            1 DIA, 2 ELL, 3 SELL (copies made at the start of the solve) */
  int ctas;              /* CTAs of the persistent launch */
} perks_cg_result;

PERKS_API void perks_cg_default_opts(perks_cg_opts* opts);

/* Solve A x = b with CG. A in CSR (int32 row_ptr[n+1], col[nnz]; values FP64
 * for PERKS_FP64/PERKS_MIXED, FP32 for PERKS_FP32). x holds the initial guess
 * on entry and the solution on return (FP64 except for PERKS_FP32). All
 * pointers are device pointers. Replaces DispatchCG::ProcessDispatchCG
 * (conjugateGradient/cg_dispatcher.cuh:559-916) and the kernel
 * gpuConjugateGradient_cub (conjugateGradient/cg_kernels.cuh:620-986). */
PERKS_API int perks_cg_csr(int n, int nnz, const int* d_row_ptr, const int* d_col, const void* d_val,
                 const void* d_b, void* d_x, const perks_cg_opts* opts, perks_cg_result* res);

/* CG with A in DIA format: `ndiag` diagonals with offsets h_offsets[ndiag]
 * (host array, |offset| < n, at most 32 diagonals), values d_data[ndiag][n]
 * diagonal-major where d_data[k*n + i] = A[i][i + offset[k]] (zero where
 * i + offset is out of range). Generalises the reference's tridiagonal DIA
 * SpMV (conjugateGradient/cg_dia_kernels.cuh:184-231) to k diagonals. */
PERKS_API int perks_cg_dia(int n, int ndiag, const int* h_offsets, const void* d_data, const void* d_b,
                 void* d_x, const perks_cg_opts* opts, perks_cg_result* res);

/* y = A x for CSR / DIA (dtype PERKS_FP32 or PERKS_FP64). Building blocks
 * exposed for tests and callers that run their own iteration. */
PERKS_API int perks_spmv_csr(int dtype, int n, int nnz, const int* d_row_ptr, const int* d_col,
                   const void* d_val, const void* d_x, void* d_y, void* stream);
PERKS_API int perks_spmv_dia(int dtype, int n, int ndiag, const int* h_offsets, const void* d_data,
                   const void* d_x, void* d_y, void* stream);

/* ---------------------------------------------------------------- batches */
/* Many independent stencil and CG instances of uneven size in ONE persistent
 * launch: CTAs take work items from a device work queue (largest jobs first).
 * A job is one item, or, for a stencil job larger than total work / (2 x SMs),
 * a run of row slices whose CTAs meet at a job barrier after each time step;
 * no grid-wide barrier is used. A stencil job whose two fields fit in one
 * CTA's shared memory stays there for all its time steps. The run is a CUDA
 * graph {reset the queue, launch}. The reference runs one instance per
 * executable (stencil/2dstencil/jacobi.driver.cpp, conjugateGradient/
 * cg_driver.cu); this interface has no counterpart there. */
typedef enum { PERKS_JOB_STENCIL = 0, PERKS_JOB_CG = 1 } perks_job_kind;

typedef struct {
  int kind;          /* perks_job_kind */
  int dtype;         /* PERKS_FP32 or PERKS_FP64; CG jobs also PERKS_MIXED (FP64 values, b and x, FP32
                        inner iteration with FP64 reliable updates, for FP64 tolerances) */
  /* stencil: shape (PERKS_2D5PT, PERKS_2DS9PT, PERKS_2D9PT or PERKS_3D7PT),
   * clamp boundary, reference evaluation order; h = 1 for 2D */
  int shape, h, wy, wx, steps;
  const void* d_in;  /* device field [h][wy][wx], not modified */
  void* d_out;       /* device field [h][wy][wx] */
  /* CG: A in CSR (device; values of dtype), b, x (device, dtype); x starts
   * at 0 (its input is ignored); stop when ||r|| <= tol ||b|| or after
   * max_iter iterations */
  int n, nnz;
  const int* d_row_ptr;
  const int* d_col;
  const void* d_val;
  const void* d_b;
  void* d_x;
  double tol;
  int max_iter;
} perks_job;

typedef struct {
  int iterations;    /* CG: iterations done; stencil: time steps done */
  int status;        /* PERKS_OK, or PERKS_ERR_BREAKDOWN / PERKS_ERR_NOT_CONVERGED for CG */
  double rel_res;    /* CG: ||r|| / ||b|| of the recursive residual */
} perks_job_result;

typedef struct {
  int threads;       /* threads per CTA (256, 512 or 1024); 0 = autotune */
  int ctas_per_sm;   /* 1 or 2; 0 = autotune */
  void* stream;      /* cudaStream_t; NULL = default stream */
  int slicing;       /* work granularity: a stencil job costlier than (total cost) / (slicing x SMs)
                        is cut into row slices run by several CTAs; 1, 2, 4, 8 or 16; 0 = autotune
                        over 2..16 */
} perks_batch_opts;

typedef struct {
  double ms;          /* device time of the last run */
  int threads, ctas_per_sm, grid;  /* the launch shape in use */
  int resident_jobs;  /* stencil jobs kept in shared memory for all steps */
  int tuned;          /* 1 if the launch shape came from the autotuner */
  int sliced_jobs;    /* stencil jobs cut into row slices run by several CTAs */
  int slicing;        /* the work granularity in use (see perks_batch_opts) */
} perks_batch_stats;

typedef struct perks_batch_plan_s* perks_batch_plan;

PERKS_API void perks_batch_default_opts(perks_batch_opts* opts);
/* Validate the jobs, order them, allocate their scratch, autotune the launch
 * shape when asked (by timing one run of each candidate), and capture the
 * graph. Job pointers must stay valid while the plan exists. */
PERKS_API int perks_batch_plan_create(const perks_job* jobs, int njobs, const perks_batch_opts* opts,
                                      perks_batch_plan* plan);
/* Run the batch once (graph launch on `stream`, or the plan's stream when
 * NULL) and wait for it; stats may be NULL. */
PERKS_API int perks_batch_plan_run(perks_batch_plan plan, void* stream, perks_batch_stats* stats);
/* Per-job results of the last run, in the caller's job order (njobs entries). */
PERKS_API int perks_batch_plan_results(perks_batch_plan plan, perks_job_result* results);
PERKS_API void perks_batch_plan_destroy(perks_batch_plan plan);

/* ------------------------------------------------------------ MatrixMarket */
/* Host code (no GPU). Reads a MatrixMarket file as the reference's
 * CooMatrix::InitMarket + CsrMatrix::Init do
 * (conjugateGradient/matrix/sparse_matrix.h:217-380, 633-730): coordinate
 * real/integer/pattern (a missing value reads as 1.0) or array files,
 * symmetric and skew-symmetric files with every off-diagonal entry mirrored,
 * entries stably sorted by (row, column), duplicates kept. perks_mtx_size
 * gives the dimensions and the entry count after mirroring; perks_mtx_read_csr
 * fills caller arrays row_ptr[rows+1], col[nnz], val[nnz]. */
PERKS_API int perks_mtx_size(const char* path, int* rows, int* cols, long long* nnz);
PERKS_API int perks_mtx_read_csr(const char* path, int rows, long long nnz_cap, int* row_ptr, int* col,
                                 double* val, long long* nnz);

/* ------------------------------------------------------------ measurement */
/* FMA throughput of this GPU in the given precision (PERKS_FP64 or
 * PERKS_FP32), in fused multiply-adds per second (a FLOP rate is twice it):
 * eight independent FMA chains per thread, four 256-thread CTAs per SM, one
 * launch of about 0.1 s. The arithmetic roofline of the FP64 stencils and
 * CG, which are bound by the FP64 pipe on GB300 rather than by HBM. `ms`
 * (may be NULL) receives the timed launch's duration. */
PERKS_API int perks_probe_fma_peak(int dtype, double* fma_per_s, double* ms);

/* ------------------------------------------------------------------ misc */
PERKS_API const char* perks_last_error(void);     /* thread-local message of the last failure */
PERKS_API const char* perks_status_string(int status);
PERKS_API int perks_abi_version(void);
/* Testing hook for the device-side timeout path (no counterpart in the
 * reference). Every device-side wait of the persistent kernels (grid barrier,
 * batch job barrier, bulk-copy mbarrier) gives up after a clock budget, sets
 * the kernel's status word and leaves; the call then returns
 * PERKS_ERR_TIMEOUT and the CUDA context stays usable. This sets, for the
 * launches that follow in this process, the budget in SM clock cycles
 * (<= 0: the default, about 2^32) and a CTA index that skips its first
 * grid-barrier arrival (batch plans: the slice index that skips its first job
 * barrier), so that every waiting CTA's budget runs out (< 0: none). Batch
 * plans take the setting when they are created. Returns PERKS_OK. */
PERKS_API int perks_debug_set_wait_fault(long long budget_cycles, int skip_cta);

/* Check of the kernels' exact FP32 division by a constant (118: the 2D star
 * shapes; 159) over all 2^32 inputs against IEEE round-to-nearest division
 * on this GPU. `form` selects the finish (0 to 3, the 2D kernels' tuning
 * table picks one per shape; 2 = the short path wherever its flag test is
 * clear, the full finish elsewhere; 3 = the branch-free short finish).
 * mismatches[2] receives the mismatch counts of
 * the two device forms (per element; packed pairs), first_bad[2] (may be
 * NULL) the lowest mismatching bit pattern of each (0xffffffff: none). */
PERKS_API int perks_debug_div_check(int divisor, int form, long long* mismatches, unsigned* first_bad);

/* Device allocations (cudaMalloc) the library's own grow-only workspace has
 * made in this process: lets a test check that an entry point allocated
 * nothing. */
PERKS_API long long perks_debug_workspace_allocs(void);

/* Kernels launched by this thread since the counter was last reset. */
PERKS_API long long perks_launch_count(void);
PERKS_API void perks_reset_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* PERKS_GB300_H */
