/* gbstencil: GB300-native temporally-blocked stencil engine, C ABI.
 *
 * This is the drop-in boundary for the AN5D artifact's per-benchmark stencil
 * time loop. Every benchmark there defines
 *
 *     double kernel_stencil(SB_TYPE *A1, int compsize, int timestep, bool scop);
 *
 * (declared at common.h:42, defined at <stencil>.c:7 and, in generated form,
 * at compiled/<prec>/<cfg>_host.cu:10). Its scop==true branch is the GPU time
 * loop that gbs_run() replaces; the artifact's C harness (common.h: main,
 * -s/-t/-n/-c, init_grid, check_result) stays as it is.
 *
 * Grid convention (the reference's): a grid of interior extent n[] per axis
 * is stored with a fixed Dirichlet halo of width r, so dimsize = n + 2r per
 * axis, and two time planes: A[2][d0][d1] (2-D) or A[2][d0][d1][d2] (3-D),
 * row-major, last index fastest. Step t reads plane t%2 and writes the
 * interior of plane (t+1)%2; the halo is never written. After T steps plane
 * T%2 holds u_T. Halo cells must hold the same values in both planes (as
 * init_grid, common.h:50-55, sets them).
 *
 * No function here allocates on the caller's behalf except gbs_run (which,
 * like the reference's host code, owns its device copy) and the batch /
 * adjoint planners, which say so. All functions return a gbs_status; none
 * aborts. gbs_last_error() describes the last failure of the calling thread.
 */
#ifndef GBSTENCIL_H
#define GBSTENCIL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gbs_status {
  GBS_OK = 0,
  GBS_ERR_INVALID = 1,     /* bad descriptor or argument */
  GBS_ERR_UNSUPPORTED = 2, /* no kernel instantiated for this combination */
  GBS_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  GBS_ERR_NOMEM = 4,       /* a device or pinned-host allocation failed */
  GBS_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  GBS_ERR_NODEVICE = 6     /* no usable sm_103 device */
} gbs_status;

enum { GBS_F32 = 0, GBS_F64 = 1 };

/* Floating-point evaluation mode.
 * GBS_FP_EXACT: every product and sum rounded separately, in the order the
 *   artifact's source writes the terms; divisions and square roots IEEE. The
 *   result is bit-identical to the artifact's CPU path (kernel_stencil with
 *   scop==false) built without floating-point contraction.
 * GBS_FP_FMA: the same terms accumulated with fused multiply-adds (one
 *   rounding per term, as the artifact's own nvcc build contracts them); the
 *   term order may differ. Results agree with the CPU path within the parity
 *   tolerance (normwise 1e-5 float, 1e-12 double). */
enum { GBS_FP_EXACT = 0, GBS_FP_FMA = 1 };

typedef struct gbs_desc {
  int stencil;       /* gbs_stencil_id("star2d1r"), ... */
  int dtype;         /* GBS_F32 | GBS_F64: the reference's SB_TYPE */
  int n[3];          /* interior extent per axis (the reference's compsize on
                        every axis); n[2] is ignored for 2-D stencils */
  int timestep;      /* T >= 0 */
  int fp_mode;       /* GBS_FP_EXACT | GBS_FP_FMA */
  int bt;            /* timesteps fused per launch (temporal degree); 0 = tuned */
  int bs1;           /* block shape. 3-D (FMA mode): tile rows per CTA, one of
                        the heights built for the degree (gbs_plan reports
                        them; 64 and 32 rows for most stencils at bt=1);
                        2-D: warps per CTA, 4; 0 = tuned */
  int bs2;           /* tile columns: 32 * (16 bytes / element size) (one
                        warp's 16-byte vector per lane); 0 = that */
  int sl;            /* stream block length in rows (2-D) / planes (3-D); 0 = tuned */
  const void *coef;  /* NULL: the source literals. Else nterms values of dtype,
                        term order as in the source (the gradient form takes
                        its numerator in coef[0]) */
  double divisor;    /* stencils with a divisor (j2d5pt: /118): 0 = source value */
  double eps;        /* gradient2d's epsilon: 0 = source value (0.0001f) */
} gbs_desc;

/* Device-side layout of a two-plane grid. Rows (the innermost axis) are
 * padded to `pitch` elements and column c of a row is stored at element
 * `shift + c`, so that every 16-byte-aligned window a kernel streams is
 * inside the allocation. */
typedef struct gbs_layout {
  size_t pitch;      /* elements between consecutive rows */
  size_t shift;      /* element offset of column 0 within a row */
  size_t rows;       /* rows per plane: d0 (2-D) or d0*d1 (3-D) */
  size_t plane;      /* elements per time plane (rows * pitch) */
  size_t bytes;      /* bytes of the two-plane device buffer */
  int dimsize[3];    /* n + 2r per axis (1 for unused axes) */
  int dim, rad;
} gbs_layout;

/* The launch sequence the engine will run for a descriptor. */
typedef struct gbs_plan_info {
  int bt;            /* temporal degree chosen */
  int bs1, bs2, sl;  /* tile / stream parameters chosen */
  int launches;      /* kernel launches for the whole time loop */
  int ctas;          /* CTAs per full-degree launch */
  int valid_w;       /* valid (non-overlap) output columns per warp strip */
  double redundancy; /* computed cells / useful cells per launch */
} gbs_plan_info;

/* ---- stencil catalogue ------------------------------------------------ */
int gbs_num_stencils(void);
const char *gbs_stencil_name(int id);
int gbs_stencil_id(const char *name); /* -1 if unknown */
/* dim, radius, terms in the update expression, BENCH_FPP (<stencil>.c:1-3) */
gbs_status gbs_stencil_info(int id, int *dim, int *rad, int *nterms, int *fpp);

/* ---- drop-in time loop ------------------------------------------------ */
/* Replaces kernel_stencil(A1, compsize, timestep, scop=true)
 * (common.h:42; generated host sequencer compiled/float/
 * star2d1r-256-10-256_host.cu:10-566). host_A is the dense two-plane grid;
 * both planes are copied to the device, advanced d->timestep steps and copied
 * back. *ms_out (may be NULL) receives the device time of the time loop only,
 * excluding allocation and copies, as the reference's return value does
 * (_host.cu:39-40,559-560). The device buffers (the grid in the engine layout
 * and a dense staging copy, through which the host copies run as single
 * contiguous transfers) are cached between calls. */
gbs_status gbs_run(const gbs_desc *d, void *host_A, double *ms_out);

/* Same time loop on a device buffer in the engine's layout (gbs_get_layout),
 * enqueued on `stream` (a cudaStream_t; NULL = legacy default stream).
 * Asynchronous: completion and device-side errors are reported by the next
 * gbs_sync(stream). */
gbs_status gbs_run_device(const gbs_desc *d, void *dev_A, void *stream);

gbs_status gbs_get_layout(const gbs_desc *d, gbs_layout *out);
gbs_status gbs_plan(const gbs_desc *d, gbs_plan_info *out);

/* ---- autotuner ---------------------------------------------------------- */
/* Replaces the artifact's offline model (Model_V100.xlsm, Formula/Macro
 * sheets) and its tuned-configuration lists (compiled/v100_float.csv:1-105,
 * columns bS1,bS2,bT,sl). gbs_tune ranks every (bt, sl) the build supports
 * for d's stencil, dtype, fp mode and size with a roofline model
 * (max(2*sizeof(T)/(bt*B_hbm), redundancy*fpp/P_fp) per cell update, plus a
 * launch gap per bt steps), times the candidates the model keeps on a scratch
 * grid of the same size (d->timestep is ignored), records the fastest in the
 * engine's tuning table and returns the candidates fastest first. When
 * d->bt / d->sl are 0, the time loop and gbs_plan resolve them through that
 * table (the entry of the same stencil, dtype and mode whose size class,
 * floor(log2(interior cells)), is nearest, within 3), else by a fixed rule.
 * The table is also loaded from the file named by the environment variable
 * GBS_TUNING at first use. Text format, one entry per line:
 * "<stencil> <f32|f64> <exact|fma> <size class> <bt> <sl> [<bs1>] <ms per step>"
 * (bs1: 3-D tile rows; absent or 0: the default shape). */
typedef struct gbs_tune_candidate {
  int bt, sl;               /* sl 0: the engine's one-wave stream length */
  double redundancy;        /* computed / useful cells per launch */
  double model_ms_per_step; /* the model's time for one timestep */
  double ms_per_step;       /* measured; < 0 if the model pruned it */
  int bs1;                  /* 3-D tile rows (block shape); 0 in 2-D */
} gbs_tune_candidate;
gbs_status gbs_tune(const gbs_desc *d, gbs_tune_candidate *cands, int max_cands, int *ncands);
gbs_status gbs_tune_set(const gbs_desc *d, int bt, int sl, double ms_per_step);
/* the model's time per step for d as planned (d->bt / d->sl or the table's) */
gbs_status gbs_tune_model(const gbs_desc *d, double *ms_per_step);
gbs_status gbs_tune_lookup(const gbs_desc *d, int *bt, int *sl); /* bt = 0: no entry */
gbs_status gbs_tune_load(const char *path);
gbs_status gbs_tune_save(const char *path);
int gbs_tune_entries(void);
void gbs_tune_clear(void);

/* Dense host grid <-> engine layout, both planes, enqueued on `stream`. */
gbs_status gbs_upload(const gbs_desc *d, const void *host_A, void *dev_A, void *stream);
gbs_status gbs_download(const gbs_desc *d, const void *dev_A, void *host_A, void *stream);

/* Waits for `stream` and turns a device-side error word (a bounded wait that
 * gave up) into GBS_ERR_TIMEOUT. */
gbs_status gbs_sync(void *stream);

/* ---- batched launch ------------------------------------------------------ */
/* Many independent grids (any mix of stencils, sizes and step counts),
 * advanced by ONE launch of a CUDA graph. No counterpart in the artifact,
 * which runs one grid per process; this replaces a loop of per-grid
 * kernel_stencil calls. */
typedef struct gbs_batch_grid {
  int stencil;        /* a stencil id (3-D stencils: GBS_BATCH_STREAMS only) */
  int n[3];           /* interior extent per axis (n[2] ignored for 2-D) */
  int timestep;       /* T >= 0 */
  void *dev_A;        /* two-plane grid in the engine layout (gbs_get_layout of
                         the same stencil, the batch's dtype and n), 128-byte
                         aligned */
  const void *coef;   /* NULL = the source literals, else nterms values of the
                         batch's dtype */
  double divisor;     /* 0 = the source value */
} gbs_batch_grid;

typedef struct gbs_batch gbs_batch; /* opaque plan */

typedef struct gbs_batch_stats {
  int grids, items, ctas;
  int plain_launches;      /* kernel launches the same work takes one grid at a time */
  long long cell_updates;  /* sum of n[0]*n[1]*timestep */
  int kernels;             /* kernel nodes in the plan's graph */
  int mode;                /* GBS_BATCH_PERSISTENT | GBS_BATCH_LAYERED | GBS_BATCH_STREAMS */
  long long hbm_bytes;     /* algorithmic HBM bytes of one run: each fused launch (time block)
                              of a grid reads and writes its interior once */
} gbs_batch_stats;

/* How a batch plan schedules its work:
 * GBS_BATCH_PERSISTENT: one persistent kernel over work items (grid, time
 *   block, strip, stream block) of 2-D float grids; CTAs take groups of
 *   consecutive items in time-block order from an atomic counter, and an
 *   item waits (bounded) until its stream block and the two beside it have
 *   finished the grid's earlier time blocks (per-block completion counters).
 * GBS_BATCH_LAYERED: the same 2-D work items, one kernel node per time block
 *   in the graph, each over every grid's items of that block; kernel
 *   boundaries order the blocks, so nothing waits on the device.
 * GBS_BATCH_STREAMS: each grid's own time loop (the single-grid kernels at
 *   the tuned degree, one kernel node per fused launch) as a chain in the
 *   graph; the chains are spread over 16 branches (environment
 *   GBS_BATCH_BRANCHES, 1..64), heaviest grid first onto the least loaded
 *   branch, so independent grids run side by side. Takes 2-D and 3-D grids,
 *   float or double. */
enum { GBS_BATCH_PERSISTENT = 0, GBS_BATCH_LAYERED = 1, GBS_BATCH_STREAMS = 2 };

/* Plans the batch: the CUDA graph, and for the work-item schedules the work
 * list and its dependency counters (device memory owned by the plan).
 * dtype: GBS_F32 for every schedule, GBS_F64 for GBS_BATCH_STREAMS; a 3-D
 * grid or GBS_F64 under a work-item schedule is GBS_ERR_UNSUPPORTED. The
 * grids' buffers must stay valid while the plan is used. */
gbs_status gbs_batch_plan(const gbs_batch_grid *grids, int ngrids, int dtype, int fp_mode, int mode,
                          gbs_batch **out);
/* Replays the plan's graph on `stream` (asynchronous; see gbs_sync). */
gbs_status gbs_batch_run(gbs_batch *plan, void *stream);
gbs_status gbs_batch_info(const gbs_batch *plan, gbs_batch_stats *out);
void gbs_batch_destroy(gbs_batch *plan);

/* Batched run that allocates nothing, for callers that may not allocate
 * device memory: code that lives inside a framework whose caching allocator
 * owns the whole device budget, or a host loop that must not call cudaMalloc
 * (it can synchronise the device and stall other work). No counterpart in
 * the artifact.
 *
 * Same result as gbs_batch_plan + gbs_batch_run with GBS_BATCH_PERSISTENT on
 * the same grids. The grid table, work list and counters live in a static
 * device array of about GBS_NOALLOC_MAX_ITEMS*32 bytes per fp mode (about
 * 1 MB each), which every GPU that loads the library holds until the process
 * exits; host staging uses static host arrays. Batches of more than
 * GBS_NOALLOC_MAX_GRIDS grids or GBS_NOALLOC_MAX_ITEMS work items are
 * rejected with GBS_ERR_INVALID. A call copies its tables in and waits for
 * the kernel on `stream`, so it cannot be part of a stream capture: on a
 * capturing stream it returns GBS_ERR_INVALID and does nothing. Every call
 * reuses the same array (its counters and
 * error word are cleared on each call), so calls that overlap on the GPU
 * race; calls from one process are serialised, and each call returns after
 * its work has finished on `stream`, reporting device-side timeouts as
 * GBS_ERR_TIMEOUT. dtype is GBS_F32. */
#define GBS_NOALLOC_MAX_GRIDS 64
#define GBS_NOALLOC_MAX_ITEMS 32768
gbs_status gbs_batch_run_noalloc(const gbs_batch_grid *grids, int ngrids, int fp_mode, void *stream);

/* ---- adjoint (gradient of the time loop) -------------------------------- */
/* No counterpart in the artifact, which only runs the forward loop. With
 * checkpoints every C steps: gbs_adjoint_forward advances dev_A (engine
 * layout, two planes) by d->timestep steps, saving u_0, u_C, u_2C, ... in the
 * caller-provided workspace (gbs_adjoint_workspace bytes, 256-byte aligned);
 * on return both planes hold u_T. gbs_adjoint_backward takes dL/du_T (one
 * plane, engine layout; its halo is ignored) and writes dL/du_0 (one plane:
 * interior and halo, since the fixed halo feeds every step) and, if
 * dev_coef_grad is not NULL, dL/dc_k (device doubles, one per term, for the
 * coefficients as the source writes them, before a divisor; stencils of at
 * most 32 terms; gradient2d: one value, for its numerator). gradient2d uses
 * its linearised update. Each chunk's
 * states are recomputed from its checkpoint, into one of two stash buffers
 * on an internal second stream while the previous chunk's adjoint steps run
 * on `stream`. Both calls are asynchronous on `stream`. */
gbs_status gbs_adjoint_workspace(const gbs_desc *d, int checkpoint_every, size_t *bytes);
gbs_status gbs_adjoint_forward(const gbs_desc *d, void *dev_A, int checkpoint_every, void *workspace,
                               void *stream);
gbs_status gbs_adjoint_backward(const gbs_desc *d, const void *dev_lamT, void *dev_grad_u0, double *dev_coef_grad,
                                int checkpoint_every, void *workspace, void *stream);

/* The same backward under a smaller memory budget: the workspace holds
 * `slots` stash planes instead of 2C. With slots >= 2C this is
 * gbs_adjoint_backward; with fewer, each chunk of C steps is reversed by the
 * binomial (revolve) checkpoint schedule over `slots` snapshot planes (plus
 * two work planes), which recomputes the fewest forward steps any schedule
 * with that many snapshots can (slots = 0: every state recomputed from the
 * chunk's checkpoint). gbs_adjoint_forward is the same for both; the
 * workspace must be sized by gbs_adjoint_workspace_slots with the same C
 * and slots. */
gbs_status gbs_adjoint_workspace_slots(const gbs_desc *d, int checkpoint_every, int slots, size_t *bytes);
gbs_status gbs_adjoint_backward_slots(const gbs_desc *d, const void *dev_lamT, void *dev_grad_u0,
                                      double *dev_coef_grad, int checkpoint_every, int slots, void *workspace,
                                      void *stream);
/* Chooses C and slots for a workspace of at most budget_bytes: the fewest
 * recomputed forward steps (ties: the smaller workspace). GBS_ERR_NOMEM if
 * nothing fits. Host arithmetic only. */
gbs_status gbs_adjoint_plan_budget(const gbs_desc *d, size_t budget_bytes, int *checkpoint_every, int *slots,
                                   size_t *bytes);
/* Forward steps the binomial schedule takes to reverse `steps` steps with
 * `slots` snapshot planes, and the most snapshots it holds at once. Host
 * arithmetic only. */
gbs_status gbs_revolve_cost(int steps, int slots, long long *forward_steps, int *peak_slots);

/* Many independent instances (any mix of stencils, sizes and dtypes, one
 * workspace each) at once: the instances' forward (or backward) calls run
 * side by side on internal branch streams, forked from `stream` and joined
 * back into it, so the calls are asynchronous on `stream` like the
 * single-instance ones. dev_coef_grad may be NULL (no coefficient gradients)
 * or hold one pointer (or NULL) per instance. */
gbs_status gbs_adjoint_forward_batch(const gbs_desc *descs, int n, void *const *dev_A, int checkpoint_every,
                                     void *const *workspaces, void *stream);
gbs_status gbs_adjoint_backward_batch(const gbs_desc *descs, int n, const void *const *dev_lamT,
                                      void *const *dev_grad_u0, double *const *dev_coef_grad, int checkpoint_every,
                                      void *const *workspaces, void *stream);

/* Measures the device's fused multiply-add throughput in GFLOP/s (2 flops per
 * FMA): the FP term of the temporally-blocked stencil roofline. */
gbs_status gbs_measure_fp_peak(int dtype, double *gflops);

/* Self-test of the engine's division by a constant divisor (used by j2d5pt,
 * j2d9pt, j2d9pt-gol and j3d27pt in GBS_FP_EXACT mode) against IEEE
 * division. checked != 0 tests the remainder-checked quotient used for any
 * divisor; checked == 0 tests the unchecked one-correction quotient that the
 * engine uses only for divisors this test proves exact (118 and 159). Float
 * checks every one of the 2^32 inputs when samples <= 0; double checks
 * `samples` random bit patterns (2^28 when samples <= 0) plus every binade
 * edge. *mismatches receives the count of inputs whose results differ. */
gbs_status gbs_check_division(int dtype, double divisor, int checked, long long samples,
                              long long *mismatches);

const char *gbs_last_error(void);
/* Frees the cached device buffers of gbs_run. */
void gbs_release_cache(void);

#ifdef __cplusplus
}
#endif
#endif /* GBSTENCIL_H */
