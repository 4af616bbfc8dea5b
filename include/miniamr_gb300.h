/*
 * miniamr_gb300.h -- C ABI of the GB300 (sm_103a) back end for miniAMR's
 * per-timestep hot path: face ghost exchange, the 7/27-point averaging
 * stencil, block split/consolidate data movement and the per-variable
 * checksum.
 *
 * The reference keeps these as four C translation units that walk a
 * host-side `double ****array` per block.  A drop-in replacement of those
 * units (miniamr_gb300/dropin/) keeps every symbol the reference's driver,
 * init and refine code call, and forwards the cell-data work here.  The
 * host keeps all octree metadata; this library keeps the cell data resident
 * in device memory as one strided pool indexed by block slot.
 *
 * Conventions
 *   - Plain C types only; every call returns MAMR_OK (0) or a negative
 *     MAMR_E* status and never exits the process.  mamr_last_error() gives
 *     a one-line description of the most recent failure on this thread.
 *   - One context = one pool on the current CUDA device, one CUDA stream.
 *     A context is not re-entrant; one host thread drives it, as the
 *     reference's single-threaded driver does.
 *   - Cell layout in host buffers (upload/download): per block, per
 *     variable, a dense (nx+2)*(ny+2)*(nz+2) array of doubles indexed
 *     [i][j][k] with k fastest and one ghost layer on each side -- the
 *     same indexing as the reference's blocks[n].array[var][i][j][k]
 *     (ref/block.h:52, allocated ref/main.c:429-450).
 *
 * The same ABI is implemented on the CPU by the oracle
 * (oracle/amr_oracle.c), which the tests use as the checker.
 */
#ifndef MINIAMR_GB300_H
#define MINIAMR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MAMR_ABI_VERSION 1

/* Storage / arithmetic precision of the cell pool. */
enum {
   MAMR_FP64 = 0,   /* bit-exact with the reference */
   MAMR_FP32 = 1    /* FP32 cells; FP64-or-better checksum and coarsening */
};

/* Status codes. */
enum {
   MAMR_OK      =  0,
   MAMR_EINVAL  = -1,  /* bad argument (size, index, null pointer) */
   MAMR_ENOMEM  = -2,  /* device or host allocation failed */
   MAMR_ECUDA   = -3,  /* CUDA runtime error */
   MAMR_EMESH   = -4,  /* misconnected mesh (ref/comm.c:198-201) */
   MAMR_EUNSUP  = -5,  /* configuration this back end does not run */
   MAMR_EDEVICE = -6   /* a device-side check set the context error word */
};

typedef struct mamr_ctx mamr_ctx;

/* Problem shape.  Field meanings follow the reference's globals
 * (ref/block.h:79-146, defaults ref/param.h). */
typedef struct {
   int32_t nx, ny, nz;   /* x/y/z_block_size: cells per block, even */
   int32_t num_vars;     /* num_vars */
   int32_t max_blocks;   /* max_num_blocks: pool capacity in block slots */
   int32_t stencil;      /* 7, 27, or 0 (variable work; FP64, plain path) */
   int32_t code;         /* ghost-exchange variant 0, 1 or 2 (1 and 2, which
                            differ only in how ranks pack messages, are one
                            exchange on one rank; plain path) */
   int32_t permute;      /* --permute: direction order cycles with stage */
   int32_t dtype;        /* MAMR_FP64 or MAMR_FP32 */
   int32_t reserved[7];  /* must be zero */
} mamr_config;

/* One active block as the hot path sees it: a projection of the
 * reference's `block` struct (ref/block.h:36-53).  An array of these in
 * sorted_list order (level ascending, block number descending within a
 * level; ref/block.c:610-625) describes the mesh. */
typedef struct {
   int32_t slot;          /* index into blocks[] == pool slot */
   int32_t level;         /* refinement level */
   int32_t nei_level[6];  /* W,E,S,N,D,U neighbour level; -2 = boundary */
   int32_t nei[6][2][2];  /* neighbour slots; [l][0][0] for a same-level or
                             coarser neighbour, all four for finer ones */
} mamr_block;

/* split_blocks(): parent slot -> 8 child slots, child[o] for octant
 * o = i1 + 2*j1 + 4*k1 (ref/block.c:128-173). */
typedef struct {
   int32_t parent;
   int32_t child[8];
} mamr_split_job;

/* consolidate_blocks(): 8 child slots (by octant) -> the slot of the
 * re-formed block (ref/block.c:370-431). */
typedef struct {
   int32_t child[8];
   int32_t target;
} mamr_consolidate_job;

/* ---- refinement marking types (ref/move.c, ref/refine.c) -------------- */

/* One refinement object after move() (ref/block.h object; ref/move.c:37-63
 * moves it on the host).  type: 0 surface / 1 solid box; 2..15 spheroid,
 * even = surface, odd = solid, 4..15 the half on one side of the centre
 * plane (4/5 x < centre dropped ... 14/15 z > centre dropped, as
 * ref/move.c:369-382 and 489-502); 20/22/24 cylinder surface along x/y/z,
 * 21/23/25 solid.  Any negative size disables the object. */
typedef struct {
   int32_t type;
   int32_t reserved;     /* must be zero */
   double cen[3];
   double size[3];
} mamr_object;

/* The globals the marking reads (ref/block.h:83-137). */
typedef struct {
   int32_t num_refine;      /* maximum level */
   int32_t refine_ghost;    /* --refine_ghost: test the extent with ghosts */
   int32_t uniform_refine;  /* --uniform_refine: every block below the
                               maximum level refines; no objects */
   int32_t mesh_size[3];    /* mesh_size[] (ref/init.c:430-437) */
   int32_t max_passes;      /* cap on the rule passes; 0 = the bound that
                               always suffices, 2 * (blocks + parents).  A
                               smaller cap the rules need more passes than
                               ends the call with MAMR_EDEVICE (no
                               counterpart in the reference: a test knob
                               for the bounded device loop) */
   int32_t reserved[9];     /* must be zero */
} mamr_mark_params;

/* One active block as the marking sees it (ref/block.h:36-53). */
typedef struct {
   int32_t slot;            /* index into blocks[] */
   int32_t level;
   int32_t parent;          /* index into parents[], -1 for an initial block */
   int32_t cen[3];          /* integer centre */
   int32_t nei_level[6];    /* W,E,S,N,D,U; -2 = boundary */
   int32_t nei[6];          /* nei[l][0][0]: blocks[] index of a same-level
                               or coarser neighbour (ignored otherwise) */
} mamr_mark_block;

/* One entry of parents[] (ref/block.h:55-70). */
typedef struct {
   int32_t active;          /* parents[p].number >= 0 */
   int32_t child[8];        /* blocks[] index, or -1 - (parents[] index)
                               for a child that is itself a parent */
} mamr_mark_parent;

/* Flags for mamr_run_timesteps(). */
enum {
   MAMR_RUN_PLAIN   = 0,  /* per-call path: comm, then stencil/check_sum per
                             variable, exactly the driver's call sequence */
   MAMR_RUN_BATCHED = 1,  /* one fused ghost+stencil(+checksum) launch per
                             stage over every block and variable */
   MAMR_RUN_GRAPH   = 2,  /* with BATCHED: replay the stages as a CUDA graph */
   MAMR_RUN_PER_BLOCK = 4, /* with PLAIN: one stencil launch per (block,
                             variable) -- the naive port, kept as a
                             baseline to measure the batched path against */
   MAMR_RUN_NO_GHOSTS = 8 /* with BATCHED and the 7-point stencil: the
                             run's last stage leaves the pool's ghost cells
                             as they were instead of writing back the ghost
                             layer it gathered -- for a caller whose next
                             work (further batched stages, splits and
                             consolidations) reads no ghost cell before a
                             run without it writes them */
};

/* ---- lifetime --------------------------------------------------------- */

/* Allocates the zero-filled cell pool for cfg->max_blocks slots on the
 * current CUDA device (replaces the per-block mallocs of
 * ref/main.c:429-450; zero fill matches the fresh-heap contents the
 * reference starts from).  The pool is never cleared afterwards. */
int mamr_create(const mamr_config *cfg, mamr_ctx **out);
int mamr_destroy(mamr_ctx *ctx);
const char *mamr_last_error(void);
/* The context's CUDA stream (a cudaStream_t) for callers that time it. */
int mamr_stream(mamr_ctx *ctx, void **stream);
/* Waits for all work queued on the context and reports device-side
 * error words. */
int mamr_sync(mamr_ctx *ctx);

/* ---- cell data in and out -------------------------------------------- */

/* Copies n blocks from a host buffer laid out [n][num_vars][nx+2][ny+2]
 * [nz+2] (doubles) into pool slots slots[0..n).  FP32 pools round to
 * nearest.  Used once after the reference's init() has filled its host
 * arrays (ref/init.c:484-495).  A pinned buffer (cudaMallocHost,
 * cudaHostAlloc) is read in place by one kernel over the host link; other
 * buffers move through a device staging area.  Both directions return
 * once the copy is complete. */
int mamr_upload_blocks(mamr_ctx *ctx, const int32_t *slots, int32_t n,
                       const double *host);
/* The reverse copy, for verification and dumps. */
int mamr_download_blocks(mamr_ctx *ctx, const int32_t *slots, int32_t n,
                         double *host);

/* ---- mesh ---------------------------------------------------------------- */

/* Replaces the active mesh: n blocks in sorted_list order.  Checks the
 * connectivity the exchange relies on and returns MAMR_EMESH where the
 * reference would print "misconnected block" (ref/comm.c:198-201).  Returns
 * once the mesh's device copies are queued on the context's stream (blocks
 * may be reused at once); a device-side failure surfaces at the next call
 * that synchronises. */
int mamr_set_mesh(mamr_ctx *ctx, const mamr_block *blocks, int32_t n);

/* ---- the hot path (reference entry point each one replaces) ----------- */

/* comm(start, num_comm, stage): ref/comm.c:42-242 on one rank --
 * on_proc_comm (ref/comm.c:1465-1580), on_proc_comm_diff
 * (ref/comm.c:1585-1908; code 1/2: whole ghost planes, level-jump edges
 * included) and apply_bc (ref/comm.c:1911-1965) for
 * variables [start, start+num_comm), directions x, y, z in order (or
 * permuted by stage when cfg.permute). */
int mamr_comm(mamr_ctx *ctx, int32_t start, int32_t num_comm, int32_t stage);

/* stencil_driver(var, calc_stage): ref/stencil.c:43-74.  Stencil 7 or 27:
 * stencil_calc(var, stencil) (ref/stencil.c:76-145).  Stencil 0: variable
 * 0 and variables >= 4*mat take stencil_calc(var, 7); the others the
 * variable-work kernel of calc_stage % 6 (stencil_0, _x, _y, _z, _7, _27;
 * ref/stencil.c:147-957) followed by stencil_check (ref/stencil.c:959-983),
 * with the coefficients mamr_set_work_params gave. */
int mamr_stencil(mamr_ctx *ctx, int32_t var, int32_t calc_stage);

/* The coefficients of the variable-work stencils: the reference's globals
 * a1 and a0[0 .. num_vars/4) (ref/init.c:418-423).  Required before the
 * first mamr_stencil of a stencil-0 context; n_a0 must be num_vars/4. */
int mamr_set_work_params(mamr_ctx *ctx, double a1, const double *a0,
                         int32_t n_a0);

/* check_sum(var): ref/check_sum.c:36-65.  FP64 pools sum each block's
 * interior serially (k fastest) and the block sums in sorted_list order,
 * the reference's exact order.  FP32 pools: when every cell v of the
 * variable lies in the window v == 0 or 2^-52 <= |v| < 2^10, each cell
 * contributes trunc(v * 2^52) exactly to a 128-bit fixed-point sum that is
 * converted to double once (order-independent; error at most 2^-52 per
 * cell); otherwise (a cell of 2^10 or more, infinite or NaN, or non-zero
 * below 2^-52) the variable takes the reference's order in FP64 with
 * Neumaier compensation -- each block serially into s + c, then the block
 * values serially in sorted_list order.  Every path is deterministic and
 * the same in mamr_run_timesteps' checksums. */
int mamr_check_sum(mamr_ctx *ctx, int32_t var, double *sum);

/* split_blocks() cell data: ref/block.c:158-173.  Jobs run in the given
 * (reference) order semantics: a child may reuse a slot freed by an
 * earlier parent in the same call.  Like mamr_consolidate, it returns once
 * the work is queued on the context's stream (jobs may be reused at once);
 * the calls that read cells or checksums back synchronise, and a
 * device-side failure surfaces there. */
int mamr_split(mamr_ctx *ctx, const mamr_split_job *jobs, int32_t n);

/* consolidate_blocks() cell data: ref/block.c:411-431, same ordering
 * semantics (a later target may be an earlier job's freed child, and a
 * later job may read an earlier job's target).  Queued as mamr_split. */
int mamr_consolidate(mamr_ctx *ctx, const mamr_consolidate_job *jobs,
                     int32_t n);

/* The stage loop of ref/driver.c:73-108 for num_ts timesteps of
 * stages_per_ts stages, comm over all variables at once (comm_vars = 0).
 * comm_stage/calc_stage of the first stage is first_stage.  When
 * checksum_freq > 0, stages with (stage % checksum_freq == 0) produce
 * num_vars checksums, appended to sums (host memory, may be NULL) in
 * stage order; *n_sums receives how many stages produced them.  The
 * tolerance check of ref/driver.c:96-101 is left to the caller. */
int mamr_run_timesteps(mamr_ctx *ctx, int32_t num_ts, int32_t stages_per_ts,
                       int32_t checksum_freq, int32_t first_stage,
                       int32_t flags, double *sums, int32_t *n_sums);

/* Number of kernels this context has launched since creation (for the
 * launch counts the benchmark reports). */
int mamr_launch_count(mamr_ctx *ctx, int64_t *count);

/* ---- refinement marking ------------------------------------------------ */

/* The refine decisions of one refinement step on one rank: what
 * reset_all() (ref/refine.c:500-527), check_objects() (ref/move.c:65-141,
 * with check_block :143-623) -- or the uniform_refine assignment
 * (ref/refine.c:68-74) -- and refine_level() (ref/refine.c:325-496) leave
 * in blocks[].refine and parents[].refine (1 refine, 0 stay, -1 coarsen),
 * computed on the device.  On one rank comm_refine(), comm_parent() and
 * comm_parent_reverse() exchange nothing, and every rule of those routines
 * only raises a flag (-1 < 0 < 1), so the result is the least fixed point
 * of the rules above the initial state whatever order they are applied
 * in; the device applies them to all blocks at once until nothing
 * changes.  blocks[] lists the active blocks (any order); block_refine[i]
 * receives blocks[i]'s flag and parent_refine[p] parents[p]'s for the
 * active entries.  The cell block size is the context's.  Returns
 * MAMR_EINVAL for indices out of range.  May be called from any host
 * thread (it makes the context's device current on that thread). */
int mamr_mark_refine(mamr_ctx *ctx, const mamr_mark_params *params,
                     const mamr_object *objects, int32_t n_objects,
                     const mamr_mark_block *blocks, int32_t n_blocks,
                     const mamr_mark_parent *parents, int32_t n_parents,
                     int32_t *block_refine, int32_t *parent_refine);

/* ---- a whole run: the driver, refinement and stage loop --------------- */

/* The run parameters of the reference's command line that the AMR driver
 * needs (ref/main.c:56-140, defaults ref/param.h); the block size,
 * variable count, pool capacity, stencil, code, permute and precision come
 * from the context's mamr_config. */
typedef struct {
   int32_t init_x, init_y, init_z;  /* --init_x/y/z: initial blocks (one rank) */
   int32_t num_refine;              /* --num_refine: maximum level */
   int32_t block_change;            /* --block_change (0: num_refine) */
   int32_t refine_freq;             /* --refine_freq: timesteps between refines */
   int32_t uniform_refine;          /* --uniform_refine */
   int32_t refine_ghost;            /* --refine_ghost */
   int32_t num_tsteps;              /* --num_tsteps */
   int32_t stages_per_ts;           /* --stages_per_ts */
   int32_t checksum_freq;           /* --checksum_freq */
   int32_t run_flags;               /* MAMR_RUN_* of the stage stretches
                                       (NO_GHOSTS is the driver's own: it
                                       sets it on the batched 7-point
                                       stretches before the last) */
   int32_t reserved[8];             /* must be zero */
} mamr_amr_params;

/* One --object of the command line (ref/main.c:118-137): type as in
 * mamr_object, bounce (1: reflect off the unit cube's faces), centre,
 * velocity per timestep, half-size, size change per timestep. */
typedef struct {
   int32_t type, bounce;
   double cen[3], move[3], size[3], inc[3];
} mamr_amr_object;

/* What the driver reports as it goes (for checking it against recorded
 * runs): kind 1 -- a split job list (data: mamr_split_job[n]); kind 2 -- a
 * consolidation job list (mamr_consolidate_job[n]); kind 3 -- the mesh a
 * refinement left (mamr_block[n] in sorted_list order, with numbers[n]
 * the blocks' numbers and cen[3n] their integer centres).  ts is the
 * timestep of the refinement (0: the initial one). */
typedef void (*mamr_amr_event)(void *user, int32_t kind, int32_t ts,
                               const void *data, int32_t n,
                               const int64_t *numbers, const int32_t *cen);

typedef struct {
   /* The refinement bookkeeping and marking depend on no cell value, so
    * they run on a second host thread (with a marking context of their
    * own) ahead of the stages; the stage side applies each refinement's
    * job lists and mesh in order.  All times leave out the caller's event
    * callback. */
   double stage_seconds;    /* wall time of the stage stretches (each
                               completed; each refinement's device work
                               is done before the next stretch starts) */
   double refine_seconds;   /* stage side's refinements: waiting for the
                               planning thread, data movement, mesh */
   double total_seconds;    /* the whole call */
   double mark_seconds;     /* planning thread: mamr_mark_refine calls */
   double bookkeeping_seconds; /* planning thread: marking lists, split
                               and consolidation records, meshes */
   double data_seconds;     /* mamr_split / mamr_consolidate calls (their
                               device work is queued) and the wait for
                               the refinement's device work (cell
                               movement, mesh upload) after its mesh */
   double mesh_seconds;     /* mamr_set_mesh calls (queued uploads) */
   double wait_seconds;     /* stage side waiting for the planning thread */
   int64_t updates;         /* cell-variable updates of the stages (the
                               reference's total_blocks x cells x vars) */
   int32_t refinements;     /* refine() calls, the initial one included */
   int32_t marking_steps;   /* refinement steps (block_change per call) */
   int32_t max_active;      /* most active blocks at any time */
   int32_t final_active;    /* active blocks at the end */
   int32_t stretches;       /* mamr_run_timesteps calls */
   int32_t plain_stretches; /* of those, on the plain path because the
                               batched path refused the configuration */
   int32_t reserved[2];
} mamr_amr_stats;

/* A whole miniAMR run on one rank (ref/driver.c:36-140): the initial
 * lattice of init() (ref/init.c:453-560) with its values (the reference's
 * rand() stream, seed 1) and checksums; the initial refinement; then each
 * timestep's stages, move() of the objects and, every refine_freq
 * timesteps, refine() (ref/refine.c:38-210) -- the marking on the device
 * (mamr_mark_refine), the split and consolidation bookkeeping of
 * ref/block.c:41-608 in this library (slots, parent records, numbers,
 * centres and neighbour tables exactly as the reference keeps them), the
 * cell data movement on the device.  Each stretch of timesteps between two
 * refinements is one mamr_run_timesteps call with params->run_flags; where
 * those ask for the batched path and it refuses the configuration
 * (MAMR_EUNSUP before any stage runs: stencil 0, code 1/2, a permuted
 * 27-point stencil, blocks no launch shape fits) the stretch and the rest
 * of the run take the plain path (stats->plain_stretches).
 * cfg must be the context's configuration.  sums receives the initial
 * checksums (num_vars) and then each checksum stage's num_vars sums, as
 * the reference's check_sum calls produce them, up to max_sums values;
 * *n_sums the count.  event (may be NULL) is called with user for each
 * split and consolidation list and each mesh, in the reference's order, on
 * the calling thread.  The refinement bookkeeping and marking run ahead of
 * the stages on a second host thread, through a marking context of their
 * own (the same block shape, one variable, max_blocks slots: one more
 * single-variable pool for the call's duration).  The tolerance check of
 * ref/driver.c:96-101 is left to the caller.  Needs lb_method 0 (the
 * reference's default) and one rank. */
int mamr_amr_run(mamr_ctx *ctx, const mamr_config *cfg,
                 const mamr_amr_params *params,
                 const mamr_amr_object *objects, int32_t n_objects,
                 double *sums, int64_t max_sums, int64_t *n_sums,
                 mamr_amr_event event, void *user, mamr_amr_stats *stats);

/* ---- launch-shape autotuner of the batched path ------------------------ */

/* No counterpart in the reference (the batched path is this library's own).
 * The stage kernel of a batched run has several launch shapes: for meshes
 * of 16^3 blocks on one level, (j-rows, i-planes) per thread = (2, 4),
 * (1, 4) or (1, 8) and a persistent or a one-CTA-per-work-item grid;
 * for 8^3 blocks and the 7-point stencil, first one or two warps per
 * (block, variable) with 4 or 2 items per CTA; otherwise threads per variable and
 * variables per CTA (1, 2, 4).  choice < 0 (the default): the first batched
 * run for each (block shape, stencil, precision, kernel, work size,
 * checksum frequency) times every candidate for a few stages into the
 * spare pool, taking checksums as the run does, and keeps the fastest for
 * the process (environment MAMR_TUNE=off keeps candidate 0).
 * choice >= 0 forces that candidate (clamped to the last) on this context.
 * Every candidate gives bit-identical results. */
int mamr_set_tuning(mamr_ctx *ctx, int32_t choice);

/* The candidate the last batched run used (-1 before one), how many there
 * were, and its shape: shape[0..4] = threads per variable (generic
 * kernel) or per tile (pencil kernel), variables per CTA, j-rows and
 * i-planes per thread (pencil kernel), CTAs.  The warp-per-block kernel
 * reports (threads per item -- a block and one or two of its variables:
 * 32 or 64, variables per CTA (items per CTA x variables per item), rows
 * of 8 cells per thread: 2 or 1, 0, CTAs): i-planes 0 marks it, -1 its
 * form whose tiles arrive by tensor copies. */
int mamr_get_tuning(const mamr_ctx *ctx, int32_t *choice,
                    int32_t *n_candidates, int32_t *shape);

/* ---- host-side helpers (no device work) -------------------------------- */

/* The coefficients init() draws for stencil 0 before any cell value
 * (ref/init.c:418-423): a1, then a0[0 .. num_vars/4), each rand()/RAND_MAX
 * from the unseeded (seed 1) stream. */
int mamr_work_coefficients(int32_t num_vars, double *a1, double *a0);

/* The cell values the reference's init() gives its first n_blocks blocks
 * on one rank (ref/init.c:484-495): per block in lattice order, per
 * variable, every cell (ghosts included) zero, then the interior filled
 * with rand()/RAND_MAX in i, j, k order (k fastest), from the C library's
 * unseeded rand() stream (seed 1) -- after the 1 + num_vars/4
 * coefficient draws when cfg->stencil is 0.  A private random_r state is
 * used, so the caller's rand() state is untouched.  out: [n_blocks]
 * [num_vars][nx+2][ny+2][nz+2] doubles.  Uses cfg's nx, ny, nz, num_vars
 * and stencil. */
int mamr_initial_values(const mamr_config *cfg, int32_t n_blocks,
                        double *out);

/* ---- diagnostics --------------------------------------------------------- */

/* Device self-test of the division routines (no counterpart in the
 * reference): mismatches[0..1] count where the FP32 kernels' x/7 and x/27
 * differ from IEEE FP32 division, over every float in [1, 2) plus 2^23
 * hashed floats of all classes; mismatches[2..3] the same for the FP64
 * kernels over n_fp64 hashed doubles.  Runs on the current device. */
int mamr_selftest_division(int64_t n_fp64, int64_t *mismatches);

/* FP64 pipe throughput of the current device (no counterpart in the
 * reference): FP64 add and FMA instructions per second over the whole GPU,
 * each from one timed launch of 8 independent dependent chains per thread
 * (a few milliseconds).  The bit-exact FP64 paths are bound by this rate,
 * not by HBM. */
int mamr_probe_fp64_rate(double *add_per_s, double *fma_per_s);

/* ---- allocation-free checksum ------------------------------------------ */

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory -- e.g. code whose device memory is all reserved up front by
 * another allocator (a framework's caching allocator, a serving process
 * with a fixed arena), or a latency-critical path that must not risk the
 * device-wide synchronisation an allocation can bring.  It computes the same
 * FP64 checksum as mamr_check_sum() (the reference's summation order, bit
 * for bit) over blocks the caller already holds on the device, and
 * allocates nothing: its only scratch, one partial sum per block, is a
 * file-scope device array of MAMR_STATIC_MAX_BLOCKS doubles (512 KiB) that
 * every GPU loading this library keeps until the process exits.
 *
 *   blocks   device pointer: FP64 cells in the dense layout of the host
 *            buffers above, [slot][num_vars][nx+2][ny+2][nz+2]
 *   cfg      nx, ny, nz and num_vars of that layout (other fields unused)
 *   slots    device pointer: n_blocks slots in sorted_list order; every
 *            slot must index a block inside the caller's blocks buffer
 *            (0 <= slot < the blocks it holds).  The slots live on the
 *            device, so they are not checked: a slot beyond the buffer is
 *            an out-of-bounds read.
 *   sum      device pointer that receives the checksum of variable var
 *   stream   cudaStream_t the two kernels are queued on (NULL: default)
 *
 * n_blocks above MAMR_STATIC_MAX_BLOCKS is rejected with MAMR_EINVAL, and
 * device ordinals from 64 up with MAMR_EUNSUP.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture.  All calls on a device share the one array:
 * calls that overlap on the GPU (other streams, other host threads) race
 * and give wrong sums, so keep them ordered.  Every partial is written
 * before it is read, so no clearing is needed between calls. */
#define MAMR_STATIC_MAX_BLOCKS 65536
int mamr_check_sum_fp64_noalloc(const double *blocks, const mamr_config *cfg,
                                const int32_t *slots, int32_t n_blocks,
                                int32_t var, double *sum, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MINIAMR_GB300_H */
