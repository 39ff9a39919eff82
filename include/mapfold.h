/*
 * mapfold.h -- C ABI of the GB300 map-folding counting engine.
 *
 * The reference (johnowhitaker/map_folding) exposes its two counting paths
 * only as process CLIs, plus one in-process C ABI (the WASM kernel's
 * solve_cases).  Each entry point below names the reference interface it
 * stands in for.  Conventions:
 *   - every function returns an mf_status (0 = MF_OK); mf_last_error()
 *     gives a one-line reason for the last failure on the calling thread;
 *   - pointers named d_* are device pointers on the current CUDA device;
 *     everything else is host memory;
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default);
 *   - counts are exact unsigned integers: uint64 per state / per case, and
 *     128-bit totals as two uint64 words {lo, hi}.
 *
 * No function here takes or returns any framework type.
 */
#ifndef MAPFOLD_H
#define MAPFOLD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MF_ABI_VERSION 1
#define MF_MAX_LEAVES 64   /* leaves (Lunnon) or cells (sym) per map */
#define MF_MAX_DIMS 8
#define MF_SYM_CYCLE_BYTES 64 /* one sym case: successor cell of each cell */

typedef enum {
    MF_OK = 0,
    MF_ERR_ARG = 1,       /* bad argument: the reference's rc 1 / status 1 */
    MF_ERR_RANGE = 2,     /* bad index range: the WASM kernel's status 2 */
    MF_ERR_CUDA = 3,      /* a CUDA runtime call failed */
    MF_ERR_NO_DEVICE = 4, /* no CUDA device visible */
    MF_ERR_CAPACITY = 5,  /* caller buffer or workspace too small */
    MF_ERR_TIMEOUT = 6    /* a bounded device-side wait ran out */
} mf_status;

/* One-line description of the last error on this thread ("" if none). */
const char *mf_last_error(void);
int32_t mf_abi_version(void);

/* Timings and work counters of one engine call (all optional outputs). */
typedef struct {
    double setup_s;       /* host-side tables, prefix or case generation */
    double h2d_s;         /* host->device copies */
    double kernel_s;      /* device time of the counting kernels (events) */
    double d2h_s;         /* device->host copies */
    double total_s;       /* wall time of the whole call */
    uint64_t units;       /* prefix states or cases counted */
    uint64_t nodes;       /* reference nodes visited (see each entry) */
    uint64_t tasks;       /* work items run, including device-side splits */
    uint64_t splits;      /* work items created by device-side splitting */
    uint64_t h2d_bytes;
    uint64_t d2h_bytes;
} mf_run_stats;

/* Launch shape and scheduling knobs of the persistent (batched) kernels.
 * Zero in any field selects the built-in default. */
typedef struct {
    uint32_t block_threads;  /* threads per CTA: 128 or 256 */
    uint32_t blocks_per_sm;  /* resident CTAs per SM (0: as many as fit) */
    uint32_t node_budget;    /* lockstep rounds (one node each) between split checks */
    uint32_t hungry_factor;  /* split while queued items < factor/8 x threads */
    uint64_t queue_capacity; /* split-item ring cells (rounded up to a power of 2) */
    uint32_t wait_limit;     /* idle rounds before an idle warp leaves */
    uint32_t stack_mode;     /* 0: DFS stack in shared memory when it fits, 1: local,
                                2: sym counts on the 128-bit kernel whatever the board */
} mf_batch_config;

/* ======================================================================
 * Lunnon backtracking DFS over leaves (any dimension count, <= 64 leaves)
 * ====================================================================== */

typedef struct mf_lunnon_plan mf_lunnon_plan;

/* Builds the coordinate and neighbour tables for a p1 x p2 x ... map and
 * uploads them to the current device.
 * Replaces: mf.c:29-75 (c/d tables), gpu_folding.cu:227-264 (host tables +
 * cudaMemcpyToSymbol), gpu_folding_v2.cu:131-163 (make_problem). */
int32_t mf_lunnon_plan_create(const int32_t *dims, int32_t ndim, mf_lunnon_plan **out);
void mf_lunnon_plan_destroy(mf_lunnon_plan *plan);
/* Number of leaves n = p1*p2*...  */
int32_t mf_lunnon_leaves(const mf_lunnon_plan *plan);
/* Bytes per packed prefix-state record: b[0..n] as uint8, zero padded to a
 * multiple of 16 so that each record loads as whole 16-byte vectors. */
uint32_t mf_lunnon_state_stride(const mf_lunnon_plan *plan);

/* Host prefix generation: every state at leaf depth `depth` that passes the
 * normal-form filter, in the reference's emission order.  Writes up to `cap`
 * records; *count_out gets the total (which may exceed cap).
 * Replaces: gpu_folding.cu:21-121 (collect_partial_states),
 * gpu_folding_v2.cu:220-256 (collect_states), mf_fast.cpp:223-259
 * (count_states, with states == NULL). */
int32_t mf_lunnon_collect(const mf_lunnon_plan *plan, int32_t depth, uint8_t *states,
                          uint64_t cap, uint64_t *count_out);

/* Plain GPU DFS, one thread per prefix state, resumed at leaf start_leaf
 * (= depth + 1) and stopped when the search returns to it.  d_per_state
 * (optional) receives each state's count; *d_total (optional) is ADDED to;
 * *d_nodes (optional) is added the number of leaf insertions the reference
 * loop would make (mf.c:136-142).
 * Replaces: gpu_folding.cu:123-207 (compute_counts) and its launch
 * :287-299; gpu_folding_v2.cu:381-453 (solve_kernel). */
int32_t mf_lunnon_count_states(const mf_lunnon_plan *plan, int32_t start_leaf,
                               const uint8_t *d_states, uint64_t num_states,
                               uint64_t *d_per_state, uint64_t *d_total, uint64_t *d_nodes,
                               void *stream);

/* Whole-map count: prefix generation to `depth`, host->device copy, plain
 * (mode 0) or batched work-stealing (mode 1) kernel, device->host copy.
 * *count_out is the folding count.  This is what `gpu_folding <n> <depth>`
 * computes (gpu_folding.cu:209-311).  depth < 0 picks a default. */
int32_t mf_lunnon_count(const mf_lunnon_plan *plan, int32_t depth, int32_t mode,
                        const mf_batch_config *cfg, uint64_t *count_out,
                        uint64_t *states_out, mf_run_stats *stats);

/* As mf_lunnon_count, over prefix states [first_state, first_state +
 * max_states) of the emission order only (max_states 0: to the end): the
 * partial count of those subtrees.  What `gpu_folding_v2 grid depth ...
 * max_states` computes (gpu_folding_v2.cu:258-325 stops after max_states). */
int32_t mf_lunnon_count_range(const mf_lunnon_plan *plan, int32_t depth, uint64_t first_state,
                              uint64_t max_states, int32_t mode, const mf_batch_config *cfg,
                              uint64_t *count_out, uint64_t *states_out, mf_run_stats *stats);

/* Batched uneven launch: all prefix states of `num_plans` maps (each at its
 * own depth) in ONE persistent work-stealing kernel that splits subtrees on
 * the device.  counts_out[k] receives map k's folding count; depths may be
 * NULL and a negative depth picks a default.
 * No reference counterpart in one call: the reference runs one map per
 * process (gpu_folding_v2.cu:476-542 batches states of a single map). */
int32_t mf_lunnon_batch_count(const mf_lunnon_plan *const *plans, int32_t num_plans,
                              const int32_t *depths, const mf_batch_config *cfg,
                              uint64_t *counts_out, mf_run_stats *stats);

/* ======================================================================
 * sym_fold: symmetry-reduced square counting (n <= 8; plans up to 9x9)
 * ====================================================================== */

/* The four edge pages of an n x n grid in centre-out spiral numbering:
 * out[page*64 + cell] = neighbour across that page's edge, or n*n.
 * Replaces: sym_fold.cpp:122-173 (build_map, make_edges). */
int32_t mf_sym_edges(int32_t n, uint8_t *out);

typedef struct mf_sym_plan mf_sym_plan;

/* Centre enumeration, D4 x stack-reversal dedup and the expansion index for
 * cases at `expanded_n` cells (0 = the reference default: 24 for n >= 7;
 * n = 6 always uses its 16-cell centre).  n must be 6..9.
 * Replaces: sym_fold.cpp:252-265, 316-408, 703-745. */
int32_t mf_sym_plan_create(int32_t n, int32_t expanded_n, mf_sym_plan **out);

/* Options of experiments/9x9/sym_fold9.cpp's setup (zero = default). */
typedef struct {
    int32_t expanded_n;   /* MF_EXPANDED_N (n >= 7): 0 = max(24, centre cells) */
    int32_t center_n;     /* MF_CENTER_N: 0 = 3 odd, 4 even, 5 for 9x9; else 3..5, n's parity */
    uint64_t seed_start;  /* MF_SEED_START: first centre representative kept */
    uint64_t seed_count;  /* MF_SEED_COUNT: representatives kept (0 = the rest) */
} mf_sym_plan_options;

/* mf_sym_plan_create with sym_fold9's setup options; n may be 9, and
 * expanded_n up to n*n as in sym_fold9 (sym_fold9.cpp:1094-1099).  Counting
 * past cell 63 runs on the 128-bit kernel.  Cases expanded past 64 cells are
 * records of 96 bytes (mf_sym_plan_case_bytes) and are streamed: there is no
 * case-count index (counting the cases below every prefix would be a large
 * part of the 9x9 search), a chunk is reached by walking the cases in
 * emission order from the first -- sym_fold9's stream mode -- the plan's
 * total is reported as 0, and max_cases must be given.  A seed slice keeps centre
 * representatives [seed_start, seed_start + seed_count) and numbers cases
 * within the slice, as sym_fold9 does.
 * Replaces: sym_fold9.cpp:969-981 (choose_center_size), :1037-1124 (setup;
 * its MF_CENTER_STREAM_DEDUP and stored dedup give the same representatives
 * in the same order). */
int32_t mf_sym_plan_create_ex(int32_t n, const mf_sym_plan_options *opts, mf_sym_plan **out);
void mf_sym_plan_destroy(mf_sym_plan *plan);
/* Board side, first searched cell (the expanded depth), centre cycles
 * enumerated, centre representatives (before any seed slice) and the plan's
 * number of cases.  Any output may be NULL. */
int32_t mf_sym_plan_info(const mf_sym_plan *plan, int32_t *n, int32_t *start_i,
                         uint64_t *center_cases, uint64_t *reduced_cases,
                         uint64_t *total_cases);

/* Bytes per case record of a plan: 64, or 96 for cases expanded past 64
 * cells.  No reference counterpart (the reference keeps cases in memory). */
uint32_t mf_sym_plan_case_bytes(const mf_sym_plan *plan);

/* Cases [start_case, start_case + max_cases) of the deterministic emission
 * order (max_cases == 0: to the end), each as a cycle record of
 * mf_sym_plan_case_bytes bytes (successor cell of each cell) plus its orbit
 * multiplier.  Seeks through a per-representative case-count index instead
 * of walking every earlier case.  *count_out gets the number selected.
 * Replaces: sym_fold.cpp:491-527 (recurse_stream_cases), :731-745. */
int32_t mf_sym_cases(const mf_sym_plan *plan, uint64_t start_case, uint64_t max_cases,
                     uint8_t *cycles, uint64_t *mults, uint64_t cap, uint64_t *count_out);

/* Plain GPU count, one thread per case: d_counts[k] = completions of case k
 * from cell start_i up to (excluding) stop_i, i.e. the number of distinct
 * cycles reaching stop_i cells (stop_i = n*n: complete foldings).  *d_nodes
 * (optional) is added the number of recurse_count calls (sym_fold.cpp:219).
 * Replaces: sym_fold.cpp:219-233 (recurse_count) run per case by
 * solve_cases_parallel :410-489. */
int32_t mf_sym_count_cases(int32_t n, int32_t start_i, int32_t stop_i,
                           const uint8_t *d_cycles, uint64_t num_cases,
                           uint64_t *d_counts, uint64_t *d_nodes, void *stream);

/* Header of a persistent (batched) launch, the first 64 bytes of its
 * workspace. */
typedef struct {
    uint64_t units_handed_out; /* initial units claimed (may exceed the count) */
    uint64_t split_head;       /* split items taken */
    uint64_t split_items;      /* split items created by device-side splitting */
    uint64_t completed;        /* units + split items finished */
    uint64_t work_items_run;
    uint32_t error;            /* 0, MF_RUN_MALFORMED or MF_RUN_WAIT_LIMIT */
    uint32_t pad;
    int64_t idle_lanes;
    uint64_t warps_out;        /* warps that have left the launch */
} mf_run_header;

#define MF_RUN_MALFORMED 1u  /* a unit's list was not a permutation */
#define MF_RUN_WAIT_LIMIT 2u /* the launch ended with work unaccounted for */

/* Device workspace the batched sym kernel needs for `cfg`. */
uint64_t mf_sym_workspace_bytes(const mf_batch_config *cfg);

/* Batched GPU count: one persistent work-stealing kernel over all cases,
 * splitting heavy subtrees on the device.  Same outputs as
 * mf_sym_count_cases.  d_workspace (256-byte aligned) must hold
 * mf_sym_workspace_bytes(cfg) bytes.  The launch is asynchronous on
 * `stream`; once it has completed, the workspace's first 64 bytes hold the
 * run's header (mf_run_header above).  The counts are valid only if its
 * error word is 0 and completed == num_cases + split_items.  Error word 1
 * (MF_RUN_MALFORMED): a case's cycle is not a permutation of its placed
 * cells; that case's count is UINT64_MAX and the kernel stopped early.
 * Error word 2 (MF_RUN_WAIT_LIMIT): the launch ended with work still
 * unaccounted for.  Every device-side wait is bounded: an idle warp leaves
 * after cfg->wait_limit idle rounds (normal while other warps finish the
 * work), and the last warp out raises this word if the work accounting has
 * not closed -- a split item that was never published, say.
 * Replaces: the same reference lines as mf_sym_count_cases; the reference
 * balances only across host threads (sym_fold.cpp:456-488). */
int32_t mf_sym_count_cases_batched(int32_t n, int32_t start_i, int32_t stop_i,
                                   const uint8_t *d_cycles, uint64_t num_cases,
                                   uint64_t *d_counts, uint64_t *d_nodes,
                                   void *d_workspace, uint64_t workspace_bytes,
                                   const mf_batch_config *cfg, void *stream);

/* Count cases [start_case, start_case + max_cases) of a plan (max_cases 0:
 * to the end): answer = n*n * sum(multiplier * count), the number
 * `sym_fold` prints for that chunk.  mode 0 = plain kernel, 1 = batched.
 * Replaces: sym_fold.cpp:410-489 / 529-620 and :764. */
int32_t mf_sym_plan_solve(const mf_sym_plan *plan, uint64_t max_cases, uint64_t start_case,
                          int32_t mode, const mf_batch_config *cfg, uint64_t *answer_lo_hi,
                          mf_run_stats *stats);

/* MF_COST_DEPTH / MF_SORT_CASES of the materialized mode: score every case
 * of the plan by its number of completions `cost_depth` cells further
 * (counted on the GPU; min, max and the uint128 total come back) and, when
 * order != 0, hold the cases in cost order (1: descending, 2: ascending,
 * ties by multiplier) so that start_case / max_cases of mf_sym_plan_solve and
 * mf_sym_cases index that order.  cost_depth <= 0 does nothing.
 * Replaces: score_and_sort_cases, sym_fold.cpp:267-314 (estimate_work
 * :235-250). */
int32_t mf_sym_plan_score(mf_sym_plan *plan, int32_t cost_depth, int32_t order, int32_t mode,
                          const mf_batch_config *cfg, uint64_t *min_score, uint64_t *max_score,
                          uint64_t *total_score_lo_hi, mf_run_stats *stats);

/* Cost estimate of the plan's cases [start_case, start_case + count) for
 * cost-weighted chunking: each case scores estimate_work at cost_depth cells
 * further, plus one for the case itself, and the scores are summed per
 * block of `block` consecutive cases into block_costs[ceil(count / block)].
 * Scoring runs on the GPU in bounded slices, so any range of an 8x8 plan
 * fits.  No counterpart in the reference, whose chunks are equal case
 * ranges (modal_sym.py:166-172); it uses estimate_work (sym_fold.cpp:235-250),
 * the lookahead its notes propose for balancing (docs/8x8-method.md:128). */
int32_t mf_sym_plan_block_costs(const mf_sym_plan *plan, uint64_t start_case, uint64_t count,
                                int32_t cost_depth, uint64_t block, int32_t mode,
                                const mf_batch_config *cfg, uint64_t *block_costs);

/* The reference's cost order on the host: perm[k] = index of the k-th case
 * after sorting by score (descending, or ascending when ascending != 0),
 * ties by multiplier ascending, with the same (unstable) std::sort the
 * reference uses, so equal keys land where they land there.
 * Replaces: sym_fold.cpp:297-310. */
int32_t mf_sym_sort_order(const uint64_t *scores, const uint64_t *mults, uint64_t count,
                          int32_t ascending, uint64_t *perm);

/* Allocation-free variant of mf_sym_count_cases_batched.  No counterpart in
 * the reference.  It is for callers that cannot allocate device memory at
 * all and therefore cannot pass a workspace: a process whose GPU memory is
 * owned by another allocator (a framework's caching pool that has reserved
 * the device), or a latency-critical caller that must not take the implicit
 * device synchronisation of cudaMalloc/cudaFree.  The split-item ring lives
 * in a fixed __device__ array of 4096 cells (416.25 KiB, plus 2.25 KiB of
 * edge pages) that every GPU loading this library holds until the process
 * exits.  The ring always has those 4096 cells: a cfg->queue_capacity above
 * 4096 is rejected with MF_ERR_CAPACITY, a smaller one is ignored, and
 * cfg->stack_mode 2 (the 128-bit kernel) is rejected with MF_ERR_ARG.
 * The caller still passes inputs and outputs (d_cycles, d_counts, d_nodes).
 * The first call on a device (and the first after a device reset) performs
 * its one-time set-up (looks up the array's device address and copies the
 * edge pages in), so make that first call before any stream capture.  All
 * calls share the array and it keeps the last call's contents; each call
 * clears what must start at zero, but calls that overlap on the GPU
 * (concurrent streams, other host threads) race on it and must be
 * serialised by the caller.  The run's header, with its error word, stays in
 * the array: read it with mf_sym_static_status after the launch (a malformed
 * case also reads UINT64_MAX in d_counts).  It calls no cudaMalloc, cudaFree
 * or other allocating routine. */
int32_t mf_sym_count_cases_batched_static(int32_t n, int32_t start_i, int32_t stop_i,
                                          const uint8_t *d_cycles, uint64_t num_cases,
                                          uint64_t *d_counts, uint64_t *d_nodes,
                                          const mf_batch_config *cfg, void *stream);

/* Copies the header of the last mf_sym_count_cases_batched_static run on
 * the current device (an mf_run_header, 64 bytes) into dst -- host or
 * device memory -- asynchronously on `stream`, after the work queued there
 * before it.  The run's counts are valid only if its error word is 0 and
 * completed == num_cases + split_items.  Allocates nothing.
 * No counterpart in the reference. */
int32_t mf_sym_static_status(void *stream, void *dst);

/* ---- CUDA-graph replay ------------------------------------------------ */

typedef struct mf_graph mf_graph;

/* Records one batched sym count on fixed device buffers -- node-counter
 * reset, split-ring reset, per-case count reset, persistent kernel -- into
 * a CUDA graph, so repeated counts (benchmark steps, chunk rounds) replay
 * with a single mf_graph_launch.  Arguments as mf_sym_count_cases_batched;
 * the buffers must stay valid for the graph's lifetime.
 * No reference counterpart (the reference relaunches per batch,
 * gpu_folding_v2.cu:512-533). */
int32_t mf_sym_graph_create(int32_t n, int32_t start_i, int32_t stop_i, const uint8_t *d_cycles,
                            uint64_t num_cases, uint64_t *d_counts, uint64_t *d_nodes,
                            void *d_workspace, uint64_t workspace_bytes,
                            const mf_batch_config *cfg, mf_graph **out);
int32_t mf_graph_launch(mf_graph *graph, void *stream);
void mf_graph_destroy(mf_graph *graph);

/* A prepared uneven batch: the maps' prefix states, tables and work queue
 * resident on the device and the batched launch recorded as a CUDA graph;
 * mf_lunnon_batch_run replays it and copies the per-map counts back.
 * Same semantics as mf_lunnon_batch_count. */
typedef struct mf_lunnon_batch mf_lunnon_batch;
int32_t mf_lunnon_batch_create(const mf_lunnon_plan *const *plans, int32_t num_plans,
                               const int32_t *depths, const mf_batch_config *cfg,
                               mf_lunnon_batch **out);
int32_t mf_lunnon_batch_run(mf_lunnon_batch *batch, uint64_t *counts_out, mf_run_stats *stats);
void mf_lunnon_batch_destroy(mf_lunnon_batch *batch);

/* ======================================================================
 * Request server: continuous batching on one resident kernel
 * ====================================================================== */

typedef struct mf_server mf_server;

typedef struct {
    uint64_t unit_capacity;  /* device unit arena, in units (power of 2; 0: 2^21) */
    uint32_t max_requests;   /* requests resident at once (0: 1024) */
    uint32_t block_threads;  /* 0: 128 */
    uint64_t table_bytes;    /* Lunnon neighbour-table arena (0: 64 MiB) */
    uint32_t node_budget;    /* rounds between split checks (0: 64) */
    uint32_t reserved;
    uint64_t queue_capacity; /* split-item ring cells (0: 2^16) */
} mf_server_config;

typedef struct {
    double submit_s;  /* monotonic clock at submission */
    double admit_s;   /* ... when its units were resident and published */
    double done_s;    /* ... when the server saw its result */
    uint64_t units;   /* cases or prefix states */
    uint64_t nodes;   /* reference nodes searched for it */
} mf_request_info;

/* Starts a server on the current device: a persistent kernel that keeps
 * running while requests come and go.  A request needs a free slot and
 * enough unit-arena memory.  Small requests (at most a quarter of the
 * resident lanes' worth of units) are admitted at once; large ones first
 * come first served, the next only once the running large ones leave 1/8
 * of the lanes idle.  Admitted units start on whichever lanes free up,
 * alongside the requests already running, and all subtrees share one
 * split-item ring, where the oldest running request keeps a stock for lanes
 * that free up.  No reference counterpart: the reference runs one chunk per
 * process or container (modal_sym.py:88-137). */
int32_t mf_server_create(const mf_server_config *cfg, mf_server **out);
/* Submit sym_fold cases [start_case, start_case + max_cases) of an n x n
 * map at MF_EXPANDED_N = expanded_n; the result is what `sym_fold` prints
 * for that chunk.  Returns at once with a request id. */
int32_t mf_server_submit_sym(mf_server *srv, int32_t n, int32_t expanded_n, uint64_t start_case,
                             uint64_t max_cases, uint64_t *request_id);
/* Submit a whole-map Lunnon count (depth < 0: default split depth). */
int32_t mf_server_submit_lunnon(mf_server *srv, const int32_t *dims, int32_t ndim, int32_t depth,
                                uint64_t *request_id);
/* *done = 1 and the answer (lo, hi) once the request has finished. */
int32_t mf_server_poll(mf_server *srv, uint64_t request_id, int32_t *done, uint64_t *answer_lo_hi,
                       mf_request_info *info);
/* Blocks until the request finishes or timeout_s passes (MF_ERR_TIMEOUT). */
int32_t mf_server_wait(mf_server *srv, uint64_t request_id, double timeout_s,
                       uint64_t *answer_lo_hi, mf_request_info *info);
/* Finishes outstanding requests, stops the kernel, frees everything. */
void mf_server_destroy(mf_server *srv);

/* The whole `sym_fold n threads max_cases start_case` computation with the
 * MF_EXPANDED_N semantics: answer = n*n * sum(multiplier * count) over the
 * selected cases (n <= 5: 2*n*n*count).  mode 0 = plain kernel, 1 =
 * batched.  Replaces: sym_fold.cpp:649-774 (main). */
int32_t mf_sym_solve(int32_t n, uint64_t max_cases, uint64_t start_case, int32_t expanded_n,
                     int32_t mode, const mf_batch_config *cfg, uint64_t *answer_lo_hi,
                     mf_run_stats *stats);

/* In-process case solver with the WASM kernel's contract: case_buffer holds
 * case_count records of 112 bytes (cycle bytes [0, n*n), uint64 LE
 * multiplier at offset 100); output_words[8] receives the 128-bit sum of
 * multiplier*count (LE words 0-3), the uint64 node count (words 4-5,
 * recurse_count calls including the stop level) and the status (word 6).
 * Status 1: n outside 2..8 or case_count > 256; status 2: start_i > stop_i
 * or stop_i > n*n.  Counting is on the GPU.
 * Replaces: mfah/wasm/sym_kernel.c:251-276 (solve_cases). */
uint32_t mf_solve_cases(uint32_t n, uint32_t start_i, uint32_t stop_i,
                        const uint8_t *case_buffer, uint32_t case_count,
                        uint32_t *output_words);

/* ======================================================================
 * Test support
 * ====================================================================== */

/* Host-side fault injection for tests of the bounded device waits.  With
 * MF_FAULT_LOST_SPLIT the next persistent launch (batched sym or Lunnon,
 * 64-bit) starts with one split-ring ticket reserved that no lane will ever
 * publish -- a donor's message lost on the way -- so the split items behind
 * it are never taken, the work accounting cannot close, the idle warps
 * leave after cfg->wait_limit rounds and the last one out raises error word
 * MF_RUN_WAIT_LIMIT (the host-buffer entry points then return
 * MF_ERR_TIMEOUT).  Nothing on the device faults or hangs.  One-shot; 0
 * clears it.  No counterpart in the reference. */
#define MF_FAULT_LOST_SPLIT 1u
void mf_test_inject_fault(uint32_t kind);

#ifdef __cplusplus
}
#endif

#endif /* MAPFOLD_H */
