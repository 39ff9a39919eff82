/*
 * oracle.h -- CPU restatement of the reference's two counting paths.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (map_folding_gb300/,
 * include/) links, loads or calls this library.  Only tests/, the smoke check
 * in __graft_entry__.py and the CPU-baseline leg of bench.py use it, and only
 * as the checker or as the timed stand-in for the reference's CPU solver.
 *
 * It restates, in plain C, the algorithms of
 *   - mf.c             (Lunnon's backtracking DFS over leaves, any dimension
 *                       count, with the res/mod split)            mf.c:14-163
 *   - gpu_folding.cu / gpu_folding_v2.cu / mf_fast.cpp (prefix-state
 *                       collection and resume-from-state)
 *                                       gpu_folding.cu:21-121,
 *                                       mf_fast.cpp:142-221
 *   - sym_fold.cpp     (spiral numbering, edge pages, get_good, recurse_count,
 *                       centre enumeration, D4 x reversal dedup, case
 *                       expansion, the threaded case solver)
 *                                       sym_fold.cpp:122-620
 * and instruments them with the algorithmic work counters the GPU throughput
 * figures are quoted in:
 *   Lunnon node  = one leaf insertion                         mf.c:136-142
 *   Lunnon step  = one iteration of the per-dimension walk    mf.c:99-107
 *                  or of the all-positions fill               mf.c:113-115
 *   sym node     = one recurse_count call                     sym_fold.cpp:219
 *   sym step     = one iteration of the cycle walk            sym_fold.cpp:189-196
 *
 * Parity is pinned against the reference's own binaries built from source by
 * oracle/Makefile (see tests/golden/make_golden.py) and against the counts the
 * reference publishes (mfah/folding.py:8-17, EXPERIMENTS.md).
 */
#ifndef MAPFOLD_ORACLE_H
#define MAPFOLD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_LEAVES 64
#define ORC_MAX_DIMS 8

typedef struct {
    uint64_t nodes;
    uint64_t steps;
} orc_work;

/* ---- Lunnon ----------------------------------------------------------- */

/* Whole-map count, mf.c:14-163 (flag = 1, normal-form filter on).
 * mod == 0 disables the res/mod split.  Returns -1 on bad input. */
int64_t orc_lunnon_count(const int32_t *dims, int32_t ndim, int32_t res,
                         int32_t mod, orc_work *work);

/* Prefix states at `depth` in the reference's emission order
 * (gpu_folding.cu:21-121).  Writes up to `cap` states: a/b arrays of
 * stride n+1 (uint8) and gapter (uint16, stride n+1).  Returns the total
 * number of states (which may exceed cap), or -1 on bad input. */
int64_t orc_lunnon_collect(const int32_t *dims, int32_t ndim, int32_t depth,
                           uint8_t *a_out, uint8_t *b_out, uint16_t *gapter_out,
                           int64_t cap);

/* Count of one prefix subtree, resumed at start_leaf and stopping when the
 * search backtracks to it (mf_fast.cpp:142-183).  The gap-stack base of the
 * resumed level is taken as 0, which does not change the count. */
uint64_t orc_lunnon_resume(const int32_t *dims, int32_t ndim, int32_t start_leaf,
                           const uint8_t *a, const uint8_t *b, orc_work *work);

/* Threaded sum over many prefix states (mf_fast.cpp:386-413). */
uint64_t orc_lunnon_resume_many(const int32_t *dims, int32_t ndim, int32_t start_leaf,
                                const uint8_t *a, const uint8_t *b, int64_t count,
                                int32_t threads, uint64_t *per_state, orc_work *work);

/* ---- sym_fold --------------------------------------------------------- */

/* Four edge pages for an n x n grid in centre-out spiral numbering
 * (sym_fold.cpp:122-173).  out[page*64 + cell]; "no neighbour" = n*n. */
void orc_sym_edges(int32_t n, uint8_t *out);

/* sym_fold.cpp:179-204. */
uint64_t orc_sym_good(const uint8_t *cycle, int32_t i, const uint8_t *edges,
                      orc_work *work);

/* sym_fold.cpp:219-233: count completions of `cycle` from cell i to n2-1.
 * cycle is modified in place and restored. */
uint64_t orc_sym_count(uint8_t *cycle, int32_t i, int32_t n2, const uint8_t *edges,
                       orc_work *work);

/* mfah/wasm/sym_kernel.c:212-230: cycles reaching `stop` cells from cell i;
 * work->nodes counts every call including those at the stop level. */
uint64_t orc_sym_count_to(uint8_t *cycle, int32_t i, int32_t stop, const uint8_t *edges,
                          orc_work *work);

/* Centre representatives after D4 x reversal dedup (sym_fold.cpp:252-265,
 * 316-408).  Writes up to cap cycles (64 bytes each) and multipliers.
 * Returns the number of representatives; *center_cases gets the number of
 * centre cycles before dedup. */
int64_t orc_sym_reps(int32_t n, uint8_t *cycles, uint64_t *mults, int64_t cap,
                     int64_t *center_cases);

/* Expand the representatives to `expanded_n` cells in the reference's
 * emission order (sym_fold.cpp:731-745 / 491-527), selecting cases
 * [start_case, start_case+max_cases) (max_cases == 0: all).  Writes up to
 * cap selected cases.  Returns the number of cases selected (or, with
 * count_only, the number that would be). */
int64_t orc_sym_expand(int32_t n, int32_t expanded_n, uint64_t start_case,
                       uint64_t max_cases, uint8_t *cycles, uint64_t *mults,
                       int64_t cap);

/* Threaded count of many cases from cell start_i (sym_fold.cpp:410-489).
 * per_case (optional) receives each raw count.  Returns sum(mult*count) as
 * two 64-bit words (lo, hi). */
void orc_sym_count_cases(int32_t n, int32_t start_i, const uint8_t *cycles,
                         const uint64_t *mults, int64_t count, int32_t threads,
                         uint64_t *per_case, uint64_t *sum_lo_hi, orc_work *work);

/* sym_fold.cpp:235-250 (estimate_work) as score_and_sort_cases applies it
 * (:274-283): scores[k] = number of cycles of case k reaching
 * min(n*n, start_i + depth) cells.  Threaded. */
void orc_sym_estimate_cases(int32_t n, int32_t start_i, int32_t depth, const uint8_t *cycles,
                            int64_t count, int32_t threads, uint64_t *scores);

/* The whole sym_fold main (sym_fold.cpp:649-774) minus printing: returns the
 * 128-bit answer in out_lo_hi.  expanded_n <= 0 means the default 24.
 * Returns 0 on success, 1 on a bad argument (as the reference's rc 1). */
int32_t orc_sym_solve(int32_t n, int32_t threads, uint64_t max_cases,
                      uint64_t start_case, int32_t expanded_n,
                      uint64_t *out_lo_hi, orc_work *work);

#ifdef __cplusplus
}
#endif

#endif
