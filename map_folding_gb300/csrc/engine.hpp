// engine.hpp -- internal declarations shared by the host code, the kernels
// and the C ABI of the map-folding engine.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mapfold.h"

namespace mf {

// ---------------------------------------------------------------- errors --
void set_error(const char *fmt, ...);
void clear_error();
const char *last_error();

#define MF_TRY_CUDA(call)                                                          \
    do {                                                                           \
        cudaError_t mf_err_ = (call);                                              \
        if (mf_err_ != cudaSuccess) {                                              \
            ::mf::set_error("%s failed: %s", #call, cudaGetErrorString(mf_err_));   \
            return MF_ERR_CUDA;                                                    \
        }                                                                          \
    } while (0)

double now_seconds();

// ------------------------------------------------------------- Lunnon ----
// Coordinate/neighbour tables of one p1 x p2 x ... map (mf.c:29-75).
struct LunnonTables {
    int n = 0;
    int dim = 0;
    int p[MF_MAX_DIMS] = {};
    int stride[MF_MAX_DIMS + 1] = {};
    // next[(i*(n+1) + l)*(n+1) + m]: leaf reached from m in dimension i when
    // leaves 1..l are placed; entry m = 0 is 0.
    std::vector<uint8_t> next;
    uint8_t at(int i, int l, int m) const { return next[(size_t(i) * (n + 1) + l) * (n + 1) + m]; }
};

bool build_lunnon_tables(const int32_t *dims, int ndim, LunnonTables &t, std::string &why);

// Bytes per packed prefix-state record (b[0..n], padded to 16).
inline uint32_t lunnon_state_stride(int n) { return uint32_t((n + 1 + 15) / 16 * 16); }

// Prefix states at leaf depth `depth` in the reference's emission order.
// Writes the records with index in [first, first + cap), `stride` bytes
// each; returns the total number of states.
uint64_t collect_lunnon_states(const LunnonTables &t, int depth, uint8_t *out, uint64_t cap,
                               uint32_t stride, uint64_t first = 0);

// A sensible default split depth for a map with n leaves.
int default_lunnon_depth(const LunnonTables &t);

// --------------------------------------------------------------- sym -----
constexpr int kSymCells = 64;
// Boards over 64 cells (9x9, experiments/9x9/sym_fold9.cpp) search with
// 128-bit masks over lists of up to kWideCells cells.
constexpr int kWideCells = 96;

void sym_edges(int n, uint8_t *out /* 4*64 */);
// The same pages with `stride` cells each (cells >= stride left out).
void sym_edges_stride(int n, uint8_t *out, int stride);
uint64_t sym_good_host(const uint8_t *cycle, int i, const uint8_t *edges);
void sym_good_host_wide(const uint8_t *cycle, int i, const uint8_t *wide_edges, uint64_t &lo,
                        uint64_t &hi);

struct SymPlan {
    int n = 0;
    int c = 0;            // centre side (3 odd, 4 even)
    int seed_i = 0;       // c*c
    int start_i = 0;      // cells placed in every case (= expanded_n)
    uint64_t center_cases = 0;
    uint64_t seed_base = 0;           // first representative kept (seed slice)
    uint64_t reduced_all = 0;         // representatives before the seed slice
    std::vector<uint8_t> edges;      // 4*64 (boards over 64 cells: cells 0..63)
    std::vector<uint8_t> wide_edges; // 4*kWideCells, boards over 64 cells only
    std::vector<uint8_t> reps;       // representatives, 64 bytes each
    std::vector<uint64_t> rep_mult;  // orbit sizes
    // Expansion index: the cases are the depth-start_i descendants of the
    // representatives, emitted in DFS order.  When mid_i > seed_i the index
    // holds every depth-mid_i prefix with the number of cases below it, so
    // a chunk start is found by binary search instead of a walk.
    int mid_i = 0;
    std::vector<uint8_t> mid_cycles;
    std::vector<uint64_t> mid_mult;
    std::vector<uint64_t> mid_first;  // prefix sums: first case index of each
    uint64_t total_cases = 0;
    // Once sorted by cost (MF_COST_DEPTH + MF_SORT_CASES, sym_fold.cpp:
    // 267-314) the cases are held materialized in sorted order, and case
    // indices refer to that order, as in the reference's materialized mode.
    std::vector<uint8_t> sorted_cycles;
    std::vector<uint64_t> sorted_mult;
    // Cases expanded past 64 cells (9x9, MF_EXPANDED_N up to 81): records of
    // kWideCells bytes, and no case-count index -- counting every case below
    // each prefix would be a large part of the 9x9 search itself -- so a chunk
    // is reached by walking the cases in emission order from the first, as
    // experiments/9x9/sym_fold9.cpp does in its stream mode (total_cases is
    // then unknown, 0).
    bool streamed = false;
    uint32_t case_bytes = kSymCells;
};

// The reference's cost order (sym_fold.cpp:297-310): std::sort of the cases
// by score, descending (ascending if `ascending`), ties by multiplier.
// std::sort is not stable; given the same input order and comparator,
// libstdc++'s introsort makes the same permutation whatever the element
// type, so sorting (score, multiplier, index) triples reproduces the
// reference's order.  perm[k] = emission index of the k-th sorted case.
void sym_sort_order(const uint64_t *scores, const uint64_t *mults, uint64_t count, bool ascending,
                    uint64_t *perm);

// Builds reps/multipliers and (host side) the expansion index at mid level
// `mid_i` (0 = none).  mid counts are filled by `count_below` when the
// index is used; see sym_plan_index().
// center_n 0: default centre; a seed slice keeps representatives
// [seed_start, seed_start + seed_count) (seed_count 0: the rest).
int build_sym_plan(int n, int expanded_n, SymPlan &plan, std::string &why, int center_n = 0,
                   uint64_t seed_start = 0, uint64_t seed_count = 0);

// Enumerate depth-`stop` descendants of `cycle` (cells < from placed) in DFS
// order, calling emit(cycle) for each; emit returns false to stop early.
// Returns false if stopped.
template <class F>
bool sym_expand(uint8_t *cycle, int from, int stop, const uint8_t *edges, F &&emit);
template <class F>
bool sym_expand_wide(uint8_t *cycle, int from, int stop, const uint8_t *wide_edges, F &&emit);

// Select cases [start, start+max) into cycles/mults; returns count selected.
uint64_t sym_select_cases(const SymPlan &plan, uint64_t start, uint64_t max_cases,
                          uint8_t *cycles, uint64_t *mults, uint64_t cap);

// build_sym_plan plus, for deep expansions, the GPU-built case index (the
// plan mf_sym_plan_create returns).  Returns an mf_status.
int build_full_sym_plan(int n, int expanded_n, SymPlan &plan);

// -------------------------------------------------------- device side ----
struct BatchKnobs {
    int block_threads;
    int blocks_per_sm;
    uint32_t node_budget;
    uint32_t hungry_factor;
    uint64_t queue_capacity;
    uint32_t wait_limit;
    uint32_t stack_mode;  // 0: shared memory when it fits, 1: local memory
};
BatchKnobs resolve_knobs(const mf_batch_config *cfg);

// Work item written by device-side splitting (96 bytes).
struct alignas(16) TaskRecord {
    uint32_t words[17];  // successor list of the placed items (byte per item)
    uint32_t owner;      // result slot
    uint64_t mask;       // remaining choices at `level`
    uint32_t level;
    uint32_t kind;       // instance / problem selector
    uint32_t pad[2];
};
static_assert(sizeof(TaskRecord) == 96, "task record layout");

struct QueueHeader {
    unsigned long long init_next;   // next initial unit to hand out
    unsigned long long spawn_head;  // next split item to hand out
    unsigned long long spawn_tail;  // split items reserved
    unsigned long long completed;   // work items finished
    unsigned long long tasks_run;
    unsigned int error;             // 0, kErrMalformed or kErrWaitLimit
    unsigned int pad;
    long long idle_lanes;           // lanes waiting for work (warps report deltas)
    unsigned long long warps_out;   // warps that have left the launch
};
static_assert(sizeof(QueueHeader) == 64, "queue header layout");

// Error words of a persistent launch (QueueHeader::error).
constexpr unsigned int kErrMalformed = 1;  // a unit's list was not a permutation
constexpr unsigned int kErrWaitLimit = 2;  // the launch ended (its warps' bounded
                                           // waits ran out) with work unaccounted for

// After a persistent launch: MF_OK, or the status its header reports --
// MF_ERR_ARG for a malformed unit, MF_ERR_TIMEOUT when a bounded wait ran
// out or the work accounting does not close (every initial unit handed out,
// completed == units + split items).  Sets the error text.
int check_queue_header(const QueueHeader &hdr, uint64_t units);

uint64_t workspace_bytes(uint64_t capacity);
uint64_t wide_workspace_bytes(uint64_t capacity);

// One Lunnon map as the batched kernel sees it.
struct LunnonInstanceDev {
    uint32_t table_offset;  // into the concatenated next-tables
    int32_t n;
    int32_t dim;
    int32_t start_leaf;
};

// d_edges: the 4 x 64 edge pages in device memory.
cudaError_t launch_sym_plain(const uint8_t *d_edges, int start_i, int stop_i,
                             const uint8_t *d_cycles, uint64_t num, uint64_t *d_counts,
                             uint64_t *d_nodes, cudaStream_t stream);
// The 128-bit batched search for boards over 64 cells (wide_kernels.cu):
// d_wide_edges holds 4 pages of kWideCells, cases are records of
// record_bytes (64, or kWideCells for expansions past 64 cells) with start_i
// <= record_bytes cells placed, stop_i <= kWideCells.
cudaError_t launch_sym_wide(const uint8_t *d_wide_edges, int start_i, int stop_i,
                            const uint8_t *d_cycles, uint32_t record_bytes, uint64_t num,
                            uint64_t *d_counts,
                            uint64_t *d_nodes, void *d_workspace, const BatchKnobs &knobs,
                            cudaStream_t stream);

cudaError_t launch_sym_batched(const uint8_t *d_edges, int start_i, int stop_i,
                               const uint8_t *d_cycles, uint64_t num, uint64_t *d_counts,
                               uint64_t *d_nodes, void *d_workspace, const BatchKnobs &knobs,
                               cudaStream_t stream);
cudaError_t launch_lunnon_plain(const uint8_t *d_table, int n, int dim, int start_leaf,
                                const uint8_t *d_states, uint32_t stride, uint64_t num,
                                uint64_t *d_per_state, uint64_t *d_total, uint64_t *d_nodes,
                                cudaStream_t stream);
// Batched multi-instance Lunnon: states of all instances concatenated;
// d_state_owner[k] = instance of state k; d_counts[instance] += count/leaf.
// d_meta holds the maps' neighbour tables followed, at inst_offset, by their
// LunnonInstanceDev records (meta_bytes in all); max_levels is the largest
// n - start_leaf over the instances.
cudaError_t launch_lunnon_batched(const uint8_t *d_meta, uint32_t meta_bytes, uint32_t inst_offset,
                                  int num_inst, int max_levels, const uint8_t *d_states,
                                  const uint32_t *d_state_owner, uint64_t num, uint64_t *d_counts,
                                  uint64_t *d_nodes, void *d_workspace, const BatchKnobs &knobs,
                                  cudaStream_t stream);

int device_sm_count();

}  // namespace mf

#include "sym_expand.inl"
