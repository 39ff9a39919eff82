// dfs_kernels.cu -- sm_103a counting kernels.
//
// Both hot paths of the reference are the same search shape: a circular
// successor list (Lunnon: b[] over leaves, mf.c:128-142; sym_fold: cycle[]
// over spiral cells, sym_fold.cpp:206-217), grown one item per level by
// inserting item `lvl` after a chosen position, with the set of admissible
// positions recomputed at every level by walking the list.  The engine below
// keeps that list per thread in shared memory (byte per item, in 128-byte
// rows shared by four warps so a warp never has a bank conflict), keeps the
// per-level choices as a 64-bit mask stack whose lowest bit is the current
// pick (in shared memory when the search is at most 48 levels deep, else in
// local memory) instead of the reference's gap[] array, walks a node's two
// constraint chains side by side, and counts the last level with a popcount.
// Gap rules:
//   LunnonRules  -- mf.c:88-124 as a bitwise AND of per-dimension walk masks
//   SymRules     -- sym_fold.cpp:179-204 (get_good)
// Kernels:
//   *_plain_kernel    one thread per unit (prefix state / case), one launch
//   *_batched_kernel  persistent grid, device work queue, subtree splitting
//
// Every unit's list is checked to be a permutation of its placed items before
// its search starts, which bounds every walk (see list_valid); the device
// queue is non-blocking (no thread ever waits on another), so malformed input
// cannot hang a kernel: a unit whose list is malformed reports UINT64_MAX
// (plain) or raises the queue error flag (batched).
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "dfs_core.cuh"
#include "engine.hpp"

namespace mf {
namespace {

// ------------------------------------------------------- plain kernels ---

// One thread per case: d_counts[k] = completions of case k (UINT64_MAX if
// its cycle is malformed).  Shared memory: 4 edge pages, then the carve.
template <int TPB, int LEVELS>
__global__ void __launch_bounds__(TPB)
    sym_plain_kernel(const uint8_t *__restrict__ edges, int start_i, int stop_i,
                     const uint8_t *__restrict__ cycles, uint64_t num,
                     unsigned long long *__restrict__ counts,
                     unsigned long long *__restrict__ nodes_out) {
    extern __shared__ __align__(16) uint8_t smem[];
    using C = Carve<TPB, 16, LEVELS>;
    const SymHopRules R = stage_sym_hop_rules<TPB>(smem, edges, start_i, stop_i - start_i);
    const size_t tables = sym_tables_bytes(stop_i - start_i);
    const List<TPB> L = C::list(smem, tables);
    typename StackOf<TPB, LEVELS>::type S;
    init_stack<TPB, 16, LEVELS>(S, smem, tables);
    const uint64_t unit = uint64_t(blockIdx.x) * TPB + threadIdx.x;
    const bool active = unit < num;
    if (active) load_list<TPB, 16>(L, cycles + unit * kSymCells, kSymCells);

    unsigned long long nodes = 0, leaves = 0;
    const bool bad = active && !list_valid(L, start_i);
    S.base = start_i;
    run_units(R, L, S, active && !bad, start_i, stop_i - 1, leaves, nodes);
    if (active) counts[unit] = bad ? ~0ULL : leaves;
    if (nodes_out) {
        const unsigned long long s = warp_sum(nodes);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(nodes_out, s);
    }
}

// One thread per prefix state.  Shared memory: the map's neighbour table,
// then the carve.
template <int TPB, int LEVELS>
__global__ void __launch_bounds__(TPB)
    lunnon_plain_kernel(const uint8_t *__restrict__ table, int table_bytes, int n, int dim,
                        int start_leaf, const uint8_t *__restrict__ states, uint32_t stride,
                        uint64_t num, unsigned long long *__restrict__ per_state,
                        unsigned long long *__restrict__ total,
                        unsigned long long *__restrict__ nodes_out) {
    extern __shared__ __align__(16) uint8_t smem[];
    using C = Carve<TPB, 17, LEVELS>;
    for (int k = threadIdx.x; k < table_bytes / 4; k += TPB)
        reinterpret_cast<uint32_t *>(smem)[k] = __ldg(reinterpret_cast<const uint32_t *>(table) + k);
    const List<TPB> L = C::list(smem, table_bytes);
    typename StackOf<TPB, LEVELS>::type S;
    init_stack<TPB, 17, LEVELS>(S, smem, table_bytes);
    const uint64_t unit = uint64_t(blockIdx.x) * TPB + threadIdx.x;
    const bool active = unit < num;
    if (active) load_list<TPB, 17>(L, states + unit * stride, stride);
    __syncthreads();

    unsigned long long nodes = 0, leaves = 0;
    const bool bad = active && !list_valid(L, start_leaf < n + 1 ? start_leaf : n + 1);
    S.base = start_leaf;
    run_units(LunnonRules{smem, n, dim}, L, S, active && !bad, start_leaf, n, leaves, nodes);
    leaves = bad ? 0 : leaves * static_cast<unsigned long long>(n);
    if (active && per_state) per_state[unit] = bad ? ~0ULL : leaves;
    if (total) {
        const unsigned long long s = warp_sum(leaves);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(total, s);
    }
    if (nodes_out) {
        const unsigned long long s = warp_sum(nodes);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(nodes_out, s);
    }
}

// ------------------------------------------------- persistent kernels ----

__global__ void ring_init_kernel(unsigned long long *seq, unsigned long long capacity) {
    for (unsigned long long k = blockIdx.x * blockDim.x + threadIdx.x; k < capacity;
         k += gridDim.x * blockDim.x)
        seq[k] = k;
}

struct SymSource {
    const uint8_t *cycles;
    int start_i;
    int last;
};

struct LunnonSource {
    const uint8_t *states;
    const uint32_t *state_owner;
    const LunnonInstanceDev *inst;
    uint32_t stride;
};

// The persistent loop, in lockstep rounds.  Each round every busy lane
// evaluates one node, consumes it and advances to its next node; a lane whose
// unit is exhausted starts its next one at once: the next unit's index is
// taken with an atomicAdd when the previous unit starts, so only the record
// load is paid when the unit is needed (holding the record in registers
// ahead of time cost 16-20 registers per thread for the whole search, which
// the occupancy needs more).  Every `period` rounds
// a warp does its bookkeeping: it reports finished units and its idle-lane
// count, lets idle lanes take split items, and -- while fewer split items are
// queued than lanes wait for work -- lets a few busy lanes give away their
// shallowest untried siblings.  A warp leaves when it is idle and all work is
// accounted for, or when it has stayed idle for wait_limit rounds; leaving is
// always safe, because the warp that owns a split item's parent keeps looping
// until it has nothing left.  The last warp out checks that the work
// accounting closed (leave_and_check).
template <int TPB, int WORDS, bool kSym, class Stk>
__device__ __forceinline__ void persistent_loop(const uint8_t *s_tables,
                                                const LunnonInstanceDev *s_inst,
                                                const SymSource &sym, const LunnonSource &lun,
                                                unsigned long long num,
                                                unsigned long long *counts,
                                                unsigned long long *nodes_out, const Queue &Q,
                                                uint32_t period, uint32_t wait_limit,
                                                const List<TPB> &L, Stk &S) {
    constexpr int kVecs = (WORDS + 3) / 4;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    bool busy = false, fresh = false;
    bool walking = false;  // a resumable walk is under way
    SymHopRules::Walk swalk{};
    LunnonRules::Walk lwalk{};
    int lvl = 0, root = 0, last = 0, eval = 0;
    uint32_t owner = 0;
    unsigned long long leaves = 0, nodes = 0, finished = 0, started = 0;
    uint32_t idle_rounds = 0, round = 0;
    int reported_idle = 0;  // lane 0: idle lanes this warp last reported
    bool ring_hint = false;  // warp-uniform: the split ring probably has items
    const SymHopRules srules{s_tables + 9 * kSymCells,
                             reinterpret_cast<const uint32_t *>(s_tables + 4 * kSymCells),
                             s_tables + 8 * kSymCells, sym.start_i};
    LunnonRules lrules{s_tables, 0, 0};

    // Prefetch state: 0 = no initial unit left for this lane, 1 = index
    // taken.  The first indices come from one warp-aggregated atomicAdd.
    unsigned long long pre_k = 0;
    {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&Q.hdr->init_next, 32ULL);
        pre_k = __shfl_sync(kFull, base, 0) + lane;
    }
    int pre_stage = 1;
    uint4 pre[kVecs];
    uint32_t pre_owner = 0;

#define MF_FETCH_RECORD()                                                                   \
    do {                                                                                   \
        const uint4 *src_ = kSym                                                           \
            ? reinterpret_cast<const uint4 *>(sym.cycles + pre_k * kSymCells)              \
            : reinterpret_cast<const uint4 *>(lun.states + pre_k * lun.stride);            \
        _Pragma("unroll") for (int q_ = 0; q_ < kVecs; ++q_) pre[q_] = __ldg(src_ + q_);   \
        if (!kSym) pre_owner = __ldg(lun.state_owner + pre_k);                             \
    } while (0)

    auto flush = [&]() {
        if (leaves) {
            const unsigned long long weight = kSym ? 1ULL : static_cast<unsigned long long>(lrules.n);
            atomicAdd(counts + owner, leaves * weight);
        }
        leaves = 0;
        ++finished;
    };

    auto set_instance = [&](uint32_t inst) -> int {
        const LunnonInstanceDev I = s_inst[inst];
        lrules = LunnonRules{s_tables + I.table_offset, I.n, I.dim};
        last = I.n;
        S.base = I.start_leaf;
        return I.start_leaf;
    };

    // Warp-cooperative intake of split items by the lanes in `need` (all 32
    // lanes call): one claim on the ring's head, then each taking lane copies
    // its item.  Returns true if fewer items were available than asked for.
    auto take_splits = [&](unsigned need) -> bool {
        const int want = __popc(need);
        unsigned long long first = 0;
        const int got = ring_claim(Q, &Q.hdr->spawn_head, want, true, first);
        const bool mine = (need >> lane) & 1u;
        const int rank = __popc(need & lt_mask);
        if (mine && rank < got) {
            uint32_t w[24];
            ring_take(Q, first + rank, w);
            ++started;
#pragma unroll
            for (int k2 = 0; k2 < WORDS; ++k2) L.set_word(k2, w[k2]);
            owner = w[17];
            root = int(w[20]);
            if (kSym) {
                last = sym.last;
                S.base = sym.start_i;
            } else {
                set_instance(owner);
            }
            lvl = root;
            S.set(root, uint64_t(w[18]) | (uint64_t(w[19]) << 32));
            eval = advance(L, S, lvl, root);  // an item's mask is never empty
            walking = false;
            fresh = false;
            busy = eval >= 0;
        }
        return got < want;
    };

    // Warp-cooperative donation (all 32 lanes call): every busy lane with an
    // untried sibling set at least kMinSplitHeight above the counted level
    // gives the shallowest such set away.  One claim on the ring's tail
    // reserves cells for all donors; each donor rolls its list back to that
    // level, copies it out, replays, and publishes.
    auto donate = [&]() {
        int s = root;
        const uint64_t m = busy && !fresh ? shallowest_siblings(S, root, lvl, s) : 0;
        const bool can = busy && !fresh && m != 0 && last - s >= kMinSplitHeight;
        const unsigned donors = __ballot_sync(kFull, can);
        if (!donors) return;
        unsigned long long first = 0;
        const int got = ring_claim(Q, &Q.hdr->spawn_tail, __popc(donors), false, first);
        const int rank = __popc(donors & lt_mask);
        if (!can || rank >= got) return;
        roll_back(L, S, s, lvl);
        uint32_t w[24];
#pragma unroll
        for (int k = 0; k < 24; ++k) w[k] = 0;
#pragma unroll
        for (int k = 0; k < WORDS; ++k) w[k] = L.word(k);
        w[17] = owner;
        w[18] = uint32_t(m);
        w[19] = uint32_t(m >> 32);
        w[20] = uint32_t(s);
        replay_keeping_pick(L, S, s, lvl);
        ring_put(Q, first + rank, w);
    };

    uint32_t nap = 256;  // idle back-off, ns
    for (;;) {
        // Start the prefetched unit on lanes whose search has ended.
        if (!busy && pre_stage != 0) {
            if (pre_k < num) {
                MF_FETCH_RECORD();
#pragma unroll
                for (int q = 0; q < kVecs; ++q) {
                    const uint32_t ws[4] = {pre[q].x, pre[q].y, pre[q].z, pre[q].w};
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (4 * q + k < WORDS) L.set_word(4 * q + k, ws[k]);
                }
                ++started;
                bool ok;
                if (kSym) {
                    owner = uint32_t(pre_k);
                    root = sym.start_i;
                    last = sym.last;
                    S.base = root;
                    ok = list_valid(L, root);
                } else {
                    owner = pre_owner;
                    root = set_instance(owner);
                    ok = list_valid(L, root < lrules.n + 1 ? root : lrules.n + 1);
                }
                if (!ok) {
                    atomicExch(&Q.hdr->error, kErrMalformed);
                    // As the plain kernel does: the case's count slot says it
                    // was not counted (a Lunnon slot is a whole map's sum and
                    // keeps only the error word).
                    if (kSym) counts[owner] = ~0ULL;
                    ++finished;
                } else if (root > last) {  // nothing left to place: one completion
                    leaves = 1;
                    flush();
                } else {
                    busy = true;
                    fresh = true;
                    walking = false;
                    lvl = root;
                    eval = root;
                }
                pre_k = atomicAdd(&Q.hdr->init_next, 1ULL);
                pre_stage = 1;
            } else {
                pre_stage = 0;
            }
        }
        // Lanes without initial units take split items while the warp's hint
        // says the ring has some (refreshed at bookkeeping, cleared by a miss).
        if (ring_hint) {
            const unsigned need = __ballot_sync(kFull, !busy && pre_stage == 0);
            if (need && take_splits(need)) ring_hint = false;
        }
        const bool bookkeeping = ++round >= period;
        if (!__any_sync(kFull, busy)) {
            // The whole warp is idle: report, look for split items, decide.
            const unsigned long long f = warp_sum(finished);
            finished = 0;
            if (lane == 0) {
                if (f) atomicAdd(&Q.hdr->completed, f);
                if (reported_idle != 32) {
                    atomicAdd(reinterpret_cast<unsigned long long *>(&Q.hdr->idle_lanes),
                              (unsigned long long)(long long)(32 - reported_idle));
                    reported_idle = 32;
                }
            }
            const unsigned need = __ballot_sync(kFull, pre_stage == 0);
            if (need) take_splits(need);
            // A lane still holding a prefetched unit keeps the warp alive.
            const bool holding = __any_sync(kFull, pre_stage != 0 && pre_k < num);
            if (__any_sync(kFull, busy) || holding) {
                idle_rounds = 0;
                nap = 256;
                continue;
            }
            int stop = 0;
            if (lane == 0) {
                const unsigned long long total = num + vload(&Q.hdr->spawn_tail);
                stop = (vload(&Q.hdr->init_next) >= num && vload(&Q.hdr->completed) >= total) ||
                       *reinterpret_cast<volatile unsigned int *>(&Q.hdr->error) != 0u ||
                       ++idle_rounds > wait_limit;
            }
            stop = __shfl_sync(kFull, stop, 0);
            if (stop) break;
            __nanosleep(nap);
            if (nap < 8192) nap <<= 1;
            continue;
        }
        idle_rounds = 0;
        nap = 256;
        // One round of evaluation per busy lane: a walk takes at most
        // kWalkCap steps and goes on in the next round if unfinished.
        if (busy) {
            uint64_t g = 0;
            bool evaluated;
            if (kSym) {
                if (!walking) {
                    srules.begin(L, eval, nodes, swalk);
                    walking = true;
                }
                evaluated = srules.run(L, swalk, kWalkCap);
                if (evaluated) g = srules.result(swalk, nodes);
            } else {
                if (!walking) {
                    lrules.begin(L, eval, nodes, lwalk);
                    walking = true;
                }
                evaluated = lrules.run(L, lwalk, kWalkCap);
                if (evaluated) g = lrules.result(lwalk, nodes);
            }
            if (evaluated) {
                walking = false;
                eval = apply_advance(L, S, lvl, eval, root, last, fresh, g, leaves);
                fresh = false;
                if (eval < 0) {
                    flush();
                    busy = false;
                }
            }
        }
        if (!bookkeeping) continue;
        round = 0;
        const unsigned idle_mask = __ballot_sync(kFull, !busy);
        const unsigned long long f = warp_sum(finished);
        finished = 0;
        long long want = 0, queued = 0;
        if (lane == 0) {
            if (f) atomicAdd(&Q.hdr->completed, f);
            const int idle_now = __popc(idle_mask);
            if (idle_now != reported_idle) {
                atomicAdd(reinterpret_cast<unsigned long long *>(&Q.hdr->idle_lanes),
                          (unsigned long long)(long long)(idle_now - reported_idle));
                reported_idle = idle_now;
            }
            if (vload(&Q.hdr->init_next) >= num) {
                queued = (long long)(vload(&Q.hdr->spawn_tail) - vload(&Q.hdr->spawn_head));
                const long long waiting = *reinterpret_cast<volatile long long *>(&Q.hdr->idle_lanes);
                want = waiting - queued;
            }
        }
        want = __shfl_sync(kFull, want, 0);
        ring_hint = __shfl_sync(kFull, queued, 0) > 0;
        // Feed waiting lanes: busy lanes give away their shallowest untried
        // siblings while lanes wait for work.
        if (want > 0) donate();
    }
#undef MF_FETCH_RECORD

    if (lane == 0 && reported_idle)
        atomicAdd(reinterpret_cast<unsigned long long *>(&Q.hdr->idle_lanes),
                  (unsigned long long)(-(long long)reported_idle));
    const unsigned long long ns = warp_sum(nodes);
    const unsigned long long st = warp_sum(started);
    if (lane == 0) {
        if (nodes_out && ns) atomicAdd(nodes_out, ns);
        if (st) atomicAdd(&Q.hdr->tasks_run, st);
        leave_and_check(Q.hdr, num);
    }
}

template <int TPB, int LEVELS>
__global__ void __launch_bounds__(TPB)
    sym_batched_kernel(const uint8_t *__restrict__ edges, SymSource src, unsigned long long num,
                       unsigned long long *counts, unsigned long long *nodes_out, Queue Q,
                       uint32_t period, uint32_t wait_limit) {
    extern __shared__ __align__(16) uint8_t smem[];
    using C = Carve<TPB, 16, LEVELS>;
    stage_sym_hop_rules<TPB>(smem, edges, src.start_i, src.last - src.start_i + 1);
    const size_t tables = sym_tables_bytes(src.last - src.start_i + 1);
    const List<TPB> L = C::list(smem, tables);
    typename StackOf<TPB, LEVELS>::type S;
    init_stack<TPB, 16, LEVELS>(S, smem, tables);
    LunnonSource none{};
    persistent_loop<TPB, 16, true>(smem, nullptr, src, none, num, counts, nodes_out, Q, period,
                                   wait_limit, L, S);
}

// Shared memory: the maps' neighbour tables and their instance records
// (meta_bytes in all, records at inst_offset), then the carve.
template <int TPB, int LEVELS>
__global__ void __launch_bounds__(TPB)
    lunnon_batched_kernel(const uint8_t *__restrict__ meta, uint32_t meta_bytes,
                          uint32_t inst_offset, LunnonSource src, unsigned long long num,
                          unsigned long long *counts, unsigned long long *nodes_out, Queue Q,
                          uint32_t period, uint32_t wait_limit) {
    extern __shared__ __align__(16) uint8_t smem[];
    using C = Carve<TPB, 17, LEVELS>;
    for (uint32_t k = threadIdx.x; k < meta_bytes / 4; k += TPB)
        reinterpret_cast<uint32_t *>(smem)[k] = __ldg(reinterpret_cast<const uint32_t *>(meta) + k);
    __syncthreads();
    const List<TPB> L = C::list(smem, meta_bytes);
    typename StackOf<TPB, LEVELS>::type S;
    init_stack<TPB, 17, LEVELS>(S, smem, meta_bytes);
    SymSource none{};
    persistent_loop<TPB, 17, false>(smem, reinterpret_cast<const LunnonInstanceDev *>(smem + inst_offset),
                                    none, src, num, counts, nodes_out, Q, period, wait_limit, L, S);
}

// ------------------------------------------------------- launch helpers --

// MF_STACK_MODE=local forces the local-memory stack (a tuning aid).
bool env_local_stack() {
    static const bool local = [] {
        const char *e = std::getenv("MF_STACK_MODE");
        return e && std::strcmp(e, "local") == 0;
    }();
    return local;
}

// Smallest compiled stack depth that holds `levels` levels (0 = local).
int pick_levels(int levels, bool local = false) {
    if (local || env_local_stack()) return 0;
    if (levels <= 24) return 24;
    if (levels <= 32) return 32;
    if (levels <= 48) return 48;
    return 0;
}

// Size a kernel's persistent grid from the occupancy calculator.  The first
// time a kernel is seen on a device its dynamic shared-memory limit is raised
// once to the device's opt-in maximum (never lowered again, so every later
// launch size stays legal); occupancy results are cached per (device,
// kernel, shared bytes), so a launch recorded into a CUDA graph makes no
// attribute or occupancy calls.
struct FitEntry {
    int dev;
    const void *fn;
    size_t smem;  // 0: the kernel's shared-memory limit has been raised
    int fit;
};
std::mutex g_fit_mu;
FitEntry g_fit[512];
int g_fit_len = 0;

template <class K>
cudaError_t prepare(K kernel, size_t smem, int tpb, int want_per_sm, int &blocks_per_sm) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const void *fn = reinterpret_cast<const void *>(kernel);
    int fit = 0;
    bool raised = false;
    {
        std::lock_guard<std::mutex> lock(g_fit_mu);
        for (int k = 0; k < g_fit_len; ++k) {
            if (g_fit[k].dev != dev || g_fit[k].fn != fn) continue;
            if (g_fit[k].smem == 0) raised = true;
            else if (g_fit[k].smem == smem) fit = g_fit[k].fit;
        }
    }
    if (!raised) {
        int optin = 0;
        e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
        if (e != cudaSuccess) return e;
        std::lock_guard<std::mutex> lock(g_fit_mu);
        if (g_fit_len < 512) g_fit[g_fit_len++] = FitEntry{dev, fn, 0, 0};
    }
    if (fit == 0) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kernel, tpb, smem);
        if (e != cudaSuccess) return e;
        if (fit < 1) return cudaErrorInvalidConfiguration;
        std::lock_guard<std::mutex> lock(g_fit_mu);
        if (g_fit_len < 512) g_fit[g_fit_len++] = FitEntry{dev, fn, smem, fit};
    }
    blocks_per_sm = want_per_sm > 0 && want_per_sm < fit ? want_per_sm : fit;
    return cudaSuccess;
}

}  // namespace

// ------------------------------------------------------------ launchers --

int device_sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return sms;
}

uint64_t workspace_bytes(uint64_t capacity) {
    return 256 + capacity * sizeof(TaskRecord) + capacity * sizeof(unsigned long long);
}

namespace {

Queue carve_queue(void *ws, uint64_t capacity) {
    uint8_t *p = static_cast<uint8_t *>(ws);
    Queue q;
    q.hdr = reinterpret_cast<QueueHeader *>(p);
    q.slots = reinterpret_cast<TaskRecord *>(p + 256);
    q.seq = reinterpret_cast<unsigned long long *>(p + 256 + capacity * sizeof(TaskRecord));
    q.capacity = capacity;
    return q;
}

// Host-side fault injection for tests (mf_test_inject_fault): the next
// persistent launch starts with one split-ring ticket reserved that no lane
// ever publishes, as if a donor's message had been lost.
std::atomic<uint32_t> g_inject{0};

__global__ void phantom_ticket_kernel(QueueHeader *hdr) { hdr->spawn_tail = 1; }

// Launch size of a persistent launch over `units` initial units searched
// `levels` levels deep: the whole resident grid, or -- for a small job, whose
// units are shallow (at most 10 levels to go, so none of them is heavy) --
// about one warp per four units, with a split ring of at most two cells per
// launched lane (at least 1024).  A tiny map then costs one small launch and
// a short ring reset instead of thousands of warps that start, find nothing
// and leave, and a 512 KB ring initialisation.  Deep units always get the
// whole grid: a single deep unit can hold most of the work.
struct LaunchShape {
    unsigned blocks;
    uint64_t ring;
};

LaunchShape persistent_shape(int sms, int bpsm, int tpb, uint64_t units, int levels,
                             uint64_t ring_knob) {
    const uint64_t full = uint64_t(sms) * uint64_t(bpsm);
    if (levels > 10) return LaunchShape{unsigned(full), ring_knob};
    const uint64_t warps = (units + 3) / 4;
    const uint64_t per_block = uint64_t(tpb / 32);
    uint64_t blocks = (warps + per_block - 1) / per_block;
    blocks = blocks < 1 ? 1 : (blocks > full ? full : blocks);
    uint64_t ring = 1024;
    while (ring < 2 * blocks * uint64_t(tpb) && ring < ring_knob) ring <<= 1;
    return LaunchShape{unsigned(blocks), ring < ring_knob ? ring : ring_knob};
}

cudaError_t reset_queue(const Queue &Q, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(Q.hdr, 0, 256, stream);
    if (e != cudaSuccess) return e;
    ring_init_kernel<<<64, 256, 0, stream>>>(Q.seq, Q.capacity);
    if (g_inject.exchange(0) == MF_FAULT_LOST_SPLIT) phantom_ticket_kernel<<<1, 1, 0, stream>>>(Q.hdr);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_sym_plain(const uint8_t *d_edges, int start_i, int stop_i,
                             const uint8_t *d_cycles, uint64_t num, uint64_t *d_counts,
                             uint64_t *d_nodes, cudaStream_t stream) {
    if (num == 0) return cudaSuccess;
    constexpr int TPB = 128;
    const uint64_t blocks = (num + TPB - 1) / TPB;
    const int levels = pick_levels(stop_i - 1 - start_i);
    const size_t tables = sym_tables_bytes(stop_i - start_i);
    auto *counts = reinterpret_cast<unsigned long long *>(d_counts);
    auto *nodes = reinterpret_cast<unsigned long long *>(d_nodes);
    int bpsm = 0;
#define MF_SYM_PLAIN(LV)                                                                        \
    do {                                                                                        \
        const size_t smem = tables + Carve<TPB, 16, LV>::kThreadBytes;                          \
        cudaError_t e = prepare(sym_plain_kernel<TPB, LV>, smem, TPB, 0, bpsm);                 \
        if (e != cudaSuccess) return e;                                                         \
        sym_plain_kernel<TPB, LV><<<unsigned(blocks), TPB, smem, stream>>>(                     \
            d_edges, start_i, stop_i, d_cycles, num, counts, nodes);                            \
    } while (0)
    switch (levels) {
        case 24: MF_SYM_PLAIN(24); break;
        case 32: MF_SYM_PLAIN(32); break;
        case 48: MF_SYM_PLAIN(48); break;
        default: MF_SYM_PLAIN(0); break;
    }
#undef MF_SYM_PLAIN
    return cudaGetLastError();
}

cudaError_t launch_lunnon_plain(const uint8_t *d_table, int n, int dim, int start_leaf,
                                const uint8_t *d_states, uint32_t stride, uint64_t num,
                                uint64_t *d_per_state, uint64_t *d_total, uint64_t *d_nodes,
                                cudaStream_t stream) {
    if (num == 0) return cudaSuccess;
    constexpr int TPB = 128;
    const int table_bytes = (dim * (n + 1) * (n + 1) + 15) / 16 * 16;
    const int levels = pick_levels(n - start_leaf);
    const uint64_t blocks = (num + TPB - 1) / TPB;
    auto *per = reinterpret_cast<unsigned long long *>(d_per_state);
    auto *tot = reinterpret_cast<unsigned long long *>(d_total);
    auto *nodes = reinterpret_cast<unsigned long long *>(d_nodes);
    int bpsm = 0;
#define MF_LUN_PLAIN(LV)                                                                        \
    do {                                                                                        \
        const size_t smem = table_bytes + Carve<TPB, 17, LV>::kThreadBytes;                     \
        cudaError_t e = prepare(lunnon_plain_kernel<TPB, LV>, smem, TPB, 0, bpsm);              \
        if (e != cudaSuccess) return e;                                                         \
        lunnon_plain_kernel<TPB, LV><<<unsigned(blocks), TPB, smem, stream>>>(                  \
            d_table, table_bytes, n, dim, start_leaf, d_states, stride, num, per, tot, nodes);   \
    } while (0)
    switch (levels) {
        case 24: MF_LUN_PLAIN(24); break;
        case 32: MF_LUN_PLAIN(32); break;
        case 48: MF_LUN_PLAIN(48); break;
        default: MF_LUN_PLAIN(0); break;
    }
#undef MF_LUN_PLAIN
    return cudaGetLastError();
}

cudaError_t launch_sym_batched(const uint8_t *d_edges, int start_i, int stop_i,
                               const uint8_t *d_cycles, uint64_t num, uint64_t *d_counts,
                               uint64_t *d_nodes, void *d_workspace, const BatchKnobs &knobs,
                               cudaStream_t stream) {
    if (num == 0) return reset_queue(carve_queue(d_workspace, knobs.queue_capacity), stream);
    cudaError_t e = cudaMemsetAsync(d_counts, 0, num * sizeof(uint64_t), stream);
    if (e != cudaSuccess) return e;
    const int sms = device_sm_count();
    const SymSource src{d_cycles, start_i, stop_i - 1};
    const int levels = pick_levels(stop_i - 1 - start_i, knobs.stack_mode == 1);
    const size_t tables = sym_tables_bytes(stop_i - start_i);
    auto *counts = reinterpret_cast<unsigned long long *>(d_counts);
    auto *nodes = reinterpret_cast<unsigned long long *>(d_nodes);
    int bpsm = 0;
#define MF_SYM_BATCHED(TPB, LV)                                                                  \
    do {                                                                                         \
        const size_t smem = tables + Carve<TPB, 16, LV>::kThreadBytes;                           \
        e = prepare(sym_batched_kernel<TPB, LV>, smem, TPB, knobs.blocks_per_sm, bpsm);          \
        if (e != cudaSuccess) return e;                                                          \
        const LaunchShape shape =                                                                \
            persistent_shape(sms, bpsm, TPB, num, stop_i - start_i, knobs.queue_capacity);       \
        const Queue Q = carve_queue(d_workspace, shape.ring);                                    \
        e = reset_queue(Q, stream);                                                              \
        if (e != cudaSuccess) return e;                                                          \
        sym_batched_kernel<TPB, LV><<<shape.blocks, TPB, smem, stream>>>(                        \
            d_edges, src, num, counts, nodes, Q, knobs.node_budget, knobs.wait_limit);          \
    } while (0)
    if (knobs.block_threads == 256) {
        switch (levels) {
            case 24: MF_SYM_BATCHED(256, 24); break;
            case 32: MF_SYM_BATCHED(256, 32); break;
            case 48: MF_SYM_BATCHED(256, 48); break;
            default: MF_SYM_BATCHED(256, 0); break;
        }
    } else {
        switch (levels) {
            case 24: MF_SYM_BATCHED(128, 24); break;
            case 32: MF_SYM_BATCHED(128, 32); break;
            case 48: MF_SYM_BATCHED(128, 48); break;
            default: MF_SYM_BATCHED(128, 0); break;
        }
    }
#undef MF_SYM_BATCHED
    return cudaGetLastError();
}

cudaError_t launch_lunnon_batched(const uint8_t *d_meta, uint32_t meta_bytes, uint32_t inst_offset,
                                  int num_inst, int max_levels, const uint8_t *d_states,
                                  const uint32_t *d_state_owner, uint64_t num, uint64_t *d_counts,
                                  uint64_t *d_nodes, void *d_workspace, const BatchKnobs &knobs,
                                  cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(d_counts, 0, size_t(num_inst) * sizeof(uint64_t), stream);
    if (e != cudaSuccess) return e;
    if (num == 0) return reset_queue(carve_queue(d_workspace, knobs.queue_capacity), stream);
    const int sms = device_sm_count();
    const uint32_t mb = (meta_bytes + 15) / 16 * 16;
    const LunnonSource src{d_states, d_state_owner, nullptr, lunnon_state_stride(64)};
    const int levels = pick_levels(max_levels, knobs.stack_mode == 1);
    auto *counts = reinterpret_cast<unsigned long long *>(d_counts);
    auto *nodes = reinterpret_cast<unsigned long long *>(d_nodes);
    int bpsm = 0;
#define MF_LUN_BATCHED(TPB, LV)                                                                  \
    do {                                                                                         \
        const size_t smem = mb + Carve<TPB, 17, LV>::kThreadBytes;                               \
        e = prepare(lunnon_batched_kernel<TPB, LV>, smem, TPB, knobs.blocks_per_sm, bpsm);       \
        if (e != cudaSuccess) return e;                                                          \
        const LaunchShape shape =                                                                \
            persistent_shape(sms, bpsm, TPB, num, max_levels, knobs.queue_capacity);             \
        const Queue Q = carve_queue(d_workspace, shape.ring);                                    \
        e = reset_queue(Q, stream);                                                              \
        if (e != cudaSuccess) return e;                                                          \
        lunnon_batched_kernel<TPB, LV><<<shape.blocks, TPB, smem, stream>>>(                     \
            d_meta, mb, inst_offset, src, num, counts, nodes, Q, knobs.node_budget,             \
            knobs.wait_limit);                                                                   \
    } while (0)
    if (knobs.block_threads == 256) {
        switch (levels) {
            case 24: MF_LUN_BATCHED(256, 24); break;
            case 32: MF_LUN_BATCHED(256, 32); break;
            case 48: MF_LUN_BATCHED(256, 48); break;
            default: MF_LUN_BATCHED(256, 0); break;
        }
    } else {
        switch (levels) {
            case 24: MF_LUN_BATCHED(128, 24); break;
            case 32: MF_LUN_BATCHED(128, 32); break;
            case 48: MF_LUN_BATCHED(128, 48); break;
            default: MF_LUN_BATCHED(128, 0); break;
        }
    }
#undef MF_LUN_BATCHED
    return cudaGetLastError();
}

}  // namespace mf

// ------------------------------------------- allocation-free entry point --
//
// mf_sym_count_cases_batched_static: the batched sym kernel with its split
// ring in a fixed device array instead of a caller-provided workspace.  For
// callers that cannot allocate device memory at all -- a process whose HBM is
// owned by another allocator, or a latency-critical caller that must not hit
// the implicit device synchronisation of cudaMalloc/cudaFree -- and therefore
// cannot hand over a workspace either.  Every GPU that loads this library
// holds these arrays until the process exits.

namespace mf {
namespace {

constexpr uint64_t kStaticRingCells = 4096;  // split-ring cells (power of two)
constexpr size_t kStaticWorkspaceBytes =
    256 + kStaticRingCells * (sizeof(TaskRecord) + sizeof(unsigned long long));  // 416.25 KiB

__device__ __align__(256) uint8_t g_static_workspace[kStaticWorkspaceBytes];
__device__ __align__(256) uint8_t g_static_edges[9][4 * kSymCells];  // edge pages per n

struct StaticState {
    bool ready = false;
    unsigned long long ctx_id = 0;  // the CUDA context the addresses belong to
    void *workspace = nullptr;
    uint8_t *edges = nullptr;
};

std::mutex g_static_mu;
StaticState g_static[64];

// Unique id of the calling thread's current CUDA context (0 if none can be
// read).  A device reset destroys the primary context and reloads this
// module with zeroed __device__ arrays; the next context gets a new id.
unsigned long long current_context_id() {
    using GetCurrent = int (*)(void **);
    using GetId = int (*)(void *, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
    });
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Once per device and context, with that device current: look up the
// arrays' device addresses (a host-side name of a __device__ array is not a
// device address) and fill the edge pages of every board size.  Done again
// if the context changed since (a device reset), so no stale address or
// zeroed edge page is ever used.
int static_setup(int dev, StaticState *&out) {
    std::lock_guard<std::mutex> lock(g_static_mu);
    StaticState &s = g_static[dev];
    void *ws = nullptr;
    MF_TRY_CUDA(cudaGetSymbolAddress(&ws, g_static_workspace));  // also brings the context up
    const unsigned long long ctx = current_context_id();
    if (!s.ready || (ctx != 0 && ctx != s.ctx_id)) {
        void *edges = nullptr;
        MF_TRY_CUDA(cudaGetSymbolAddress(&edges, g_static_edges));
        uint8_t host[9][4 * kSymCells] = {};
        for (int n = 2; n <= 8; ++n) sym_edges(n, host[n]);
        MF_TRY_CUDA(cudaMemcpy(edges, host, sizeof(host), cudaMemcpyHostToDevice));
        s.workspace = ws;
        s.edges = static_cast<uint8_t *>(edges);
        s.ctx_id = ctx;
        s.ready = true;
    }
    out = &s;
    return MF_OK;
}

int current_static_state(StaticState *&s) {
    int dev = 0;
    MF_TRY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return MF_ERR_ARG;
    }
    return static_setup(dev, s);
}

}  // namespace
}  // namespace mf

extern "C" int32_t mf_sym_count_cases_batched_static(int32_t n, int32_t start_i, int32_t stop_i,
                                                     const uint8_t *d_cycles, uint64_t num_cases,
                                                     uint64_t *d_counts, uint64_t *d_nodes,
                                                     const mf_batch_config *cfg, void *stream) {
    using namespace mf;
    clear_error();
    if (n < 2 || n > 8) {
        set_error("n must be between 2 and 8");
        return MF_ERR_ARG;
    }
    if (start_i < 0 || start_i > stop_i || stop_i > n * n) {
        set_error("need 0 <= start_i <= stop_i <= n*n");
        return MF_ERR_RANGE;
    }
    if (cfg && cfg->queue_capacity > kStaticRingCells) {
        set_error("queue_capacity %llu exceeds the fixed split ring of %llu cells",
                  (unsigned long long)cfg->queue_capacity, (unsigned long long)kStaticRingCells);
        return MF_ERR_CAPACITY;
    }
    if (num_cases > 0xffffffffULL) {
        set_error("at most 2^32-1 cases per call");
        return MF_ERR_ARG;
    }
    if (num_cases && (!d_cycles || !d_counts)) {
        set_error("d_cycles and d_counts are required");
        return MF_ERR_ARG;
    }
    if (reinterpret_cast<uintptr_t>(d_cycles) % 16) {
        set_error("d_cycles must be 16-byte aligned");
        return MF_ERR_ARG;
    }
    if (cfg && cfg->stack_mode == 2) {
        set_error("stack_mode 2 (the 128-bit kernel) has no allocation-free form");
        return MF_ERR_ARG;
    }
    StaticState *s = nullptr;
    if (int rc = current_static_state(s)) return rc;
    BatchKnobs knobs = resolve_knobs(cfg);
    knobs.queue_capacity = kStaticRingCells;
    MF_TRY_CUDA(launch_sym_batched(s->edges + size_t(n) * 4 * kSymCells, start_i, stop_i, d_cycles,
                                   num_cases, d_counts, d_nodes, s->workspace, knobs,
                                   static_cast<cudaStream_t>(stream)));
    return MF_OK;
}

extern "C" int32_t mf_sym_static_status(void *stream, void *dst) {
    using namespace mf;
    clear_error();
    if (!dst) {
        set_error("dst is required");
        return MF_ERR_ARG;
    }
    StaticState *s = nullptr;
    if (int rc = current_static_state(s)) return rc;
    MF_TRY_CUDA(cudaMemcpyAsync(dst, s->workspace, sizeof(QueueHeader), cudaMemcpyDefault,
                                static_cast<cudaStream_t>(stream)));
    return MF_OK;
}

extern "C" void mf_test_inject_fault(uint32_t kind) { mf::g_inject.store(kind); }
