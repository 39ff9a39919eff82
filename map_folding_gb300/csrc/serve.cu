// serve.cu -- continuous-batching request server.
//
// One persistent kernel keeps running while requests come and go.  The host
// admits a request (an 8x8 sym chunk, a whole small Lunnon map, ...) by
// copying its units into a device unit arena, filling the request's slot
// record and pending counter, and publishing one range of units on a device
// ring; lanes claim units from the oldest range with units left, so a
// request admitted while others are running starts on the lanes that free
// up, and its subtrees share the split ring with everybody else's.  Each
// finished unit or split item decrements its request's pending counter; the
// lane that brings it to zero writes the request's result into mapped host
// memory, where the host sees it without a copy.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "dfs_core.cuh"
#include "engine.hpp"

namespace mf {
namespace {

struct alignas(16) ServeUnit {  // 96 bytes
    uint32_t words[17];         // successor list of the placed items
    uint32_t slot;              // request slot
    uint64_t mult;              // multiplier of this unit's count
    uint32_t root;              // first level to search
    uint32_t pad[3];
};
static_assert(sizeof(ServeUnit) == 96, "serve unit layout");

struct alignas(16) SlotInfo {  // 32 bytes
    uint32_t kind;             // 0 = sym, 1 = Lunnon
    int32_t n;                 // sym: board side; Lunnon: leaves
    int32_t dim;               // Lunnon dimensions
    int32_t base;              // first level of the request's units
    int32_t last;              // level counted by popcount
    uint32_t table_off;        // Lunnon: neighbour table in the table arena
    uint32_t weight;           // leaves per counted position (Lunnon: n)
    uint32_t seq;              // request sequence number
};

struct alignas(16) ServeRange {  // 32 bytes
    unsigned long long first;    // first arena unit
    unsigned long long count;
    unsigned long long taken;    // units claimed so far (may overshoot)
    uint32_t slot;
    uint32_t pad;
};

struct alignas(16) DoneRec {  // 32 bytes, mapped host memory
    unsigned long long sum;
    unsigned long long nodes;
    unsigned long long units;
    volatile unsigned long long seq;  // written last
};

struct ServeCtl {
    unsigned long long published;  // ranges published by the host
    unsigned long long head;       // oldest range that may have units left
    unsigned int stop;             // host: leave once idle
    unsigned int error;
    long long idle_lanes;
    unsigned int oldest_seq;       // host: oldest running request while others run, else 0
    unsigned int pad0;
    unsigned long long pad[3];
};

// Split items the oldest running request keeps in the ring while newer
// requests share the GPU: lanes that free up (and find no unclaimed range)
// take them before newer requests' subtrees, so the oldest request's heavy
// subtrees spread over the lanes instead of finishing serially.
constexpr long long kServeStock = 1024;

struct ServeArgs {
    ServeCtl *ctl;
    ServeRange *ranges;
    unsigned long long range_cap;  // power of two
    const ServeUnit *units;
    unsigned long long unit_cap;
    const SlotInfo *slots;
    long long *pending;
    unsigned long long *sum;
    unsigned long long *nodes;
    DoneRec *done;                 // device view of mapped host memory
    const uint8_t *tables;         // Lunnon tables (append-only arena)
    const uint8_t *edges;          // sym edge pages for n = 6, 7, 8
    Queue Q;
    uint32_t period;
    uint32_t wait_limit;
};

template <int TPB, int LEVELS>
__global__ void __launch_bounds__(TPB) serve_kernel(ServeArgs A) {
    extern __shared__ __align__(16) uint8_t smem[];
    constexpr size_t kTables = 3 * kSymTables;  // n = 6, 7, 8
    for (int b = 0; b < 3; ++b) stage_sym_tables<TPB>(smem + b * kSymTables, A.edges + b * 4 * kSymCells);
    __syncthreads();
    using C = Carve<TPB, 17, LEVELS>;
    const List<TPB> L = C::list(smem, kTables);
    SmemStack<TPB, LEVELS> S = C::stack(smem, kTables);

    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    bool busy = false, fresh = false;
    int lvl = 0, root = 0, last = 0, eval = 0;
    uint32_t slot = 0, kind = 0, weight = 1, my_seq = 0;
    uint64_t mult = 1;
    SymRules srules = sym_rules(smem);
    LunnonRules lrules{A.tables, 0, 0};
    unsigned long long leaves = 0, nodes = 0, unit_nodes0 = 0;
    uint32_t idle_rounds = 0, stuck_rounds = 0, round = 0, nap = 256;
    int reported_idle = 0;
    bool ring_hint = false;

    // Slot records are rewritten when a slot is reused, so they are read
    // through L2 (never from a possibly stale L1 line).
    auto read_slot = [&](uint32_t s) {
        SlotInfo I;
        const uint4 *src = reinterpret_cast<const uint4 *>(A.slots + s);
        uint4 *dst = reinterpret_cast<uint4 *>(&I);
        dst[0] = __ldcg(src);
        dst[1] = __ldcg(src + 1);
        return I;
    };

    auto set_slot = [&](uint32_t s) {
        const SlotInfo I = read_slot(s);  // written before the range was published
        slot = s;
        kind = I.kind;
        weight = I.weight;
        my_seq = I.seq;
        last = I.last;
        S.base = I.base;
        if (kind == 0) srules = sym_rules(smem + (I.n - 6) * kSymTables);
        else lrules = LunnonRules{A.tables + I.table_off, I.n, I.dim};
    };

    // Count a finished unit or split item into its request; the lane that
    // finishes a request's last piece publishes the result.
    auto finish = [&]() {
        if (leaves) atomicAdd(A.sum + slot, leaves * weight * mult);
        atomicAdd(A.nodes + slot, nodes - unit_nodes0);
        leaves = 0;
        __threadfence();
        const long long before = atomicAdd(reinterpret_cast<unsigned long long *>(A.pending + slot),
                                           (unsigned long long)(-1LL));
        if (before == 1) {
            __threadfence();
            DoneRec *d = A.done + slot;
            d->sum = atomicAdd(A.sum + slot, 0ULL);
            d->nodes = atomicAdd(A.nodes + slot, 0ULL);
            __threadfence_system();
            d->seq = read_slot(slot).seq;
            __threadfence_system();
        }
    };

    auto evaluate = [&]() -> uint64_t {
        return kind == 0 ? srules.gaps(L, eval, nodes) : lrules.gaps(L, eval, nodes);
    };

    for (;;) {
        // Refill idle lanes: units of the oldest published range first (a
        // small request, or a large one admitted because lanes were idle),
        // then split items, which come oldest request first while newer
        // requests share the GPU.
        const unsigned need = __ballot_sync(kFull, !busy);
        if (need) {
            unsigned long long first = 0;
            int got = 0;
            if (lane == __ffs(need) - 1) {
                const int want = __popc(need);
                unsigned long long h = vload(&A.ctl->head);
                for (int tries = 0; tries < 8; ++tries) {
                    if (h >= vload(&A.ctl->published)) break;
                    ServeRange *R = A.ranges + (h & (A.range_cap - 1));
                    const unsigned long long count = __ldcg(&R->count);
                    const unsigned long long t = atomicAdd(&R->taken, (unsigned long long)want);
                    if (t + want >= count) atomicCAS(&A.ctl->head, h, h + 1);
                    if (t < count) {
                        first = __ldcg(&R->first) + t;
                        got = int(count - t < (unsigned long long)want ? count - t : want);
                        break;
                    }
                    h = vload(&A.ctl->head);
                }
            }
            const int leader = __ffs(need) - 1;
            first = __shfl_sync(kFull, first, leader);
            got = __shfl_sync(kFull, got, leader);
            const int rank = __popc(need & lt_mask);
            if (!busy && rank < got) {
                const ServeUnit *u = A.units + ((first + rank) & (A.unit_cap - 1));
                uint32_t w[24];
                const uint4 *src = reinterpret_cast<const uint4 *>(u);
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const uint4 x = __ldcg(src + q);
                    w[4 * q] = x.x;
                    w[4 * q + 1] = x.y;
                    w[4 * q + 2] = x.z;
                    w[4 * q + 3] = x.w;
                }
#pragma unroll
                for (int k = 0; k < 17; ++k) L.set_word(k, w[k]);
                set_slot(w[17]);
                mult = uint64_t(w[18]) | (uint64_t(w[19]) << 32);
                root = int(w[20]);
                unit_nodes0 = nodes;
                const int placed = kind == 0 ? root : (root < lrules.n + 1 ? root : lrules.n + 1);
                if (!list_valid(L, placed)) {
                    atomicExch(&A.ctl->error, kErrMalformed);
                    finish();
                } else if (root > last) {
                    leaves = 1;
                    finish();
                } else {
                    busy = true;
                    fresh = true;
                    lvl = root;
                    eval = root;
                }
            }
        }
        if (ring_hint && __any_sync(kFull, !busy)) {
            const unsigned rest = __ballot_sync(kFull, !busy);
            unsigned long long f2 = 0;
            const int g2 = ring_claim(A.Q, &A.Q.hdr->spawn_head, __popc(rest), true, f2);
            const int r2 = __popc(rest & lt_mask);
            if (((rest >> lane) & 1u) && r2 < g2) {
                uint32_t w[24];
                ring_take(A.Q, f2 + r2, w);
#pragma unroll
                for (int k = 0; k < 17; ++k) L.set_word(k, w[k]);
                set_slot(w[17]);
                mult = uint64_t(w[22]) | (uint64_t(w[23]) << 32);
                root = int(w[20]);
                unit_nodes0 = nodes;
                lvl = root;
                S.set(root, uint64_t(w[18]) | (uint64_t(w[19]) << 32));
                eval = advance(L, S, lvl, root);
                fresh = false;
                busy = eval >= 0;
                if (!busy) finish();
            }
            if (g2 < __popc(rest)) ring_hint = false;
        }
        const bool bookkeeping = ++round >= A.period;
        if (!__any_sync(kFull, busy)) {
            int stop = 0;
            if (lane == 0) {
                if (reported_idle != 32) {
                    atomicAdd(reinterpret_cast<unsigned long long *>(&A.ctl->idle_lanes),
                              (unsigned long long)(long long)(32 - reported_idle));
                    reported_idle = 32;
                }
                const bool work = vload(&A.ctl->head) < vload(&A.ctl->published) ||
                                  vload(&A.Q.hdr->spawn_tail) != vload(&A.Q.hdr->spawn_head);
                stop = !work && (*reinterpret_cast<volatile unsigned int *>(&A.ctl->stop) != 0u ||
                                 ++idle_rounds > A.wait_limit);
                if (work) {
                    idle_rounds = 0;
                    // Work is pending but this idle warp got none of it this
                    // round.  A published unit or split item is claimable at
                    // once, so wait_limit such rounds in a row mean an item
                    // that is never published: report it and leave.
                    if (++stuck_rounds > A.wait_limit) {
                        atomicCAS(&A.ctl->error, 0u, kErrWaitLimit);
                        stop = 1;
                    }
                }
            }
            stop = __shfl_sync(kFull, stop, 0);
            if (stop) break;
            ring_hint = true;
            __nanosleep(nap);
            if (nap < 8192) nap <<= 1;
            continue;
        }
        nap = 256;
        stuck_rounds = 0;
        if (busy) {
            const uint64_t g = evaluate();
            eval = apply_advance(L, S, lvl, eval, root, last, fresh, g, leaves);
            fresh = false;
            if (eval < 0) {
                finish();
                busy = false;
            }
        }
        if (!bookkeeping) continue;
        round = 0;
        const unsigned idle_mask = __ballot_sync(kFull, !busy);
        long long want = 0, queued = 0;
        unsigned oldest = 0;
        if (lane == 0) {
            const int idle_now = __popc(idle_mask);
            if (idle_now != reported_idle) {
                atomicAdd(reinterpret_cast<unsigned long long *>(&A.ctl->idle_lanes),
                          (unsigned long long)(long long)(idle_now - reported_idle));
                reported_idle = idle_now;
            }
            queued = (long long)(vload(&A.Q.hdr->spawn_tail) - vload(&A.Q.hdr->spawn_head));
            const bool ranges_left = vload(&A.ctl->head) < vload(&A.ctl->published);
            if (!ranges_left)
                want = *reinterpret_cast<volatile long long *>(&A.ctl->idle_lanes) - queued;
            if (queued < kServeStock)
                oldest = *reinterpret_cast<volatile unsigned int *>(&A.ctl->oldest_seq);
        }
        want = __shfl_sync(kFull, want, 0);
        oldest = __shfl_sync(kFull, oldest, 0);
        ring_hint = __shfl_sync(kFull, queued, 0) > 0;
        if (want > 0 || oldest != 0) {
            // Donate, as the batched kernels do, carrying slot and multiplier:
            // every lane when lanes are idle, else the oldest request's lanes
            // to keep its stock of split items.
            int s = root;
            const uint64_t m = busy && !fresh ? shallowest_siblings(S, root, lvl, s) : 0;
            const bool can = busy && !fresh && m != 0 && last - s >= kMinSplitHeight &&
                             (want > 0 || my_seq == oldest);
            const unsigned donors = __ballot_sync(kFull, can);
            if (donors) {
                unsigned long long first = 0;
                const int got = ring_claim(A.Q, &A.Q.hdr->spawn_tail, __popc(donors), false, first);
                const int rank = __popc(donors & lt_mask);
                if (can && rank < got) {
                    roll_back(L, S, s, lvl);
                    uint32_t w[24];
#pragma unroll
                    for (int k = 0; k < 24; ++k) w[k] = 0;
#pragma unroll
                    for (int k = 0; k < 17; ++k) w[k] = L.word(k);
                    w[17] = slot;
                    w[18] = uint32_t(m);
                    w[19] = uint32_t(m >> 32);
                    w[20] = uint32_t(s);
                    w[22] = uint32_t(mult);
                    w[23] = uint32_t(mult >> 32);
                    replay_keeping_pick(L, S, s, lvl);
                    atomicAdd(reinterpret_cast<unsigned long long *>(A.pending + slot), 1ULL);
                    ring_put(A.Q, first + rank, w);
                }
            }
        }
    }
    if (lane == 0 && reported_idle)
        atomicAdd(reinterpret_cast<unsigned long long *>(&A.ctl->idle_lanes),
                  (unsigned long long)(-(long long)reported_idle));
}


__global__ void serve_ring_init(unsigned long long *seq, unsigned long long capacity) {
    for (unsigned long long k = blockIdx.x * blockDim.x + threadIdx.x; k < capacity;
         k += gridDim.x * blockDim.x)
        seq[k] = k;
}

constexpr int kServeTPB = 128;
constexpr double kBigHoldS = 0.05;
constexpr int kServeLevels = 32;

double mono() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

uint64_t pow2_at_least(uint64_t v, uint64_t lo) {
    uint64_t p = lo;
    while (p < v) p <<= 1;
    return p;
}

struct Request {
    uint64_t id = 0;
    SlotInfo info{};
    std::vector<ServeUnit> units;
    std::vector<uint8_t> table;    // Lunnon neighbour table
    unsigned __int128 factor = 1;  // answer = sum * factor
    double t_submit = 0, t_admit = 0, t_done = 0;
    unsigned long long sum = 0, nodes = 0;
    uint64_t unit_count = 0;
    int state = 0;  // 0 waiting, 1 running, 2 done
    int slot = -1;
    uint64_t arena_off = 0;
};

}  // namespace
}  // namespace mf

using namespace mf;

struct mf_server {
    mf_server_config cfg{};
    int device = 0;
    int sms = 0;
    int blocks_per_sm = 0;
    size_t smem = 0;
    uint64_t range_cap = 0;
    cudaStream_t kstream = nullptr, cstream = nullptr;
    ServeCtl *d_ctl = nullptr;
    ServeRange *d_ranges = nullptr;
    ServeUnit *d_units = nullptr;
    SlotInfo *d_slots = nullptr;
    long long *d_pending = nullptr;
    unsigned long long *d_sum = nullptr, *d_nodes = nullptr;
    uint8_t *d_tables = nullptr, *d_edges = nullptr;
    void *d_ring = nullptr;
    Queue Q{};
    DoneRec *h_done = nullptr, *d_done = nullptr;
    ServeUnit *h_stage = nullptr;
    uint64_t stage_cap = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::thread pump;
    bool quit = false;
    bool kernel_live = false;
    std::deque<std::shared_ptr<Request>> waiting;
    std::vector<std::shared_ptr<Request>> slot_req;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> by_id;
    std::vector<std::pair<uint64_t, uint64_t>> free_units;  // sorted [off, len)
    uint64_t next_id = 1;
    uint32_t next_seq = 1;
    uint32_t oldest_written = 0;
    uint64_t published = 0;
    uint64_t table_cursor = 0;
    int running = 0;
    int running_big = 0;        // running requests with more than small_units units
    uint64_t small_units = 0;   // a quarter of the resident lanes
    uint64_t lanes = 0;         // resident lanes of the server kernel
    long long *h_idle = nullptr;  // pinned copy of the kernel's idle-lane count
    double idle_checked = 0;
    double big_admitted = 0;      // when the last large request was admitted
    bool idle_seen = false;
    std::string failure;
    std::unordered_map<uint64_t, std::shared_ptr<SymPlan>> plans;
};

namespace {

bool alloc_units(mf_server *s, uint64_t need, uint64_t &off) {
    for (size_t k = 0; k < s->free_units.size(); ++k) {
        auto &f = s->free_units[k];
        if (f.second >= need) {
            off = f.first;
            f.first += need;
            f.second -= need;
            if (f.second == 0) s->free_units.erase(s->free_units.begin() + long(k));
            return true;
        }
    }
    return false;
}

void free_units(mf_server *s, uint64_t off, uint64_t len) {
    auto &v = s->free_units;
    auto it = std::lower_bound(v.begin(), v.end(), std::make_pair(off, uint64_t(0)));
    it = v.insert(it, {off, len});
    // merge with neighbours
    size_t k = size_t(it - v.begin());
    if (k + 1 < v.size() && v[k].first + v[k].second == v[k + 1].first) {
        v[k].second += v[k + 1].second;
        v.erase(v.begin() + long(k) + 1);
    }
    if (k > 0 && v[k - 1].first + v[k - 1].second == v[k].first) {
        v[k - 1].second += v[k].second;
        v.erase(v.begin() + long(k));
    }
}

cudaError_t launch_server_kernel(mf_server *s) {
    ServeArgs A;
    A.ctl = s->d_ctl;
    A.ranges = s->d_ranges;
    A.range_cap = s->range_cap;
    A.units = s->d_units;
    A.unit_cap = s->cfg.unit_capacity;
    A.slots = s->d_slots;
    A.pending = s->d_pending;
    A.sum = s->d_sum;
    A.nodes = s->d_nodes;
    A.done = s->d_done;
    A.tables = s->d_tables;
    A.edges = s->d_edges;
    A.Q = s->Q;
    A.period = s->cfg.node_budget;
    A.wait_limit = 1u << 20;
    serve_kernel<kServeTPB, kServeLevels>
        <<<unsigned(s->sms * s->blocks_per_sm), kServeTPB, s->smem, s->kstream>>>(A);
    return cudaGetLastError();
}

// Admit a request: copy its units and table in, fill its slot, publish its
// range.  Called with the lock held; returns false if it does not fit now.
bool admit(mf_server *s, const std::shared_ptr<Request> &r) {
    int slot = -1;
    for (size_t k = 0; k < s->slot_req.size(); ++k)
        if (!s->slot_req[k]) {
            slot = int(k);
            break;
        }
    if (slot < 0) return false;
    const uint64_t n = r->units.size();
    uint64_t off = 0;
    if (!alloc_units(s, n, off)) return false;
    uint64_t table_off = 0;
    if (r->info.kind == 1) {
        // Whole 256-byte blocks: no cache line ever holds bytes of two
        // tables, so a line cached for an older table cannot be stale for
        // a newer one.
        const uint64_t tb = (r->table.size() + 255) / 256 * 256;
        if (s->table_cursor + tb > s->cfg.table_bytes) {
            free_units(s, off, n);
            return false;  // the table arena is append-only while the kernel runs
        }
        table_off = s->table_cursor;
        s->table_cursor += tb;
    }
    // Units go through the fixed pinned staging buffer in pieces (freeing or
    // growing pinned memory would wait for the resident kernel).
    cudaStream_t c = s->cstream;
    bool ok = true;
    for (uint64_t k0 = 0; ok && k0 < n; k0 += s->stage_cap) {
        const uint64_t m = std::min<uint64_t>(s->stage_cap, n - k0);
        for (uint64_t k = 0; k < m; ++k) {
            s->h_stage[k] = r->units[k0 + k];
            s->h_stage[k].slot = uint32_t(slot);
        }
        ok = cudaMemcpyAsync(s->d_units + off + k0, s->h_stage, m * sizeof(ServeUnit),
                             cudaMemcpyHostToDevice, c) == cudaSuccess &&
             cudaStreamSynchronize(c) == cudaSuccess;
    }
    r->info.seq = s->next_seq++;
    r->info.table_off = uint32_t(table_off);
    ServeRange range{};
    range.first = off;
    range.count = n;
    range.taken = 0;
    range.slot = uint32_t(slot);
    const long long pend = (long long)n;
    const unsigned long long zero = 0;
    const uint64_t pub = s->published + 1;
    if (r->info.kind == 1)
        ok = ok && cudaMemcpyAsync(s->d_tables + table_off, r->table.data(), r->table.size(),
                                   cudaMemcpyHostToDevice, c) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(s->d_slots + slot, &r->info, sizeof(SlotInfo), cudaMemcpyHostToDevice, c) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(s->d_pending + slot, &pend, sizeof(pend), cudaMemcpyHostToDevice, c) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(s->d_sum + slot, &zero, sizeof(zero), cudaMemcpyHostToDevice, c) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(s->d_nodes + slot, &zero, sizeof(zero), cudaMemcpyHostToDevice, c) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(s->d_ranges + (s->published & (s->range_cap - 1)), &range,
                               sizeof(range), cudaMemcpyHostToDevice, c) == cudaSuccess;
    // The counter goes last: once the kernel sees it, everything above is in place.
    ok = ok && cudaMemcpyAsync(&s->d_ctl->published, &pub, sizeof(pub), cudaMemcpyHostToDevice, c) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(c) == cudaSuccess;
    if (!ok) {
        s->failure = "copying a request to the device failed";
        return false;
    }
    s->published = pub;
    r->slot = slot;
    r->arena_off = off;
    r->state = 1;
    r->t_admit = mono();
    s->slot_req[size_t(slot)] = r;
    ++s->running;
    if (r->unit_count > s->small_units) ++s->running_big;
    return true;
}

// Tell the kernel which request is the oldest while two or more share the
// GPU (0 otherwise); its lanes then keep split items in stock.
void publish_oldest(mf_server *s) {
    uint32_t oldest = 0;
    if (s->running >= 2)
        for (const auto &r : s->slot_req)
            if (r && (oldest == 0 || r->info.seq < oldest)) oldest = r->info.seq;
    if (oldest == s->oldest_written) return;
    if (cudaMemcpyAsync(&s->d_ctl->oldest_seq, &oldest, sizeof(oldest), cudaMemcpyHostToDevice,
                        s->cstream) != cudaSuccess ||
        cudaStreamSynchronize(s->cstream) != cudaSuccess) {
        s->failure = "publishing the oldest request failed";
        return;
    }
    s->oldest_written = oldest;
}

// True once at least 1/8 of the resident lanes are idle (sampled at most
// every 0.5 ms): the running requests no longer fill the GPU.
bool lanes_idle(mf_server *s) {
    const double now = mono();
    if (now - s->idle_checked < 5e-4) return s->idle_seen;
    s->idle_checked = now;
    if (cudaMemcpyAsync(s->h_idle, &s->d_ctl->idle_lanes, sizeof(long long),
                        cudaMemcpyDeviceToHost, s->cstream) != cudaSuccess ||
        cudaStreamSynchronize(s->cstream) != cudaSuccess) {
        s->failure = "reading the idle-lane count failed";
        return false;
    }
    s->idle_seen = *s->h_idle >= (long long)(s->lanes / 8);
    return s->idle_seen;
}

void pump_loop(mf_server *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lock(s->mu);
    while (!s->quit || s->running > 0 || !s->waiting.empty()) {
        if (s->quit && !s->failure.empty()) break;  // nothing more can complete
        // Completions: a lane wrote the result and then the sequence number.
        for (size_t k = 0; k < s->slot_req.size(); ++k) {
            auto &r = s->slot_req[k];
            if (!r) continue;
            const DoneRec &d = s->h_done[k];
            if (d.seq != r->info.seq) continue;
            std::atomic_thread_fence(std::memory_order_acquire);
            r->sum = d.sum;
            r->nodes = d.nodes;
            r->t_done = mono();
            r->state = 2;
            free_units(s, r->arena_off, r->units.size());
            r->units.clear();
            r->units.shrink_to_fit();
            if (r->unit_count > s->small_units) --s->running_big;
            --s->running;
            r.reset();
            s->cv.notify_all();
        }
        // Admissions. Large requests go first come first served, and the next
        // one only once the running large requests leave lanes idle (work-
        // conserving FIFO: a large request gets the whole GPU instead of
        // sharing it and stretching everybody's latency). Small requests
        // (whole small maps) are admitted at once.
        bool big_blocked = false;
        for (auto it = s->waiting.begin(); it != s->waiting.end();) {
            const std::shared_ptr<Request> r = *it;
            const bool big = r->unit_count > s->small_units;
            // After a large admission the idle count needs a moment (its
            // units being claimed) before it means anything again.
            if (big && (big_blocked ||
                        (s->running_big > 0 &&
                         (mono() - s->big_admitted < kBigHoldS || !lanes_idle(s))))) {
                big_blocked = true;
                ++it;
                continue;
            }
            if (!admit(s, r)) break;  // no slot or memory: keep the order
            it = s->waiting.erase(it);
            if (big) {
                s->big_admitted = mono();
                s->idle_checked = 0;  // sample afresh before the next one
            }
        }
        publish_oldest(s);
        // Keep the kernel alive while work is resident.
        if (s->running > 0) {
            if (s->kernel_live && cudaStreamQuery(s->kstream) == cudaSuccess) {
                s->kernel_live = false;
                // A kernel that left with requests still running either ran
                // out of work to wait for (relaunch it) or reported an error.
                unsigned int err = 0;
                if (cudaMemcpy(&err, &s->d_ctl->error, sizeof(err), cudaMemcpyDeviceToHost) != cudaSuccess)
                    s->failure = "reading the server kernel's error word failed";
                else if (err == kErrWaitLimit)
                    s->failure = "the server kernel gave up waiting for a split item that was never published";
                else if (err)
                    s->failure = "the server kernel saw a malformed unit";
            }
            if (!s->kernel_live && s->failure.empty()) {
                const unsigned int zero = 0;
                cudaMemcpy(&s->d_ctl->stop, &zero, sizeof(zero), cudaMemcpyHostToDevice);
                if (launch_server_kernel(s) == cudaSuccess) s->kernel_live = true;
                else s->failure = "launching the server kernel failed";
            }
        }
        if (!s->waiting.empty() && s->running == 0 && s->table_cursor > 0) {
            // Nothing is resident but the head request still does not fit:
            // its Lunnon table needs the append-only table arena restarted,
            // which is only safe once no kernel can hold stale cached tables.
            if (s->kernel_live) {
                const unsigned int one = 1;
                cudaMemcpy(&s->d_ctl->stop, &one, sizeof(one), cudaMemcpyHostToDevice);
                lock.unlock();
                cudaStreamSynchronize(s->kstream);
                lock.lock();
                s->kernel_live = false;
            }
            s->table_cursor = 0;
            continue;
        }
        s->cv.wait_for(lock, std::chrono::microseconds(50));
    }
}

int make_server(const mf_server_config *cfg, mf_server **out) {
    auto s = std::make_unique<mf_server>();
    mf_server_config c{};
    if (cfg) c = *cfg;
    c.unit_capacity = pow2_at_least(c.unit_capacity ? c.unit_capacity : (1ULL << 21), 1024);
    if (!c.max_requests) c.max_requests = 1024;
    if (!c.block_threads) c.block_threads = kServeTPB;
    if (!c.table_bytes) c.table_bytes = 64ULL << 20;
    if (!c.node_budget) c.node_budget = 64;
    c.queue_capacity = pow2_at_least(c.queue_capacity ? c.queue_capacity : (1ULL << 16), 16);
    s->cfg = c;
    s->range_cap = pow2_at_least(2ULL * c.max_requests, 4096);
    MF_TRY_CUDA(cudaGetDevice(&s->device));
    s->sms = device_sm_count();
    MF_TRY_CUDA(cudaStreamCreateWithFlags(&s->kstream, cudaStreamNonBlocking));
    MF_TRY_CUDA(cudaStreamCreateWithFlags(&s->cstream, cudaStreamNonBlocking));
    MF_TRY_CUDA(cudaMalloc(&s->d_ctl, sizeof(ServeCtl)));
    MF_TRY_CUDA(cudaMemset(s->d_ctl, 0, sizeof(ServeCtl)));
    MF_TRY_CUDA(cudaMalloc(&s->d_ranges, s->range_cap * sizeof(ServeRange)));
    MF_TRY_CUDA(cudaMemset(s->d_ranges, 0, s->range_cap * sizeof(ServeRange)));
    MF_TRY_CUDA(cudaMalloc(&s->d_units, c.unit_capacity * sizeof(ServeUnit)));
    MF_TRY_CUDA(cudaMalloc(&s->d_slots, c.max_requests * sizeof(SlotInfo)));
    MF_TRY_CUDA(cudaMalloc(&s->d_pending, c.max_requests * sizeof(long long)));
    MF_TRY_CUDA(cudaMalloc(&s->d_sum, c.max_requests * sizeof(unsigned long long)));
    MF_TRY_CUDA(cudaMalloc(&s->d_nodes, c.max_requests * sizeof(unsigned long long)));
    MF_TRY_CUDA(cudaMalloc(&s->d_tables, c.table_bytes));
    MF_TRY_CUDA(cudaMalloc(&s->d_edges, 3 * 4 * kSymCells));
    uint8_t edges[3][4 * kSymCells];
    for (int b = 0; b < 3; ++b) sym_edges(6 + b, edges[b]);
    MF_TRY_CUDA(cudaMemcpy(s->d_edges, edges, sizeof(edges), cudaMemcpyHostToDevice));
    const uint64_t ring_bytes = 256 + c.queue_capacity * (sizeof(TaskRecord) + 8);
    MF_TRY_CUDA(cudaMalloc(&s->d_ring, ring_bytes));
    MF_TRY_CUDA(cudaMemset(s->d_ring, 0, 256));
    s->Q.hdr = static_cast<QueueHeader *>(s->d_ring);
    s->Q.slots = reinterpret_cast<TaskRecord *>(static_cast<uint8_t *>(s->d_ring) + 256);
    s->Q.seq = reinterpret_cast<unsigned long long *>(static_cast<uint8_t *>(s->d_ring) + 256 +
                                                      c.queue_capacity * sizeof(TaskRecord));
    s->Q.capacity = c.queue_capacity;
    serve_ring_init<<<64, 256>>>(s->Q.seq, s->Q.capacity);
    MF_TRY_CUDA(cudaGetLastError());
    MF_TRY_CUDA(cudaHostAlloc(&s->h_done, c.max_requests * sizeof(DoneRec), cudaHostAllocMapped));
    s->stage_cap = std::min<uint64_t>(c.unit_capacity, 1ULL << 16);
    MF_TRY_CUDA(cudaMallocHost(&s->h_idle, sizeof(long long)));
    MF_TRY_CUDA(cudaMallocHost(&s->h_stage, s->stage_cap * sizeof(ServeUnit)));
    std::memset(static_cast<void *>(s->h_done), 0, c.max_requests * sizeof(DoneRec));
    MF_TRY_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&s->d_done), s->h_done, 0));
    s->smem = 3 * kSymTables + Carve<kServeTPB, 17, kServeLevels>::kThreadBytes;
    int optin = 0;
    MF_TRY_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
    MF_TRY_CUDA(cudaFuncSetAttribute(serve_kernel<kServeTPB, kServeLevels>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    MF_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &s->blocks_per_sm, serve_kernel<kServeTPB, kServeLevels>, kServeTPB, s->smem));
    if (s->blocks_per_sm < 1) {
        set_error("the server kernel does not fit on an SM");
        return MF_ERR_CUDA;
    }
    s->lanes = uint64_t(s->sms) * uint64_t(s->blocks_per_sm) * kServeTPB;
    s->small_units = s->lanes / 4;
    MF_TRY_CUDA(cudaDeviceSynchronize());
    s->slot_req.assign(c.max_requests, nullptr);
    s->free_units.push_back({0, c.unit_capacity});
    mf_server *raw = s.get();
    s->pump = std::thread(pump_loop, raw);
    *out = s.release();
    return MF_OK;
}

int submit(mf_server *s, std::shared_ptr<Request> r, uint64_t *id) {
    if (r->units.size() > s->cfg.unit_capacity) {
        set_error("request needs %zu units; the arena holds %llu", r->units.size(),
                  (unsigned long long)s->cfg.unit_capacity);
        return MF_ERR_CAPACITY;
    }
    if (r->table.size() > s->cfg.table_bytes) {
        set_error("request's table does not fit the table arena");
        return MF_ERR_CAPACITY;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    r->id = s->next_id++;
    r->t_submit = mono();
    r->unit_count = r->units.size();
    if (r->units.empty()) {
        r->state = 2;
        r->t_admit = r->t_done = r->t_submit;
    } else {
        s->waiting.push_back(r);
    }
    s->by_id[r->id] = r;
    *id = r->id;
    s->cv.notify_all();
    return MF_OK;
}

}  // namespace

extern "C" {

int32_t mf_server_create(const mf_server_config *cfg, mf_server **out) {
    clear_error();
    if (!out) {
        set_error("out is NULL");
        return MF_ERR_ARG;
    }
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        set_error("no CUDA device");
        return MF_ERR_NO_DEVICE;
    }
    return make_server(cfg, out);
}

int32_t mf_server_submit_sym(mf_server *s, int32_t n, int32_t expanded_n, uint64_t start_case,
                             uint64_t max_cases, uint64_t *request_id) {
    clear_error();
    if (!s || !request_id) {
        set_error("server and request_id are required");
        return MF_ERR_ARG;
    }
    if (n < 6 || n > 8) {
        set_error("the server counts sym chunks of 6x6 .. 8x8 maps");
        return MF_ERR_ARG;
    }
    const uint64_t key = uint64_t(n) * 1000 + uint64_t(expanded_n < 0 ? 0 : expanded_n);
    std::shared_ptr<SymPlan> plan;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        auto it = s->plans.find(key);
        if (it != s->plans.end()) plan = it->second;
    }
    if (!plan) {
        // Building a deep expansion index runs a count kernel, which needs
        // SMs: let the (then idle) server kernel leave first.
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait(lock, [&] { return s->running == 0 && s->waiting.empty(); });
            if (s->kernel_live) {
                const unsigned int one = 1;
                cudaMemcpy(&s->d_ctl->stop, &one, sizeof(one), cudaMemcpyHostToDevice);
                cudaStreamSynchronize(s->kstream);
                s->kernel_live = false;
            }
        }
        auto p = std::make_shared<SymPlan>();
        int rc = build_full_sym_plan(n, expanded_n, *p);
        if (rc) return rc;
        std::lock_guard<std::mutex> lock(s->mu);
        s->plans[key] = p;
        plan = p;
    }
    const int levels = n * n - 1 - plan->start_i;
    if (levels > kServeLevels) {
        set_error("the server searches at most %d levels below a case; expand to at least %d cells",
                  kServeLevels, n * n - 1 - kServeLevels);
        return MF_ERR_ARG;
    }
    auto r = std::make_shared<Request>();
    uint64_t avail = plan->total_cases > start_case ? plan->total_cases - start_case : 0;
    if (max_cases && max_cases < avail) avail = max_cases;
    std::vector<uint8_t> cycles(std::max<uint64_t>(avail, 1) * kSymCells);
    std::vector<uint64_t> mults(std::max<uint64_t>(avail, 1));
    const uint64_t got = sym_select_cases(*plan, start_case, avail, cycles.data(), mults.data(), avail);
    r->units.resize(got);
    for (uint64_t k = 0; k < got; ++k) {
        ServeUnit &u = r->units[k];
        std::memset(&u, 0, sizeof(u));
        std::memcpy(u.words, &cycles[k * kSymCells], kSymCells);
        u.mult = mults[k];
        u.root = uint32_t(plan->start_i);
    }
    r->info.kind = 0;
    r->info.n = n;
    r->info.base = plan->start_i;
    r->info.last = n * n - 1;
    r->info.weight = 1;
    r->factor = (unsigned __int128)(n * n);
    return submit(s, r, request_id);
}

int32_t mf_server_submit_lunnon(mf_server *s, const int32_t *dims, int32_t ndim, int32_t depth,
                                uint64_t *request_id) {
    clear_error();
    if (!s || !request_id) {
        set_error("server and request_id are required");
        return MF_ERR_ARG;
    }
    LunnonTables t;
    std::string why;
    if (!build_lunnon_tables(dims, ndim, t, why)) {
        set_error("%s", why.c_str());
        return MF_ERR_ARG;
    }
    if (depth < 0) depth = default_lunnon_depth(t);
    if (depth > t.n) depth = t.n;
    if (t.n - (depth + 1) > kServeLevels) {
        set_error("the server searches at most %d levels below a prefix state", kServeLevels);
        return MF_ERR_ARG;
    }
    const uint32_t stride = lunnon_state_stride(t.n);
    const uint64_t total = collect_lunnon_states(t, depth, nullptr, 0, stride);
    std::vector<uint8_t> states(std::max<uint64_t>(total, 1) * stride);
    collect_lunnon_states(t, depth, states.data(), total, stride);
    auto r = std::make_shared<Request>();
    r->units.resize(total);
    for (uint64_t k = 0; k < total; ++k) {
        ServeUnit &u = r->units[k];
        std::memset(&u, 0, sizeof(u));
        std::memcpy(u.words, &states[k * stride], size_t(t.n) + 1);
        u.mult = 1;
        u.root = uint32_t(depth + 1);
    }
    r->table.assign(t.next.begin(), t.next.end());
    r->table.resize((r->table.size() + 15) / 16 * 16, 0);
    r->info.kind = 1;
    r->info.n = t.n;
    r->info.dim = t.dim;
    r->info.base = depth + 1;
    r->info.last = t.n;
    r->info.weight = uint32_t(t.n);
    r->factor = 1;
    return submit(s, r, request_id);
}

static void fill_answer(const Request &r, uint64_t *ans, mf_request_info *info) {
    const unsigned __int128 a = (unsigned __int128)r.sum * r.factor;
    if (ans) {
        ans[0] = uint64_t(a);
        ans[1] = uint64_t(a >> 64);
    }
    if (info) {
        info->submit_s = r.t_submit;
        info->admit_s = r.t_admit;
        info->done_s = r.t_done;
        info->units = r.unit_count;
        info->nodes = r.nodes;
    }
}

int32_t mf_server_poll(mf_server *s, uint64_t id, int32_t *done, uint64_t *answer_lo_hi,
                       mf_request_info *info) {
    clear_error();
    if (!s || !done) {
        set_error("server and done are required");
        return MF_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->by_id.find(id);
    if (it == s->by_id.end()) {
        set_error("unknown request %llu", (unsigned long long)id);
        return MF_ERR_ARG;
    }
    if (!s->failure.empty()) {
        set_error("%s", s->failure.c_str());
        return MF_ERR_CUDA;
    }
    *done = it->second->state == 2;
    if (*done) fill_answer(*it->second, answer_lo_hi, info);
    return MF_OK;
}

int32_t mf_server_wait(mf_server *s, uint64_t id, double timeout_s, uint64_t *answer_lo_hi,
                       mf_request_info *info) {
    clear_error();
    if (!s) {
        set_error("server is required");
        return MF_ERR_ARG;
    }
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->by_id.find(id);
    if (it == s->by_id.end()) {
        set_error("unknown request %llu", (unsigned long long)id);
        return MF_ERR_ARG;
    }
    auto r = it->second;
    const auto deadline = std::chrono::steady_clock::now() +
                          std::chrono::microseconds(int64_t(timeout_s * 1e6));
    while (r->state != 2 && s->failure.empty()) {
        if (s->cv.wait_until(lock, deadline) == std::cv_status::timeout && r->state != 2) {
            set_error("request %llu still running after %.3f s", (unsigned long long)id, timeout_s);
            return MF_ERR_TIMEOUT;
        }
    }
    if (!s->failure.empty()) {
        set_error("%s", s->failure.c_str());
        return MF_ERR_CUDA;
    }
    fill_answer(*r, answer_lo_hi, info);
    return MF_OK;
}

void mf_server_destroy(mf_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->quit = true;
        s->cv.notify_all();
    }
    if (s->pump.joinable()) s->pump.join();
    const unsigned int one = 1;
    cudaMemcpy(&s->d_ctl->stop, &one, sizeof(one), cudaMemcpyHostToDevice);
    cudaStreamSynchronize(s->kstream);
    cudaFree(s->d_ctl);
    cudaFree(s->d_ranges);
    cudaFree(s->d_units);
    cudaFree(s->d_slots);
    cudaFree(s->d_pending);
    cudaFree(s->d_sum);
    cudaFree(s->d_nodes);
    cudaFree(s->d_tables);
    cudaFree(s->d_edges);
    cudaFree(s->d_ring);
    cudaFreeHost(s->h_done);
    if (s->h_stage) cudaFreeHost(s->h_stage);
    if (s->h_idle) cudaFreeHost(s->h_idle);
    cudaStreamDestroy(s->kstream);
    cudaStreamDestroy(s->cstream);
    delete s;
}

}  // extern "C"
