// wide_kernels.cu -- the sym_fold search on boards over 64 cells (9x9).
//
// experiments/9x9/sym_fold9.cpp runs sym_fold's recursion with 128-bit masks
// (sym_fold9.cpp:34, 261-312) so that cells past 63 can be counted.  This is
// the same search as the 64-bit batched kernel -- lockstep rounds, the
// unified page-start/step walk, a persistent grid fed by a warp-cooperative
// split ring -- with 128-bit position masks, 96-cell successor lists and
// 128-byte split records.  Cases arrive as the 64-byte records of the 64-bit
// path (the host expands them to at most 64 cells); the list bytes past the
// record start as zeros and are written by insertions before they are read.
#include <cuda_runtime.h>

#include <mutex>

#include "dfs_core.cuh"
#include "engine.hpp"

namespace mf {
namespace {

struct Mask128 {
    uint64_t lo, hi;
};

__device__ __forceinline__ bool w_zero(const Mask128 &m) { return (m.lo | m.hi) == 0; }
__device__ __forceinline__ int w_low(const Mask128 &m) {
    return m.lo ? __ffsll(static_cast<long long>(m.lo)) - 1
                : 63 + __ffsll(static_cast<long long>(m.hi));
}
__device__ __forceinline__ Mask128 w_drop_low(Mask128 m) {
    if (m.lo) m.lo &= m.lo - 1;
    else m.hi &= m.hi - 1;
    return m;
}
__device__ __forceinline__ int w_popc(const Mask128 &m) { return __popcll(m.lo) + __popcll(m.hi); }
__device__ __forceinline__ Mask128 w_low_bits(int k) {
    return Mask128{low_bits(k), k <= 64 ? 0ULL : low_bits(k - 64)};
}
__device__ __forceinline__ void w_set(Mask128 &m, int x) {
    const uint64_t b = 1ULL << (x & 63);
    m.lo |= x < 64 ? b : 0ULL;
    m.hi |= x < 64 ? 0ULL : b;
}

// Shared tables: 4 edge pages of kWideCells, then per cell the packed list of
// pages whose neighbour has a smaller number (9 bits each: page << 7 |
// neighbour) and its length.
constexpr size_t kWidePages = 4 * kWideCells;
constexpr size_t kWideTables = 1280;
static_assert(kWidePages + 8 * kWideCells + kWideCells <= kWideTables, "wide table layout");
constexpr int kWideWords = kWideCells / 4;  // list words per lane
constexpr int kWideRecordWords = 32;        // 128-byte split records
static_assert(kWideWords + 4 + 2 <= kWideRecordWords, "wide record layout");

template <int TPB>
__device__ __forceinline__ void stage_wide_tables(uint8_t *smem, const uint8_t *__restrict__ edges) {
    for (int k = threadIdx.x; k < int(kWidePages / 4); k += TPB)
        reinterpret_cast<uint32_t *>(smem)[k] = __ldg(reinterpret_cast<const uint32_t *>(edges) + k);
    for (int k = threadIdx.x; k < kWideCells; k += TPB) {
        uint64_t q = 0;
        int c = 0;
        for (int p = 0; p < 4; ++p) {
            const int nb = __ldg(edges + p * kWideCells + k);
            if (nb < k) q |= uint64_t(nb | (p << 7)) << (9 * c++);
        }
        reinterpret_cast<uint64_t *>(smem + kWidePages)[k] = q;
        smem[kWidePages + 8 * kWideCells + k] = uint8_t(c);
    }
}

// get_good with 128-bit masks (sym_fold9.cpp:286-312), in the two-chain form
// of SymRules::gaps: the (at most two) placed-neighbour pages of cell i are
// walked side by side, a chain that is back at its start retracing itself
// until the other is done.
struct SymRulesW {
    const uint8_t *edge;
    const uint64_t *pages;
    const uint8_t *count;
    template <int TPB>
    __device__ __forceinline__ Mask128 gaps(const List<TPB> &L, int i,
                                            unsigned long long &nodes) const {
        ++nodes;
        Mask128 good = w_low_bits(i);
        uint64_t q = pages[i];
        for (int left = count[i]; left > 0 && !w_zero(good); left -= 2, q >>= 18) {
            const uint64_t qb = left > 1 ? (q >> 9) : q;
            const int oA = int(q & 127), oB = int(qb & 127);
            const uint8_t *eA = edge + int((q >> 7) & 3) * kWideCells;
            const uint8_t *eB = edge + int((qb >> 7) & 3) * kWideCells;
            Mask128 aA{0, 0}, aB{0, 0};
            w_set(aA, oA);
            w_set(aB, oB);
            int jA = L.get(oA), jB = L.get(oB);
            bool dA = jA == oA, dB = jB == oB;
            while (!(dA && dB)) {
                const int pA = eA[jA];
                const int pB = eB[jB];
                const int xA = pA < i ? pA : jA;
                const int xB = pB < i ? pB : jB;
                w_set(aA, xA);
                w_set(aB, xB);
                jA = L.get(xA);
                jB = L.get(xB);
                dA |= jA == oA;
                dB |= jB == oB;
            }
            good.lo &= aA.lo & aB.lo;
            good.hi &= aA.hi & aB.hi;
        }
        return good;
    }
};

__device__ __forceinline__ SymRulesW wide_rules(const uint8_t *smem) {
    return SymRulesW{smem, reinterpret_cast<const uint64_t *>(smem + kWidePages),
                     smem + kWidePages + 8 * kWideCells};
}

// 128-bit mask stack.  The mask of level lvl holds positions below lvl, so
// its high word can be non-zero only for lvl > 64: low words get one row per
// level (level k at lo[k*TPB]), high words rows only for levels 65 ..
// 64 + kWideHiRows (after the low rows), and the other levels read zero.
// The chosen positions are interleaved bytes.
constexpr int kWideHiRows = 16;  // levels 65..80: enough below 82 cells

template <int TPB, int LEVELS>
struct StackW {
    uint64_t *lo;
    List<TPB> chosen;
    int base;
    __device__ __forceinline__ Mask128 get(int lvl) const {
        const uint64_t hi = lvl > 64 ? lo[(LEVELS + lvl - 65) * TPB] : 0ULL;
        return Mask128{lo[(lvl - base) * TPB], hi};
    }
    __device__ __forceinline__ void set(int lvl, const Mask128 &v) const {
        lo[(lvl - base) * TPB] = v.lo;
        if (lvl > 64) lo[(LEVELS + lvl - 65) * TPB] = v.hi;
    }
    __device__ __forceinline__ int pick(int lvl) const { return chosen.get(lvl - base); }
    __device__ __forceinline__ void set_pick(int lvl, int j) const { chosen.put(lvl - base, j); }
};

template <int TPB, int LEVELS>
struct CarveW {
    static constexpr size_t kList = size_t(kWideWords) * 4 * TPB;
    static constexpr size_t kMask = size_t(LEVELS + kWideHiRows) * 8 * TPB;
    static constexpr size_t kPick = size_t((LEVELS + 3) / 4) * 4 * TPB;
    static constexpr size_t kBytes = kWideTables + kList + kMask + kPick;
};

// advance of dfs_core.cuh with 128-bit masks (a taken split item starts here).
template <int TPB, int LEVELS>
__device__ __forceinline__ int advance_w(const List<TPB> &L, const StackW<TPB, LEVELS> &S, int &lvl,
                                         int root) {
    for (;;) {
        const Mask128 cur = S.get(lvl);
        if (w_zero(cur)) {
            if (lvl == root) return -1;
            --lvl;
            L.put(S.pick(lvl), L.get(lvl));  // detach item lvl
            continue;
        }
        const int j = w_low(cur);
        S.set(lvl, w_drop_low(cur));
        L.put(lvl, L.get(j));  // insert item lvl after j
        L.put(j, lvl);
        S.set_pick(lvl, j);
        return lvl + 1;
    }
}

// apply_advance of dfs_core.cuh with 128-bit masks: consume level eval's
// mask g (handed over in registers) and move to the next node; -1 when the
// unit's subtree is exhausted.
template <int TPB, int LEVELS>
__device__ __forceinline__ int apply_advance_w(const List<TPB> &L, const StackW<TPB, LEVELS> &S,
                                               int &lvl, int eval, int root, int last, bool fresh,
                                               const Mask128 &g, unsigned long long &leaves) {
    Mask128 cur;
    if (eval == last) {
        leaves += w_popc(g);
        if (fresh) return -1;
        L.put(S.pick(lvl), L.get(lvl));  // detach item lvl (= eval - 1)
        cur = S.get(lvl);
    } else {
        lvl = eval;
        cur = g;
    }
    for (;;) {
        if (w_zero(cur)) {
            if (lvl == root) return -1;
            --lvl;
            L.put(S.pick(lvl), L.get(lvl));  // detach item lvl
            cur = S.get(lvl);
            continue;
        }
        const int j = w_low(cur);
        S.set(lvl, w_drop_low(cur));
        L.put(lvl, L.get(j));  // insert item lvl after j
        L.put(j, lvl);
        S.set_pick(lvl, j);
        return lvl + 1;
    }
}

__device__ __forceinline__ void wide_take(const uint4 *slots, const Queue &Q, unsigned long long t,
                                          uint32_t (&w)[kWideRecordWords]) {
    const unsigned long long cell = t & (Q.capacity - 1);
    __threadfence();
    const uint4 *src = slots + cell * (kWideRecordWords / 4);
#pragma unroll
    for (int q = 0; q < kWideRecordWords / 4; ++q) {
        const uint4 x = __ldcg(src + q);
        w[4 * q] = x.x;
        w[4 * q + 1] = x.y;
        w[4 * q + 2] = x.z;
        w[4 * q + 3] = x.w;
    }
    __threadfence();
    atomicExch(Q.seq + cell, t + Q.capacity);
}

__device__ __forceinline__ void wide_put(uint4 *slots, const Queue &Q, unsigned long long t,
                                         const uint32_t (&w)[kWideRecordWords]) {
    const unsigned long long cell = t & (Q.capacity - 1);
    uint4 *dst = slots + cell * (kWideRecordWords / 4);
#pragma unroll
    for (int q = 0; q < kWideRecordWords / 4; ++q)
        __stcg(dst + q, make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]));
    __threadfence();
    atomicExch(Q.seq + cell, t + 1);
}

// The persistent loop of the 64-bit batched kernel (dfs_kernels.cu), for
// 128-bit masks: initial units by a warp-aggregated atomicAdd, lockstep
// rounds, bookkeeping every `period` rounds (idle-lane report, donation of
// the shallowest untried siblings while lanes wait), split items taken by
// idle lanes, and the same leaving rule.  Split record: list words
// 0..kWideWords-1, owner, untried mask (4 words), level.
template <int TPB, int LEVELS>
__global__ void __launch_bounds__(TPB)
    sym_wide_kernel(const uint8_t *__restrict__ edges, int start_i, int last,
                    const uint8_t *__restrict__ cycles, uint32_t record_bytes, unsigned long long num,
                    unsigned long long *counts, unsigned long long *nodes_out, Queue Q,
                    uint4 *slots, uint32_t period, uint32_t wait_limit) {
    extern __shared__ __align__(16) uint8_t smem[];
    stage_wide_tables<TPB>(smem, edges);
    __syncthreads();
    using C = CarveW<TPB, LEVELS>;
    const SymRulesW R = wide_rules(smem);
    const List<TPB> L{smem + kWideTables + 4 * threadIdx.x};
    StackW<TPB, LEVELS> S;
    S.lo = reinterpret_cast<uint64_t *>(smem + kWideTables + C::kList) + threadIdx.x;
    S.chosen = List<TPB>{smem + kWideTables + C::kList + C::kMask + 4 * threadIdx.x};
    S.base = start_i;

    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    constexpr int kOwner = kWideWords, kMaskW = kWideWords + 1, kRoot = kWideWords + 5;
    bool busy = false, fresh = false, init_left = true;
    int lvl = start_i, root = start_i, eval = start_i;
    uint32_t owner = 0;
    unsigned long long leaves = 0, nodes = 0, finished = 0, started = 0;
    uint32_t idle_rounds = 0, round = 0, nap = 256;
    int reported_idle = 0;
    bool ring_hint = false;

    auto flush = [&]() {
        if (leaves) atomicAdd(counts + owner, leaves);
        leaves = 0;
        ++finished;
    };

    auto take_splits = [&](unsigned need) -> bool {
        const int want = __popc(need);
        unsigned long long first = 0;
        const int got = ring_claim(Q, &Q.hdr->spawn_head, want, true, first);
        const int rank = __popc(need & lt_mask);
        if (((need >> lane) & 1u) && rank < got) {
            uint32_t w[kWideRecordWords];
            wide_take(slots, Q, first + rank, w);
            ++started;
#pragma unroll
            for (int k = 0; k < kWideWords; ++k) L.set_word(k, w[k]);
            owner = w[kOwner];
            root = int(w[kRoot]);
            lvl = root;
            S.set(root, Mask128{uint64_t(w[kMaskW]) | (uint64_t(w[kMaskW + 1]) << 32),
                                uint64_t(w[kMaskW + 2]) | (uint64_t(w[kMaskW + 3]) << 32)});
            eval = advance_w(L, S, lvl, root);  // an item's mask is never empty
            fresh = false;
            busy = eval >= 0;
            if (!busy) ++finished;
        }
        return got < want;
    };

    auto donate = [&]() {
        int s = root;
        Mask128 m{0, 0};
        if (busy && !fresh) {
            while (s < lvl && w_zero(S.get(s))) ++s;
            m = S.get(s);
        }
        const bool can = busy && !fresh && !w_zero(m) && last - s >= kMinSplitHeight;
        const unsigned donors = __ballot_sync(kFull, can);
        if (!donors) return;
        unsigned long long first = 0;
        const int got = ring_claim(Q, &Q.hdr->spawn_tail, __popc(donors), false, first);
        const int rank = __popc(donors & lt_mask);
        if (!can || rank >= got) return;
        for (int l = lvl; l >= s; --l) L.put(S.pick(l), L.get(l));
        uint32_t w[kWideRecordWords];
#pragma unroll
        for (int k = 0; k < kWideRecordWords; ++k) w[k] = 0;
#pragma unroll
        for (int k = 0; k < kWideWords; ++k) w[k] = L.word(k);
        w[kOwner] = owner;
        w[kMaskW] = uint32_t(m.lo);
        w[kMaskW + 1] = uint32_t(m.lo >> 32);
        w[kMaskW + 2] = uint32_t(m.hi);
        w[kMaskW + 3] = uint32_t(m.hi >> 32);
        w[kRoot] = uint32_t(s);
        for (int l = s; l <= lvl; ++l) {
            const int j = S.pick(l);
            L.put(l, L.get(j));
            L.put(j, l);
        }
        S.set(s, Mask128{0, 0});
        wide_put(slots, Q, first + rank, w);
    };

    for (;;) {
        // Initial units for lanes without work, one warp-aggregated claim.
        const unsigned want_init = __ballot_sync(kFull, !busy && init_left);
        if (want_init) {
            const int leader = __ffs(want_init) - 1;
            unsigned long long base = 0;
            if (lane == leader)
                base = atomicAdd(&Q.hdr->init_next, (unsigned long long)__popc(want_init));
            base = __shfl_sync(kFull, base, leader);
            if (!busy && init_left) {
                const unsigned long long k = base + __popc(want_init & lt_mask);
                if (k < num) {
                    // 64-byte records (cases of at most 64 cells) or 96-byte
                    // ones (deeper 9x9 expansions); list words past the
                    // record start as zeros.
                    const uint4 *src = reinterpret_cast<const uint4 *>(cycles + k * record_bytes);
                    const int vecs = int(record_bytes / 16);
#pragma unroll
                    for (int q = 0; q < kWideWords / 4; ++q) {
                        const uint4 x = q < vecs ? __ldg(src + q) : make_uint4(0, 0, 0, 0);
                        L.set_word(4 * q, x.x);
                        L.set_word(4 * q + 1, x.y);
                        L.set_word(4 * q + 2, x.z);
                        L.set_word(4 * q + 3, x.w);
                    }
                    owner = uint32_t(k);
                    root = start_i;
                    ++started;
                    if (!list_valid(L, start_i)) {
                        atomicExch(&Q.hdr->error, kErrMalformed);
                        ++finished;
                    } else if (start_i > last) {
                        leaves = 1;
                        flush();
                    } else {
                        busy = true;
                        fresh = true;
                        lvl = start_i;
                        eval = start_i;
                    }
                } else {
                    init_left = false;
                }
            }
        }
        if (ring_hint) {
            const unsigned need = __ballot_sync(kFull, !busy && !init_left);
            if (need && take_splits(need)) ring_hint = false;
        }
        const bool bookkeeping = ++round >= period;
        if (!__any_sync(kFull, busy)) {
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
            const unsigned need = __ballot_sync(kFull, !init_left);
            if (need) take_splits(need);
            if (__any_sync(kFull, busy) || __any_sync(kFull, init_left)) {
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
        if (busy) {
            const Mask128 g = R.gaps(L, eval, nodes);
            eval = apply_advance_w(L, S, lvl, eval, root, last, fresh, g, leaves);
            fresh = false;
            if (eval < 0) {
                flush();
                busy = false;
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
                want = *reinterpret_cast<volatile long long *>(&Q.hdr->idle_lanes) - queued;
            }
        }
        want = __shfl_sync(kFull, want, 0);
        ring_hint = __shfl_sync(kFull, queued, 0) > 0;
        if (want > 0) donate();
    }

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

__global__ void wide_ring_init(unsigned long long *seq, unsigned long long capacity) {
    for (unsigned long long k = blockIdx.x * blockDim.x + threadIdx.x; k < capacity;
         k += gridDim.x * blockDim.x)
        seq[k] = k;
}

constexpr int kWideTPB = 64;

template <int LEVELS>
cudaError_t launch_wide_levels(const uint8_t *d_edges, int start_i, int last, const uint8_t *d_cycles,
                               uint32_t record_bytes, uint64_t num, uint64_t *d_counts, uint64_t *d_nodes, const Queue &Q,
                               uint4 *slots, const BatchKnobs &knobs, cudaStream_t stream) {
    static std::mutex mu;
    static bool raised[16] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    constexpr size_t smem = CarveW<kWideTPB, LEVELS>::kBytes;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (dev < 0 || dev >= 16) return cudaErrorInvalidDevice;
        if (!raised[dev]) {
            e = cudaFuncSetAttribute(sym_wide_kernel<kWideTPB, LEVELS>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if (e != cudaSuccess) return e;
            raised[dev] = true;
        }
    }
    int fit = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, sym_wide_kernel<kWideTPB, LEVELS>,
                                                      kWideTPB, smem);
    if (e != cudaSuccess) return e;
    if (fit < 1) return cudaErrorInvalidConfiguration;
    if (knobs.blocks_per_sm > 0 && int(knobs.blocks_per_sm) < fit) fit = int(knobs.blocks_per_sm);
    sym_wide_kernel<kWideTPB, LEVELS><<<unsigned(device_sm_count() * fit), kWideTPB, smem, stream>>>(
        d_edges, start_i, last, d_cycles, record_bytes, num,
        reinterpret_cast<unsigned long long *>(d_counts),
        reinterpret_cast<unsigned long long *>(d_nodes), Q, slots, knobs.node_budget,
        knobs.wait_limit);
    return cudaGetLastError();
}

}  // namespace

uint64_t wide_workspace_bytes(uint64_t capacity) {
    return 256 + capacity * (4 * kWideRecordWords) + capacity * sizeof(unsigned long long);
}

cudaError_t launch_sym_wide(const uint8_t *d_wide_edges, int start_i, int stop_i,
                            const uint8_t *d_cycles, uint32_t record_bytes, uint64_t num,
                            uint64_t *d_counts,
                            uint64_t *d_nodes, void *d_workspace, const BatchKnobs &knobs,
                            cudaStream_t stream) {
    const uint64_t cap = knobs.queue_capacity;
    uint8_t *p = static_cast<uint8_t *>(d_workspace);
    Queue Q{};
    Q.hdr = reinterpret_cast<QueueHeader *>(p);
    Q.slots = nullptr;  // wide records live in `slots` below
    Q.seq = reinterpret_cast<unsigned long long *>(p + 256 + cap * (4 * kWideRecordWords));
    Q.capacity = cap;
    auto *slots = reinterpret_cast<uint4 *>(p + 256);
    cudaError_t e = cudaMemsetAsync(Q.hdr, 0, 256, stream);
    if (e != cudaSuccess) return e;
    wide_ring_init<<<64, 256, 0, stream>>>(Q.seq, cap);
    e = cudaGetLastError();
    if (e != cudaSuccess || num == 0) return e;
    e = cudaMemsetAsync(d_counts, 0, num * sizeof(uint64_t), stream);
    if (e != cudaSuccess) return e;
    const int levels = stop_i - 1 - start_i;
    // Stored levels run up to stop_i - 2; their high words need rows up to
    // stop_i - 2 - 65 < kWideHiRows.
    if ((record_bytes != kSymCells && record_bytes != kWideCells) || start_i > int(record_bytes) ||
        stop_i > 66 + kWideHiRows || stop_i > kWideCells)
        return cudaErrorInvalidValue;
    if (levels <= 40)
        return launch_wide_levels<40>(d_wide_edges, start_i, stop_i - 1, d_cycles, record_bytes, num,
                                      d_counts,
                                      d_nodes, Q, slots, knobs, stream);
    if (levels <= 56)
        return launch_wide_levels<56>(d_wide_edges, start_i, stop_i - 1, d_cycles, record_bytes, num,
                                      d_counts,
                                      d_nodes, Q, slots, knobs, stream);
    return cudaErrorInvalidValue;  // deeper searches need a deeper expansion first
}

}  // namespace mf
