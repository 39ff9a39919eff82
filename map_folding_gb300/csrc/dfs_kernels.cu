// dfs_kernels.cu -- sm_103a counting kernels.
//
// Both hot paths of the reference are the same search shape: a circular
// successor list (Lunnon: b[] over leaves, mf.c:128-142; sym_fold: cycle[]
// over spiral cells, sym_fold.cpp:206-217), grown one item per level by
// inserting item `lvl` after a chosen position, with the set of admissible
// positions recomputed at every level by walking the list.  The engine below
// keeps that list per thread in shared memory (byte per item, word-interleaved
// across the CTA so a warp never has a bank conflict), keeps the per-level
// choices as a 64-bit mask stack instead of the reference's gap[] array, and
// counts the last level with a popcount.  Gap rules:
//   LunnonRules  -- mf.c:88-124 as a bitwise AND of per-dimension walk masks
//   SymRules     -- sym_fold.cpp:179-204 (get_good)
// Kernels:
//   *_plain_kernel    one thread per unit (prefix state / case), one launch
//   *_batched_kernel  persistent grid, device work queue, subtree splitting
//
// Every unit's list is checked to be a permutation of its placed items before
// its search starts, which bounds every walk (see list_valid), and every
// device wait has a limit, so malformed input cannot hang a kernel: a unit
// whose list is malformed reports UINT64_MAX (plain) or raises the queue
// error flag (batched).
#include <cuda_runtime.h>

#include <cstdint>

#include "engine.hpp"

namespace mf {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxLevels = 66;      // levels 0..65 (Lunnon up to n + 1 = 65)
constexpr int kMinSplitHeight = 3;  // never hand out subtrees shallower than this

__device__ __forceinline__ uint64_t low_bits(int k) {
    return k >= 64 ? ~0ULL : ((1ULL << k) - 1ULL);
}

// Per-thread successor list in shared memory.  Byte j of thread t lives in
// 32-bit word (j/4)*TPB + t, so a warp's 32 lanes always address 32
// different banks, whatever items they touch.
template <int TPB>
struct List {
    uint8_t *base;  // smem + 4 * threadIdx.x
    __device__ __forceinline__ int get(int j) const { return base[(j & ~3) * TPB + (j & 3)]; }
    __device__ __forceinline__ void put(int j, int v) const {
        base[(j & ~3) * TPB + (j & 3)] = static_cast<uint8_t>(v);
    }
    __device__ __forceinline__ uint32_t word(int w) const {
        return reinterpret_cast<const uint32_t *>(base)[w * TPB];
    }
    __device__ __forceinline__ void set_word(int w, uint32_t v) const {
        reinterpret_cast<uint32_t *>(base)[w * TPB] = v;
    }
};

// A unit's list is usable only if it is a permutation of the placed items
// (items >= placed are written before they are read).  That is also what
// makes every walk below terminate without a step bound: each walk iterates
// an injective map (the list composed with an involution -- the page's
// partner matching for sym, the dimension's neighbour table d[l][.] for
// Lunnon) from a point with no preimage, so it reaches its end in fewer
// than `placed` + 1 steps.  Insertions keep the list a permutation.
template <int TPB>
__device__ __forceinline__ bool list_valid(const List<TPB> &L, int placed) {
    bool ok = true;
    uint64_t seen_lo = 0, seen_hi = 0;
    for (int k = 0; k < placed; ++k) {
        const int v = L.get(k);
        ok &= v < placed;
        if (v < 64) seen_lo |= 1ULL << v;
        else seen_hi |= 1ULL << (v & 63);
    }
    const uint64_t want_lo = low_bits(placed);
    const uint64_t want_hi = placed > 64 ? low_bits(placed - 64) : 0;
    return ok && seen_lo == want_lo && seen_hi == want_hi;
}

// ------------------------------------------------------------- rules -----

// sym_fold.cpp:179-204: positions j < i after which cell i may follow in the
// stack.  For each edge page whose neighbour `other` of i is placed, walk the
// cycle from `other`, hopping over every placed partner pair, and keep the
// positions landed on; AND the pages.  The pages' walks run as one flat loop
// (a lane moves on to its next page inside the same loop), so a warp waits
// for its longest lane's total walk, not for the sum of per-page maxima.
struct SymRules {
    const uint8_t *edge;  // 4 pages x 64, shared memory
    template <int TPB>
    __device__ __forceinline__ uint64_t gaps(const List<TPB> &L, int i, unsigned long long &nodes,
                                             bool &) const {
        ++nodes;
        uint64_t good = low_bits(i);
        unsigned pend = 0;  // pages whose neighbour of i is placed
#pragma unroll
        for (int p = 0; p < 4; ++p) pend |= unsigned(edge[p * kSymCells + i] < i) << p;
        const uint8_t *e = edge;
        uint64_t allowed = ~0ULL;
        int other = 0, j = 0;
        for (;;) {
            if (j == other) {  // current page finished (or none started)
                good &= allowed;
                if (!good || !pend) break;
                const int p = __ffs(pend) - 1;
                pend &= pend - 1;
                e = edge + p * kSymCells;
                other = e[i];
                allowed = 1ULL << other;
                j = L.get(other);
                continue;
            }
            const int partner = e[j];
            j = partner < i ? partner : j;
            allowed |= 1ULL << j;
            j = L.get(j);
        }
        return good;
    }
};

// mf.c:88-124 with the gap stack replaced by masks: for every constrained
// dimension walk m = d[l][l], d[l][b[m]], ... up to l and collect the walked
// positions; a gap is a position every constrained dimension walked (the
// reference's count[m] == dim - dd); with no constrained dimension every
// position 0..l-1 is a gap.  Position 0 (insert on top of the sentinel) is
// dropped for l >= 2: it makes b[0] = l != 1 and the normal-form filter
// (mf.c:83) would prune the whole subtree.  `nodes` counts the insertions
// the reference loop would make (mf.c:136-142), position 0 included.  As for
// sym, the dimensions' walks run as one flat loop.
struct LunnonRules {
    const uint8_t *table;  // [dim][n+1][n+1]
    int n;
    int dim;
    template <int TPB>
    __device__ __forceinline__ uint64_t gaps(const List<TPB> &L, int l, unsigned long long &nodes,
                                             bool &) const {
        const int w = n + 1;
        uint64_t mask = ~0ULL, walked = ~0ULL;
        int bound = 0, d = -1, m = l;
        const uint8_t *row = table;
        for (;;) {
            if (m == l) {  // current dimension finished (or none started)
                mask &= walked;
                if (!mask) break;
                int first = l;
                while (++d < dim) {
                    row = table + (d * w + l) * w;
                    first = row[l];
                    if (first != l) break;
                }
                if (d >= dim) break;
                ++bound;
                m = first;
                walked = 0;
                continue;
            }
            walked |= 1ULL << m;
            m = row[L.get(m)];
        }
        if (!bound) mask = low_bits(l);
        nodes += __popcll(mask);
        if (l >= 2) mask &= ~1ULL;
        return mask;
    }
};

// ---------------------------------------------------------- DFS core -----

struct Stack {
    uint64_t mask[kMaxLevels];   // untried positions per level
    uint8_t chosen[kMaxLevels];  // position the level's item was inserted after
};

// Advance one unit's search by at most `budget` gap evaluations.  On entry
// items root..lvl-1 are inserted and mask[lvl] holds lvl's untried
// positions.  The last level is never entered: its positions are counted.
// Returns true when the unit's subtree is exhausted.
template <class Rules, int TPB>
__device__ __forceinline__ bool dfs_run(const Rules &R, const List<TPB> &L, Stack &S, int &lvl,
                                        int root, int last, unsigned long long &leaves,
                                        unsigned long long &nodes, uint32_t budget, bool &bad) {
    for (;;) {
        const uint64_t cur = S.mask[lvl];
        if (cur == 0) {
            if (lvl == root) return true;
            --lvl;
            L.put(S.chosen[lvl], L.get(lvl));  // detach item lvl
            continue;
        }
        if (budget == 0) return false;
        --budget;
        const int j = __ffsll(static_cast<long long>(cur)) - 1;
        S.mask[lvl] = cur & (cur - 1);
        const int after = L.get(j);
        L.put(lvl, after);  // insert item lvl after j
        L.put(j, lvl);
        const int nxt = lvl + 1;
        const uint64_t g = R.gaps(L, nxt, nodes, bad);
        if (bad) return true;
        if (nxt == last) {
            leaves += __popcll(g);
            L.put(j, after);
            continue;
        }
        S.chosen[lvl] = static_cast<uint8_t>(j);
        lvl = nxt;
        S.mask[lvl] = g;
    }
}

// Start a unit whose list is loaded: evaluate the root level.  Returns true
// if the unit still needs a search (mask[root] set), false if it is already
// counted into `leaves`.
template <class Rules, int TPB>
__device__ __forceinline__ bool dfs_begin(const Rules &R, const List<TPB> &L, Stack &S, int root,
                                          int last, unsigned long long &leaves,
                                          unsigned long long &nodes, bool &bad) {
    if (root > last) {  // nothing left to place: the unit is one completion
        leaves += 1;
        return false;
    }
    const uint64_t g = R.gaps(L, root, nodes, bad);
    if (bad) return false;
    if (root == last) {
        leaves += __popcll(g);
        return false;
    }
    S.mask[root] = g;
    return true;
}

template <int TPB, int WORDS>
__device__ __forceinline__ void load_list(const List<TPB> &L, const uint8_t *__restrict__ src,
                                          uint32_t stride) {
    // Records are 16-byte aligned with 16-byte multiple strides: whole-vector
    // loads, then scatter the words into the interleaved layout.
    const uint4 *v = reinterpret_cast<const uint4 *>(src);
    const int vecs = (stride / 16) < (WORDS + 3) / 4 ? int(stride / 16) : (WORDS + 3) / 4;
    for (int q = 0; q < vecs; ++q) {
        const uint4 x = __ldg(v + q);
        const uint32_t ws[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (4 * q + k < WORDS) L.set_word(4 * q + k, ws[k]);
    }
    for (int w = 4 * vecs; w < WORDS; ++w) L.set_word(w, 0);
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

// ------------------------------------------------------- plain kernels ---

struct EdgePages {
    uint32_t w[64];  // 4 pages x 64 bytes
};

template <int TPB>
__global__ void __launch_bounds__(TPB)
    sym_plain_kernel(EdgePages pages, int start_i, int stop_i, const uint8_t *__restrict__ cycles,
                     uint64_t num, unsigned long long *__restrict__ counts,
                     unsigned long long *__restrict__ nodes_out) {
    __shared__ uint32_t s_edge[64];
    __shared__ uint32_t s_list[16 * TPB];
    const int tid = threadIdx.x;
    for (int k = tid; k < 64; k += TPB) s_edge[k] = pages.w[k];
    const List<TPB> L{reinterpret_cast<uint8_t *>(s_list) + 4 * tid};
    const uint64_t unit = uint64_t(blockIdx.x) * TPB + tid;
    const bool active = unit < num;
    if (active) load_list<TPB, 16>(L, cycles + unit * kSymCells, kSymCells);
    __syncthreads();

    unsigned long long nodes = 0;
    if (active) {
        const SymRules R{reinterpret_cast<const uint8_t *>(s_edge)};
        Stack S;
        bool bad = !list_valid(L, start_i);
        unsigned long long leaves = 0;
        const int last = stop_i - 1;
        if (!bad && dfs_begin(R, L, S, start_i, last, leaves, nodes, bad)) {
            int lvl = start_i;
            while (!dfs_run(R, L, S, lvl, start_i, last, leaves, nodes, 0xffffffffu, bad)) {
            }
        }
        counts[unit] = bad ? ~0ULL : leaves;
    }
    if (nodes_out) {
        const unsigned long long s = warp_sum(nodes);
        if ((tid & 31) == 0 && s) atomicAdd(nodes_out, s);
    }
}

template <int TPB>
__global__ void __launch_bounds__(TPB)
    lunnon_plain_kernel(const uint8_t *__restrict__ table, int table_bytes, int n, int dim,
                        int start_leaf, const uint8_t *__restrict__ states, uint32_t stride,
                        uint64_t num, unsigned long long *__restrict__ per_state,
                        unsigned long long *__restrict__ total,
                        unsigned long long *__restrict__ nodes_out) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint32_t *s_list = reinterpret_cast<uint32_t *>(smem);  // 17 * TPB words
    uint8_t *s_table = smem + 17 * 4 * TPB;
    const int tid = threadIdx.x;
    for (int k = tid; k < table_bytes / 4; k += TPB)
        reinterpret_cast<uint32_t *>(s_table)[k] = __ldg(reinterpret_cast<const uint32_t *>(table) + k);
    const List<TPB> L{reinterpret_cast<uint8_t *>(s_list) + 4 * tid};
    const uint64_t unit = uint64_t(blockIdx.x) * TPB + tid;
    const bool active = unit < num;
    if (active) load_list<TPB, 17>(L, states + unit * stride, stride);
    __syncthreads();

    unsigned long long nodes = 0;
    unsigned long long leaves = 0;
    if (active) {
        const LunnonRules R{s_table, n, dim};
        Stack S;
        bool bad = !list_valid(L, start_leaf < n + 1 ? start_leaf : n + 1);
        if (!bad && dfs_begin(R, L, S, start_leaf, n, leaves, nodes, bad)) {
            int lvl = start_leaf;
            while (!dfs_run(R, L, S, lvl, start_leaf, n, leaves, nodes, 0xffffffffu, bad)) {
            }
        }
        leaves = bad ? 0 : leaves * static_cast<unsigned long long>(n);
        if (per_state) per_state[unit] = bad ? ~0ULL : leaves;
    }
    if (total) {
        const unsigned long long s = warp_sum(leaves);
        if ((tid & 31) == 0 && s) atomicAdd(total, s);
    }
    if (nodes_out) {
        const unsigned long long s = warp_sum(nodes);
        if ((tid & 31) == 0 && s) atomicAdd(nodes_out, s);
    }
}

// ------------------------------------------------- persistent kernels ----

struct Queue {
    QueueHeader *hdr;
    TaskRecord *slots;
    unsigned int *ready;
    unsigned long long capacity;
};

__device__ __forceinline__ unsigned long long vload(const unsigned long long *p) {
    return *reinterpret_cast<const volatile unsigned long long *>(p);
}

// Hand out one work item: an initial unit while any are left (an atomicAdd
// that may overshoot harmlessly), otherwise a split subtree (a CAS that never
// hands out an index that has not been reserved).  Returns 0 = none,
// 1 = initial unit k, 2 = split item k.
__device__ __forceinline__ int take_item(const Queue &Q, unsigned long long num,
                                         unsigned long long &k) {
    if (vload(&Q.hdr->init_next) < num) {
        k = atomicAdd(&Q.hdr->init_next, 1ULL);
        if (k < num) return 1;
    }
    unsigned long long h = vload(&Q.hdr->spawn_head);
    for (int attempt = 0; attempt < 32; ++attempt) {
        const unsigned long long t = vload(&Q.hdr->spawn_tail);
        if (h >= t) return 0;
        const unsigned long long seen = atomicCAS(&Q.hdr->spawn_head, h, h + 1);
        if (seen == h) {
            k = h;
            return 2;
        }
        h = seen;
    }
    return 0;
}

// Wait (bounded) until split item k is published, then copy it out.
template <int TPB, int WORDS>
__device__ __forceinline__ bool fetch_split(const Queue &Q, unsigned long long k, const List<TPB> &L,
                                            uint32_t &owner, uint64_t &mask, int &level,
                                            uint32_t wait_limit) {
    const volatile unsigned int *flag = Q.ready + k;
    uint32_t spins = 0;
    while (*flag == 0u) {
        if (++spins > wait_limit) {
            atomicExch(&Q.hdr->error, 1u);
            return false;
        }
        __nanosleep(64);
    }
    __threadfence();
    const uint4 *src = reinterpret_cast<const uint4 *>(Q.slots + k);
    uint32_t w[24];
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const uint4 x = __ldcg(src + q);
        w[4 * q] = x.x;
        w[4 * q + 1] = x.y;
        w[4 * q + 2] = x.z;
        w[4 * q + 3] = x.w;
    }
#pragma unroll
    for (int k2 = 0; k2 < WORDS; ++k2) L.set_word(k2, w[k2]);
    owner = w[17];
    mask = uint64_t(w[18]) | (uint64_t(w[19]) << 32);
    level = int(w[20]);
    return true;
}

// Give away the shallowest untried sibling set of this unit as a new work
// item.  The list is rolled back to that level, copied, and replayed.
template <int TPB, int WORDS>
__device__ __forceinline__ bool donate(const Queue &Q, const List<TPB> &L, Stack &S, int lvl,
                                       int root, int last, uint32_t owner) {
    int s = root;
    while (s <= lvl && S.mask[s] == 0) ++s;
    if (s > lvl || last - s < kMinSplitHeight) return false;
    // Reserve a slot without ever overshooting the capacity.
    unsigned long long t = vload(&Q.hdr->spawn_tail);
    bool got = false;
    for (int attempt = 0; attempt < 32 && t < Q.capacity; ++attempt) {
        const unsigned long long seen = atomicCAS(&Q.hdr->spawn_tail, t, t + 1);
        if (seen == t) {
            got = true;
            break;
        }
        t = seen;
    }
    if (!got) return false;
    for (int l = lvl - 1; l >= s; --l) L.put(S.chosen[l], L.get(l));
    uint32_t w[24];
#pragma unroll
    for (int k = 0; k < 24; ++k) w[k] = 0;
#pragma unroll
    for (int k = 0; k < WORDS; ++k) w[k] = L.word(k);
    w[17] = owner;
    w[18] = uint32_t(S.mask[s]);
    w[19] = uint32_t(S.mask[s] >> 32);
    w[20] = uint32_t(s);
    uint4 *dst = reinterpret_cast<uint4 *>(Q.slots + t);
#pragma unroll
    for (int q = 0; q < 6; ++q) __stcg(dst + q, make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]));
    for (int l = s; l < lvl; ++l) {
        const int j = S.chosen[l];
        const int after = L.get(j);
        L.put(l, after);
        L.put(j, l);
    }
    S.mask[s] = 0;
    __threadfence();
    atomicExch(Q.ready + t, 1u);
    return true;
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
    const uint8_t *tables;
    uint32_t stride;
};

// The persistent loop.  Every lane holds at most one unit; lanes that run out
// of work refill individually inside their slice, and at the slice boundary
// the warp (re)converges to refill, check whether the queue is running dry
// and, if so, let each busy lane give away its shallowest untried siblings.
// A warp leaves when it is idle and all work is accounted for, or when it has
// stayed idle for wait_limit rounds -- leaving is always safe, because the
// warp that owns a split item's parent keeps looping until it has nothing.
template <int TPB, int WORDS, bool kSym>
__device__ __forceinline__ void persistent_loop(const uint8_t *s_tables, const SymSource &sym,
                                                const LunnonSource &lun, unsigned long long num,
                                                unsigned long long *counts,
                                                unsigned long long *nodes_out, const Queue &Q,
                                                uint32_t budget, unsigned long long hungry_level,
                                                uint32_t wait_limit, const List<TPB> &L) {
    const int lane = threadIdx.x & 31;
    Stack S;
    bool busy = false;
    bool bad = false;
    int lvl = 0, root = 0, last = 0;
    uint32_t owner = 0;
    unsigned long long leaves = 0, nodes = 0, finished = 0, started = 0;
    uint32_t idle_rounds = 0;
    SymRules srules{s_tables};
    LunnonRules lrules{nullptr, 0, 0};

    // Count a finished unit into its owner's slot.
    auto flush = [&]() {
        if (bad) {
            atomicExch(&Q.hdr->error, 1u);
            bad = false;
        } else if (leaves) {
            const unsigned long long weight = kSym ? 1ULL : static_cast<unsigned long long>(lrules.n);
            atomicAdd(counts + owner, leaves * weight);
        }
        leaves = 0;
        ++finished;
    };

    // Acquire work until a unit needs a search or nothing is available.
    auto acquire = [&]() -> bool {
        for (int tries = 0; tries < 64; ++tries) {
            unsigned long long k = 0;
            const int kind = take_item(Q, num, k);
            if (kind == 0) return false;
            ++started;
            if (kind == 1) {
                if (kSym) {
                    load_list<TPB, WORDS>(L, sym.cycles + k * kSymCells, kSymCells);
                    owner = uint32_t(k);
                    root = sym.start_i;
                    last = sym.last;
                    bad = !list_valid(L, root);
                } else {
                    load_list<TPB, WORDS>(L, lun.states + k * lun.stride, lun.stride);
                    owner = lun.state_owner[k];
                    const LunnonInstanceDev I = lun.inst[owner];
                    lrules = LunnonRules{s_tables + I.table_offset, I.n, I.dim};
                    root = I.start_leaf;
                    last = I.n;
                    bad = !list_valid(L, root < I.n + 1 ? root : I.n + 1);
                }
                if (bad) {
                    flush();
                    continue;
                }
                bool more;
                if (kSym) more = dfs_begin(srules, L, S, root, last, leaves, nodes, bad);
                else more = dfs_begin(lrules, L, S, root, last, leaves, nodes, bad);
                if (more && !bad) {
                    lvl = root;
                    return true;
                }
                flush();
            } else {
                uint64_t mask = 0;
                int level = 0;
                if (!fetch_split<TPB, WORDS>(Q, k, L, owner, mask, level, wait_limit)) {
                    ++finished;
                    continue;
                }
                if (kSym) {
                    last = sym.last;
                } else {
                    const LunnonInstanceDev I = lun.inst[owner];
                    lrules = LunnonRules{s_tables + I.table_offset, I.n, I.dim};
                    last = I.n;
                }
                root = level;
                lvl = level;
                S.mask[level] = mask;
                return true;
            }
        }
        return false;
    };

    for (;;) {
        if (!busy) busy = acquire();
        const unsigned any = __ballot_sync(kFull, busy);
        if (any == 0) {
            // Account this warp's finished units first, then decide.
            const unsigned long long f = warp_sum(finished);
            finished = 0;
            int stop = 0;
            if (lane == 0) {
                if (f) atomicAdd(&Q.hdr->completed, f);
                const unsigned long long total = num + vload(&Q.hdr->spawn_tail);
                stop = (vload(&Q.hdr->init_next) >= num && vload(&Q.hdr->completed) >= total) ||
                       *reinterpret_cast<volatile unsigned int *>(&Q.hdr->error) != 0u ||
                       ++idle_rounds > wait_limit;
            }
            stop = __shfl_sync(kFull, stop, 0);
            if (stop) break;
            __nanosleep(200);
            continue;
        }
        idle_rounds = 0;
        if (busy) {
            // Run the slice; a lane whose unit ends refills and keeps going.
            uint32_t left = budget;
            for (;;) {
                bool done;
                if (kSym) done = dfs_run(srules, L, S, lvl, root, last, leaves, nodes, left, bad);
                else done = dfs_run(lrules, L, S, lvl, root, last, leaves, nodes, left, bad);
                if (!done) break;
                flush();
                busy = acquire();
                if (!busy) break;
                left = budget / 2;  // a fresh unit gets a shorter remaining slice
            }
        }
        // Slice boundary: account finished units, then split if the queue is
        // running dry.
        const unsigned long long f = warp_sum(finished);
        int hungry = 0;
        if (lane == 0) {
            if (f) atomicAdd(&Q.hdr->completed, f);
            const unsigned long long in = vload(&Q.hdr->init_next);
            const unsigned long long init_left = in < num ? num - in : 0;
            const unsigned long long split_left =
                vload(&Q.hdr->spawn_tail) - vload(&Q.hdr->spawn_head);
            hungry = (init_left + split_left) < hungry_level;
        }
        finished = 0;
        hungry = __shfl_sync(kFull, hungry, 0);
        if (hungry && busy) donate<TPB, WORDS>(Q, L, S, lvl, root, last, owner);
    }

    const unsigned long long ns = warp_sum(nodes);
    const unsigned long long st = warp_sum(started);
    if (lane == 0) {
        if (nodes_out && ns) atomicAdd(nodes_out, ns);
        if (st) atomicAdd(&Q.hdr->tasks_run, st);
    }
}

template <int TPB>
__global__ void __launch_bounds__(TPB)
    sym_batched_kernel(EdgePages pages, SymSource src, unsigned long long num,
                       unsigned long long *counts, unsigned long long *nodes_out, Queue Q,
                       uint32_t budget, unsigned long long hungry_level, uint32_t wait_limit) {
    __shared__ uint32_t s_edge[64];
    __shared__ uint32_t s_list[16 * TPB];
    for (int k = threadIdx.x; k < 64; k += TPB) s_edge[k] = pages.w[k];
    __syncthreads();
    const List<TPB> L{reinterpret_cast<uint8_t *>(s_list) + 4 * threadIdx.x};
    LunnonSource none{};
    persistent_loop<TPB, 16, true>(reinterpret_cast<const uint8_t *>(s_edge), src, none, num, counts,
                                   nodes_out, Q, budget, hungry_level, wait_limit, L);
}

template <int TPB>
__global__ void __launch_bounds__(TPB)
    lunnon_batched_kernel(LunnonSource src, uint32_t tables_bytes, unsigned long long num,
                          unsigned long long *counts, unsigned long long *nodes_out, Queue Q,
                          uint32_t budget, unsigned long long hungry_level, uint32_t wait_limit) {
    extern __shared__ __align__(16) uint8_t smem[];
    uint32_t *s_list = reinterpret_cast<uint32_t *>(smem);
    uint8_t *s_tables = smem + 17 * 4 * TPB;
    for (uint32_t k = threadIdx.x; k < tables_bytes / 4; k += TPB)
        reinterpret_cast<uint32_t *>(s_tables)[k] =
            __ldg(reinterpret_cast<const uint32_t *>(src.tables) + k);
    __syncthreads();
    const List<TPB> L{reinterpret_cast<uint8_t *>(s_list) + 4 * threadIdx.x};
    SymSource none{};
    persistent_loop<TPB, 17, false>(s_tables, none, src, num, counts, nodes_out, Q, budget,
                                    hungry_level, wait_limit, L);
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
    const uint64_t slots = capacity * sizeof(TaskRecord);
    const uint64_t flags = (capacity * sizeof(unsigned int) + 255) / 256 * 256;
    return 256 + slots + flags;
}

namespace {

Queue carve_queue(void *ws, uint64_t capacity) {
    uint8_t *p = static_cast<uint8_t *>(ws);
    Queue q;
    q.hdr = reinterpret_cast<QueueHeader *>(p);
    q.slots = reinterpret_cast<TaskRecord *>(p + 256);
    q.ready = reinterpret_cast<unsigned int *>(p + 256 + capacity * sizeof(TaskRecord));
    q.capacity = capacity;
    return q;
}

EdgePages pack_pages(const uint8_t *edges) {
    EdgePages e;
    for (int k = 0; k < 64; ++k)
        e.w[k] = uint32_t(edges[4 * k]) | (uint32_t(edges[4 * k + 1]) << 8) |
                 (uint32_t(edges[4 * k + 2]) << 16) | (uint32_t(edges[4 * k + 3]) << 24);
    return e;
}

}  // namespace

cudaError_t launch_sym_plain(const uint8_t *edges, int start_i, int stop_i, const uint8_t *d_cycles,
                             uint64_t num, uint64_t *d_counts, uint64_t *d_nodes,
                             cudaStream_t stream) {
    if (num == 0) return cudaSuccess;
    constexpr int TPB = 128;
    const uint64_t blocks = (num + TPB - 1) / TPB;
    sym_plain_kernel<TPB><<<unsigned(blocks), TPB, 0, stream>>>(
        pack_pages(edges), start_i, stop_i, d_cycles, num,
        reinterpret_cast<unsigned long long *>(d_counts),
        reinterpret_cast<unsigned long long *>(d_nodes));
    return cudaGetLastError();
}

cudaError_t launch_lunnon_plain(const uint8_t *d_table, int n, int dim, int start_leaf,
                                const uint8_t *d_states, uint32_t stride, uint64_t num,
                                uint64_t *d_per_state, uint64_t *d_total, uint64_t *d_nodes,
                                cudaStream_t stream) {
    if (num == 0) return cudaSuccess;
    constexpr int TPB = 128;
    const int table_bytes = (dim * (n + 1) * (n + 1) + 15) / 16 * 16;
    const size_t smem = size_t(17) * 4 * TPB + table_bytes;
    cudaError_t e = cudaFuncSetAttribute(lunnon_plain_kernel<TPB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
    if (e != cudaSuccess) return e;
    const uint64_t blocks = (num + TPB - 1) / TPB;
    lunnon_plain_kernel<TPB><<<unsigned(blocks), TPB, smem, stream>>>(
        d_table, table_bytes, n, dim, start_leaf, d_states, stride, num,
        reinterpret_cast<unsigned long long *>(d_per_state),
        reinterpret_cast<unsigned long long *>(d_total),
        reinterpret_cast<unsigned long long *>(d_nodes));
    return cudaGetLastError();
}

cudaError_t launch_sym_batched(const uint8_t *edges, int start_i, int stop_i,
                               const uint8_t *d_cycles, uint64_t num, uint64_t *d_counts,
                               uint64_t *d_nodes, void *d_workspace, const BatchKnobs &knobs,
                               cudaStream_t stream) {
    Queue Q = carve_queue(d_workspace, knobs.queue_capacity);
    cudaError_t e = cudaMemsetAsync(d_workspace, 0, 256, stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(Q.ready, 0, knobs.queue_capacity * sizeof(unsigned int), stream);
    if (e != cudaSuccess) return e;
    if (num == 0) return cudaSuccess;
    e = cudaMemsetAsync(d_counts, 0, num * sizeof(uint64_t), stream);
    if (e != cudaSuccess) return e;
    const int sms = device_sm_count();
    SymSource src{d_cycles, start_i, stop_i - 1};
    const unsigned long long threads = 1ULL * sms * knobs.blocks_per_sm * knobs.block_threads;
    const unsigned long long hungry = threads * knobs.hungry_factor / 8;
    const unsigned grid = unsigned(sms * knobs.blocks_per_sm);
#define MF_SYM_BATCHED(TPB)                                                                      \
    sym_batched_kernel<TPB><<<grid, TPB, 0, stream>>>(                                           \
        pack_pages(edges), src, num, reinterpret_cast<unsigned long long *>(d_counts),           \
        reinterpret_cast<unsigned long long *>(d_nodes), Q, knobs.node_budget, hungry,           \
        knobs.wait_limit)
    switch (knobs.block_threads) {
        case 64: MF_SYM_BATCHED(64); break;
        case 256: MF_SYM_BATCHED(256); break;
        default: MF_SYM_BATCHED(128); break;
    }
#undef MF_SYM_BATCHED
    return cudaGetLastError();
}

cudaError_t launch_lunnon_batched(const uint8_t *d_tables, uint32_t tables_bytes,
                                  const LunnonInstanceDev *d_inst, int num_inst,
                                  const uint8_t *d_states, const uint32_t *d_state_owner,
                                  uint64_t num, uint64_t *d_counts, uint64_t *d_nodes,
                                  void *d_workspace, const BatchKnobs &knobs, cudaStream_t stream) {
    Queue Q = carve_queue(d_workspace, knobs.queue_capacity);
    cudaError_t e = cudaMemsetAsync(d_workspace, 0, 256, stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(Q.ready, 0, knobs.queue_capacity * sizeof(unsigned int), stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(d_counts, 0, size_t(num_inst) * sizeof(uint64_t), stream);
    if (e != cudaSuccess) return e;
    if (num == 0) return cudaSuccess;
    const int sms = device_sm_count();
    const uint32_t tb = (tables_bytes + 15) / 16 * 16;
    const unsigned long long threads = 1ULL * sms * knobs.blocks_per_sm * knobs.block_threads;
    const unsigned long long hungry = threads * knobs.hungry_factor / 8;
    const unsigned grid = unsigned(sms * knobs.blocks_per_sm);
    const size_t smem = size_t(17) * 4 * knobs.block_threads + tb;
#define MF_LUN_BATCHED(TPB)                                                                     \
    do {                                                                                        \
        cudaFuncSetAttribute(lunnon_batched_kernel<TPB>,                                        \
                             cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);          \
        lunnon_batched_kernel<TPB><<<grid, TPB, smem, stream>>>(                                \
            LunnonSource{d_states, d_state_owner, d_inst, d_tables, lunnon_state_stride(64)},   \
            tb, num, reinterpret_cast<unsigned long long *>(d_counts),                          \
            reinterpret_cast<unsigned long long *>(d_nodes), Q, knobs.node_budget, hungry,      \
            knobs.wait_limit);                                                                  \
    } while (0)
    switch (knobs.block_threads) {
        case 64: MF_LUN_BATCHED(64); break;
        case 256: MF_LUN_BATCHED(256); break;
        default: MF_LUN_BATCHED(128); break;
    }
#undef MF_LUN_BATCHED
    return cudaGetLastError();
}

}  // namespace mf
