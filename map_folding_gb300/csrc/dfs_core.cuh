// dfs_core.cuh -- device building blocks shared by the counting kernels
// (dfs_kernels.cu) and the request server (serve.cu): the per-thread
// successor lists, the gap rules of both paths, the DFS stacks, the lockstep
// advance/apply steps and the warp-cooperative split-item ring.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "engine.hpp"

namespace mf {
namespace {


constexpr unsigned kFull = 0xffffffffu;
constexpr int kLocalLevels = 66;    // local-memory stack: levels 0..65
constexpr int kMinSplitHeight = 4;  // never hand out subtrees shallower than this
// Steps a resumable walk may take per lockstep round (measured on the 7x7
// cases: 6 steps gave 8 % more nodes per second than uncapped walks, 8 steps
// 6.5 %, 10 steps 2 %).
constexpr int kWalkCap = 6;

__device__ __forceinline__ uint64_t low_bits(int k) {
    return k >= 64 ? ~0ULL : ((1ULL << k) - 1ULL);
}

// Per-thread byte array in shared memory, laid out so that a warp's 32 lanes
// always address 32 different banks, whatever indices they touch.
//
// CTAs of a multiple of 128 threads (the 64-bit kernels): each group of four
// warps shares 128-byte rows, row j holding byte j of all 128 threads --
// lane l of warp w at byte 4*l + w, so lane l always reads bank l.  Byte j of
// a thread is then at its base + 128*j: one shift-add per access, which the
// walks make twice per step.  Other CTA sizes (the 64-thread 128-bit
// kernel): byte j of thread t in 32-bit word (j/4)*TPB + t.
template <int TPB>
struct List {
    static constexpr bool kRows = TPB % 128 == 0;
    uint8_t *base;  // this thread's byte 0
    // The list of the calling thread in an area of `bytes` bytes per thread.
    __device__ static List at(uint8_t *area, int bytes) {
        const int t = threadIdx.x;
        if constexpr (kRows) return List{area + (t >> 7) * bytes * 128 + 4 * (t & 31) + ((t >> 5) & 3)};
        else return List{area + 4 * t};
    }
    __device__ __forceinline__ int offset(int j) const {
        if constexpr (kRows) return j << 7;
        else return (j & ~3) * TPB + (j & 3);
    }
    __device__ __forceinline__ int get(int j) const { return base[offset(j)]; }
    __device__ __forceinline__ void put(int j, int v) const { base[offset(j)] = static_cast<uint8_t>(v); }
    // Bytes 4w .. 4w+3 as one little-endian word.
    __device__ __forceinline__ uint32_t word(int w) const {
        if constexpr (kRows) {
            return uint32_t(get(4 * w)) | uint32_t(get(4 * w + 1)) << 8 |
                   uint32_t(get(4 * w + 2)) << 16 | uint32_t(get(4 * w + 3)) << 24;
        } else {
            return reinterpret_cast<const uint32_t *>(base)[w * TPB];
        }
    }
    __device__ __forceinline__ void set_word(int w, uint32_t v) const {
        if constexpr (kRows) {
#pragma unroll
            for (int b = 0; b < 4; ++b) put(4 * w + b, int((v >> (8 * b)) & 0xffu));
        } else {
            reinterpret_cast<uint32_t *>(base)[w * TPB] = v;
        }
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

// 1 << m with PTX shift semantics: 0 for m >= 64 (a walk may pass through
// position 64, the last leaf of a 64-leaf map, which is never a gap).
__device__ __forceinline__ uint64_t bit64(int m) {
    uint64_t r;
    asm("shl.b64 %0, %1, %2;" : "=l"(r) : "l"(1ULL), "r"(m));
    return r;
}

// sym_fold.cpp:179-204: positions j < i after which cell i may follow in the
// stack.  For each edge page whose neighbour `other` of i is placed, walk the
// cycle from `other`, hopping over every placed partner pair, and keep the
// positions landed on; AND the pages.
//
// The pages are walked two at a time, side by side in one loop (on the
// spiral numbering every cell has at most two placed neighbours, so that is
// one pass): two independent dependent-load chains per lane instead of one,
// and no page-start logic inside the loop.  A chain that has come back to its
// start keeps stepping until the other one has too, which changes nothing:
// from `other` the walk goes to L[other] again (other's partner on this page
// is i itself, never placed), so it retraces the same positions.  With one
// page the second chain is a copy of the first.  The pages to walk for cell i
// come packed from a per-cell table: byte k = page << 6 | neighbour (so the
// page's 64-byte row starts at byte & 0xC0), `count` entries.
struct SymRules {
    const uint8_t *edge;     // 4 pages x 64, shared memory
    const uint32_t *pages;   // per cell: its placed-neighbour pages, packed
    const uint8_t *count;    // per cell: how many
    template <class List>
    __device__ __forceinline__ uint64_t gaps(const List &L, int i,
                                             unsigned long long &nodes) const {
        ++nodes;
        uint64_t good = low_bits(i);
        uint32_t q = pages[i];
        for (int left = count[i]; left > 0 && good; left -= 2, q >>= 16) {
            const uint32_t qb = left > 1 ? (q >> 8) : q;
            const int oA = q & 63, oB = qb & 63;
            const uint8_t *eA = edge + (q & 0xC0);
            const uint8_t *eB = edge + (qb & 0xC0);
            uint64_t aA = 1ULL << oA, aB = 1ULL << oB;
            int jA = L.get(oA), jB = L.get(oB);
            bool dA = jA == oA, dB = jB == oB;
            while (!(dA && dB)) {
                const int pA = eA[jA];
                const int pB = eB[jB];
                const int xA = pA < i ? pA : jA;
                const int xB = pB < i ? pB : jB;
                aA |= 1ULL << xA;
                aB |= 1ULL << xB;
                jA = L.get(xA);
                jB = L.get(xB);
                dA |= jA == oA;
                dB |= jB == oB;
            }
            good &= aA & aB;
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
// the reference loop would make (mf.c:136-142), position 0 included.
//
// As for sym, the dimensions are walked two at a time side by side.  Setting
// b[l] = l first (leaf l is not placed, so its slot is free until it is
// inserted) makes every walk periodic: after reaching l it goes on to
// d[l][b[l]] = d[l][l], its first position, and retraces itself, so a chain
// that is done can keep stepping while the other finishes.  Bit l, picked up
// on the way through, is not a position and is masked off.
struct LunnonRules {
    const uint8_t *table;  // [dim][n+1][n+1]
    int n;
    int dim;

    // The resumable-walk interface of SymHopRules, with the whole walk done
    // in begin(): capping the Lunnon walks per round measured slower (6x6 at
    // depth 18: 272 -> 387 ms batched), the dimension walks being short and
    // the pair switch inside the capped loop costing more than it saves.
    struct Walk {
        uint64_t mask;
    };
    template <class List>
    __device__ __forceinline__ void begin(const List &L, int l, unsigned long long &nodes,
                                          Walk &w) const {
        w.mask = gaps(L, l, nodes);
    }
    template <class List>
    __device__ __forceinline__ bool run(const List &, Walk &, int) const { return true; }
    __device__ __forceinline__ uint64_t result(const Walk &w, unsigned long long &) const {
        return w.mask;
    }
    template <class List>
    __device__ __forceinline__ uint64_t gaps(const List &L, int l,
                                             unsigned long long &nodes) const {
        const int w = n + 1;
        uint64_t mask = low_bits(l);
        int bound = 0, d = 0;
        L.put(l, l);
        while (mask) {
            const uint8_t *rA = nullptr, *rB = nullptr;
            for (; d < dim && !rB; ++d) {
                const uint8_t *row = table + (d * w + l) * w;
                if (row[l] == l) continue;  // unconstrained dimension
                if (!rA) rA = row;
                else rB = row;
            }
            if (!rA) break;
            if (!rB) rB = rA;
            ++bound;
            int mA = rA[l], mB = rB[l];
            uint64_t wA = 0, wB = 0;
            bool dA = false, dB = false;
            while (!(dA && dB)) {
                wA |= bit64(mA);
                wB |= bit64(mB);
                dA |= mA == l;
                dB |= mB == l;
                mA = rA[L.get(mA)];
                mB = rB[L.get(mB)];
            }
            mask &= wA & wB;
        }
        if (!bound) mask = low_bits(l);
        nodes += __popcll(mask);
        if (l >= 2) mask &= ~1ULL;
        return mask;
    }
};

// ------------------------------------------------------------- stacks ----

// Per-level search state, one 64-bit mask per level: the position the
// level's item is inserted after is the mask's lowest set bit, and the
// higher bits are its untried siblings.  (No separate pick byte: the pick is
// a count-trailing-zeros away, one shared-memory store less per insertion.)
// Levels are stored relative to `base`, the unit's first level.
template <int TPB, int LEVELS>
struct SmemStack {
    static constexpr int kLevels = LEVELS;
    uint64_t *mask;  // &s_mask[threadIdx.x], level k at mask[k * TPB]
    int base;
    __device__ __forceinline__ uint64_t get(int lvl) const { return mask[(lvl - base) * TPB]; }
    __device__ __forceinline__ void set(int lvl, uint64_t v) const { mask[(lvl - base) * TPB] = v; }
};

struct LocalStack {
    static constexpr int kLevels = kLocalLevels;
    uint64_t mask[kLocalLevels];
    int base;
    __device__ __forceinline__ uint64_t get(int lvl) const { return mask[lvl - base]; }
    __device__ __forceinline__ void set(int lvl, uint64_t v) { mask[lvl - base] = v; }
};

__device__ __forceinline__ int low_bit(uint64_t m) { return __ffsll(static_cast<long long>(m)) - 1; }

// ---------------------------------------------------------- DFS core -----
//
// Lockstep form: in every round each busy lane evaluates exactly one node
// (one gaps() call), so a warp's lanes run the expensive walk together no
// matter where each is in its own tree.  Between evaluations a lane
// advances: it backtracks over exhausted levels and inserts its next untried
// item, which names the level to evaluate next.

// Insert item lvl after the lowest position of `cur` (cur != 0) and record
// cur as the level's mask; returns the level to evaluate next.
template <class Stk, class List>
__device__ __forceinline__ int descend(const List &L, Stk &S, int lvl, uint64_t cur) {
    const int j = low_bit(cur);
    S.set(lvl, cur);
    L.put(lvl, L.get(j));  // insert item lvl after j
    L.put(j, lvl);
    return lvl + 1;
}

// Start a split item: S[root] holds the untried positions of level root (never
// empty), no item of level root is inserted yet.  Returns root + 1.
template <class Stk, class List>
__device__ __forceinline__ int advance(const List &L, Stk &S, int &lvl, int root) {
    lvl = root;
    return descend(L, S, root, S.get(root));
}

// Consume the evaluation g of level `eval` and advance to the next node, with
// g handed over in a register.  Items root..eval-1 are inserted.  The last
// level is never entered: its positions are counted.  After a counted last
// level or a dead end the item above is detached and its next sibling, if
// any, inserted; exhausted levels are backtracked over.  Returns the next
// level to evaluate, or -1 when the unit's subtree is exhausted (or a fresh
// unit had nothing left to place).
template <class Stk, class List>
__device__ __forceinline__ int apply_advance(const List &L, Stk &S, int &lvl, int eval,
                                             int root, int last, bool fresh, uint64_t g,
                                             unsigned long long &leaves) {
    if (eval != last && g) {
        lvl = eval;
        return descend(L, S, lvl, g);
    }
    if (eval == last) leaves += __popcll(g);
    if (fresh) return -1;  // a fresh unit: nothing above it to go back to
    lvl = eval - 1;
    for (;;) {
        const uint64_t m = S.get(lvl);
        L.put(low_bit(m), L.get(lvl));  // detach item lvl
        const uint64_t rest = m & (m - 1);
        if (rest) return descend(L, S, lvl, rest);
        if (lvl == root) return -1;
        --lvl;
    }
}

// Donation (splitting a lane's subtree on the device).  Items root..lvl are
// inserted.  The shallowest level s with untried siblings, and those
// siblings (0 if no level has any).
template <class Stk>
__device__ __forceinline__ uint64_t shallowest_siblings(const Stk &S, int root, int lvl, int &s) {
    s = root;
    uint64_t m = S.get(s);
    while (s < lvl && (m & (m - 1)) == 0) m = S.get(++s);
    return m & (m - 1);
}

// Detach items lvl..s, leaving the list as it was before item s was placed.
template <class Stk, class List>
__device__ __forceinline__ void roll_back(const List &L, const Stk &S, int s, int lvl) {
    for (int l = lvl; l >= s; --l) L.put(low_bit(S.get(l)), L.get(l));
}

// Re-insert items s..lvl after roll_back; level s keeps only its current
// pick (its untried siblings have been given away).
template <class Stk, class List>
__device__ __forceinline__ void replay_keeping_pick(const List &L, Stk &S, int s, int lvl) {
    for (int l = s; l <= lvl; ++l) {
        const int j = low_bit(S.get(l));
        L.put(l, L.get(j));
        L.put(j, l);
    }
    const uint64_t ms = S.get(s);
    S.set(s, ms & (~ms + 1));
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

// Shared-memory carve-up of one CTA: [tables][lists][mask stack].
template <int TPB, int WORDS, int LEVELS>
struct Carve {
    static constexpr size_t kList = size_t(WORDS) * 4 * TPB;
    static constexpr size_t kMask = size_t(LEVELS) * 8 * TPB;
    static constexpr size_t kThreadBytes = kList + kMask;
    __device__ static List<TPB> list(uint8_t *smem, size_t tables) {
        return List<TPB>::at(smem + tables, 4 * WORDS);
    }
    __device__ static SmemStack<TPB, LEVELS> stack(uint8_t *smem, size_t tables) {
        SmemStack<TPB, LEVELS> s;
        s.mask = reinterpret_cast<uint64_t *>(smem + tables + kList) + threadIdx.x;
        s.base = 0;
        return s;
    }
};

template <int TPB, int WORDS>
struct Carve<TPB, WORDS, 0> {  // local-memory stack
    static constexpr size_t kList = size_t(WORDS) * 4 * TPB;
    static constexpr size_t kThreadBytes = kList;
    __device__ static List<TPB> list(uint8_t *smem, size_t tables) {
        return List<TPB>::at(smem + tables, 4 * WORDS);
    }
};

template <int TPB, int LEVELS>
struct StackOf {
    using type = SmemStack<TPB, LEVELS>;
};
template <int TPB>
struct StackOf<TPB, 0> {
    using type = LocalStack;
};

template <int TPB, int WORDS, int LEVELS>
__device__ __forceinline__ void init_stack(SmemStack<TPB, LEVELS> &S, uint8_t *smem, size_t tables) {
    S = Carve<TPB, WORDS, LEVELS>::stack(smem, tables);
}
template <int TPB, int WORDS, int LEVELS>
__device__ __forceinline__ void init_stack(LocalStack &S, uint8_t *, size_t) {
    S.base = 0;
}

// Run one loaded unit per lane to completion in lockstep rounds (no refill):
// the plain one-thread-per-unit kernels.  Walks are resumable and take at
// most kWalkCap steps per round.
template <class Rules, class Stk, int TPB>
__device__ __forceinline__ void run_units(const Rules &R, const List<TPB> &L, Stk &S, bool busy,
                                          int root, int last, unsigned long long &leaves,
                                          unsigned long long &nodes) {
    int lvl = root, eval = root;
    bool fresh = true;
    if (busy && root > last) {  // nothing left to place: one completion
        leaves += 1;
        busy = false;
    }
    bool walking = false;
    typename Rules::Walk w;
    while (__any_sync(kFull, busy)) {
        if (busy) {
            if (!walking) {
                R.begin(L, eval, nodes, w);
                walking = true;
            }
            if (R.run(L, w, kWalkCap)) {
                walking = false;
                const uint64_t g = R.result(w, nodes);
                eval = apply_advance(L, S, lvl, eval, root, last, fresh, g, leaves);
                fresh = false;
                busy = eval >= 0;
            }
        }
    }
}

// ---------------------------------------------------------- sym tables ---

// Sym tables in shared memory: the 4 edge pages (256 B), then per cell the
// packed list of pages whose neighbour has a smaller number (256 B) and its
// length (64 B).
constexpr size_t kSymTables = 9 * kSymCells;

template <int TPB>
__device__ __forceinline__ void stage_sym_tables(uint8_t *smem, const uint8_t *__restrict__ edges) {
    for (int k = threadIdx.x; k < 64; k += TPB) {
        reinterpret_cast<uint32_t *>(smem)[k] = __ldg(reinterpret_cast<const uint32_t *>(edges) + k);
        uint32_t q = 0;
        int c = 0;
        for (int p = 0; p < 4; ++p) {
            const int nb = __ldg(edges + p * kSymCells + k);
            if (nb < k) q |= uint32_t(nb | (p << 6)) << (8 * c++);
        }
        reinterpret_cast<uint32_t *>(smem + 4 * kSymCells)[k] = q;
        smem[8 * kSymCells + k] = uint8_t(c);
    }
}

// The counting kernels precompute, per searched level i and per chain k (the
// cell's first or second placed-neighbour page), the position the walk lands
// on from each position j: hop[(i - first) * 128 + k * 64 + j] = j's partner
// on that page if the partner is placed (< i), else j.  A walk step is then
// one table byte and one list byte -- the compare-and-select of get_good's
// `edge[j] < i` test is gone from the walk, which is bound by the integer
// (ALU) pipe.  128 bytes per level: 3.2 KB for the 7x7 search from 24 cells.
__host__ __device__ constexpr size_t sym_hop_bytes(int levels) {
    return size_t(levels > 0 ? levels : 0) * 128;
}

template <int TPB>
__device__ __forceinline__ void stage_sym_hops(uint8_t *hop, const uint8_t *tables, int first,
                                               int levels) {
    const uint32_t *pages = reinterpret_cast<const uint32_t *>(tables + 4 * kSymCells);
    const uint8_t *count = tables + 8 * kSymCells;
    for (int k = threadIdx.x; k < levels * 128; k += TPB) {
        const int i = first + (k >> 7), chain = (k >> 6) & 1, j = k & 63;
        const int c = count[i];
        const uint32_t q = (chain && c > 1) ? (pages[i] >> 8) : pages[i];
        const int p = tables[(q & 0xC0) + j];
        hop[k] = uint8_t(c != 0 && p < i ? p : j);
    }
}

// SymRules with the precomputed hop rows (levels first .. first + levels - 1),
// and a walk that can stop and resume: begin() sets up a node's two chains,
// run() takes at most `cap` steps and says whether both are done, result()
// is the node's mask.  The counting kernels give every walk at most a few
// steps per lockstep round and let unfinished walks go on in the next round:
// a round then lasts as long as that cap, not as long as the longest walk of
// the warp's 32 nodes (about 6 steps per node on average against 14 for the
// longest lane of a round on the 7x7 cases).
struct SymHopRules {
    const uint8_t *hop;
    const uint32_t *pages;
    const uint8_t *count;
    int first;

    struct Walk {
        const uint8_t *hA, *hB;
        uint64_t aA, aB;
        int jA, jB, oA, oB, i;
        bool dA, dB;
    };

    template <class List>
    __device__ __forceinline__ void begin(const List &L, int i, unsigned long long &nodes,
                                          Walk &w) const {
        ++nodes;
        const uint32_t q = pages[i];
        const int c = count[i];
        w.i = i;
        if (c == 0) {
            w.aA = w.aB = ~0ULL;
            w.dA = w.dB = true;
            return;
        }
        const uint32_t qb = c > 1 ? (q >> 8) : q;
        w.oA = q & 63;
        w.oB = qb & 63;
        w.hA = hop + (i - first) * 128;
        w.hB = w.hA + 64;
        w.aA = 1ULL << w.oA;
        w.aB = 1ULL << w.oB;
        w.jA = L.get(w.oA);
        w.jB = L.get(w.oB);
        w.dA = w.jA == w.oA;
        w.dB = w.jB == w.oB;
    }

    template <class List>
    __device__ __forceinline__ bool run(const List &L, Walk &w, int cap) const {
        for (int k = 0; k < cap && !(w.dA && w.dB); ++k) {
            const int xA = w.hA[w.jA];
            const int xB = w.hB[w.jB];
            w.aA |= 1ULL << xA;
            w.aB |= 1ULL << xB;
            w.jA = L.get(xA);
            w.jB = L.get(xB);
            w.dA |= w.jA == w.oA;
            w.dB |= w.jB == w.oB;
        }
        return w.dA && w.dB;
    }

    __device__ __forceinline__ uint64_t result(const Walk &w, unsigned long long &) const {
        return low_bits(w.i) & w.aA & w.aB;
    }

    template <class List>
    __device__ __forceinline__ uint64_t gaps(const List &L, int i,
                                             unsigned long long &nodes) const {
        Walk w;
        begin(L, i, nodes, w);
        run(L, w, 1 << 30);
        return result(w, nodes);
    }
};



// Shared-memory size of the sym tables plus the hop rows of `levels` levels.
__host__ __device__ constexpr size_t sym_tables_bytes(int levels) {
    return 9 * kSymCells + sym_hop_bytes(levels);
}

// Stage the tables and the hop rows of levels first .. first + levels - 1
// (ends with __syncthreads).
template <int TPB>
__device__ __forceinline__ SymHopRules stage_sym_hop_rules(uint8_t *smem,
                                                           const uint8_t *__restrict__ edges,
                                                           int first, int levels) {
    stage_sym_tables<TPB>(smem, edges);
    __syncthreads();
    stage_sym_hops<TPB>(smem + 9 * kSymCells, smem, first, levels);
    __syncthreads();
    return SymHopRules{smem + 9 * kSymCells, reinterpret_cast<const uint32_t *>(smem + 4 * kSymCells),
                       smem + 8 * kSymCells, first};
}

__device__ __forceinline__ SymRules sym_rules(const uint8_t *smem) {
    return SymRules{smem, reinterpret_cast<const uint32_t *>(smem + 4 * kSymCells),
                    smem + 8 * kSymCells};
}

// --------------------------------------------------------- split ring ----

// Bounded multi-producer multi-consumer ring of split items (the sequence-
// numbered cell scheme of D. Vyukov's bounded MPMC queue): cell c holds
// seq == ticket when free for the producer of `ticket`, ticket + 1 once that
// producer has published it, and ticket + capacity once its consumer has
// copied it out.  Producers and consumers only ever claim a cell whose
// sequence already says it is ready for them, so nobody waits on anybody.
struct Queue {
    QueueHeader *hdr;
    TaskRecord *slots;
    unsigned long long *seq;
    unsigned long long capacity;  // power of two
};

__device__ __forceinline__ unsigned long long vload(const unsigned long long *p) {
    return *reinterpret_cast<const volatile unsigned long long *>(p);
}

// Warp-cooperative claim of up to `want` (<= 32) consecutive tickets at the
// ring's head (pop) or tail (push): each lane checks one cell's sequence, and
// one CAS by lane 0 takes the run of ready cells for the whole warp, so a
// warp makes at most one atomic per refill or donation round.  All 32 lanes
// call it; returns the number of tickets taken (warp-uniform), the first in
// `first`.
__device__ __forceinline__ int ring_claim(const Queue &Q, unsigned long long *counter, int want,
                                          bool pop, unsigned long long &first) {
    const int lane = threadIdx.x & 31;
    unsigned long long pos = 0;
    if (lane == 0) pos = vload(counter);
    pos = __shfl_sync(kFull, pos, 0);
    const unsigned long long t = pos + lane;
    const bool ready =
        lane < want && vload(Q.seq + (t & (Q.capacity - 1))) == (pop ? t + 1 : t);
    const unsigned ok = __ballot_sync(kFull, ready);
    const int run = ok == kFull ? 32 : __ffs(~ok) - 1;  // ready cells from lane 0 on
    int got = 0;
    if (lane == 0 && run > 0) got = atomicCAS(counter, pos, pos + run) == pos ? run : 0;
    first = pos;
    return __shfl_sync(kFull, got, 0);
}

// Called once per warp (lane 0) as it leaves a persistent launch, after all
// of its counters are in.  Warps leave early on purpose (idle for wait_limit
// rounds while others still work), so only the last warp out can tell
// whether the launch ended with work unaccounted for -- every initial unit
// handed out and completed == units + split items -- and, if not, raises
// error word kErrWaitLimit: some bounded wait ran out before the work was
// done (a split item that was never published, say).
__device__ __forceinline__ void leave_and_check(QueueHeader *hdr, unsigned long long units) {
    __threadfence();
    const unsigned long long warps = (unsigned long long)gridDim.x * (blockDim.x / 32);
    const unsigned long long out = atomicAdd(&hdr->warps_out, 1ULL) + 1;
    if (out != warps) return;
    __threadfence();
    const bool closed = vload(&hdr->init_next) >= units &&
                        vload(&hdr->completed) == units + vload(&hdr->spawn_tail);
    if (!closed) atomicCAS(&hdr->error, 0u, kErrWaitLimit);
}

// Copy ticket t's item out and free its cell for the producer of t + capacity.
__device__ __forceinline__ void ring_take(const Queue &Q, unsigned long long t, uint32_t (&w)[24]) {
    const unsigned long long cell = t & (Q.capacity - 1);
    __threadfence();
    const uint4 *src = reinterpret_cast<const uint4 *>(Q.slots + cell);
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const uint4 x = __ldcg(src + q);
        w[4 * q] = x.x;
        w[4 * q + 1] = x.y;
        w[4 * q + 2] = x.z;
        w[4 * q + 3] = x.w;
    }
    __threadfence();
    atomicExch(Q.seq + cell, t + Q.capacity);
}

// Write ticket t's item and publish it to its consumer.
__device__ __forceinline__ void ring_put(const Queue &Q, unsigned long long t, const uint32_t (&w)[24]) {
    const unsigned long long cell = t & (Q.capacity - 1);
    uint4 *dst = reinterpret_cast<uint4 *>(Q.slots + cell);
#pragma unroll
    for (int q = 0; q < 6; ++q)
        __stcg(dst + q, make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]));
    __threadfence();
    atomicExch(Q.seq + cell, t + 1);
}

}  // namespace
}  // namespace mf
