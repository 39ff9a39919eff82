// host.cpp -- host-side tables, prefix-state generation and sym case setup.
//
// Everything here is one-time or per-request setup that the reference also
// runs on the host; the counting itself runs in the kernels (dfs_kernels.cu).
#include <algorithm>
#include <array>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <set>
#include <thread>
#include <unordered_set>

#include "engine.hpp"

namespace mf {

// ------------------------------------------------------------- errors ----
namespace {
thread_local char g_error[512] = {0};
}

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}

void clear_error() { g_error[0] = '\0'; }
const char *last_error() { return g_error; }

double now_seconds() {
    using clock = std::chrono::steady_clock;
    return std::chrono::duration<double>(clock::now().time_since_epoch()).count();
}

// ------------------------------------------------------------- Lunnon ----

// mf.c:29-75.  Leaf m (1-based) has mixed-radix digits (m-1) in the radices
// p1, p2, ...; coordinate = digit + 1.  Moving from m along dimension i goes
// down a stride when m and l have coordinates of equal parity (unless m is
// on the low face), otherwise up a stride (unless m is on the high face or
// the leaf above is not yet placed).
bool build_lunnon_tables(const int32_t *dims, int ndim, LunnonTables &t, std::string &why) {
    if (dims == nullptr || ndim < 1 || ndim > MF_MAX_DIMS) {
        why = "dimension count must be 1.." + std::to_string(MF_MAX_DIMS);
        return false;
    }
    long long n = 1;
    for (int i = 0; i < ndim; ++i) {
        if (dims[i] < 1) {
            why = "every dimension must be >= 1";
            return false;
        }
        n *= dims[i];
        if (n > MF_MAX_LEAVES) {
            why = "map too large: at most 64 leaves";
            return false;
        }
    }
    t.n = int(n);
    t.dim = ndim;
    t.stride[0] = 1;
    for (int i = 0; i < ndim; ++i) {
        t.p[i] = dims[i];
        t.stride[i + 1] = t.stride[i] * dims[i];
    }
    const int w = t.n + 1;
    t.next.assign(size_t(ndim) * w * w, 0);
    std::vector<int> coord(w);
    for (int i = 0; i < ndim; ++i) {
        const int step = t.stride[i];
        const int side = dims[i];
        for (int m = 1; m <= t.n; ++m) coord[m] = ((m - 1) / step) % side + 1;
        for (int l = 1; l <= t.n; ++l) {
            uint8_t *row = &t.next[(size_t(i) * w + l) * w];
            for (int m = 1; m <= l; ++m) {
                int to = m;
                if (((coord[l] ^ coord[m]) & 1) == 0) {
                    if (coord[m] != 1) to = m - step;
                } else if (coord[m] != side && m + step <= l) {
                    to = m + step;
                }
                row[m] = uint8_t(to);
            }
        }
    }
    return true;
}

int default_lunnon_depth(const LunnonTables &t) {
    // Enough prefixes to fill the GPU several times over for the larger maps,
    // few enough that host generation stays in the millisecond range.
    int d = t.n / 2 + 3;
    if (t.n >= 30) d = t.n / 2;
    if (d > t.n) d = t.n;
    return d;
}

namespace {

// One level of the host search: the surviving gap positions for the leaf of
// this level, in the order mf.c:118-124 leaves them on its stack; the search
// consumes them from the end (mf.c:137, `gap[--g]`).
struct GapFrame {
    uint8_t pos[MF_MAX_LEAVES + 1];
    int count = 0;
    int left = 0;
};

void compute_frame(const LunnonTables &t, const uint8_t *b, int l, GapFrame &f, int *hits) {
    f.count = 0;
    uint8_t order[MF_MAX_LEAVES + 1];
    int distinct = 0;
    int bound = 0;
    for (int i = 0; i < t.dim; ++i) {
        int m = t.at(i, l, l);
        if (m == l) continue;
        ++bound;
        while (m != l) {
            if (hits[m]++ == 0) order[distinct++] = uint8_t(m);
            m = t.at(i, l, b[m]);
        }
    }
    if (bound == 0) {
        for (int m = 0; m < l; ++m) f.pos[f.count++] = uint8_t(m);
    } else {
        for (int k = 0; k < distinct; ++k) {
            int m = order[k];
            if (hits[m] == bound) f.pos[f.count++] = uint8_t(m);
            hits[m] = 0;
        }
    }
    f.left = f.count;
}

}  // namespace

uint64_t collect_lunnon_states(const LunnonTables &t, int depth, uint8_t *out, uint64_t cap,
                               uint32_t stride, uint64_t first) {
    const int n = t.n;
    if (depth < 0) depth = 0;
    if (depth > n) depth = n;
    uint8_t a[MF_MAX_LEAVES + 2] = {0};
    uint8_t b[MF_MAX_LEAVES + 2] = {0};
    int hits[MF_MAX_LEAVES + 2] = {0};
    std::vector<GapFrame> frames(n + 2);
    uint64_t found = 0;

    auto enter = [&](int l) {
        GapFrame &f = frames[l];
        f.count = f.left = 0;
        if (l >= 2 && b[0] != 1) return;  // normal-form filter, mf.c:83
        if (l > depth) {
            if (out != nullptr && found >= first && found - first < cap) {
                uint8_t *rec = out + (found - first) * stride;
                std::memset(rec, 0, stride);
                std::memcpy(rec, b, size_t(n) + 1);
            }
            ++found;
            return;
        }
        compute_frame(t, b, l, f, hits);
    };

    int l = 1;
    enter(1);
    for (;;) {
        GapFrame &f = frames[l];
        if (f.left > 0) {
            const int m = f.pos[--f.left];
            a[l] = uint8_t(m);
            b[l] = b[m];
            b[m] = uint8_t(l);
            a[b[l]] = uint8_t(l);
            ++l;
            enter(l);
        } else {
            --l;
            if (l == 0) break;
            b[a[l]] = b[l];
            a[b[l]] = a[l];
        }
    }
    return found;
}

// ---------------------------------------------------------------- sym ----

namespace {

// Inward spiral from (0,0), heading +x, turning left-handed when the next
// cell is off the board or taken; numbers count down to 0 at the centre.
// sym_fold.cpp:122-145.  Result indexed [x*h + y].
std::vector<int> spiral_numbers(int w, int h) {
    const int cells = w * h;
    std::vector<int> num(cells, -1);
    int x = 0, y = 0, dx = 1, dy = 0;
    for (int v = cells - 1; v >= 0; --v) {
        num[x * h + y] = v;
        int nx = x + dx, ny = y + dy;
        bool blocked = nx < 0 || nx >= w || ny < 0 || ny >= h || num[nx * h + ny] >= 0;
        if (blocked) {
            std::swap(dx, dy);
            dx = -dx;
            nx = x + dx;
            ny = y + dy;
        }
        x = nx;
        y = ny;
    }
    return num;
}

}  // namespace

void sym_edges_stride(int n, uint8_t *out, int stride) {
    const int cells = n * n;
    std::memset(out, cells, 4 * size_t(stride));
    auto num = spiral_numbers(n, n);
    // Cells at or beyond `stride` get no entry (a 64-cell projection of a
    // 9x9 board keeps cells 0..63 with partners up to 80, which every search
    // below 64 cells treats as not yet placed).
    auto link = [&](int page, int u, int v) {
        if (u < stride) out[page * stride + u] = uint8_t(v);
        if (v < stride) out[page * stride + v] = uint8_t(u);
    };
    // sym_fold.cpp:147-173: x-edges go to page x%2, y-edges to page 2+y%2.
    for (int x = 0; x < n; ++x)
        for (int y = 0; y < n; ++y) {
            if (x > 0) link(x % 2, num[x * n + y], num[(x - 1) * n + y]);
            if (y > 0) link(2 + y % 2, num[x * n + y], num[x * n + y - 1]);
        }
}

void sym_edges(int n, uint8_t *out) { sym_edges_stride(n, out, kSymCells); }

// sym_fold.cpp:179-204.
uint64_t sym_good_host(const uint8_t *cycle, int i, const uint8_t *edges) {
    uint64_t good = i >= 64 ? ~0ULL : ((1ULL << i) - 1);
    for (int page = 0; page < 4; ++page) {
        const uint8_t *e = edges + page * kSymCells;
        const int other = e[i];
        if (other >= i) continue;
        uint64_t allowed = 1ULL << other;
        for (int j = cycle[other]; j != other; j = cycle[j]) {
            if (e[j] < i) j = e[j];
            allowed |= 1ULL << j;
        }
        good &= allowed;
        if (!good) return 0;
    }
    return good;
}

// sym_fold9.cpp:286-312: get_good with 128-bit masks over kWideCells cells.
void sym_good_host_wide(const uint8_t *cycle, int i, const uint8_t *wide_edges, uint64_t &lo,
                        uint64_t &hi) {
    lo = i >= 64 ? ~0ULL : ((1ULL << i) - 1);
    hi = i <= 64 ? 0 : (i >= 128 ? ~0ULL : ((1ULL << (i - 64)) - 1));
    for (int page = 0; page < 4; ++page) {
        const uint8_t *e = wide_edges + page * kWideCells;
        const int other = e[i];
        if (other >= i) continue;
        uint64_t alo = 0, ahi = 0;
        auto mark = [&](int x) {
            if (x < 64) alo |= 1ULL << x;
            else ahi |= 1ULL << (x - 64);
        };
        mark(other);
        for (int j = cycle[other]; j != other; j = cycle[j]) {
            if (e[j] < i) j = e[j];
            mark(j);
        }
        lo &= alo;
        hi &= ahi;
        if (!lo && !hi) return;
    }
}

namespace {

constexpr int kMaxCentre = 25;  // 5 x 5 centre (experiments/9x9/sym_fold9.cpp:33)

size_t host_threads() {
    const unsigned hw = std::thread::hardware_concurrency();
    return hw ? hw : 1;
}

// A centre cycle packed into one integer: cell v's successor (< 25, 5 bits)
// at bits 5v..5v+4.  Equal cycles give equal keys.
using CentreKey = unsigned __int128;

struct CentreKeyHash {
    size_t operator()(CentreKey k) const {
        const uint64_t lo = uint64_t(k), hi = uint64_t(k >> 64);
        uint64_t h = lo * 0x9E3779B97F4A7C15ULL ^ (hi + 0x632BE59BD9B4E019ULL) * 0xC2B2AE3D27D4EB4FULL;
        return size_t(h ^ (h >> 29));
    }
};

// The eight symmetries of the c x c centre as permutations of its own
// spiral numbering (sym_fold.cpp:316-350).
std::vector<std::array<uint8_t, kMaxCentre>> centre_symmetries(int c) {
    auto num = spiral_numbers(c, c);
    std::vector<int> px(c * c), py(c * c);
    for (int x = 0; x < c; ++x)
        for (int y = 0; y < c; ++y) {
            px[num[x * c + y]] = x;
            py[num[x * c + y]] = y;
        }
    const int e = c - 1;
    std::vector<std::array<uint8_t, kMaxCentre>> out;
    for (int t = 0; t < 8; ++t) {
        std::array<uint8_t, kMaxCentre> perm;
        perm.fill(255);
        for (int v = 0; v < c * c; ++v) {
            int x = px[v], y = py[v];
            // identity, transpose, and their compositions with the flips
            int u = (t & 1) ? y : x;
            int w = (t & 1) ? x : y;
            int tx, ty;
            switch (t >> 1) {
                case 0: tx = u; ty = w; break;
                case 1: tx = u; ty = e - w; break;
                case 2: tx = e - u; ty = w; break;
                default: tx = e - u; ty = e - w; break;
            }
            perm[v] = uint8_t(num[tx * c + ty]);
        }
        out.push_back(perm);
    }
    return out;
}

}  // namespace

int build_sym_plan(int n, int expanded_n, SymPlan &plan, std::string &why, int center_n,
                   uint64_t seed_start, uint64_t seed_count) {
    if (n < 6 || n > 9) {
        why = "symmetry plan needs n in 6..9";
        return MF_ERR_ARG;
    }
    plan = SymPlan{};
    plan.n = n;
    // sym_fold.cpp:703 (c = 3 odd, 4 even); experiments/9x9/sym_fold9.cpp:
    // 969-981 adds MF_CENTER_N and a 5x5 default for 9x9.
    plan.c = center_n > 0 ? center_n : (n >= 9 ? 5 : ((n % 2 == 0) ? 4 : 3));
    if (plan.c < 3 || plan.c > n || plan.c * plan.c > kMaxCentre || (plan.c % 2) != (n % 2)) {
        why = "MF_CENTER_N must be between 3 and " + std::to_string(n) +
              ", have the same parity as n, and fit a 5x5 centre";
        return MF_ERR_ARG;
    }
    plan.seed_i = plan.c * plan.c;
    const int n2 = n * n;
    if (n >= 7) {
        if (expanded_n <= 0) expanded_n = std::max(24, plan.seed_i);
        if (expanded_n < plan.seed_i || expanded_n > n2) {
            why = "MF_EXPANDED_N must be between " + std::to_string(plan.seed_i) + " and " +
                  std::to_string(n2);
            return MF_ERR_ARG;
        }
        plan.start_i = expanded_n;
    } else {
        plan.start_i = plan.seed_i;
    }
    if (plan.start_i > kSymCells) {  // only boards over 64 cells get here (9x9)
        plan.streamed = true;
        plan.case_bytes = kWideCells;
    }
    plan.edges.resize(4 * kSymCells);
    sym_edges(n, plan.edges.data());  // boards over 64 cells: the 64-cell projection
    if (n2 > kSymCells) {
        plan.wide_edges.resize(4 * kWideCells);
        sym_edges_stride(n, plan.wide_edges.data(), kWideCells);
    }
    const uint8_t *edges = plan.edges.data();

    // Centre cycles: every cycle of the c*c centre cells (sym_fold.cpp:703-707),
    // deduplicated in generation order (sym_fold9.cpp:601-627 gives the same
    // representatives in the same order as deduplicating the stored list):
    // orbit representatives under the square's symmetries and reversal of the
    // stack, sym_fold.cpp:361-408; the multiplier is the orbit size.  An
    // orbit's canonical key is the least of its 16 images.
    uint8_t cyc[kSymCells] = {0};
    cyc[0] = 1;
    cyc[1] = 2;
    cyc[2] = 0;
    const int c2 = plan.seed_i;
    const auto perms = centre_symmetries(plan.c);
    // 1. Every centre cycle in DFS order (c2 bytes each; cells past c2 stay 0).
    std::vector<uint8_t> centres;
    sym_expand(cyc, 3, c2, edges, [&](const uint8_t *cy) {
        centres.insert(centres.end(), cy, cy + c2);
        return true;
    });
    const size_t count = centres.size() / size_t(c2);
    plan.center_cases = count;
    // 2. Canonical key and orbit size of each, on all host threads.  The
    // image under a symmetry maps perm[u] to perm[cy[u]]; the reversed stack
    // is its inverse (the centre is one cycle over all c2 cells), mapping
    // perm[cy[u]] to perm[u].  Both keys in one pass.
    std::vector<CentreKey> canon(count);
    std::vector<uint8_t> orbit_size(count);
    auto keys = [&](size_t lo, size_t hi) {
        for (size_t k = lo; k < hi; ++k) {
            const uint8_t *cy = &centres[k * size_t(c2)];
            std::array<CentreKey, 16> orbit{};
            int orbit_len = 0;
            for (const auto &perm : perms) {
                CentreKey img = 0, rev = 0;
                for (int u = 0; u < c2; ++u) {
                    const int pu = perm[u], pc = perm[cy[u]];
                    img |= CentreKey(pc) << (5 * pu);
                    rev |= CentreKey(pu) << (5 * pc);
                }
                orbit[orbit_len++] = img;
                orbit[orbit_len++] = rev;
            }
            std::sort(orbit.begin(), orbit.begin() + orbit_len);
            canon[k] = orbit[0];
            orbit_size[k] =
                uint8_t(std::unique(orbit.begin(), orbit.begin() + orbit_len) - orbit.begin());
        }
    };
    const size_t workers = count < 65536 ? 1 : std::min<size_t>(host_threads(), 64);
    if (workers <= 1) {
        keys(0, count);
    } else {
        std::vector<std::thread> pool;
        const size_t step = (count + workers - 1) / workers;
        for (size_t lo = 0; lo < count; lo += step)
            pool.emplace_back(keys, lo, std::min(count, lo + step));
        for (auto &t : pool) t.join();
    }
    // 3. In DFS order, a cycle is a representative when its orbit's key is
    // new: the orbits partition the cycles, so that is the same test as
    // looking the cycle up among all earlier orbits' members.
    std::unordered_set<CentreKey, CentreKeyHash> seen;
    seen.reserve(count / 4 + 16);
    for (size_t k = 0; k < count; ++k) {
        if (!seen.insert(canon[k]).second) continue;
        const size_t at = plan.reps.size();
        plan.reps.resize(at + kSymCells, 0);
        std::memcpy(&plan.reps[at], &centres[k * size_t(c2)], size_t(c2));
        plan.rep_mult.push_back(orbit_size[k]);
    }
    plan.reduced_all = plan.rep_mult.size();
    // sym_fold9.cpp:1071-1088: MF_SEED_START / MF_SEED_COUNT slice the
    // representatives; case indices then run within the slice.
    if (seed_start > 0 || seed_count > 0) {
        const uint64_t reps = plan.rep_mult.size();
        const uint64_t lo = std::min(seed_start, reps);
        // Saturating: a count past the end (or one that would wrap) runs to it.
        const uint64_t hi = seed_count && seed_count < reps - lo ? lo + seed_count : reps;
        plan.reps = std::vector<uint8_t>(plan.reps.begin() + long(lo * kSymCells),
                                         plan.reps.begin() + long(hi * kSymCells));
        plan.rep_mult = std::vector<uint64_t>(plan.rep_mult.begin() + long(lo),
                                              plan.rep_mult.begin() + long(hi));
        plan.seed_base = lo;
    }

    // Expansion index.  Up to depth 24 the prefixes are few enough (~0.4 M
    // for 7x7 and 8x8) to list on the host; deeper cases are counted per
    // depth-24 prefix on the GPU when the index is completed.
    plan.mid_i = std::min(plan.start_i, 24);
    if (plan.mid_i < plan.seed_i) plan.mid_i = plan.seed_i;
    const size_t reps = plan.rep_mult.size();
    for (size_t r = 0; r < reps; ++r) {
        std::memcpy(cyc, &plan.reps[r * kSymCells], kSymCells);
        const uint64_t mult = plan.rep_mult[r];
        sym_expand(cyc, plan.seed_i, plan.mid_i, edges, [&](const uint8_t *c) {
            plan.mid_cycles.insert(plan.mid_cycles.end(), c, c + kSymCells);
            plan.mid_mult.push_back(mult);
            return true;
        });
    }
    const uint64_t mids = plan.mid_mult.size();
    if (plan.mid_i == plan.start_i) {
        plan.mid_first.resize(mids + 1);
        for (uint64_t k = 0; k <= mids; ++k) plan.mid_first[k] = k;
        plan.total_cases = mids;
    }
    // else: mid_first is filled by the index completion (needs the GPU),
    // except for streamed plans, which have none.
    return MF_OK;
}

void sym_sort_order(const uint64_t *scores, const uint64_t *mults, uint64_t count, bool ascending,
                    uint64_t *perm) {
    struct Scored {
        uint64_t score;
        uint64_t mult;
        uint64_t index;
    };
    std::vector<Scored> v(count);
    for (uint64_t k = 0; k < count; ++k) v[k] = Scored{scores[k], mults[k], k};
    std::sort(v.begin(), v.end(), [&](const Scored &a, const Scored &b) {
        if (a.score == b.score) return a.mult < b.mult;
        return ascending ? a.score < b.score : a.score > b.score;
    });
    for (uint64_t k = 0; k < count; ++k) perm[k] = v[k].index;
}

uint64_t sym_select_cases(const SymPlan &plan, uint64_t start, uint64_t max_cases,
                          uint8_t *cycles, uint64_t *mults, uint64_t cap) {
    if (!plan.sorted_mult.empty()) {  // cost-sorted order
        const uint64_t total = plan.sorted_mult.size();
        if (start >= total) return 0;
        uint64_t end = total;
        if (max_cases != 0 && max_cases < end - start) end = start + max_cases;
        for (uint64_t k = start; k < end && k - start < cap; ++k) {
            if (cycles) std::memcpy(cycles + (k - start) * kSymCells, &plan.sorted_cycles[k * kSymCells],
                                    kSymCells);
            if (mults) mults[k - start] = plan.sorted_mult[k];
        }
        return end - start;
    }
    if (plan.streamed) {
        // Walk the cases in emission order from the first (sym_fold9's stream
        // mode), expanding each depth-mid prefix past 64 cells with 128-bit
        // masks; max_cases must be given (the total is unknown).
        if (max_cases == 0) return 0;
        uint64_t skip = start, got = 0;
        const uint64_t mids = plan.mid_mult.size();
        uint8_t cyc[kWideCells];
        for (uint64_t k = 0; k < mids && got < max_cases; ++k) {
            std::memset(cyc, 0, sizeof(cyc));
            std::memcpy(cyc, &plan.mid_cycles[k * kSymCells], kSymCells);
            const uint64_t mult = plan.mid_mult[k];
            sym_expand_wide(cyc, plan.mid_i, plan.start_i, plan.wide_edges.data(),
                            [&](const uint8_t *c) {
                                if (skip > 0) {
                                    --skip;
                                    return true;
                                }
                                if (got < cap) {
                                    if (cycles) std::memcpy(cycles + got * kWideCells, c, kWideCells);
                                    if (mults) mults[got] = mult;
                                }
                                ++got;
                                return got < max_cases;
                            });
        }
        return got;
    }
    if (plan.mid_first.empty() || start >= plan.total_cases) return 0;
    uint64_t end = plan.total_cases;
    if (max_cases != 0 && max_cases < end - start) end = start + max_cases;
    const uint64_t want = end - start;
    uint64_t got = 0;
    if (plan.mid_i == plan.start_i) {
        for (uint64_t k = start; k < end; ++k, ++got) {
            if (got < cap) {
                if (cycles) std::memcpy(cycles + got * kSymCells, &plan.mid_cycles[k * kSymCells],
                                        kSymCells);
                if (mults) mults[got] = plan.mid_mult[k];
            }
        }
        return got;
    }
    // First depth-mid prefix whose case range contains `start`.
    auto it = std::upper_bound(plan.mid_first.begin(), plan.mid_first.end(), start);
    uint64_t k = uint64_t(it - plan.mid_first.begin()) - 1;
    uint64_t skip = start - plan.mid_first[k];
    const uint64_t mids = plan.mid_mult.size();
    uint8_t cyc[kSymCells];
    for (; k < mids && got < want; ++k) {
        std::memcpy(cyc, &plan.mid_cycles[k * kSymCells], kSymCells);
        const uint64_t mult = plan.mid_mult[k];
        sym_expand(cyc, plan.mid_i, plan.start_i, plan.edges.data(), [&](const uint8_t *c) {
            if (skip > 0) {
                --skip;
                return true;
            }
            if (got < cap) {
                if (cycles) std::memcpy(cycles + got * kSymCells, c, kSymCells);
                if (mults) mults[got] = mult;
            }
            ++got;
            return got < want;
        });
        skip = 0;
    }
    return got;
}

}  // namespace mf
