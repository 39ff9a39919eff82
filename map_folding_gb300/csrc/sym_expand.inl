// sym_expand.inl -- DFS expansion of sym cases in emission order.
#pragma once

namespace mf {

namespace detail {
template <class F>
bool sym_expand_rec(uint8_t *cycle, int i, int stop, const uint8_t *edges, F &emit) {
    if (i == stop) return emit(static_cast<const uint8_t *>(cycle));
    uint64_t good = sym_good_host(cycle, i, edges);
    while (good) {
        int j = __builtin_ctzll(good);
        good &= good - 1;
        uint8_t after = cycle[j];
        cycle[i] = after;
        cycle[j] = static_cast<uint8_t>(i);
        bool go_on = sym_expand_rec(cycle, i + 1, stop, edges, emit);
        cycle[j] = after;
        if (!go_on) return false;
    }
    return true;
}
}  // namespace detail

// Cases are emitted lowest insertion position first, the order in which
// sym_fold.cpp:491-527 numbers them.
template <class F>
bool sym_expand(uint8_t *cycle, int from, int stop, const uint8_t *edges, F &&emit) {
    return detail::sym_expand_rec(cycle, from, stop, edges, emit);
}

namespace detail {
template <class F>
bool sym_expand_wide_rec(uint8_t *cycle, int i, int stop, const uint8_t *wide_edges, F &emit) {
    if (i == stop) return emit(static_cast<const uint8_t *>(cycle));
    uint64_t lo = 0, hi = 0;
    sym_good_host_wide(cycle, i, wide_edges, lo, hi);
    for (int half = 0; half < 2; ++half) {
        uint64_t good = half ? hi : lo;
        while (good) {
            const int j = __builtin_ctzll(good) + 64 * half;
            good &= good - 1;
            const uint8_t after = cycle[j];
            cycle[i] = after;
            cycle[j] = static_cast<uint8_t>(i);
            const bool go_on = sym_expand_wide_rec(cycle, i + 1, stop, wide_edges, emit);
            cycle[j] = after;
            if (!go_on) return false;
        }
    }
    return true;
}
}  // namespace detail

// sym_expand on boards over 64 cells with 128-bit masks
// (experiments/9x9/sym_fold9.cpp:286-312): `cycle` holds kWideCells cells,
// `wide_edges` the 4 pages of kWideCells.  Same emission order.
template <class F>
bool sym_expand_wide(uint8_t *cycle, int from, int stop, const uint8_t *wide_edges, F &&emit) {
    return detail::sym_expand_wide_rec(cycle, from, stop, wide_edges, emit);
}

}  // namespace mf
