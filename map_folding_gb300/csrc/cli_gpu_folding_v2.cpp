// cli_gpu_folding_v2.cpp -- drop-in for the reference's `gpu_folding_v2`.
//
//   gpu_folding_v2 grid depth [batch_size] [threads_per_block] [blocks_per_sm]
//                  [max_gpus] [max_queued_batches] [max_states]
//
// Argument checks, exit codes and output follow gpu_folding_v2.cu:544-699:
// stdout is the decimal count only; stderr carries the key=value lines.
// threads_per_block and blocks_per_sm shape the persistent kernel; batch
// size, GPU count and queue depth are accepted and reported (one GPU, one
// resident launch).  max_states > 0 counts only the first max_states prefix
// states, as the reference's producer stops after them.  Grids are limited to
// 8 (64 leaves) instead of the reference's 9.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "mapfold.h"

namespace {

bool parse_long(const char *text, long &out) {
    char *end = nullptr;
    out = std::strtol(text, &end, 10);
    return *text != '\0' && *end == '\0';
}

bool parse_size(const char *text, unsigned long long &out) {
    char *end = nullptr;
    out = std::strtoull(text, &end, 10);
    return *text != '\0' && *end == '\0';
}

int need_int(const char *text, const char *name, long &out) {
    if (!parse_long(text, out)) {
        std::fprintf(stderr, "Invalid %s: %s\n", name, text);
        std::exit(2);
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 3 || argc > 9) {
        std::fprintf(stderr,
                     "Usage: %s grid depth [batch_size] [threads_per_block] [blocks_per_sm] "
                     "[max_gpus] [max_queued_batches] [max_states]\nExample: %s 6 18 5000 128 8 4 8 0\n",
                     argv[0], argv[0]);
        return 1;
    }
    long grid = 0, depth = 0, batch = 100000, tpb = 128, bpsm = 8, gpus = 0, queued = 8;
    unsigned long long max_states = 0;
    need_int(argv[1], "grid", grid);
    need_int(argv[2], "depth", depth);
    if (argc >= 4) need_int(argv[3], "batch_size", batch);
    if (argc >= 5) need_int(argv[4], "threads_per_block", tpb);
    if (argc >= 6) need_int(argv[5], "blocks_per_sm", bpsm);
    if (argc >= 7) need_int(argv[6], "max_gpus", gpus);
    if (argc >= 8) need_int(argv[7], "max_queued_batches", queued);
    if (argc >= 9 && !parse_size(argv[8], max_states)) {
        std::fprintf(stderr, "Invalid max_states: %s\n", argv[8]);
        return 2;
    }
    // gpu_folding_v2.cu:594-607 (MAX_GRID 9); the engine's Lunnon search
    // holds at most 64 leaves, so a 9x9 grid is refused after these checks.
    if (grid < 1 || grid > 9) {
        std::fprintf(stderr, "grid must be between 1 and 9\n");
        return 1;
    }
    const long n = grid * grid;
    if (depth < 1 || depth > n) {
        std::fprintf(stderr, "depth must be between 1 and %ld\n", n);
        return 1;
    }
    if (batch < 1 || tpb < 1 || bpsm < 1 || queued < 1) {
        std::fprintf(stderr,
                     "batch_size, threads_per_block, blocks_per_sm, and max_queued_batches must be positive\n");
        return 1;
    }
    if (n > 64) {
        std::fprintf(stderr, "a %ldx%ld map has %ld leaves; this engine counts maps of up to 64\n",
                     grid, grid, n);
        return 1;
    }
    const auto t0 = std::chrono::steady_clock::now();
    std::fprintf(stderr, "gpus=1 batch_size=%ld threads_per_block=%ld blocks_per_sm=%ld "
                 "max_queued_batches=%ld max_states=%llu\n",
                 batch, tpb, bpsm, queued, max_states);
    const int32_t dims[2] = {int32_t(grid), int32_t(grid)};
    mf_lunnon_plan *plan = nullptr;
    if (mf_lunnon_plan_create(dims, 2, &plan) != MF_OK) {
        std::fprintf(stderr, "%s\n", mf_last_error());
        return 1;
    }
    mf_batch_config cfg{};
    cfg.block_threads = uint32_t(tpb);
    cfg.blocks_per_sm = uint32_t(bpsm);
    uint64_t count = 0, states = 0;
    mf_run_stats st{};
    const int rc = mf_lunnon_count_range(plan, int32_t(depth), 0, max_states, 1, &cfg, &count,
                                         &states, &st);
    mf_lunnon_plan_destroy(plan);
    if (rc != MF_OK) {
        std::fprintf(stderr, "%s\n", mf_last_error());
        return 1;
    }
    const double total_s =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::fprintf(stderr, "grid=%ld depth=%ld states=%llu collect_s=%g\n", grid, depth,
                 (unsigned long long)states, st.setup_s);
    std::printf("%llu\n", (unsigned long long)count);
    std::fprintf(stderr, "solve_s=%g total_s=%g\n", st.total_s - st.setup_s, total_s);
    return 0;
}
