// cli_gpu_folding.cpp -- drop-in for the reference's `gpu_folding` binary.
//
//   gpu_folding <grid_size> <partition_depth> [plain|batched] [p1xp2x...]
//
// With the two reference arguments the output is the reference's
// (gpu_folding.cu:209-311): the prefix-state count line and the total line on
// stdout, usage / size errors with rc 1.  Extensions, after them: the kernel
// (default: batched) and an explicit map shape (default grid_size x grid_size).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mapfold.h"

static bool parse_shape(const char *text, std::vector<int32_t> &dims) {
    dims.clear();
    std::string s(text);
    size_t at = 0;
    while (at <= s.size()) {
        size_t x = s.find('x', at);
        std::string part = s.substr(at, x == std::string::npos ? std::string::npos : x - at);
        char *end = nullptr;
        long v = std::strtol(part.c_str(), &end, 10);
        if (part.empty() || *end != '\0' || v < 1) return false;
        dims.push_back(int32_t(v));
        if (x == std::string::npos) break;
        at = x + 1;
    }
    return !dims.empty();
}

int main(int argc, char **argv) {
    if (argc < 3) {
        std::printf("Usage: ./gpu_folding grid_size partition_depth\n");
        std::printf("Example: ./gpu_folding 20 8\n");
        return 1;
    }
    const int grid = std::atoi(argv[1]);
    int depth = std::atoi(argv[2]);
    const long long n_sq = 1LL * grid * grid;
    if (n_sq > MF_MAX_LEAVES) {
        std::printf("Grid too large, max 8 (64 stamps)\n");
        return 1;
    }
    int mode = 1;
    std::vector<int32_t> dims = {grid, grid};
    for (int k = 3; k < argc; ++k) {
        if (std::strcmp(argv[k], "plain") == 0) mode = 0;
        else if (std::strcmp(argv[k], "batched") == 0) mode = 1;
        else if (!parse_shape(argv[k], dims)) {
            std::fprintf(stderr, "bad map shape: %s\n", argv[k]);
            return 1;
        }
    }
    long long n = 1;
    for (int32_t d : dims) n *= d;
    if (grid <= 0 || n <= 0) {
        // The reference collects nothing for an empty map.
        std::printf("Number of partial states at depth %d: %d\n", depth, 0);
        std::printf("Total number of ways: %llu\n", 0ULL);
        return 0;
    }
    if (n > MF_MAX_LEAVES) {
        std::printf("Grid too large, max 8 (64 stamps)\n");
        return 1;
    }
    if (depth < 0) depth = 0;
    if (depth > n) depth = int(n);

    mf_lunnon_plan *plan = nullptr;
    if (mf_lunnon_plan_create(dims.data(), int32_t(dims.size()), &plan) != MF_OK) {
        std::fprintf(stderr, "error: %s\n", mf_last_error());
        return 1;
    }
    uint64_t states = 0;
    mf_lunnon_collect(plan, depth, nullptr, 0, &states);
    std::printf("Number of partial states at depth %d: %llu\n", depth, (unsigned long long)states);
    std::fflush(stdout);
    uint64_t total = 0;
    mf_run_stats st{};
    int rc = mf_lunnon_count(plan, depth, mode, nullptr, &total, nullptr, &st);
    mf_lunnon_plan_destroy(plan);
    if (rc != MF_OK) {
        std::fprintf(stderr, "error: %s\n", mf_last_error());
        return 2;
    }
    std::printf("Total number of ways: %llu\n", (unsigned long long)total);
    std::fprintf(stderr, "mode=%s states=%llu kernel_s=%.6f setup_s=%.6f total_s=%.6f\n",
                 mode ? "batched" : "plain", (unsigned long long)st.units, st.kernel_s, st.setup_s,
                 st.total_s);
    return 0;
}
