// cli_sym_fold.cpp -- drop-in for the reference's `sym_fold` binary.
//
//   sym_fold n [threads] [max_cases] [start_case]
//
// Same argument checks, exit codes, stdout (one decimal line) and stderr
// key=value lines as sym_fold.cpp:622-774, including MF_STREAM_CASES,
// MF_EXPANDED_N and MF_SETUP_ONLY.  The counting runs on the GPU; `threads`
// is accepted and echoed.  MF_GPU_MODE=plain selects the one-thread-per-case
// kernel instead of the batched work-stealing one.  A long chunk runs as
// consecutive pieces of about 5 s, so that a progress thread can print the
// reference's progress lines with exact finished-case counts.
//
// Built with -DMF_SYM_FOLD9 this is the drop-in for
// experiments/9x9/sym_fold9.cpp instead: n up to 9, MF_CENTER_N (5x5 centre
// by default on 9x9), MF_SEED_START / MF_SEED_COUNT and its stderr lines
// (sym_fold9.cpp:963-1198); counting past cell 63 uses the 128-bit kernel.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>

#include "mapfold.h"

namespace {

using Clock = std::chrono::steady_clock;

double since(Clock::time_point t) {
    return std::chrono::duration<double>(Clock::now() - t).count();
}

std::string decimal(uint64_t lo, uint64_t hi) {
    unsigned __int128 v = (static_cast<unsigned __int128>(hi) << 64) | lo;
    if (v == 0) return "0";
    std::string s;
    while (v) {
        s.insert(s.begin(), char('0' + int(v % 10)));
        v /= 10;
    }
    return s;
}

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

// Cases selected for the device and cases whose count is back, for the
// progress lines.
struct Progress {
    std::atomic<unsigned long long> selected{0}, completed{0};
    std::atomic<int> producer_done{0};
};

// The reference's progress thread (sym_fold.cpp:442-454 materialized,
// :574-589 streaming): a line every 5 s while the count runs, none after.
class ProgressPrinter {
  public:
    ProgressPrinter(const Progress &p, bool stream, unsigned long long planned)
        : p_(p), stream_(stream), planned_(planned), start_(Clock::now()), thread_([this] { run(); }) {}
    ~ProgressPrinter() {
        {
            std::lock_guard<std::mutex> lock(mu_);
            done_ = true;
        }
        cv_.notify_all();
        thread_.join();
    }

  private:
    void run() {
        std::unique_lock<std::mutex> lock(mu_);
        while (!done_) {
            if (cv_.wait_for(lock, std::chrono::seconds(5), [this] { return done_; })) break;
            const unsigned long long c = p_.completed.load();
            const double el = since(start_);
            const double rate = el > 0.0 ? double(c) / el : 0.0;
            if (stream_)
                std::fprintf(stderr,
                             "stream selected=%llu completed=%llu producer_done=%d rate=%g/s elapsed_s=%g\n",
                             p_.selected.load(), c, p_.producer_done.load(), rate, el);
            else
                std::fprintf(stderr, "progress=%llu/%llu rate=%g/s elapsed_s=%g\n", c, planned_, rate, el);
        }
    }

    const Progress &p_;
    const bool stream_;
    const unsigned long long planned_;
    const Clock::time_point start_;
    std::mutex mu_;
    std::condition_variable cv_;
    bool done_ = false;
    std::thread thread_;  // last: starts once the members above exist
};

void usage(const char *exe) {
    std::fprintf(stderr, "Usage: %s n [threads] [max_cases] [start_case]\nExample: %s 6 12\n", exe,
                 exe);
}

}  // namespace

#ifdef MF_SYM_FOLD9
constexpr long kMaxN = 9;
#else
constexpr long kMaxN = 8;
#endif

int main(int argc, char **argv) {
    if (argc < 2 || argc > 5) {
        usage(argv[0]);
        return 1;
    }
    long n = 0;
    if (!parse_long(argv[1], n)) {
        std::fprintf(stderr, "Invalid n: %s\n", argv[1]);
        return 2;
    }
    if (n < 1 || n > kMaxN) {
        std::fprintf(stderr, "n must be between 1 and %ld\n", kMaxN);
        return 1;
    }
    unsigned hw = std::thread::hardware_concurrency();
    long threads = hw == 0 ? 1 : long(hw);
    if (argc >= 3 && !parse_long(argv[2], threads)) {
        std::fprintf(stderr, "Invalid threads: %s\n", argv[2]);
        return 2;
    }
    if (threads < 1) {
        std::fprintf(stderr, "threads must be positive\n");
        return 1;
    }
    unsigned long long max_cases = 0, start_case = 0;
    if (argc >= 4 && !parse_size(argv[3], max_cases)) {
        std::fprintf(stderr, "Invalid max_cases: %s\n", argv[3]);
        return 2;
    }
    if (argc >= 5 && !parse_size(argv[4], start_case)) {
        std::fprintf(stderr, "Invalid start_case: %s\n", argv[4]);
        return 2;
    }
    const auto t0 = Clock::now();
    if (n <= 1) {
        std::printf("1\n");
        return 0;
    }
    if (n == 2) {
        std::printf("8\n");
        return 0;
    }
    const char *mode_env = std::getenv("MF_GPU_MODE");
    const int mode = (mode_env && std::strcmp(mode_env, "plain") == 0) ? 0 : 1;
    const bool stream = std::getenv("MF_STREAM_CASES") != nullptr;
    int expanded_n = 24;
    if (const char *e = std::getenv("MF_EXPANDED_N")) expanded_n = std::atoi(e);

    uint64_t answer[2] = {0, 0};
    mf_run_stats st{};
    if (n <= 5) {
        if (mf_sym_solve(int32_t(n), 0, 0, 0, mode, nullptr, answer, &st) != MF_OK) {
            std::fprintf(stderr, "error: %s\n", mf_last_error());
            return 2;
        }
        // answer = 2 n^2 raw
        unsigned __int128 a = (static_cast<unsigned __int128>(answer[1]) << 64) | answer[0];
        unsigned __int128 raw = a / (2 * n * n);
        std::fprintf(stderr, "raw_count=%s\n", decimal(uint64_t(raw), uint64_t(raw >> 64)).c_str());
    } else {
        mf_sym_plan_options opts{};
        int c = (n % 2 == 0) ? 4 : 3;
        std::string bad_seed;  // reported after the centre lines, as the reference does
#ifdef MF_SYM_FOLD9
        // sym_fold9.cpp:969-981.
        if (n >= 9) c = 5;
        if (const char *text = std::getenv("MF_CENTER_N")) c = std::atoi(text);
        if (c < 3 || c > n || c * c > 25 || (c % 2) != (n % 2)) {
            std::fprintf(stderr,
                         "MF_CENTER_N must be between 3 and %ld, have the same parity as n, and fit "
                         "MAX_CENTER=25\n", n);
            return 2;
        }
        opts.center_n = c;
        unsigned long long seed_start = 0, seed_count = 0;
        const char *seed_start_text = std::getenv("MF_SEED_START");
        // sym_fold9.cpp:1071-1086 parses the slice after the centre setup and
        // exits 2 on bad text there.
        if (seed_start_text) {
            const char *count_text = std::getenv("MF_SEED_COUNT");
            if (!parse_size(seed_start_text, seed_start))
                bad_seed = std::string("Invalid MF_SEED_START: ") + seed_start_text;
            else if (count_text && !parse_size(count_text, seed_count))
                bad_seed = std::string("Invalid MF_SEED_COUNT: ") + count_text;
            if (bad_seed.empty()) {
                opts.seed_start = seed_start;
                opts.seed_count = seed_count;
            }
        }
        if (!std::getenv("MF_EXPANDED_N") && n >= 7) expanded_n = std::max(24, c * c);
#endif
        const int c2 = c * c;
        // The reference reports the centre before it checks MF_EXPANDED_N
        // (sym_fold.cpp:703-724): on a bad depth, set up the centre alone,
        // print its lines, then the error.
        const bool bad_expanded = n >= 7 && (expanded_n < c2 || expanded_n > n * n);
        opts.expanded_n = n >= 7 ? (bad_expanded || !bad_seed.empty() ? c2 : expanded_n) : 0;
        mf_sym_plan *plan = nullptr;
        if (mf_sym_plan_create_ex(int32_t(n), &opts, &plan) != MF_OK) {
            std::fprintf(stderr, "error: %s\n", mf_last_error());
            return 2;
        }
        int32_t start_i = 0;
        uint64_t centers = 0, reduced = 0, total = 0;
        mf_sym_plan_info(plan, nullptr, &start_i, &centers, &reduced, &total);
        unsigned long long seeds = reduced;  // representatives the cases come from
#ifdef MF_SYM_FOLD9
        std::fprintf(stderr, "center_size=%d center_cases=%llu%s\n", c, (unsigned long long)centers,
                     std::getenv("MF_CENTER_STREAM_DEDUP") ? " center_stream_dedup=1" : "");
        std::fprintf(stderr, "reduced_cases=%llu\n", (unsigned long long)reduced);
        if (!bad_seed.empty()) {
            std::fprintf(stderr, "%s\n", bad_seed.c_str());
            mf_sym_plan_destroy(plan);
            return 2;
        }
        if (seed_start_text) {
            const unsigned long long lo = std::min<unsigned long long>(seed_start, reduced);
            const unsigned long long hi =
                seed_count && seed_count < reduced - lo ? lo + seed_count : reduced;
            seeds = hi - lo;
            std::fprintf(stderr, "seed_slice_start=%llu seed_slice_count=%llu\n", seed_start, seeds);
        }
#else
        std::fprintf(stderr, "center_cases=%llu\n", (unsigned long long)centers);
        std::fprintf(stderr, "reduced_cases=%llu\n", (unsigned long long)reduced);
#endif
        if (bad_expanded) {
            std::fprintf(stderr, "MF_EXPANDED_N must be between %d and %ld\n", c2, n * n);
            mf_sym_plan_destroy(plan);
            return 1;
        }
        if (n >= 7) {
            if (stream)
                std::fprintf(stderr, "stream_seed_cases=%llu stream_from=%d stream_to=%d\n", seeds, c2,
                             expanded_n);
            else
                std::fprintf(stderr, "expanded_cases=%llu\n", (unsigned long long)total);
        }
        // sym_fold.cpp:267-314 (materialized mode only): score by
        // MF_COST_DEPTH, optionally reorder by MF_SORT_CASES.
        const char *depth_text = std::getenv("MF_COST_DEPTH");
        const int cost_depth = depth_text ? std::atoi(depth_text) : 0;
        if (!stream && cost_depth > 0) {
            const char *sort_text = std::getenv("MF_SORT_CASES");
            int order = 0;
            if (sort_text && *sort_text && std::strcmp(sort_text, "0") != 0)
                order = std::strcmp(sort_text, "asc") == 0 ? 2 : 1;
            uint64_t lo = 0, hi = 0, tot[2] = {0, 0};
            const auto ts = Clock::now();
            if (mf_sym_plan_score(plan, cost_depth, order, mode, nullptr, &lo, &hi, tot, nullptr) != MF_OK) {
                std::fprintf(stderr, "error: %s\n", mf_last_error());
                mf_sym_plan_destroy(plan);
                return 2;
            }
            std::fprintf(stderr, "cost_depth=%d min_score=%llu max_score=%llu total_score=%s score_s=%g\n",
                         cost_depth, (unsigned long long)lo, (unsigned long long)hi,
                         decimal(tot[0], tot[1]).c_str(), since(ts));
            if (order) std::fprintf(stderr, "sorted_cases=%s\n", order == 2 ? "asc" : "desc");
        }
        if (std::getenv("MF_SETUP_ONLY") != nullptr) {
            // The reference prints the number of cases it holds: the centre
            // representatives in stream mode, the expanded cases otherwise.
#ifdef MF_SYM_FOLD9
            // sym_fold9.cpp:1145-1172: streaming past the centre prints the
            // number of generated cases, otherwise the number of cases held.
            const uint64_t held = (stream && start_i == c2) ? seeds : total;
#else
            const uint64_t held = (n >= 7 && !stream) ? total : reduced;
#endif
            std::printf("%llu\n", (unsigned long long)held);
#ifdef MF_SYM_FOLD9
            std::fprintf(stderr,
                         "n=%ld threads=%ld center_n=%d max_cases=%llu start_case=%llu setup_only=1 "
                         "total_s=%g\n", n, threads, c, max_cases, start_case, since(t0));
#else
            std::fprintf(stderr, "n=%ld threads=%ld max_cases=%llu start_case=%llu setup_only=1 total_s=%g\n",
                         n, threads, max_cases, start_case, since(t0));
#endif
            mf_sym_plan_destroy(plan);
            return 0;
        }
        // sym_fold.cpp:539-542: the streaming solver reads MF_QUEUE_SIZE (its
        // host case queue's bound; nothing to size here) and rejects bad text.
        if (stream) {
            if (const char *q = std::getenv("MF_QUEUE_SIZE")) {
                unsigned long long ignored = 0;
                if (!parse_size(q, ignored)) {
                    std::fprintf(stderr, "Invalid MF_QUEUE_SIZE: %s\n", q);
                    mf_sym_plan_destroy(plan);
                    return 2;
                }
            }
        }
        // The chunk runs as consecutive pieces so that finished cases can be
        // reported: the first piece is at most 4096 cases, later ones are
        // sized from the measured rate to take about 5 s.  Counts add up
        // exactly (the answer is linear in the cases).
        unsigned long long planned = total > start_case ? total - start_case : 0;
        if (max_cases && max_cases < planned) planned = max_cases;
        // Cases past 64 cells have no index: the chunk is walked to from the
        // first case, so it runs as one piece (each piece would walk again).
        const bool deep = mf_sym_plan_case_bytes(plan) > 64;
        if (deep) {
            if (!max_cases) {
                std::fprintf(stderr, "error: cases expanded past 64 cells are streamed: give max_cases\n");
                mf_sym_plan_destroy(plan);
                return 2;
            }
            planned = max_cases;
        }
        int rc = MF_OK;
        {
            Progress prog;
            ProgressPrinter printer(prog, stream, planned);
            unsigned __int128 sum = 0;
            unsigned long long done = 0;
            unsigned long long piece = deep ? planned : std::min<unsigned long long>(planned, 4096);
            while (done < planned) {
                prog.selected = done + piece;
                if (done + piece == planned) prog.producer_done = 1;
                const auto ts = Clock::now();
                uint64_t part[2] = {0, 0};
                mf_run_stats ps{};
                rc = mf_sym_plan_solve(plan, piece, start_case + done, mode, nullptr, part, &ps);
                if (rc != MF_OK) break;
                sum += (static_cast<unsigned __int128>(part[1]) << 64) | part[0];
                st.kernel_s += ps.kernel_s;
                st.units += ps.units;
                st.nodes += ps.nodes;
                st.splits += ps.splits;
                done += piece;
                if (deep) done = planned;  // a short final chunk ends the stream
                prog.completed = done;
                const double el = since(ts);
                const double rate = el > 0.0 ? double(piece) / el : 1e9;
                const double next = std::max(4096.0, std::min(5.0 * rate, 1e15));
                piece = std::min<unsigned long long>(planned - done, (unsigned long long)next);
            }
            answer[0] = uint64_t(sum);
            answer[1] = uint64_t(sum >> 64);
        }
        mf_sym_plan_destroy(plan);
        if (rc != MF_OK) {
            std::fprintf(stderr, "error: %s\n", mf_last_error());
            return 2;
        }
        const double el = since(t0);
        if (stream)
            std::fprintf(stderr, "stream selected=%llu completed=%llu producer_done=1 rate=%g/s elapsed_s=%g\n",
                         (unsigned long long)st.units, (unsigned long long)st.units,
                         el > 0 ? double(st.units) / el : 0.0, el);
        else
            std::fprintf(stderr, "progress=%llu/%llu rate=%g/s elapsed_s=%g\n",
                         (unsigned long long)st.units, (unsigned long long)st.units,
                         el > 0 ? double(st.units) / el : 0.0, el);
    }
    std::printf("%s\n", decimal(answer[0], answer[1]).c_str());
    std::fprintf(stderr, "n=%ld threads=%ld max_cases=%llu start_case=%llu total_s=%g\n", n, threads,
                 max_cases, start_case, since(t0));
    std::fprintf(stderr, "gpu_mode=%s kernel_s=%g nodes=%llu splits=%llu\n", mode ? "batched" : "plain",
                 st.kernel_s, (unsigned long long)st.nodes, (unsigned long long)st.splits);
    return 0;
}
