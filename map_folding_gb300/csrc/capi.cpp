// capi.cpp -- the extern "C" entry points declared in include/mapfold.h.
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "engine.hpp"

using mf::set_error;

namespace mf {

BatchKnobs resolve_knobs(const mf_batch_config *cfg) {
    BatchKnobs k;
    k.block_threads = 128;
    k.blocks_per_sm = 0;  // as many as fit (occupancy calculator)
    k.node_budget = 64;
    k.hungry_factor = 2;
    k.queue_capacity = 1ULL << 16;
    k.wait_limit = 1u << 20;
    k.stack_mode = 0;
    if (cfg) {
        k.stack_mode = cfg->stack_mode;
        if (cfg->block_threads == 128 || cfg->block_threads == 256)
            k.block_threads = int(cfg->block_threads);
        if (cfg->blocks_per_sm) k.blocks_per_sm = int(std::min<uint32_t>(cfg->blocks_per_sm, 32));
        if (cfg->node_budget) k.node_budget = cfg->node_budget;
        if (cfg->hungry_factor) k.hungry_factor = cfg->hungry_factor;
        if (cfg->queue_capacity) k.queue_capacity = cfg->queue_capacity;
        if (cfg->wait_limit) k.wait_limit = cfg->wait_limit;
    }
    // The split ring indexes cells by ticket & (capacity - 1).
    uint64_t cap = 16;
    while (cap < k.queue_capacity && cap < (1ULL << 26)) cap <<= 1;
    k.queue_capacity = cap;
    return k;
}

static_assert(sizeof(QueueHeader) == sizeof(mf_run_header), "mf_run_header mirrors QueueHeader");
static_assert(offsetof(QueueHeader, error) == offsetof(mf_run_header, error), "error word offset");
static_assert(offsetof(QueueHeader, completed) == offsetof(mf_run_header, completed),
              "completed offset");
static_assert(kErrMalformed == MF_RUN_MALFORMED && kErrWaitLimit == MF_RUN_WAIT_LIMIT,
              "error words");

int check_queue_header(const QueueHeader &hdr, uint64_t units) {
    if (hdr.error == kErrMalformed) {
        set_error("a unit's list is not a permutation of its placed items (malformed input)");
        return MF_ERR_ARG;
    }
    if (hdr.error == kErrWaitLimit) {
        set_error("a bounded device-side wait ran out with work still unaccounted for");
        return MF_ERR_TIMEOUT;
    }
    if (hdr.error) {
        set_error("the persistent kernel reported error word %u", hdr.error);
        return MF_ERR_TIMEOUT;
    }
    if (units && (hdr.init_next < units || hdr.completed != units + hdr.spawn_tail)) {
        set_error("work accounting does not close: %llu of %llu units handed out, %llu items "
                  "completed of %llu units + %llu split items",
                  (unsigned long long)hdr.init_next, (unsigned long long)units,
                  (unsigned long long)hdr.completed, (unsigned long long)units,
                  (unsigned long long)hdr.spawn_tail);
        return MF_ERR_TIMEOUT;
    }
    return MF_OK;
}

namespace {

// Grow-only device and pinned-host buffers reused across calls, so the
// host-buffer entry points do not pay cudaMalloc inside a timed loop.
struct Scratch {
    void *ptr = nullptr;
    size_t bytes = 0;
    bool pinned = false;
};

// Every entry point that uses the scratch buffers holds this lock for its
// whole run (recursive: one such entry point may call another), so calls
// from several host threads are serialised instead of reallocating buffers
// under each other's kernels.
std::recursive_mutex g_scratch_mu;
Scratch g_scratch[8];

enum Slot { kDevUnits = 0, kDevCounts, kDevWork, kDevAux, kHostUnits, kHostCounts, kDevAux2, kSlots };

void *scratch(int slot, size_t bytes, bool pinned) {
    Scratch &s = g_scratch[slot];
    if (s.bytes >= bytes && s.ptr) return s.ptr;
    if (s.ptr) {
        if (s.pinned) cudaFreeHost(s.ptr);
        else cudaFree(s.ptr);
        s.ptr = nullptr;
        s.bytes = 0;
    }
    size_t want = std::max<size_t>(bytes, 4096);
    want = (want + 4095) / 4096 * 4096;
    cudaError_t e = pinned ? cudaMallocHost(&s.ptr, want) : cudaMalloc(&s.ptr, want);
    if (e != cudaSuccess) {
        s.ptr = nullptr;
        set_error("allocating %zu bytes failed: %s", want, cudaGetErrorString(e));
        return nullptr;
    }
    s.bytes = want;
    s.pinned = pinned;
    return s.ptr;
}

int ensure_device() {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        set_error("no CUDA device: %s", e == cudaSuccess ? "none visible" : cudaGetErrorString(e));
        return MF_ERR_NO_DEVICE;
    }
    return MF_OK;
}

// Edge pages of each board size, uploaded once per device.
std::mutex g_edges_mu;
uint8_t *g_edges[16][10] = {};
uint8_t *g_wide_edges[16][10] = {};

// Boards over 64 cells get the 64-cell projection here (cells 0..63; the
// host-side expansion and the index never go past 64 cells).
const uint8_t *device_edges(int n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16 || n < 1 || n > 9) return nullptr;
    std::lock_guard<std::mutex> lock(g_edges_mu);
    if (!g_edges[dev][n]) {
        uint8_t host[4 * kSymCells];
        sym_edges(n, host);
        uint8_t *d = nullptr;
        if (cudaMalloc(&d, sizeof(host)) != cudaSuccess) return nullptr;
        if (cudaMemcpy(d, host, sizeof(host), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFree(d);
            return nullptr;
        }
        g_edges[dev][n] = d;
    }
    return g_edges[dev][n];
}

// Full edge pages (kWideCells per page) for the 128-bit kernel.
const uint8_t *device_wide_edges(int n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16 || n < 1 || n > 9) return nullptr;
    std::lock_guard<std::mutex> lock(g_edges_mu);
    if (!g_wide_edges[dev][n]) {
        uint8_t host[4 * kWideCells];
        sym_edges_stride(n, host, kWideCells);
        uint8_t *d = nullptr;
        if (cudaMalloc(&d, sizeof(host)) != cudaSuccess) return nullptr;
        if (cudaMemcpy(d, host, sizeof(host), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFree(d);
            return nullptr;
        }
        g_wide_edges[dev][n] = d;
    }
    return g_wide_edges[dev][n];
}

struct Timer {
    cudaEvent_t a = nullptr, b = nullptr;
    Timer() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~Timer() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    double seconds() {
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        return ms * 1e-3;
    }
};

using u128 = unsigned __int128;

}  // namespace
}  // namespace mf

using namespace mf;

struct mf_lunnon_plan {
    LunnonTables t;
    uint8_t *d_table = nullptr;
    uint32_t table_bytes = 0;
};

struct mf_sym_plan {
    SymPlan p;
};

extern "C" {

const char *mf_last_error(void) { return mf::last_error(); }
int32_t mf_abi_version(void) { return MF_ABI_VERSION; }

// ------------------------------------------------------------- Lunnon ----

int32_t mf_lunnon_plan_create(const int32_t *dims, int32_t ndim, mf_lunnon_plan **out) {
    clear_error();
    if (!out) {
        set_error("out is NULL");
        return MF_ERR_ARG;
    }
    *out = nullptr;
    auto plan = std::make_unique<mf_lunnon_plan>();
    std::string why;
    if (!build_lunnon_tables(dims, ndim, plan->t, why)) {
        set_error("%s", why.c_str());
        return MF_ERR_ARG;
    }
    *out = plan.release();
    return MF_OK;
}

void mf_lunnon_plan_destroy(mf_lunnon_plan *plan) {
    if (!plan) return;
    if (plan->d_table) cudaFree(plan->d_table);
    delete plan;
}

int32_t mf_lunnon_leaves(const mf_lunnon_plan *plan) { return plan ? plan->t.n : 0; }

uint32_t mf_lunnon_state_stride(const mf_lunnon_plan *plan) {
    return plan ? lunnon_state_stride(plan->t.n) : 0;
}

int32_t mf_lunnon_collect(const mf_lunnon_plan *plan, int32_t depth, uint8_t *states, uint64_t cap,
                          uint64_t *count_out) {
    clear_error();
    if (!plan || !count_out) {
        set_error("plan and count_out are required");
        return MF_ERR_ARG;
    }
    if (depth < 0 || depth > plan->t.n) {
        set_error("depth must be between 0 and %d", plan->t.n);
        return MF_ERR_ARG;
    }
    *count_out = collect_lunnon_states(plan->t, depth, states, states ? cap : 0,
                                       lunnon_state_stride(plan->t.n));
    return MF_OK;
}

static int upload_table(mf_lunnon_plan *plan) {
    if (plan->d_table) return MF_OK;
    int rc = ensure_device();
    if (rc) return rc;
    plan->table_bytes = uint32_t((plan->t.next.size() + 15) / 16 * 16);
    MF_TRY_CUDA(cudaMalloc(&plan->d_table, plan->table_bytes));
    MF_TRY_CUDA(cudaMemset(plan->d_table, 0, plan->table_bytes));
    MF_TRY_CUDA(cudaMemcpy(plan->d_table, plan->t.next.data(), plan->t.next.size(),
                           cudaMemcpyHostToDevice));
    return MF_OK;
}

int32_t mf_lunnon_count_states(const mf_lunnon_plan *cplan, int32_t start_leaf,
                               const uint8_t *d_states, uint64_t num_states, uint64_t *d_per_state,
                               uint64_t *d_total, uint64_t *d_nodes, void *stream) {
    clear_error();
    auto *plan = const_cast<mf_lunnon_plan *>(cplan);
    if (!plan || (!d_states && num_states)) {
        set_error("plan and d_states are required");
        return MF_ERR_ARG;
    }
    if (start_leaf < 1 || start_leaf > plan->t.n + 1) {
        set_error("start_leaf must be between 1 and %d", plan->t.n + 1);
        return MF_ERR_ARG;
    }
    if (reinterpret_cast<uintptr_t>(d_states) % 16) {
        set_error("d_states must be 16-byte aligned");
        return MF_ERR_ARG;
    }
    int rc = upload_table(plan);
    if (rc) return rc;
    MF_TRY_CUDA(launch_lunnon_plain(plan->d_table, plan->t.n, plan->t.dim, start_leaf, d_states,
                                    lunnon_state_stride(plan->t.n), num_states, d_per_state,
                                    d_total, d_nodes, static_cast<cudaStream_t>(stream)));
    return MF_OK;
}

static int32_t lunnon_batch_impl(const mf_lunnon_plan *const *plans, int32_t num_plans,
                                 const int32_t *depths, const uint64_t *firsts,
                                 const uint64_t *limits, const mf_batch_config *cfg,
                                 uint64_t *counts_out, mf_run_stats *stats);

int32_t mf_lunnon_count(const mf_lunnon_plan *plan, int32_t depth, int32_t mode,
                        const mf_batch_config *cfg, uint64_t *count_out, uint64_t *states_out,
                        mf_run_stats *stats) {
    return mf_lunnon_count_range(plan, depth, 0, 0, mode, cfg, count_out, states_out, stats);
}

int32_t mf_lunnon_count_range(const mf_lunnon_plan *cplan, int32_t depth, uint64_t first_state,
                              uint64_t max_states, int32_t mode, const mf_batch_config *cfg,
                              uint64_t *count_out, uint64_t *states_out, mf_run_stats *stats) {
    clear_error();
    std::lock_guard<std::recursive_mutex> scratch_lock(g_scratch_mu);
    auto *plan = const_cast<mf_lunnon_plan *>(cplan);
    if (!plan || !count_out) {
        set_error("plan and count_out are required");
        return MF_ERR_ARG;
    }
    if (depth < 0) depth = default_lunnon_depth(plan->t);
    if (depth > plan->t.n) {
        set_error("depth must be between 0 and %d", plan->t.n);
        return MF_ERR_ARG;
    }
    if (mode == 1) {
        const mf_lunnon_plan *one[1] = {plan};
        int32_t d[1] = {depth};
        mf_run_stats local{};
        mf_run_stats *st = stats ? stats : &local;
        int rc = lunnon_batch_impl(one, 1, d, &first_state, &max_states, cfg, count_out, st);
        if (rc == MF_OK && states_out) *states_out = st->units;
        return rc;
    }
    int rc = ensure_device();
    if (rc) return rc;
    rc = upload_table(plan);
    if (rc) return rc;
    const double t0 = now_seconds();
    const uint32_t stride = lunnon_state_stride(plan->t.n);
    const uint64_t all = collect_lunnon_states(plan->t, depth, nullptr, 0, stride);
    uint64_t total = all > first_state ? all - first_state : 0;
    if (max_states && max_states < total) total = max_states;
    auto *h_states = static_cast<uint8_t *>(scratch(kHostUnits, total * stride, true));
    if (!h_states) return MF_ERR_CUDA;
    collect_lunnon_states(plan->t, depth, h_states, total, stride, first_state);
    const double t1 = now_seconds();
    auto *d_states = static_cast<uint8_t *>(scratch(kDevUnits, total * stride, false));
    auto *d_acc = static_cast<uint64_t *>(scratch(kDevCounts, 2 * sizeof(uint64_t), false));
    auto *h_acc = static_cast<uint64_t *>(scratch(kHostCounts, 2 * sizeof(uint64_t), true));
    if (!d_states || !d_acc || !h_acc) return MF_ERR_CUDA;
    Timer th, tk, td;
    cudaStream_t st = nullptr;
    cudaEventRecord(th.a, st);
    MF_TRY_CUDA(cudaMemcpyAsync(d_states, h_states, total * stride, cudaMemcpyHostToDevice, st));
    MF_TRY_CUDA(cudaMemsetAsync(d_acc, 0, 2 * sizeof(uint64_t), st));
    cudaEventRecord(th.b, st);
    cudaEventRecord(tk.a, st);
    MF_TRY_CUDA(launch_lunnon_plain(plan->d_table, plan->t.n, plan->t.dim, depth + 1, d_states,
                                    stride, total, nullptr, d_acc, d_acc + 1, st));
    cudaEventRecord(tk.b, st);
    cudaEventRecord(td.a, st);
    MF_TRY_CUDA(cudaMemcpyAsync(h_acc, d_acc, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    cudaEventRecord(td.b, st);
    MF_TRY_CUDA(cudaStreamSynchronize(st));
    *count_out = h_acc[0];
    if (states_out) *states_out = total;
    if (stats) {
        *stats = mf_run_stats{};
        stats->setup_s = t1 - t0;
        stats->h2d_s = th.seconds();
        stats->kernel_s = tk.seconds();
        stats->d2h_s = td.seconds();
        stats->total_s = now_seconds() - t0;
        stats->units = total;
        stats->nodes = h_acc[1];
        stats->tasks = total;
        stats->h2d_bytes = total * stride;
        stats->d2h_bytes = 2 * sizeof(uint64_t);
    }
    return MF_OK;
}

static int32_t lunnon_batch_impl(const mf_lunnon_plan *const *plans, int32_t num_plans,
                                 const int32_t *depths, const uint64_t *firsts,
                                 const uint64_t *limits, const mf_batch_config *cfg,
                                 uint64_t *counts_out, mf_run_stats *stats) {
    std::lock_guard<std::recursive_mutex> scratch_lock(g_scratch_mu);
    if (!plans || num_plans < 1 || !counts_out) {
        set_error("plans, num_plans >= 1 and counts_out are required");
        return MF_ERR_ARG;
    }
    int rc = ensure_device();
    if (rc) return rc;
    const double t0 = now_seconds();
    const uint32_t stride = lunnon_state_stride(64);
    // Concatenate tables and states of all maps.
    std::vector<LunnonInstanceDev> inst(num_plans);
    std::vector<uint8_t> tables;
    std::vector<uint64_t> per_plan(num_plans), first(num_plans, 0);
    uint64_t total = 0;
    for (int k = 0; k < num_plans; ++k) {
        const mf_lunnon_plan *p = plans[k];
        if (!p) {
            set_error("plan %d is NULL", k);
            return MF_ERR_ARG;
        }
        int d = depths ? depths[k] : -1;
        if (d < 0) d = default_lunnon_depth(p->t);
        if (d > p->t.n) d = p->t.n;
        inst[k].table_offset = uint32_t(tables.size());
        inst[k].n = p->t.n;
        inst[k].dim = p->t.dim;
        inst[k].start_leaf = d + 1;
        tables.insert(tables.end(), p->t.next.begin(), p->t.next.end());
        tables.resize((tables.size() + 15) / 16 * 16, 0);
        const uint64_t all = collect_lunnon_states(p->t, d, nullptr, 0, stride);
        first[k] = firsts ? firsts[k] : 0;
        per_plan[k] = all > first[k] ? all - first[k] : 0;
        if (limits && limits[k] && limits[k] < per_plan[k]) per_plan[k] = limits[k];
        total += per_plan[k];
    }
    if (tables.size() > 160 * 1024) {
        set_error("batched maps' tables total %zu bytes; at most 163840 fit on chip",
                  tables.size());
        return MF_ERR_CAPACITY;
    }
    const size_t unit_bytes = total * stride;
    const size_t owner_bytes = total * sizeof(uint32_t);
    auto *h_units = static_cast<uint8_t *>(scratch(kHostUnits, unit_bytes + owner_bytes, true));
    if (!h_units) return MF_ERR_CUDA;
    auto *h_owner = reinterpret_cast<uint32_t *>(h_units + unit_bytes);
    uint64_t at = 0;
    for (int k = 0; k < num_plans; ++k) {
        collect_lunnon_states(plans[k]->t, inst[k].start_leaf - 1, h_units + at * stride,
                              per_plan[k], stride, first[k]);
        for (uint64_t s = 0; s < per_plan[k]; ++s) h_owner[at + s] = uint32_t(k);
        at += per_plan[k];
    }
    const double t1 = now_seconds();
    const BatchKnobs knobs = resolve_knobs(cfg);
    const size_t ws = workspace_bytes(knobs.queue_capacity);
    const size_t meta_bytes = (tables.size() + inst.size() * sizeof(LunnonInstanceDev) + 255) / 256 * 256;
    auto *d_units = static_cast<uint8_t *>(scratch(kDevUnits, unit_bytes + owner_bytes, false));
    auto *d_work = scratch(kDevWork, ws, false);
    auto *d_meta = static_cast<uint8_t *>(scratch(kDevAux, meta_bytes, false));
    auto *d_counts = static_cast<uint64_t *>(scratch(kDevCounts, (num_plans + 1) * 8, false));
    auto *h_counts = static_cast<uint64_t *>(scratch(kHostCounts, (num_plans + 1) * 8 + 64, true));
    if (!d_units || !d_work || !d_meta || !d_counts || !h_counts) return MF_ERR_CUDA;
    cudaStream_t st = nullptr;
    Timer th, tk, td;
    cudaEventRecord(th.a, st);
    MF_TRY_CUDA(cudaMemcpyAsync(d_units, h_units, unit_bytes + owner_bytes, cudaMemcpyHostToDevice, st));
    MF_TRY_CUDA(cudaMemcpyAsync(d_meta, tables.data(), tables.size(), cudaMemcpyHostToDevice, st));
    auto *d_inst = reinterpret_cast<LunnonInstanceDev *>(d_meta + tables.size());
    MF_TRY_CUDA(cudaMemcpyAsync(d_inst, inst.data(), inst.size() * sizeof(LunnonInstanceDev),
                                cudaMemcpyHostToDevice, st));
    MF_TRY_CUDA(cudaMemsetAsync(d_counts + num_plans, 0, 8, st));
    cudaEventRecord(th.b, st);
    cudaEventRecord(tk.a, st);
    int max_levels = 0;
    for (const auto &I : inst) max_levels = std::max(max_levels, I.n - I.start_leaf);
    const uint32_t meta_used = uint32_t(tables.size() + inst.size() * sizeof(LunnonInstanceDev));
    MF_TRY_CUDA(launch_lunnon_batched(d_meta, meta_used, uint32_t(tables.size()), num_plans,
                                      max_levels, d_units,
                                      reinterpret_cast<uint32_t *>(d_units + unit_bytes), total,
                                      d_counts, d_counts + num_plans, d_work, knobs, st));
    cudaEventRecord(tk.b, st);
    cudaEventRecord(td.a, st);
    MF_TRY_CUDA(cudaMemcpyAsync(h_counts, d_counts, (num_plans + 1) * 8, cudaMemcpyDeviceToHost, st));
    MF_TRY_CUDA(cudaMemcpyAsync(h_counts + num_plans + 1, d_work, sizeof(QueueHeader),
                                cudaMemcpyDeviceToHost, st));
    cudaEventRecord(td.b, st);
    MF_TRY_CUDA(cudaStreamSynchronize(st));
    const QueueHeader *hdr = reinterpret_cast<const QueueHeader *>(h_counts + num_plans + 1);
    if (int rc = check_queue_header(*hdr, total)) return rc;
    for (int k = 0; k < num_plans; ++k) counts_out[k] = h_counts[k];
    if (stats) {
        *stats = mf_run_stats{};
        stats->setup_s = t1 - t0;
        stats->h2d_s = th.seconds();
        stats->kernel_s = tk.seconds();
        stats->d2h_s = td.seconds();
        stats->total_s = now_seconds() - t0;
        stats->units = total;
        stats->nodes = h_counts[num_plans];
        stats->tasks = hdr->tasks_run;
        stats->splits = hdr->spawn_tail;
        stats->h2d_bytes = unit_bytes + owner_bytes + tables.size();
        stats->d2h_bytes = (num_plans + 1) * 8 + sizeof(QueueHeader);
    }
    return MF_OK;
}

int32_t mf_lunnon_batch_count(const mf_lunnon_plan *const *plans, int32_t num_plans,
                              const int32_t *depths, const mf_batch_config *cfg,
                              uint64_t *counts_out, mf_run_stats *stats) {
    clear_error();
    return lunnon_batch_impl(plans, num_plans, depths, nullptr, nullptr, cfg, counts_out, stats);
}

}  // extern "C"

// ------------------------------------------------------- graph replay ----

struct mf_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// Record what `body` enqueues on a private stream into an instantiated graph.
template <class F>
int capture_graph(F &&body, mf_graph **out) {
    cudaStream_t s = nullptr;
    MF_TRY_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        set_error("cudaStreamBeginCapture failed: %s", cudaGetErrorString(e));
        return MF_ERR_CUDA;
    }
    const cudaError_t eb = body(s);
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(s, &g);
    cudaStreamDestroy(s);
    if (eb != cudaSuccess || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        set_error("recording the launch failed: %s",
                  cudaGetErrorString(eb != cudaSuccess ? eb : ee));
        return MF_ERR_CUDA;
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        set_error("cudaGraphInstantiate failed: %s", cudaGetErrorString(e));
        return MF_ERR_CUDA;
    }
    auto *gr = new mf_graph;
    gr->graph = g;
    gr->exec = exec;
    *out = gr;
    return MF_OK;
}

}  // namespace

struct mf_lunnon_batch {
    int num_plans = 0;
    uint64_t units = 0;
    uint64_t h2d_bytes = 0;
    uint8_t *d_units = nullptr;
    uint8_t *d_meta = nullptr;
    uint64_t *d_counts = nullptr;  // num_plans counts + node counter
    void *d_work = nullptr;
    uint64_t *h_out = nullptr;     // pinned: counts + node counter + queue header
    mf_graph *graph = nullptr;
    cudaStream_t stream = nullptr;
};

extern "C" {

static int check_sym_range(int32_t n, int32_t start_i, int32_t stop_i);

int32_t mf_sym_graph_create(int32_t n, int32_t start_i, int32_t stop_i, const uint8_t *d_cycles,
                            uint64_t num_cases, uint64_t *d_counts, uint64_t *d_nodes,
                            void *d_workspace, uint64_t workspace_bytes_,
                            const mf_batch_config *cfg, mf_graph **out) {
    clear_error();
    if (!out) {
        set_error("out is NULL");
        return MF_ERR_ARG;
    }
    *out = nullptr;
    int rc = check_sym_range(n, start_i, stop_i);
    if (rc) return rc;
    const BatchKnobs knobs = resolve_knobs(cfg);
    if (!d_workspace || workspace_bytes_ < workspace_bytes(knobs.queue_capacity)) {
        set_error("workspace must hold %llu bytes",
                  (unsigned long long)workspace_bytes(knobs.queue_capacity));
        return MF_ERR_CAPACITY;
    }
    if (num_cases && (!d_cycles || !d_counts)) {
        set_error("d_cycles and d_counts are required");
        return MF_ERR_ARG;
    }
    if (reinterpret_cast<uintptr_t>(d_cycles) % 16 || reinterpret_cast<uintptr_t>(d_workspace) % 256) {
        set_error("d_cycles must be 16-byte and d_workspace 256-byte aligned");
        return MF_ERR_ARG;
    }
    const uint8_t *edges = device_edges(n);
    if (!edges) {
        set_error("uploading the edge pages failed");
        return MF_ERR_CUDA;
    }
    return capture_graph(
        [&](cudaStream_t s) -> cudaError_t {
            if (d_nodes) {
                cudaError_t e = cudaMemsetAsync(d_nodes, 0, sizeof(uint64_t), s);
                if (e != cudaSuccess) return e;
            }
            return launch_sym_batched(edges, start_i, stop_i, d_cycles, num_cases, d_counts,
                                      d_nodes, d_workspace, knobs, s);
        },
        out);
}

int32_t mf_graph_launch(mf_graph *graph, void *stream) {
    clear_error();
    if (!graph) {
        set_error("graph is NULL");
        return MF_ERR_ARG;
    }
    MF_TRY_CUDA(cudaGraphLaunch(graph->exec, static_cast<cudaStream_t>(stream)));
    return MF_OK;
}

void mf_graph_destroy(mf_graph *graph) {
    if (!graph) return;
    if (graph->exec) cudaGraphExecDestroy(graph->exec);
    if (graph->graph) cudaGraphDestroy(graph->graph);
    delete graph;
}

void mf_lunnon_batch_destroy(mf_lunnon_batch *b) {
    if (!b) return;
    mf_graph_destroy(b->graph);
    if (b->d_units) cudaFree(b->d_units);
    if (b->d_meta) cudaFree(b->d_meta);
    if (b->d_counts) cudaFree(b->d_counts);
    if (b->d_work) cudaFree(b->d_work);
    if (b->h_out) cudaFreeHost(b->h_out);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int32_t mf_lunnon_batch_create(const mf_lunnon_plan *const *plans, int32_t num_plans,
                               const int32_t *depths, const mf_batch_config *cfg,
                               mf_lunnon_batch **out) {
    clear_error();
    if (!out || !plans || num_plans < 1) {
        set_error("out, plans and num_plans >= 1 are required");
        return MF_ERR_ARG;
    }
    *out = nullptr;
    int rc = ensure_device();
    if (rc) return rc;
    const uint32_t stride = lunnon_state_stride(64);
    std::vector<LunnonInstanceDev> inst(num_plans);
    std::vector<uint8_t> meta;
    std::vector<uint64_t> per_plan(num_plans);
    uint64_t total = 0;
    int max_levels = 0;
    for (int k = 0; k < num_plans; ++k) {
        const mf_lunnon_plan *p = plans[k];
        if (!p) {
            set_error("plan %d is NULL", k);
            return MF_ERR_ARG;
        }
        int d = depths ? depths[k] : -1;
        if (d < 0) d = default_lunnon_depth(p->t);
        if (d > p->t.n) d = p->t.n;
        inst[k] = LunnonInstanceDev{uint32_t(meta.size()), p->t.n, p->t.dim, d + 1};
        meta.insert(meta.end(), p->t.next.begin(), p->t.next.end());
        meta.resize((meta.size() + 15) / 16 * 16, 0);
        per_plan[k] = collect_lunnon_states(p->t, d, nullptr, 0, stride);
        total += per_plan[k];
        max_levels = std::max(max_levels, p->t.n - d - 1);
    }
    if (meta.size() > 160 * 1024) {
        set_error("batched maps' tables total %zu bytes; at most 163840 fit on chip", meta.size());
        return MF_ERR_CAPACITY;
    }
    const uint32_t inst_offset = uint32_t(meta.size());
    const uint8_t *ib = reinterpret_cast<const uint8_t *>(inst.data());
    meta.insert(meta.end(), ib, ib + inst.size() * sizeof(LunnonInstanceDev));
    const size_t unit_bytes = total * stride, owner_bytes = total * sizeof(uint32_t);
    std::vector<uint8_t> host(unit_bytes + owner_bytes);
    auto *owner = reinterpret_cast<uint32_t *>(host.data() + unit_bytes);
    uint64_t at = 0;
    for (int k = 0; k < num_plans; ++k) {
        collect_lunnon_states(plans[k]->t, inst[k].start_leaf - 1, host.data() + at * stride,
                              per_plan[k], stride);
        for (uint64_t s = 0; s < per_plan[k]; ++s) owner[at + s] = uint32_t(k);
        at += per_plan[k];
    }
    auto b = std::unique_ptr<mf_lunnon_batch, void (*)(mf_lunnon_batch *)>(new mf_lunnon_batch,
                                                                           mf_lunnon_batch_destroy);
    b->num_plans = num_plans;
    b->units = total;
    b->h2d_bytes = host.size() + meta.size();
    const BatchKnobs knobs = resolve_knobs(cfg);
    MF_TRY_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    MF_TRY_CUDA(cudaMalloc(&b->d_units, std::max<size_t>(host.size(), 16)));
    MF_TRY_CUDA(cudaMalloc(&b->d_meta, (meta.size() + 255) / 256 * 256));
    MF_TRY_CUDA(cudaMalloc(&b->d_counts, (num_plans + 1) * sizeof(uint64_t)));
    MF_TRY_CUDA(cudaMalloc(&b->d_work, workspace_bytes(knobs.queue_capacity)));
    MF_TRY_CUDA(cudaMallocHost(&b->h_out, (num_plans + 1) * sizeof(uint64_t) + sizeof(QueueHeader)));
    MF_TRY_CUDA(cudaMemcpy(b->d_units, host.data(), host.size(), cudaMemcpyHostToDevice));
    MF_TRY_CUDA(cudaMemcpy(b->d_meta, meta.data(), meta.size(), cudaMemcpyHostToDevice));
    mf_lunnon_batch *raw = b.get();
    rc = capture_graph(
        [&](cudaStream_t s) -> cudaError_t {
            cudaError_t e = cudaMemsetAsync(raw->d_counts + num_plans, 0, sizeof(uint64_t), s);
            if (e != cudaSuccess) return e;
            return launch_lunnon_batched(raw->d_meta, uint32_t(meta.size()), inst_offset, num_plans,
                                         max_levels, raw->d_units,
                                         reinterpret_cast<uint32_t *>(raw->d_units + unit_bytes),
                                         total, raw->d_counts, raw->d_counts + num_plans,
                                         raw->d_work, knobs, s);
        },
        &b->graph);
    if (rc) return rc;
    *out = b.release();
    return MF_OK;
}

int32_t mf_lunnon_batch_run(mf_lunnon_batch *b, uint64_t *counts_out, mf_run_stats *stats) {
    clear_error();
    if (!b || !counts_out) {
        set_error("batch and counts_out are required");
        return MF_ERR_ARG;
    }
    const double t0 = now_seconds();
    const int np = b->num_plans;
    Timer tk, td;
    cudaEventRecord(tk.a, b->stream);
    MF_TRY_CUDA(cudaGraphLaunch(b->graph->exec, b->stream));
    cudaEventRecord(tk.b, b->stream);
    cudaEventRecord(td.a, b->stream);
    MF_TRY_CUDA(cudaMemcpyAsync(b->h_out, b->d_counts, (np + 1) * sizeof(uint64_t),
                                cudaMemcpyDeviceToHost, b->stream));
    MF_TRY_CUDA(cudaMemcpyAsync(b->h_out + np + 1, b->d_work, sizeof(QueueHeader),
                                cudaMemcpyDeviceToHost, b->stream));
    cudaEventRecord(td.b, b->stream);
    MF_TRY_CUDA(cudaStreamSynchronize(b->stream));
    const QueueHeader *hdr = reinterpret_cast<const QueueHeader *>(b->h_out + np + 1);
    if (int rc = check_queue_header(*hdr, b->units)) return rc;
    for (int k = 0; k < np; ++k) counts_out[k] = b->h_out[k];
    if (stats) {
        *stats = mf_run_stats{};
        stats->kernel_s = tk.seconds();
        stats->d2h_s = td.seconds();
        stats->total_s = now_seconds() - t0;
        stats->units = b->units;
        stats->nodes = b->h_out[np];
        stats->tasks = hdr->tasks_run;
        stats->splits = hdr->spawn_tail;
        stats->h2d_bytes = 0;
        stats->d2h_bytes = (np + 1) * sizeof(uint64_t) + sizeof(QueueHeader);
    }
    return MF_OK;
}

// ---------------------------------------------------------------- sym ----

int32_t mf_sym_edges(int32_t n, uint8_t *out) {
    clear_error();
    if (n < 1 || n > 8 || !out) {
        set_error("n must be 1..8 and out non-NULL");
        return MF_ERR_ARG;
    }
    sym_edges(n, out);
    return MF_OK;
}

static int complete_index(SymPlan &p);

int32_t mf_sym_plan_create(int32_t n, int32_t expanded_n, mf_sym_plan **out) {
    mf_sym_plan_options o{};
    o.expanded_n = expanded_n;
    return mf_sym_plan_create_ex(n, &o, out);
}

int32_t mf_sym_plan_create_ex(int32_t n, const mf_sym_plan_options *opts, mf_sym_plan **out) {
    clear_error();
    if (!out) {
        set_error("out is NULL");
        return MF_ERR_ARG;
    }
    *out = nullptr;
    mf_sym_plan_options o{};
    if (opts) o = *opts;
    auto plan = std::make_unique<mf_sym_plan>();
    std::string why;
    int rc = build_sym_plan(n, o.expanded_n, plan->p, why, o.center_n, o.seed_start, o.seed_count);
    if (rc) {
        set_error("%s", why.c_str());
        return rc;
    }
    if (plan->p.mid_first.empty() && !plan->p.streamed) {
        rc = complete_index(plan->p);
        if (rc) return rc;
    }
    *out = plan.release();
    return MF_OK;
}

void mf_sym_plan_destroy(mf_sym_plan *plan) { delete plan; }

}  // extern "C"

namespace mf {
int build_full_sym_plan(int n, int expanded_n, SymPlan &plan) {
    std::string why;
    int rc = build_sym_plan(n, expanded_n, plan, why);
    if (rc) {
        set_error("%s", why.c_str());
        return rc;
    }
    if (plan.mid_first.empty() && !plan.streamed) return complete_index(plan);
    return MF_OK;
}
}  // namespace mf

extern "C" {

int32_t mf_sym_plan_info(const mf_sym_plan *plan, int32_t *n, int32_t *start_i,
                         uint64_t *center_cases, uint64_t *reduced_cases, uint64_t *total_cases) {
    clear_error();
    if (!plan) {
        set_error("plan is NULL");
        return MF_ERR_ARG;
    }
    if (n) *n = plan->p.n;
    if (start_i) *start_i = plan->p.start_i;
    if (center_cases) *center_cases = plan->p.center_cases;
    if (reduced_cases) *reduced_cases = plan->p.reduced_all;  // before any seed slice
    if (total_cases) *total_cases = plan->p.total_cases;
    return MF_OK;
}

int32_t mf_sym_cases(const mf_sym_plan *plan, uint64_t start_case, uint64_t max_cases,
                     uint8_t *cycles, uint64_t *mults, uint64_t cap, uint64_t *count_out) {
    clear_error();
    if (!plan || !count_out) {
        set_error("plan and count_out are required");
        return MF_ERR_ARG;
    }
    if (plan->p.streamed && !max_cases) {
        set_error("cases expanded past 64 cells are streamed: max_cases must be given");
        return MF_ERR_ARG;
    }
    *count_out = sym_select_cases(plan->p, start_case, max_cases, cycles, mults,
                                  (cycles || mults) ? cap : 0);
    return MF_OK;
}

uint32_t mf_sym_plan_case_bytes(const mf_sym_plan *plan) {
    return plan ? plan->p.case_bytes : 0;
}

static int check_sym_range(int32_t n, int32_t start_i, int32_t stop_i) {
    if (n < 2 || n > 8) {
        set_error("n must be between 2 and 8");
        return MF_ERR_ARG;
    }
    if (start_i < 0 || start_i > stop_i || stop_i > n * n) {
        set_error("need 0 <= start_i <= stop_i <= n*n");
        return MF_ERR_RANGE;
    }
    return MF_OK;
}

int32_t mf_sym_count_cases(int32_t n, int32_t start_i, int32_t stop_i, const uint8_t *d_cycles,
                           uint64_t num_cases, uint64_t *d_counts, uint64_t *d_nodes, void *stream) {
    clear_error();
    int rc = check_sym_range(n, start_i, stop_i);
    if (rc) return rc;
    if (num_cases && (!d_cycles || !d_counts)) {
        set_error("d_cycles and d_counts are required");
        return MF_ERR_ARG;
    }
    if (reinterpret_cast<uintptr_t>(d_cycles) % 16) {
        set_error("d_cycles must be 16-byte aligned");
        return MF_ERR_ARG;
    }
    const uint8_t *edges = device_edges(n);
    if (!edges) {
        set_error("uploading the edge pages failed");
        return MF_ERR_CUDA;
    }
    MF_TRY_CUDA(launch_sym_plain(edges, start_i, stop_i, d_cycles, num_cases, d_counts, d_nodes,
                                 static_cast<cudaStream_t>(stream)));
    return MF_OK;
}

uint64_t mf_sym_workspace_bytes(const mf_batch_config *cfg) {
    return workspace_bytes(resolve_knobs(cfg).queue_capacity);
}

int32_t mf_sym_count_cases_batched(int32_t n, int32_t start_i, int32_t stop_i,
                                   const uint8_t *d_cycles, uint64_t num_cases, uint64_t *d_counts,
                                   uint64_t *d_nodes, void *d_workspace, uint64_t workspace_bytes_,
                                   const mf_batch_config *cfg, void *stream) {
    clear_error();
    int rc = check_sym_range(n, start_i, stop_i);
    if (rc) return rc;
    const BatchKnobs knobs = resolve_knobs(cfg);
    if (!d_workspace || workspace_bytes_ < workspace_bytes(knobs.queue_capacity)) {
        set_error("workspace must hold %llu bytes",
                  (unsigned long long)workspace_bytes(knobs.queue_capacity));
        return MF_ERR_CAPACITY;
    }
    if (num_cases && (!d_cycles || !d_counts)) {
        set_error("d_cycles and d_counts are required");
        return MF_ERR_ARG;
    }
    if (reinterpret_cast<uintptr_t>(d_cycles) % 16 || reinterpret_cast<uintptr_t>(d_workspace) % 256) {
        set_error("d_cycles must be 16-byte and d_workspace 256-byte aligned");
        return MF_ERR_ARG;
    }
    if (num_cases > 0xffffffffULL) {
        set_error("at most 2^32-1 cases per call");
        return MF_ERR_ARG;
    }
    const uint8_t *edges = device_edges(n);
    if (!edges) {
        set_error("uploading the edge pages failed");
        return MF_ERR_CUDA;
    }
    MF_TRY_CUDA(launch_sym_batched(edges, start_i, stop_i, d_cycles, num_cases, d_counts, d_nodes,
                                   d_workspace, knobs, static_cast<cudaStream_t>(stream)));
    return MF_OK;
}

}  // extern "C"

namespace {

// Count `num` cases (host cycles) on the device.  mode 0: plain kernel,
// 1: batched.  Per-case counts land in h_counts.  Returns mf_status.
int count_cases_host(int n, int start_i, int stop_i, const uint8_t *h_cycles, uint64_t num,
                     int mode, const mf_batch_config *cfg, uint64_t *h_counts, mf_run_stats *st,
                     QueueHeader *hdr_out, uint32_t record_bytes = kSymCells) {
    std::lock_guard<std::recursive_mutex> scratch_lock(g_scratch_mu);
    const size_t in_bytes = num * record_bytes;
    const BatchKnobs knobs = resolve_knobs(cfg);
    // Searches past cell 63 run on the 128-bit kernel (batched only);
    // stack_mode 2 selects it for any board.
    const bool wide = stop_i > kSymCells || knobs.stack_mode == 2;
    if (wide) mode = 1;
    auto *d_cycles = static_cast<uint8_t *>(scratch(kDevUnits, in_bytes, false));
    auto *d_counts = static_cast<uint64_t *>(scratch(kDevCounts, (num + 1) * 8, false));
    const uint64_t ws_bytes = wide ? wide_workspace_bytes(knobs.queue_capacity)
                                   : workspace_bytes(knobs.queue_capacity);
    void *d_work = mode == 1 ? scratch(kDevWork, ws_bytes, false) : nullptr;
    auto *h_hdr = static_cast<uint8_t *>(scratch(kHostCounts, 256, true));
    if (!d_cycles || !d_counts || (mode == 1 && !d_work) || !h_hdr) return MF_ERR_CUDA;
    const uint8_t *edges = wide ? device_wide_edges(n) : device_edges(n);
    if (!edges) {
        set_error("uploading the edge pages failed");
        return MF_ERR_CUDA;
    }
    cudaStream_t s = nullptr;
    Timer th, tk, td;
    cudaEventRecord(th.a, s);
    MF_TRY_CUDA(cudaMemcpyAsync(d_cycles, h_cycles, in_bytes, cudaMemcpyHostToDevice, s));
    MF_TRY_CUDA(cudaMemsetAsync(d_counts + num, 0, 8, s));
    cudaEventRecord(th.b, s);
    cudaEventRecord(tk.a, s);
    if (wide)
        MF_TRY_CUDA(launch_sym_wide(edges, start_i, stop_i, d_cycles, record_bytes, num, d_counts,
                                    d_counts + num,
                                    d_work, knobs, s));
    else if (mode == 1)
        MF_TRY_CUDA(launch_sym_batched(edges, start_i, stop_i, d_cycles, num, d_counts,
                                       d_counts + num, d_work, knobs, s));
    else
        MF_TRY_CUDA(launch_sym_plain(edges, start_i, stop_i, d_cycles, num, d_counts, d_counts + num, s));
    cudaEventRecord(tk.b, s);
    cudaEventRecord(td.a, s);
    MF_TRY_CUDA(cudaMemcpyAsync(h_counts, d_counts, (num + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (mode == 1)
        MF_TRY_CUDA(cudaMemcpyAsync(h_hdr, d_work, sizeof(QueueHeader), cudaMemcpyDeviceToHost, s));
    cudaEventRecord(td.b, s);
    MF_TRY_CUDA(cudaStreamSynchronize(s));
    QueueHeader hdr{};
    if (mode == 1) std::memcpy(&hdr, h_hdr, sizeof(hdr));
    if (hdr_out) *hdr_out = hdr;
    if (mode == 1)
        if (int rc = check_queue_header(hdr, num)) return rc;
    for (uint64_t k = 0; k < num; ++k)
        if (h_counts[k] == ~0ULL) {
            set_error("case %llu is not a consistent cycle", (unsigned long long)k);
            return MF_ERR_ARG;
        }
    if (st) {
        st->h2d_s += th.seconds();
        st->kernel_s += tk.seconds();
        st->d2h_s += td.seconds();
        st->nodes += h_counts[num];
        st->units += num;
        st->tasks += mode == 1 ? hdr.tasks_run : num;
        st->splits += hdr.spawn_tail;
        st->h2d_bytes += in_bytes;
        st->d2h_bytes += (num + 1) * 8;
    }
    return MF_OK;
}

}  // namespace

namespace mf {
namespace {
int complete_index_impl(SymPlan &p) {
    int rc = ensure_device();
    if (rc) return rc;
    const uint64_t mids = p.mid_mult.size();
    std::vector<uint64_t> below(mids + 1);
    rc = count_cases_host(p.n, p.mid_i, p.start_i, p.mid_cycles.data(), mids, 1, nullptr,
                          below.data(), nullptr, nullptr);
    if (rc) return rc;
    p.mid_first.assign(mids + 1, 0);
    for (uint64_t k = 0; k < mids; ++k) p.mid_first[k + 1] = p.mid_first[k] + below[k];
    p.total_cases = p.mid_first[mids];
    return MF_OK;
}
}  // namespace
}  // namespace mf

static int complete_index(SymPlan &p) { return mf::complete_index_impl(p); }

extern "C" {

int32_t mf_sym_solve(int32_t n, uint64_t max_cases, uint64_t start_case, int32_t expanded_n,
                     int32_t mode, const mf_batch_config *cfg, uint64_t *answer_lo_hi,
                     mf_run_stats *stats) {
    clear_error();
    if (!answer_lo_hi) {
        set_error("answer_lo_hi is required");
        return MF_ERR_ARG;
    }
    answer_lo_hi[0] = answer_lo_hi[1] = 0;
    if (n < 1 || n > 8) {
        set_error("n must be between 1 and 8");
        return MF_ERR_ARG;
    }
    mf_run_stats local{};
    mf_run_stats *st = stats ? stats : &local;
    *st = mf_run_stats{};
    const double t0 = now_seconds();
    u128 answer = 0;
    if (n <= 2) {
        answer = n == 1 ? 1 : 8;  // sym_fold.cpp:680-687
    } else if (n <= 5) {
        // sym_fold.cpp:698-701: 2*n^2 * completions of the 3-cell cycle.
        // The single root is split on the host into its depth-k descendants
        // so the device has enough independent units.
        const int n2 = n * n;
        const int split = std::min(n2 - 1, n == 5 ? 12 : 5);
        uint8_t edges[4 * kSymCells];
        sym_edges(n, edges);
        uint8_t cyc[kSymCells] = {0};
        cyc[0] = 1;
        cyc[1] = 2;
        cyc[2] = 0;
        std::vector<uint8_t> units;
        sym_expand(cyc, 3, split, edges, [&](const uint8_t *c) {
            units.insert(units.end(), c, c + kSymCells);
            return true;
        });
        const uint64_t num = units.size() / kSymCells;
        st->setup_s = now_seconds() - t0;
        int rc = ensure_device();
        if (rc) return rc;
        std::vector<uint64_t> counts(num + 1);
        rc = count_cases_host(n, split, n2, units.data(), num, mode, cfg, counts.data(), st, nullptr);
        if (rc) return rc;
        u128 raw = 0;
        for (uint64_t k = 0; k < num; ++k) raw += counts[k];
        answer = u128(2) * u128(n2) * raw;
    } else {
        int rc = ensure_device();
        if (rc) return rc;
        mf_sym_plan *plan = nullptr;
        rc = mf_sym_plan_create(n, expanded_n, &plan);
        if (rc) return rc;
        std::unique_ptr<mf_sym_plan, void (*)(mf_sym_plan *)> hold(plan, mf_sym_plan_destroy);
        const double setup = now_seconds() - t0;
        rc = mf_sym_plan_solve(plan, max_cases, start_case, mode, cfg, answer_lo_hi, st);
        st->setup_s += setup;
        st->total_s = now_seconds() - t0;
        return rc;
    }
    answer_lo_hi[0] = uint64_t(answer);
    answer_lo_hi[1] = uint64_t(answer >> 64);
    st->total_s = now_seconds() - t0;
    return MF_OK;
}

int32_t mf_sym_plan_solve(const mf_sym_plan *plan, uint64_t max_cases, uint64_t start_case,
                          int32_t mode, const mf_batch_config *cfg, uint64_t *answer_lo_hi,
                          mf_run_stats *stats) {
    clear_error();
    if (!plan || !answer_lo_hi) {
        set_error("plan and answer_lo_hi are required");
        return MF_ERR_ARG;
    }
    answer_lo_hi[0] = answer_lo_hi[1] = 0;
    std::lock_guard<std::recursive_mutex> scratch_lock(g_scratch_mu);
    mf_run_stats local{};
    mf_run_stats *st = stats ? stats : &local;
    *st = mf_run_stats{};
    int rc = ensure_device();
    if (rc) return rc;
    const double t0 = now_seconds();
    const SymPlan &p = plan->p;
    uint64_t want = p.total_cases > start_case ? p.total_cases - start_case : 0;
    if (max_cases && max_cases < want) want = max_cases;
    if (p.streamed) {
        // No index past 64 cells: the chunk is walked to from the first case
        // (as sym_fold9's stream mode does), so its size must be given.
        if (!max_cases) {
            set_error("cases expanded past 64 cells are streamed: max_cases must be given");
            return MF_ERR_ARG;
        }
        want = max_cases;
    }
    auto *cycles = static_cast<uint8_t *>(
        scratch(kHostUnits, std::max<uint64_t>(want, 1) * p.case_bytes, true));
    std::vector<uint64_t> mults(std::max<uint64_t>(want, 1));
    if (!cycles) return MF_ERR_CUDA;
    const uint64_t got = sym_select_cases(p, start_case, want, cycles, mults.data(), want);
    st->setup_s = now_seconds() - t0;
    std::vector<uint64_t> counts(got + 1);
    if (got) {
        rc = count_cases_host(p.n, p.start_i, p.n * p.n, cycles, got, mode, cfg, counts.data(), st,
                              nullptr, p.case_bytes);
        if (rc) return rc;
    }
    u128 sum = 0;
    for (uint64_t k = 0; k < got; ++k) sum += u128(mults[k]) * u128(counts[k]);
    const u128 answer = sum * u128(p.n * p.n);
    answer_lo_hi[0] = uint64_t(answer);
    answer_lo_hi[1] = uint64_t(answer >> 64);
    st->total_s = now_seconds() - t0;
    return MF_OK;
}

int32_t mf_sym_plan_block_costs(const mf_sym_plan *plan, uint64_t start_case, uint64_t count,
                                int32_t cost_depth, uint64_t block, int32_t mode,
                                const mf_batch_config *cfg, uint64_t *block_costs) {
    clear_error();
    if (!plan || !block_costs || block == 0 || cost_depth < 0) {
        set_error("plan, block_costs, block > 0 and cost_depth >= 0 are required");
        return MF_ERR_ARG;
    }
    const SymPlan &p = plan->p;
    if (start_case > p.total_cases || count > p.total_cases - start_case) {
        set_error("case range [%llu, +%llu) is outside the plan's %llu cases",
                  (unsigned long long)start_case, (unsigned long long)count,
                  (unsigned long long)p.total_cases);
        return MF_ERR_RANGE;
    }
    const uint64_t blocks = (count + block - 1) / block;
    std::fill(block_costs, block_costs + blocks, 0ULL);
    if (count == 0) return MF_OK;
    int rc = ensure_device();
    if (rc) return rc;
    const int stop = std::min(p.n * p.n, p.start_i + cost_depth);
    // Slices of whole blocks, about 2^21 cases each.
    const uint64_t slice = std::max<uint64_t>(block, (uint64_t(1) << 21) / block * block);
    std::vector<uint8_t> cycles(std::min(slice, count) * kSymCells);
    std::vector<uint64_t> scores(std::min(slice, count) + 1);
    for (uint64_t off = 0; off < count; off += slice) {
        const uint64_t m = std::min(slice, count - off);
        const uint64_t got = sym_select_cases(p, start_case + off, m, cycles.data(), nullptr, m);
        if (got != m) {
            set_error("case selection returned %llu of %llu cases", (unsigned long long)got,
                      (unsigned long long)m);
            return MF_ERR_RANGE;
        }
        mf_run_stats st{};
        rc = count_cases_host(p.n, p.start_i, stop, cycles.data(), m, mode, cfg, scores.data(), &st,
                              nullptr);
        if (rc) return rc;
        for (uint64_t k = 0; k < m; ++k) block_costs[(off + k) / block] += scores[k] + 1;
    }
    return MF_OK;
}

int32_t mf_sym_sort_order(const uint64_t *scores, const uint64_t *mults, uint64_t count,
                          int32_t ascending, uint64_t *perm) {
    clear_error();
    if (count && (!scores || !mults || !perm)) {
        set_error("scores, mults and perm are required");
        return MF_ERR_ARG;
    }
    sym_sort_order(scores, mults, count, ascending != 0, perm);
    return MF_OK;
}

int32_t mf_sym_plan_score(mf_sym_plan *plan, int32_t cost_depth, int32_t order, int32_t mode,
                          const mf_batch_config *cfg, uint64_t *min_score, uint64_t *max_score,
                          uint64_t *total_score_lo_hi, mf_run_stats *stats) {
    clear_error();
    if (!plan) {
        set_error("plan is required");
        return MF_ERR_ARG;
    }
    if (order < 0 || order > 2) {
        set_error("order must be 0 (keep), 1 (descending) or 2 (ascending)");
        return MF_ERR_ARG;
    }
    mf_run_stats local{};
    mf_run_stats *st = stats ? stats : &local;
    *st = mf_run_stats{};
    if (min_score) *min_score = 0;
    if (max_score) *max_score = 0;
    if (total_score_lo_hi) total_score_lo_hi[0] = total_score_lo_hi[1] = 0;
    SymPlan &p = plan->p;
    // The cases in the order the plan holds them (the reference scores the
    // list it holds: the expanded cases in emission order).
    const uint64_t total = p.sorted_mult.empty() ? p.total_cases : p.sorted_mult.size();
    if (cost_depth <= 0 || total == 0) return MF_OK;
    int rc = ensure_device();
    if (rc) return rc;
    const double t0 = now_seconds();
    std::vector<uint8_t> cycles(total * kSymCells);
    std::vector<uint64_t> mults(total);
    sym_select_cases(p, 0, total, cycles.data(), mults.data(), total);
    // estimate_work counts the cycles that reach min(n2, start + depth)
    // cells: the count kernels' partial-depth form.
    const int stop = std::min(p.n * p.n, p.start_i + cost_depth);
    std::vector<uint64_t> scores(total + 1);
    rc = count_cases_host(p.n, p.start_i, stop, cycles.data(), total, mode, cfg, scores.data(), st,
                          nullptr);
    if (rc) return rc;
    uint64_t lo = ~0ULL, hi = 0;
    u128 sum = 0;
    for (uint64_t k = 0; k < total; ++k) {
        lo = std::min(lo, scores[k]);
        hi = std::max(hi, scores[k]);
        sum += scores[k];
    }
    if (min_score) *min_score = lo;
    if (max_score) *max_score = hi;
    if (total_score_lo_hi) {
        total_score_lo_hi[0] = uint64_t(sum);
        total_score_lo_hi[1] = uint64_t(sum >> 64);
    }
    if (order != 0) {
        std::vector<uint64_t> perm(total);
        sym_sort_order(scores.data(), mults.data(), total, order == 2, perm.data());
        std::vector<uint8_t> sc(total * kSymCells);
        std::vector<uint64_t> sm(total);
        for (uint64_t k = 0; k < total; ++k) {
            std::memcpy(&sc[k * kSymCells], &cycles[perm[k] * kSymCells], kSymCells);
            sm[k] = mults[perm[k]];
        }
        p.sorted_cycles = std::move(sc);
        p.sorted_mult = std::move(sm);
    }
    st->units = total;
    st->total_s = now_seconds() - t0;
    return MF_OK;
}

uint32_t mf_solve_cases(uint32_t n, uint32_t start_i, uint32_t stop_i, const uint8_t *case_buffer,
                        uint32_t case_count, uint32_t *output_words) {
    clear_error();
    if (!output_words) {
        set_error("output_words is required");
        return 1;
    }
    auto write = [&](u128 count, uint64_t nodes, uint32_t status) {
        output_words[0] = uint32_t(uint64_t(count));
        output_words[1] = uint32_t(uint64_t(count) >> 32);
        output_words[2] = uint32_t(uint64_t(count >> 64));
        output_words[3] = uint32_t(uint64_t(count >> 64) >> 32);
        output_words[4] = uint32_t(nodes);
        output_words[5] = uint32_t(nodes >> 32);
        output_words[6] = status;
        output_words[7] = 0;
        return status;
    };
    // mfah/wasm/sym_kernel.c:251-260
    if (n < 2 || n > 8 || case_count > 256) {
        set_error("n must be 2..8 and case_count <= 256");
        return write(0, 0, 1);
    }
    const uint32_t n2 = n * n;
    if (start_i > stop_i || stop_i > n2) {
        set_error("need start_i <= stop_i <= n*n");
        return write(0, 0, 2);
    }
    if (case_count && !case_buffer) {
        set_error("case_buffer is required");
        return write(0, 0, 1);
    }
    if (ensure_device()) return write(0, 0, 3);
    std::vector<uint8_t> cycles(std::max<uint32_t>(case_count, 1) * kSymCells, 0);
    std::vector<uint64_t> mults(case_count);
    for (uint32_t k = 0; k < case_count; ++k) {
        const uint8_t *rec = case_buffer + size_t(k) * 112;
        std::memcpy(&cycles[size_t(k) * kSymCells], rec, n2);
        uint64_t m = 0;
        for (int b = 7; b >= 0; --b) m = (m << 8) | rec[100 + b];
        mults[k] = m;
    }
    std::vector<uint64_t> counts(case_count + 1);
    mf_run_stats st{};
    if (case_count) {
        int rc = count_cases_host(int(n), int(start_i), int(stop_i), cycles.data(), case_count, 0,
                                  nullptr, counts.data(), &st, nullptr);
        if (rc) return write(0, 0, 3);
    }
    u128 total = 0;
    uint64_t leaves = 0;
    for (uint32_t k = 0; k < case_count; ++k) {
        total += u128(mults[k]) * u128(counts[k]);
        leaves += counts[k];
    }
    // sym_kernel.c counts one call per leaf reached as well (:213-216).
    return write(total, st.nodes + leaves, 0);
}

}  // extern "C"
