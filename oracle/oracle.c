/*
 * oracle.c -- CPU restatement of the reference's counting paths.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  The product never links this
 * file.  Each function names the reference lines whose behaviour it restates.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ======================================================================= */
/* Lunnon                                                                  */
/* ======================================================================= */

typedef struct {
    int n;
    int dim;
    int p[ORC_MAX_DIMS];
    int stride[ORC_MAX_DIMS + 1];              /* bigP, mf.c:30-34 */
    int coord[ORC_MAX_DIMS][ORC_MAX_LEAVES + 1];   /* c, mf.c:41-45 */
    uint8_t next[ORC_MAX_DIMS][ORC_MAX_LEAVES + 1][ORC_MAX_LEAVES + 1]; /* d */
} lun_tables;

/* mf.c:29-75.  coord[i][m] is the 1-based coordinate of leaf m along
 * dimension i; next[i][l][m] is the leaf the dimension-i walk moves to from
 * m when leaves 1..l are placed.  next[i][l][0] stays 0, as the
 * zero-initialised tables of mf_fast.cpp:24 / gpu_folding_v2.cu:36 leave it. */
static int lun_build(const int32_t *dims, int32_t ndim, lun_tables *t) {
    if (ndim < 1 || ndim > ORC_MAX_DIMS) return -1;
    memset(t, 0, sizeof(*t));
    int n = 1;
    for (int i = 0; i < ndim; ++i) {
        if (dims[i] < 1) return -1;
        n *= dims[i];
        if (n > ORC_MAX_LEAVES) return -1;
        t->p[i] = dims[i];
    }
    t->n = n;
    t->dim = ndim;
    t->stride[0] = 1;
    for (int i = 1; i <= ndim; ++i) t->stride[i] = t->stride[i - 1] * dims[i - 1];
    for (int i = 0; i < ndim; ++i)
        for (int m = 1; m <= n; ++m)
            t->coord[i][m] = ((m - 1) / t->stride[i]) % dims[i] + 1;
    for (int i = 0; i < ndim; ++i) {
        int P = t->stride[i];
        for (int l = 1; l <= n; ++l) {
            for (int m = 1; m <= l; ++m) {
                int cm = t->coord[i][m];
                int same_parity = ((t->coord[i][l] - cm) & 1) == 0;
                int to;
                if (same_parity) to = (cm == 1) ? m : m - P;
                else to = (cm == dims[i] || m + P > l) ? m : m + P;
                t->next[i][l][m] = (uint8_t)to;
            }
        }
    }
    return 0;
}

/* Gap computation for leaf l, mf.c:88-124.  The gap stack grows from
 * *top; on return *top is the new top after the common-gap filter. */
static void lun_gaps(const lun_tables *t, const int *b, int l, int res, int mod,
                     int *gap, int *cnt, int *top, orc_work *w) {
    int free_dims = 0;
    int base = *top;
    int sp = base;
    for (int i = 0; i < t->dim; ++i) {
        int m = t->next[i][l][l];
        if (m == l) {
            ++free_dims;
            continue;
        }
        while (m != l) {
            if (w) ++w->steps;
            if (mod == 0 || l != mod || m % mod == res) {
                gap[sp] = m;
                if (cnt[m]++ == 0) ++sp;
            }
            m = t->next[i][l][b[m]];
        }
    }
    if (free_dims == t->dim) {
        for (int m = 0; m < l; ++m) {
            if (w) ++w->steps;
            gap[sp++] = m;
        }
    }
    int keep = base;
    int need = t->dim - free_dims;
    for (int j = base; j < sp; ++j) {
        int x = gap[j];
        gap[keep] = x;
        if (cnt[x] == need) ++keep;
        cnt[x] = 0;
    }
    *top = keep;
}

typedef struct {
    int a[ORC_MAX_LEAVES + 2];
    int b[ORC_MAX_LEAVES + 2];
    int gapter[ORC_MAX_LEAVES + 2];
    int cnt[ORC_MAX_LEAVES + 2];
    int gap[ORC_MAX_LEAVES * ORC_MAX_LEAVES + 2];
} lun_search;

int64_t orc_lunnon_count(const int32_t *dims, int32_t ndim, int32_t res, int32_t mod,
                         orc_work *work) {
    lun_tables *t = malloc(sizeof(*t));
    lun_search *s = calloc(1, sizeof(*s));
    if (!t || !s || lun_build(dims, ndim, t) != 0) {
        free(t);
        free(s);
        return -1;
    }
    const int n = t->n;
    int64_t total = 0;
    int g = 0;
    int l = 1;
    /* mf.c:82-143 */
    while (l > 0) {
        if (l <= 1 || s->b[0] == 1) {
            if (l > n) {
                total += n;
            } else {
                g = s->gapter[l - 1];
                lun_gaps(t, s->b, l, res, mod, s->gap, s->cnt, &g, work);
            }
        }
        while (l > 0 && g == s->gapter[l - 1]) {
            --l;
            s->b[s->a[l]] = s->b[l];
            s->a[s->b[l]] = s->a[l];
        }
        if (l > 0) {
            int m = s->gap[--g];
            s->a[l] = m;
            s->b[l] = s->b[m];
            s->b[m] = l;
            s->a[s->b[l]] = l;
            s->gapter[l++] = g;
            if (work) ++work->nodes;
        }
    }
    free(t);
    free(s);
    return total;
}

/* gpu_folding.cu:21-121 / gpu_folding_v2.cu:220-256, with the search state
 * initialised to zero as mf.c:22-27 and gpu_folding_v2.cu:221 do. */
int64_t orc_lunnon_collect(const int32_t *dims, int32_t ndim, int32_t depth,
                           uint8_t *a_out, uint8_t *b_out, uint16_t *gapter_out,
                           int64_t cap) {
    lun_tables *t = malloc(sizeof(*t));
    lun_search *s = calloc(1, sizeof(*s));
    if (!t || !s || lun_build(dims, ndim, t) != 0 || depth < 0) {
        free(t);
        free(s);
        return -1;
    }
    const int n = t->n;
    if (depth > n) depth = n;
    const int stride = n + 1;
    int64_t found = 0;
    int g = 0;
    int l = 1;
    while (l > 0) {
        if (l <= 1 || s->b[0] == 1) {
            if (l > depth) {
                if (found < cap) {
                    for (int k = 0; k <= n; ++k) {
                        if (a_out) a_out[found * stride + k] = (uint8_t)s->a[k];
                        if (b_out) b_out[found * stride + k] = (uint8_t)s->b[k];
                        if (gapter_out) gapter_out[found * stride + k] = (uint16_t)s->gapter[k];
                    }
                }
                ++found;
                g = s->gapter[l - 1];
            } else {
                g = s->gapter[l - 1];
                lun_gaps(t, s->b, l, 0, 0, s->gap, s->cnt, &g, NULL);
            }
        }
        while (l > 0 && g == s->gapter[l - 1]) {
            --l;
            s->b[s->a[l]] = s->b[l];
            s->a[s->b[l]] = s->a[l];
        }
        if (l > 0) {
            int m = s->gap[--g];
            s->a[l] = m;
            s->b[l] = s->b[m];
            s->b[m] = l;
            s->a[s->b[l]] = l;
            s->gapter[l++] = g;
        }
    }
    free(t);
    free(s);
    return found;
}

static uint64_t lun_resume(const lun_tables *t, lun_search *s, int start_leaf,
                           const uint8_t *a, const uint8_t *b, orc_work *work) {
    const int n = t->n;
    memset(s, 0, sizeof(*s));
    for (int k = 0; k <= n; ++k) {
        s->a[k] = a[k];
        s->b[k] = b[k];
    }
    if (start_leaf < 1) start_leaf = 1;
    if (start_leaf > n + 1) start_leaf = n + 1;
    /* mf_fast.cpp:153-182: resume at start_leaf, stop when it is exhausted. */
    uint64_t total = 0;
    int l = start_leaf;
    int g = 0;
    s->gapter[start_leaf - 1] = 0;
    for (;;) {
        if (l <= 1 || s->b[0] == 1) {
            if (l > n) {
                total += (uint64_t)n;
            } else {
                g = s->gapter[l - 1];
                lun_gaps(t, s->b, l, 0, 0, s->gap, s->cnt, &g, work);
            }
        }
        while (g == s->gapter[l - 1]) {
            if (l == start_leaf) return total;
            --l;
            s->b[s->a[l]] = s->b[l];
            s->a[s->b[l]] = s->a[l];
        }
        int m = s->gap[--g];
        s->a[l] = m;
        s->b[l] = s->b[m];
        s->b[m] = l;
        s->a[s->b[l]] = l;
        s->gapter[l++] = g;
        if (work) ++work->nodes;
    }
}

uint64_t orc_lunnon_resume(const int32_t *dims, int32_t ndim, int32_t start_leaf,
                           const uint8_t *a, const uint8_t *b, orc_work *work) {
    lun_tables *t = malloc(sizeof(*t));
    lun_search *s = malloc(sizeof(*s));
    uint64_t r = 0;
    if (t && s && lun_build(dims, ndim, t) == 0) r = lun_resume(t, s, start_leaf, a, b, work);
    free(t);
    free(s);
    return r;
}

typedef struct {
    const lun_tables *t;
    int start_leaf;
    const uint8_t *a;
    const uint8_t *b;
    int64_t count;
    uint64_t *per_state;
    atomic_llong next;
    pthread_mutex_t mu;
    uint64_t total;
    orc_work work;
} lun_pool;

static void *lun_worker(void *arg) {
    lun_pool *pool = arg;
    lun_search *s = malloc(sizeof(*s));
    const int stride = pool->t->n + 1;
    uint64_t local = 0;
    orc_work w = {0, 0};
    for (;;) {
        long long k = atomic_fetch_add(&pool->next, 1);
        if (k >= pool->count) break;
        uint64_t c = lun_resume(pool->t, s, pool->start_leaf, pool->a + k * stride,
                                pool->b + k * stride, &w);
        if (pool->per_state) pool->per_state[k] = c;
        local += c;
    }
    pthread_mutex_lock(&pool->mu);
    pool->total += local;
    pool->work.nodes += w.nodes;
    pool->work.steps += w.steps;
    pthread_mutex_unlock(&pool->mu);
    free(s);
    return NULL;
}

uint64_t orc_lunnon_resume_many(const int32_t *dims, int32_t ndim, int32_t start_leaf,
                                const uint8_t *a, const uint8_t *b, int64_t count,
                                int32_t threads, uint64_t *per_state, orc_work *work) {
    lun_tables *t = malloc(sizeof(*t));
    if (!t || lun_build(dims, ndim, t) != 0) {
        free(t);
        return 0;
    }
    if (threads < 1) threads = 1;
    lun_pool pool;
    pool.t = t;
    pool.start_leaf = start_leaf;
    pool.a = a;
    pool.b = b;
    pool.count = count;
    pool.per_state = per_state;
    atomic_init(&pool.next, 0);
    pthread_mutex_init(&pool.mu, NULL);
    pool.total = 0;
    pool.work.nodes = pool.work.steps = 0;
    pthread_t *tid = malloc(sizeof(pthread_t) * (size_t)threads);
    for (int i = 0; i < threads; ++i) pthread_create(&tid[i], NULL, lun_worker, &pool);
    for (int i = 0; i < threads; ++i) pthread_join(tid[i], NULL);
    free(tid);
    pthread_mutex_destroy(&pool.mu);
    if (work) {
        work->nodes += pool.work.nodes;
        work->steps += pool.work.steps;
    }
    free(t);
    return pool.total;
}

/* ======================================================================= */
/* sym_fold                                                                */
/* ======================================================================= */

#define SYM_CELLS 64

/* sym_fold.cpp:122-145: cells numbered n*n-1 down to 0 along an inward
 * spiral that starts at (0,0) heading +x and turns when blocked.
 * map[x*h + y]. */
static void sym_spiral(int w, int h, int *map) {
    const int unset = w * h;
    for (int k = 0; k < w * h; ++k) map[k] = unset;
    int x = 0, y = 0, dx = 1, dy = 0;
    for (int v = w * h - 1; v >= 0; --v) {
        map[x * h + y] = v;
        int nx = x + dx, ny = y + dy;
        if (nx < 0 || nx >= w || ny < 0 || ny >= h || map[nx * h + ny] != unset) {
            int t = dx;
            dx = -dy;
            dy = t;
            nx = x + dx;
            ny = y + dy;
        }
        x = nx;
        y = ny;
    }
}

/* sym_fold.cpp:147-173. */
void orc_sym_edges(int32_t n, uint8_t *out) {
    const int cells = n * n;
    int map[SYM_CELLS];
    for (int k = 0; k < 4 * SYM_CELLS; ++k) out[k] = (uint8_t)cells;
    sym_spiral(n, n, map);
    for (int x = 0; x < n; ++x) {
        for (int y = 0; y < n; ++y) {
            int here = map[x * n + y];
            if (x > 0) {
                uint8_t *page = out + (x % 2) * SYM_CELLS;
                int there = map[(x - 1) * n + y];
                page[here] = (uint8_t)there;
                page[there] = (uint8_t)here;
            }
            if (y > 0) {
                uint8_t *page = out + (2 + y % 2) * SYM_CELLS;
                int there = map[x * n + y - 1];
                page[here] = (uint8_t)there;
                page[there] = (uint8_t)here;
            }
        }
    }
}

static inline uint64_t sym_low(int k) { return k >= 64 ? ~0ULL : ((1ULL << k) - 1ULL); }

/* sym_fold.cpp:179-204. */
uint64_t orc_sym_good(const uint8_t *cycle, int32_t i, const uint8_t *edges, orc_work *w) {
    uint64_t good = sym_low(i);
    for (int page = 0; page < 4; ++page) {
        const uint8_t *e = edges + page * SYM_CELLS;
        int other = e[i];
        if (other >= i) continue;
        uint64_t allowed = 1ULL << other;
        int j = cycle[other];
        while (j != other) {
            if (w) ++w->steps;
            int partner = e[j];
            if (partner < i) j = partner;
            allowed |= 1ULL << j;
            j = cycle[j];
        }
        good &= allowed;
        if (good == 0) return 0;
    }
    return good;
}

/* sym_fold.cpp:206-233. */
uint64_t orc_sym_count(uint8_t *cycle, int32_t i, int32_t n2, const uint8_t *edges,
                       orc_work *w) {
    if (w) ++w->nodes;
    uint64_t good = orc_sym_good(cycle, i, edges, w);
    if (good == 0) return 0;
    if (i == n2 - 1) return (uint64_t)__builtin_popcountll(good);
    uint64_t total = 0;
    while (good) {
        int j = __builtin_ctzll(good);
        good &= good - 1;
        uint8_t after = cycle[j];
        cycle[i] = after;
        cycle[j] = (uint8_t)i;
        total += orc_sym_count(cycle, i + 1, n2, edges, w);
        cycle[j] = after;
    }
    return total;
}

/* mfah/wasm/sym_kernel.c:212-230 and mfah/folding.py:179-197: the number of
 * cycles reaching `stop` cells; nodes counts every call, the stop level's
 * included. */
uint64_t orc_sym_count_to(uint8_t *cycle, int32_t i, int32_t stop, const uint8_t *edges,
                          orc_work *w) {
    if (w) ++w->nodes;
    if (i == stop) return 1;
    uint64_t good = orc_sym_good(cycle, i, edges, w);
    uint64_t total = 0;
    while (good) {
        int j = __builtin_ctzll(good);
        good &= good - 1;
        uint8_t after = cycle[j];
        cycle[i] = after;
        cycle[j] = (uint8_t)i;
        total += orc_sym_count_to(cycle, i + 1, stop, edges, w);
        cycle[j] = after;
    }
    return total;
}

/* Growable list of 64-byte cycles. */
typedef struct {
    uint8_t *data;
    int64_t len;
    int64_t cap;
} cyc_list;

static void cyc_push(cyc_list *lst, const uint8_t *cycle) {
    if (lst->len == lst->cap) {
        lst->cap = lst->cap ? lst->cap * 2 : 1024;
        lst->data = realloc(lst->data, (size_t)lst->cap * SYM_CELLS);
    }
    memcpy(lst->data + lst->len * SYM_CELLS, cycle, SYM_CELLS);
    ++lst->len;
}

/* sym_fold.cpp:252-265. */
static void sym_generate(uint8_t *cycle, int i, int stop, const uint8_t *edges,
                         cyc_list *out) {
    if (i == stop) {
        cyc_push(out, cycle);
        return;
    }
    uint64_t good = orc_sym_good(cycle, i, edges, NULL);
    while (good) {
        int j = __builtin_ctzll(good);
        good &= good - 1;
        uint8_t after = cycle[j];
        cycle[i] = after;
        cycle[j] = (uint8_t)i;
        sym_generate(cycle, i + 1, stop, edges, out);
        cycle[j] = after;
    }
}

static void sym_initial(uint8_t *cycle) {
    memset(cycle, 0, SYM_CELLS);
    cycle[0] = 1;
    cycle[1] = 2;
    cycle[2] = 0;
}

/* 16-byte centre key (sym_fold.cpp:352-359): first c2 successors, rest 255. */
typedef struct {
    uint8_t k[16];
} ckey;

static void key_of(const uint8_t *cycle, int c2, ckey *key) {
    memset(key->k, 255, 16);
    for (int i = 0; i < c2; ++i) key->k[i] = cycle[i];
}

/* Small open-addressing set of centre keys. */
typedef struct {
    ckey *slot;
    uint8_t *used;
    int64_t cap;
    int64_t len;
} key_set;

static uint64_t key_hash(const ckey *key) {
    uint64_t h = 0x9E3779B97F4A7C15ULL;
    for (int i = 0; i < 16; ++i) h = (h ^ key->k[i]) * 0x100000001B3ULL;
    return h ^ (h >> 29);
}

static void set_init(key_set *s, int64_t cap) {
    s->cap = cap;
    s->len = 0;
    s->slot = calloc((size_t)cap, sizeof(ckey));
    s->used = calloc((size_t)cap, 1);
}

static void set_free(key_set *s) {
    free(s->slot);
    free(s->used);
}

static int set_has(const key_set *s, const ckey *key) {
    uint64_t h = key_hash(key) % (uint64_t)s->cap;
    while (s->used[h]) {
        if (memcmp(s->slot[h].k, key->k, 16) == 0) return 1;
        h = (h + 1) % (uint64_t)s->cap;
    }
    return 0;
}

static int set_add(key_set *s, const ckey *key) {
    uint64_t h = key_hash(key) % (uint64_t)s->cap;
    while (s->used[h]) {
        if (memcmp(s->slot[h].k, key->k, 16) == 0) return 0;
        h = (h + 1) % (uint64_t)s->cap;
    }
    s->used[h] = 1;
    s->slot[h] = *key;
    ++s->len;
    return 1;
}

/* sym_fold.cpp:316-350: the eight square symmetries as permutations of the
 * centre's own spiral numbering. */
static void sym_perms(int c, uint8_t perms[8][16]) {
    int map[16];
    int rx[16], ry[16];
    sym_spiral(c, c, map);
    for (int x = 0; x < c; ++x)
        for (int y = 0; y < c; ++y) {
            rx[map[x * c + y]] = x;
            ry[map[x * c + y]] = y;
        }
    const int d = c - 1;
    for (int t = 0; t < 8; ++t) {
        memset(perms[t], 255, 16);
        for (int i = 0; i < c * c; ++i) {
            int x = rx[i], y = ry[i], tx, ty;
            switch (t) {
            case 0: tx = x; ty = y; break;
            case 1: tx = y; ty = x; break;
            case 2: tx = x; ty = d - y; break;
            case 3: tx = y; ty = d - x; break;
            case 4: tx = d - x; ty = y; break;
            case 5: tx = d - y; ty = x; break;
            case 6: tx = d - x; ty = d - y; break;
            default: tx = d - y; ty = d - x; break;
            }
            perms[t][i] = (uint8_t)map[tx * c + ty];
        }
    }
}

int64_t orc_sym_reps(int32_t n, uint8_t *cycles, uint64_t *mults, int64_t cap,
                     int64_t *center_cases) {
    if (n < 6 || n > 8) return -1;
    const int c = (n % 2 == 0) ? 4 : 3;
    const int c2 = c * c;
    uint8_t edges[4 * SYM_CELLS];
    orc_sym_edges(n, edges);
    uint8_t cycle[SYM_CELLS];
    sym_initial(cycle);
    cyc_list centers = {0};
    sym_generate(cycle, 3, c2, edges, &centers);
    if (center_cases) *center_cases = centers.len;

    uint8_t perms[8][16];
    sym_perms(c, perms);
    key_set seen;
    set_init(&seen, 1 << 20);
    int64_t reps = 0;
    /* sym_fold.cpp:361-408 */
    for (int64_t k = 0; k < centers.len; ++k) {
        const uint8_t *cy = centers.data + k * SYM_CELLS;
        ckey key;
        key_of(cy, c2, &key);
        if (set_has(&seen, &key)) continue;
        key_set orbit;
        set_init(&orbit, 64);
        for (int t = 0; t < 8; ++t) {
            uint8_t mapped[SYM_CELLS], rev[SYM_CELLS];
            memcpy(mapped, cy, SYM_CELLS);
            for (int i = 0; i < c2; ++i) mapped[perms[t][i]] = perms[t][cy[i]];
            memcpy(rev, mapped, SYM_CELLS);
            int i = 0;
            do {
                rev[mapped[i]] = (uint8_t)i;
                i = mapped[i];
            } while (i != 0);
            ckey km, kr;
            key_of(mapped, c2, &km);
            key_of(rev, c2, &kr);
            set_add(&orbit, &km);
            set_add(&orbit, &kr);
        }
        if (reps < cap) {
            memcpy(cycles + reps * SYM_CELLS, cy, SYM_CELLS);
            mults[reps] = (uint64_t)orbit.len;
        }
        ++reps;
        for (int64_t h = 0; h < orbit.cap; ++h)
            if (orbit.used[h]) set_add(&seen, &orbit.slot[h]);
        set_free(&orbit);
    }
    set_free(&seen);
    free(centers.data);
    return reps;
}

typedef struct {
    const uint8_t *edges;
    int stop;
    uint64_t start, end;
    uint64_t index;
    uint64_t mult;
    uint8_t *cycles;
    uint64_t *mults;
    int64_t cap;
    int64_t selected;
} expand_ctx;

/* sym_fold.cpp:491-527: emit cases in DFS order (lowest set bit first);
 * returns 1 once the selection window is exhausted. */
static int sym_expand_rec(uint8_t *cycle, int i, expand_ctx *ctx) {
    if (i == ctx->stop) {
        if (ctx->index >= ctx->start && ctx->index < ctx->end) {
            if (ctx->selected < ctx->cap) {
                memcpy(ctx->cycles + ctx->selected * SYM_CELLS, cycle, SYM_CELLS);
                ctx->mults[ctx->selected] = ctx->mult;
            }
            ++ctx->selected;
        }
        ++ctx->index;
        return ctx->index >= ctx->end;
    }
    uint64_t good = orc_sym_good(cycle, i, ctx->edges, NULL);
    while (good) {
        int j = __builtin_ctzll(good);
        good &= good - 1;
        uint8_t after = cycle[j];
        cycle[i] = after;
        cycle[j] = (uint8_t)i;
        int stop = sym_expand_rec(cycle, i + 1, ctx);
        cycle[j] = after;
        if (stop) return 1;
    }
    return 0;
}

int64_t orc_sym_expand(int32_t n, int32_t expanded_n, uint64_t start_case,
                       uint64_t max_cases, uint8_t *cycles, uint64_t *mults,
                       int64_t cap) {
    if (n < 6 || n > 8) return -1;
    const int c = (n % 2 == 0) ? 4 : 3;
    const int c2 = c * c;
    if (expanded_n < c2 || expanded_n > n * n) return -1;
    int64_t nreps = orc_sym_reps(n, NULL, NULL, 0, NULL);
    uint8_t *reps = malloc((size_t)nreps * SYM_CELLS);
    uint64_t *rmult = malloc((size_t)nreps * sizeof(uint64_t));
    orc_sym_reps(n, reps, rmult, nreps, NULL);
    uint8_t edges[4 * SYM_CELLS];
    orc_sym_edges(n, edges);
    expand_ctx ctx;
    ctx.edges = edges;
    ctx.stop = expanded_n;
    ctx.start = start_case;
    ctx.end = max_cases == 0 ? UINT64_MAX : start_case + max_cases;
    ctx.index = 0;
    ctx.cycles = cycles;
    ctx.mults = mults;
    ctx.cap = cap;
    ctx.selected = 0;
    for (int64_t r = 0; r < nreps; ++r) {
        uint8_t cy[SYM_CELLS];
        memcpy(cy, reps + r * SYM_CELLS, SYM_CELLS);
        ctx.mult = rmult[r];
        if (sym_expand_rec(cy, c2, &ctx)) break;
    }
    free(reps);
    free(rmult);
    return ctx.selected;
}

typedef struct {
    const uint8_t *edges;
    int start_i, n2;
    int stop;  /* count cycles reaching this many cells (n2: complete ones) */
    const uint8_t *cycles;
    const uint64_t *mults;
    int64_t count;
    uint64_t *per_case;
    atomic_llong next;
    pthread_mutex_t mu;
    u128 total;
    orc_work work;
} sym_pool;

static void *sym_worker(void *arg) {
    sym_pool *pool = arg;
    u128 local = 0;
    orc_work w = {0, 0};
    for (;;) {
        long long k = atomic_fetch_add(&pool->next, 1);
        if (k >= pool->count) break;
        uint8_t cy[SYM_CELLS];
        memcpy(cy, pool->cycles + k * SYM_CELLS, SYM_CELLS);
        uint64_t c = pool->stop >= pool->n2
                         ? orc_sym_count(cy, pool->start_i, pool->n2, pool->edges, &w)
                         : orc_sym_count_to(cy, pool->start_i, pool->stop, pool->edges, &w);
        if (pool->per_case) pool->per_case[k] = c;
        local += (u128)(pool->mults ? pool->mults[k] : 1) * (u128)c;
    }
    pthread_mutex_lock(&pool->mu);
    pool->total += local;
    pool->work.nodes += w.nodes;
    pool->work.steps += w.steps;
    pthread_mutex_unlock(&pool->mu);
    return NULL;
}

static void sym_run_pool(int32_t n, int32_t start_i, int32_t stop, const uint8_t *cycles,
                         const uint64_t *mults, int64_t count, int32_t threads,
                         uint64_t *per_case, uint64_t *sum_lo_hi, orc_work *work);

void orc_sym_count_cases(int32_t n, int32_t start_i, const uint8_t *cycles,
                         const uint64_t *mults, int64_t count, int32_t threads,
                         uint64_t *per_case, uint64_t *sum_lo_hi, orc_work *work) {
    sym_run_pool(n, start_i, n * n, cycles, mults, count, threads, per_case, sum_lo_hi, work);
}

/* sym_fold.cpp:235-250 (estimate_work), scored as score_and_sort_cases does
 * at :274-283: each case's number of cycles reaching min(n2, start_i + depth)
 * cells. */
void orc_sym_estimate_cases(int32_t n, int32_t start_i, int32_t depth, const uint8_t *cycles,
                            int64_t count, int32_t threads, uint64_t *scores) {
    const int32_t n2 = n * n;
    const int32_t stop = start_i + depth < n2 ? start_i + depth : n2;
    sym_run_pool(n, start_i, stop, cycles, NULL, count, threads, scores, NULL, NULL);
}

static void sym_run_pool(int32_t n, int32_t start_i, int32_t stop, const uint8_t *cycles,
                         const uint64_t *mults, int64_t count, int32_t threads,
                         uint64_t *per_case, uint64_t *sum_lo_hi, orc_work *work) {
    uint8_t edges[4 * SYM_CELLS];
    orc_sym_edges(n, edges);
    if (threads < 1) threads = 1;
    sym_pool pool;
    pool.edges = edges;
    pool.start_i = start_i;
    pool.n2 = n * n;
    pool.stop = stop;
    pool.cycles = cycles;
    pool.mults = mults;
    pool.count = count;
    pool.per_case = per_case;
    atomic_init(&pool.next, 0);
    pthread_mutex_init(&pool.mu, NULL);
    pool.total = 0;
    pool.work.nodes = pool.work.steps = 0;
    pthread_t *tid = malloc(sizeof(pthread_t) * (size_t)threads);
    for (int i = 0; i < threads; ++i) pthread_create(&tid[i], NULL, sym_worker, &pool);
    for (int i = 0; i < threads; ++i) pthread_join(tid[i], NULL);
    free(tid);
    pthread_mutex_destroy(&pool.mu);
    if (sum_lo_hi) {
        sum_lo_hi[0] = (uint64_t)pool.total;
        sum_lo_hi[1] = (uint64_t)(pool.total >> 64);
    }
    if (work) {
        work->nodes += pool.work.nodes;
        work->steps += pool.work.steps;
    }
}

int32_t orc_sym_solve(int32_t n, int32_t threads, uint64_t max_cases, uint64_t start_case,
                      int32_t expanded_n, uint64_t *out_lo_hi, orc_work *work) {
    u128 answer = 0;
    out_lo_hi[0] = out_lo_hi[1] = 0;
    if (n < 1 || n > 8) return 1;
    if (n == 1) {
        out_lo_hi[0] = 1;
        return 0;
    }
    if (n == 2) {
        out_lo_hi[0] = 8;
        return 0;
    }
    const int n2 = n * n;
    uint8_t edges[4 * SYM_CELLS];
    orc_sym_edges(n, edges);
    if (n <= 5) {
        /* sym_fold.cpp:698-701 */
        uint8_t cy[SYM_CELLS];
        sym_initial(cy);
        uint64_t raw = orc_sym_count(cy, 3, n2, edges, work);
        answer = (u128)2 * (u128)n2 * (u128)raw;
    } else {
        const int c = (n % 2 == 0) ? 4 : 3;
        int solve_i = c * c;
        if (n >= 7) {
            if (expanded_n <= 0) expanded_n = 24;
            if (expanded_n < solve_i || expanded_n > n2) return 1;
            solve_i = expanded_n;
        }
        int64_t count = orc_sym_expand(n, solve_i, start_case, max_cases, NULL, NULL, 0);
        uint8_t *cycles = malloc((size_t)(count ? count : 1) * SYM_CELLS);
        uint64_t *mults = malloc((size_t)(count ? count : 1) * sizeof(uint64_t));
        orc_sym_expand(n, solve_i, start_case, max_cases, cycles, mults, count);
        uint64_t sum[2];
        orc_sym_count_cases(n, solve_i, cycles, mults, count, threads, NULL, sum, work);
        u128 s = ((u128)sum[1] << 64) | sum[0];
        answer = s * (u128)n2;
        free(cycles);
        free(mults);
    }
    out_lo_hi[0] = (uint64_t)answer;
    out_lo_hi[1] = (uint64_t)(answer >> 64);
    return 0;
}
