/*
 * oracle_levels.c -- level-synchronous, multi-threaded restatement of the
 * reference's branchless IDDFS, for the configurations its single-threaded
 * depth-first form (pca_oracle.c) cannot finish: 32 tests at kernel depth 4.
 *
 * TEST INFRASTRUCTURE ONLY: the tests, the fixture generators and the smoke
 * check call it as the checker; the product library never links it.
 *
 * What it restates. tools/enumerate.c:316-402 walks the kernel depth-first:
 * at position p it generates the candidates of the current state
 * (src/search_state.c:280-330), steps each (src/search_state.c:49-187),
 * counts it ("tried"), and prunes it when the OEP table of position p has
 * already seen its key (tools/enumerate.c:379-384, the table cleared per
 * target depth at :631). The first child in that walk's order represents
 * its key. The walk reaches the children of position p in lexicographic
 * order of their paths, which is the order (rank of the parent among the
 * kept states of position p-1, candidate index): so the kept states of each
 * position are obtained level by level, each level's children taken in
 * parent order and candidate order, the first of every key kept. That is
 * what this file computes, with the exact keys of pca_oracle.c (regs+flags,
 * or regs+flags+live), compared in full on every hash hit.
 *
 * The split. Levels 1..S are deduplicated; positions S+1..K are enumerated
 * without pruning, every generated child counted, and every (kernel, output
 * register) whose state holds the target in a live register on every test
 * (src/search_state.c:223-239) is a solution. The iterative deepening
 * (tools/enumerate.c:624-662) tries K = 0, 1, ... and stops at the first K
 * with a solution; for each K the deduplicated prefix is S = min(K-1,
 * split). With S = K-1 the solutions at K are all solving children of the
 * kept states of position K-1, in the walk's order: the reference's
 * canonical set at the last position.
 */
#define _POSIX_C_SOURCE 199309L
#include "pca_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define OP_ADD 0x02
#define OP_SUB 0x03
#define OP_MUL 0x04
#define OP_AND 0x07
#define OP_OR 0x08
#define OP_XOR 0x09
#define OP_SHL 0x0A
#define OP_SHR 0x0B
#define OP_ASR 0x0C
#define OP_LDI 0x10
#define OP_ADDI 0x12
#define OP_IN 0x17
#define OP_OUT 0x18
#define OP_HLT 0x01
#define I_OP(i) (((i) >> 11) & 0x1F)
#define I_RD(i) (((i) >> 8) & 7)
#define I_RS(i) (((i) >> 5) & 7)
#define I_RT(i) (((i) >> 2) & 7)
#define I_IMM(i) ((i) & 0xFF)
#define ENC_I(op, rd, imm) ((uint16_t)(((op) & 0x1F) << 11 | ((rd) & 7) << 8 | ((imm) & 0xFF)))

/* ---- candidate lists per liveness mask (src/search_state.c:280-330) ----- */

typedef struct {
    uint16_t cand[128][4096];
    int nc[128];
} gen_cache_t;

static void gen_cache_init(gen_cache_t *g)
{
    for (int m = 0; m < 128; m++) g->nc[m] = orc_gen_candidates(g->cand[m], 4096, (uint8_t)(m << 1));
}

/* ---- a level: the kept states of one position, in the walk's order ------ */

typedef struct {
    size_t n;
    uint16_t *regs;     /* [n][T][8] */
    uint8_t *flags;     /* [n][T] */
    uint8_t *live;      /* [n] */
    uint32_t *parent;   /* [n] rank in the level above */
    uint16_t *cidx;     /* [n] candidate index in the parent's list */
} lvl_t;

static void lvl_free(lvl_t *L)
{
    free(L->regs); free(L->flags); free(L->live); free(L->parent); free(L->cidx);
    memset(L, 0, sizeof *L);
}

static int lvl_alloc(lvl_t *L, size_t n, int T)
{
    memset(L, 0, sizeof *L);
    L->n = n;
    size_t m = n ? n : 1;
    L->regs = malloc(m * (size_t)T * 16);
    L->flags = malloc(m * (size_t)T);
    L->live = malloc(m);
    L->parent = malloc(m * 4);
    L->cidx = malloc(m * 2);
    return L->regs && L->flags && L->live && L->parent && L->cidx ? 0 : -1;
}

static void lvl_get(const lvl_t *L, size_t i, int T, orc_state_t *s)
{
    memset(s, 0, sizeof *s);
    memcpy(s->regs, L->regs + i * (size_t)T * 8, (size_t)T * 16);
    memcpy(s->flags, L->flags + i * (size_t)T, (size_t)T);
    s->live = L->live[i];
}

static void lvl_put(lvl_t *L, size_t i, int T, const orc_state_t *s, uint32_t parent, uint16_t c)
{
    memcpy(L->regs + i * (size_t)T * 8, s->regs, (size_t)T * 16);
    memcpy(L->flags + i * (size_t)T, s->flags, (size_t)T);
    L->live[i] = s->live;
    L->parent[i] = parent;
    L->cidx[i] = c;
}

/* ---- a parallel for over [0, n) in blocks, on POSIX threads ------------- */

typedef void (*range_fn)(void *arg, size_t lo, size_t hi, int thread);

typedef struct {
    range_fn fn;
    void *arg;
    size_t n, block;
    volatile size_t next;
    int thread;
} pfor_t;

typedef struct { pfor_t *p; int id; } pfor_arg_t;

static void *pfor_worker(void *a_)
{
    pfor_arg_t *a = a_;
    pfor_t *p = a->p;
    for (;;) {
        size_t lo = __sync_fetch_and_add(&p->next, p->block);
        if (lo >= p->n) break;
        size_t hi = lo + p->block < p->n ? lo + p->block : p->n;
        p->fn(p->arg, lo, hi, a->id);
    }
    return NULL;
}

static void parallel_for(int nthreads, size_t n, size_t block, range_fn fn, void *arg)
{
    pfor_t p = {fn, arg, n, block ? block : 1, 0, 0};
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    pfor_arg_t args[256];
    for (int i = 0; i < nthreads; i++) {
        args[i] = (pfor_arg_t){&p, i};
        pthread_create(&th[i], NULL, pfor_worker, &args[i]);
    }
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
}

/* ---- exact keys --------------------------------------------------------- */

static size_t key_bytes(const orc_state_t *s, int T, int with_live, uint8_t *k)
{
    size_t n = 0;
    for (int t = 0; t < T; t++) { memcpy(k + n, s->regs[t], 16); n += 16; }
    memcpy(k + n, s->flags, (size_t)T);
    n += (size_t)T;
    if (with_live) k[n++] = s->live;
    return n;
}

static uint64_t key_hash(const uint8_t *k, size_t n)
{
    uint64_t h = 0x243F6A8885A308D3ULL;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t w;
        memcpy(&w, k + i, 8);
        h = (h ^ w) * 0x9E3779B97F4A7C15ULL;
        h ^= h >> 31;
    }
    for (; i < n; i++) { h = (h ^ k[i]) * 0x100000001B3ULL; h ^= h >> 29; }
    h ^= h >> 33;
    h *= 0xFF51AFD7ED558CCDULL;
    h ^= h >> 33;
    return h;
}

/* ---- building level d+1 from level d ------------------------------------ */

typedef struct {
    const orc_ctx_t *ctx;
    const gen_cache_t *g;
    const lvl_t *P;
    lvl_t *C;
    int mode, T, nshards;
    const uint64_t *off;      /* [P.n + 1] first child of each parent */
    uint64_t *hash;           /* [children] */
    uint8_t *win;             /* [children] 1 = first of its key */
    uint64_t *rank;           /* [P.n + 1] kept children before each parent */
} build_t;

static void child_of(const build_t *b, size_t p, int c, orc_state_t *ps, orc_state_t *out)
{
    lvl_get(b->P, p, b->T, ps);
    const int m = (ps->live >> 1) & 127;
    orc_step(b->ctx, ps, b->g->cand[m][c], out);
}

static void build_hash_range(void *a, size_t lo, size_t hi, int thread)
{
    (void)thread;
    build_t *b = a;
    uint8_t key[ORC_MAX_TESTS * 17 + 1];
    for (size_t p = lo; p < hi; p++) {
        orc_state_t ps, cs;
        lvl_get(b->P, p, b->T, &ps);
        const int m = (ps.live >> 1) & 127;
        for (int c = 0; c < b->g->nc[m]; c++) {
            orc_step(b->ctx, &ps, b->g->cand[m][c], &cs);
            size_t n = key_bytes(&cs, b->T, b->mode == ORC_OEP_EXACT_LIVE, key);
            b->hash[b->off[p] + c] = key_hash(key, n);
        }
    }
}

typedef struct { uint64_t hash; uint32_t parent; uint16_t cand; uint16_t used; } slot_t;

/* Shard j keeps the first child of every key whose hash falls in it,
   scanning the children in the walk's order. */
static void build_shard_range(void *a, size_t lo, size_t hi, int thread)
{
    (void)thread;
    build_t *b = a;
    const uint64_t M = b->off[b->P->n];
    uint8_t k1[ORC_MAX_TESTS * 17 + 1], k2[ORC_MAX_TESTS * 17 + 1];
    for (size_t j = lo; j < hi; j++) {
        size_t cap = 1024, used = 0;
        slot_t *tab = calloc(cap, sizeof *tab);
        size_t p = 0;
        for (uint64_t i = 0; i < M; i++) {
            const uint64_t h = b->hash[i];
            if ((h >> 40) % (uint64_t)b->nshards != j) continue;
            while (b->off[p + 1] <= i) p++;
            const int c = (int)(i - b->off[p]);
            if ((used + 1) * 2 > cap) {
                size_t nc = cap * 2;
                slot_t *nt = calloc(nc, sizeof *nt);
                for (size_t q = 0; q < cap; q++) {
                    if (!tab[q].used) continue;
                    size_t x = tab[q].hash & (nc - 1);
                    while (nt[x].used) x = (x + 1) & (nc - 1);
                    nt[x] = tab[q];
                }
                free(tab);
                tab = nt;
                cap = nc;
            }
            size_t x = h & (cap - 1);
            int dup = 0;
            orc_state_t ps, cs;
            size_t n1 = 0;
            int have1 = 0;
            while (tab[x].used) {
                if (tab[x].hash == h) {
                    if (!have1) {
                        child_of(b, p, c, &ps, &cs);
                        n1 = key_bytes(&cs, b->T, b->mode == ORC_OEP_EXACT_LIVE, k1);
                        have1 = 1;
                    }
                    orc_state_t ps2, cs2;
                    child_of(b, tab[x].parent, tab[x].cand, &ps2, &cs2);
                    size_t n2 = key_bytes(&cs2, b->T, b->mode == ORC_OEP_EXACT_LIVE, k2);
                    if (n1 == n2 && memcmp(k1, k2, n1) == 0) { dup = 1; break; }
                }
                x = (x + 1) & (cap - 1);
            }
            if (dup) continue;
            tab[x].hash = h;
            tab[x].parent = (uint32_t)p;
            tab[x].cand = (uint16_t)c;
            tab[x].used = 1;
            used++;
            b->win[i] = 1;
        }
        free(tab);
    }
}

static void build_write_range(void *a, size_t lo, size_t hi, int thread)
{
    (void)thread;
    build_t *b = a;
    for (size_t p = lo; p < hi; p++) {
        orc_state_t ps, cs;
        lvl_get(b->P, p, b->T, &ps);
        const int m = (ps.live >> 1) & 127;
        uint64_t r = b->rank[p];
        for (int c = 0; c < b->g->nc[m]; c++) {
            if (!b->win[b->off[p] + c]) continue;
            orc_step(b->ctx, &ps, b->g->cand[m][c], &cs);
            lvl_put(b->C, r++, b->T, &cs, (uint32_t)p, (uint16_t)c);
        }
    }
}

static void count_children_range(void *a, size_t lo, size_t hi, int thread)
{
    (void)thread;
    build_t *b = a;
    for (size_t p = lo; p < hi; p++) {
        const int m = (b->P->live[p] >> 1) & 127;
        ((uint64_t *)b->off)[p + 1] = (uint64_t)b->g->nc[m];
    }
}

/* Returns 0, or -1 when memory runs out. */
static int build_level(const orc_ctx_t *ctx, const gen_cache_t *g, const lvl_t *P, lvl_t *C,
                       int mode, int nthreads, uint64_t *children_out)
{
    const int T = ctx->num_tests;
    build_t b = {ctx, g, P, C, mode, T, nthreads * 8, NULL, NULL, NULL, NULL};
    uint64_t *off = calloc(P->n + 1, 8);
    if (!off) return -1;
    b.off = off;
    parallel_for(nthreads, P->n, 4096, count_children_range, &b);
    for (size_t p = 0; p < P->n; p++) off[p + 1] += off[p];
    const uint64_t M = off[P->n];
    *children_out = M;
    b.win = calloc(M ? M : 1, 1);
    b.rank = calloc(P->n + 1, 8);
    if (!b.win || !b.rank) { free(off); free(b.win); free(b.rank); return -1; }
    if (mode == ORC_OEP_NONE) {
        memset(b.win, 1, M);
    } else {
        b.hash = malloc((M ? M : 1) * 8);
        if (!b.hash) { free(off); free(b.win); free(b.rank); return -1; }
        parallel_for(nthreads, P->n, 64, build_hash_range, &b);
        parallel_for(nthreads, (size_t)b.nshards, 1, build_shard_range, &b);
        free(b.hash);
        b.hash = NULL;
    }
    for (size_t p = 0; p < P->n; p++) {
        uint64_t k = 0;
        for (uint64_t i = off[p]; i < off[p + 1]; i++) k += b.win[i];
        b.rank[p + 1] = b.rank[p] + k;
    }
    if (lvl_alloc(C, b.rank[P->n], T)) { free(off); free(b.win); free(b.rank); return -1; }
    parallel_for(nthreads, P->n, 256, build_write_range, &b);
    free(off);
    free(b.win);
    free(b.rank);
    return 0;
}

/* ---- the unpruned positions S+1..K -------------------------------------- */

typedef struct {
    uint32_t state;      /* rank in level S */
    uint16_t c[4];       /* candidate indices of positions S+1.. */
    uint8_t out_reg;
} osol_t;

typedef struct {
    osol_t *v;
    size_t n, cap;
    uint64_t children;
} tsols_t;

typedef struct {
    const orc_ctx_t *ctx;
    const gen_cache_t *g;
    const lvl_t *L;
    int T, s;            /* suffix depth */
    uint16_t target[ORC_MAX_TESTS];
    tsols_t *per;        /* [nthreads] */
} suffix_t;

static void push_sol(tsols_t *ts, uint32_t state, const uint16_t *c, int s, uint8_t r)
{
    if (ts->n == ts->cap) {
        ts->cap = ts->cap ? ts->cap * 2 : 1024;
        ts->v = realloc(ts->v, ts->cap * sizeof *ts->v);
    }
    osol_t *o = &ts->v[ts->n++];
    memset(o, 0, sizeof *o);
    o->state = state;
    for (int i = 0; i < s; i++) o->c[i] = c[i];
    o->out_reg = r;
}

/* Live registers of s other than `skip` that hold the target on every test. */
static uint8_t matching_regs(const suffix_t *sx, const orc_state_t *s, int skip)
{
    uint8_t m = 0;
    for (int r = 1; r < 8; r++) {
        if (r == skip || !(s->live >> r & 1)) continue;
        int ok = 1;
        for (int t = 0; t < sx->T && ok; t++) ok = s->regs[t][r] == sx->target[t];
        if (ok) m |= (uint8_t)(1u << r);
    }
    return m;
}

/* Does the value candidate `insn` writes equal the target on every test?
   The value half of src/search_state.c:49-187, stopping at the first test
   that differs. */
static int writes_target(const suffix_t *sx, const orc_state_t *s, uint16_t insn)
{
    const int op = I_OP(insn), rd = I_RD(insn), rs = I_RS(insn), rt = I_RT(insn);
    const uint8_t imm = I_IMM(insn);
    const int T = sx->T;
    for (int t = 0; t < T; t++) {
        const uint16_t a = s->regs[t][rs], b = s->regs[t][rt];
        uint16_t v;
        switch (op) {
        case OP_ADD: v = (uint16_t)(a + b); break;
        case OP_SUB: v = (uint16_t)(a - b); break;
        case OP_MUL: v = (uint16_t)((uint32_t)a * b); break;
        case OP_AND: v = a & b; break;
        case OP_OR: v = a | b; break;
        case OP_XOR: v = a ^ b; break;
        case OP_SHL: v = (uint16_t)(a << (b & 0xF)); break;
        case OP_SHR: v = (uint16_t)(a >> (b & 0xF)); break;
        case OP_ASR: v = (uint16_t)((int16_t)a >> (b & 0xF)); break;
        case OP_LDI: v = imm; break;
        case OP_ADDI: v = (uint16_t)(s->regs[t][rd] + (uint16_t)(int16_t)(int8_t)imm); break;
        default: return 0;
        }
        if (v != sx->target[t]) return 0;
    }
    return 1;
}

static void suffix_dfs(const suffix_t *sx, tsols_t *ts, uint32_t state, const orc_state_t *s,
                       int pos, uint16_t *path)
{
    const int m = (s->live >> 1) & 127;
    const int nc = sx->g->nc[m];
    ts->children += (uint64_t)nc;
    if (pos == sx->s - 1) {
        for (int c = 0; c < nc; c++) {
            const uint16_t insn = sx->g->cand[m][c];
            const int rd = I_RD(insn);
            uint8_t solving = matching_regs(sx, s, rd);
            if (rd && writes_target(sx, s, insn)) solving |= (uint8_t)(1u << rd);
            if (!solving) continue;
            path[pos] = (uint16_t)c;
            for (int r = 1; r < 8; r++)
                if (solving >> r & 1) push_sol(ts, state, path, sx->s, (uint8_t)r);
        }
        return;
    }
    for (int c = 0; c < nc; c++) {
        orc_state_t ch;
        if (!orc_step(sx->ctx, s, sx->g->cand[m][c], &ch)) continue;
        path[pos] = (uint16_t)c;
        suffix_dfs(sx, ts, state, &ch, pos + 1, path);
    }
}

static void suffix_range(void *a, size_t lo, size_t hi, int thread)
{
    suffix_t *sx = a;
    tsols_t *ts = &sx->per[thread];
    uint16_t path[4];
    for (size_t i = lo; i < hi; i++) {
        orc_state_t s;
        lvl_get(sx->L, i, sx->T, &s);
        suffix_dfs(sx, ts, (uint32_t)i, &s, 0, path);
    }
}

static int osol_cmp(const void *x, const void *y)
{
    const osol_t *a = x, *b = y;
    if (a->state != b->state) return a->state < b->state ? -1 : 1;
    for (int i = 0; i < 4; i++)
        if (a->c[i] != b->c[i]) return a->c[i] < b->c[i] ? -1 : 1;
    return (int)a->out_reg - (int)b->out_reg;
}

int orc_enumerate_split(const orc_task_t *task, int max_depth, int split, int oep_mode,
                        int nthreads, int sol_cap, uint16_t *sol_progs, int *sol_lens,
                        orc_result_t *res)
{
    memset(res, 0, sizeof *res);
    res->optimal_depth = -1;
    if (task->num_outputs != 1 || task->num_tests < 1 || task->num_tests > ORC_MAX_TESTS ||
        task->num_inputs > 7 || max_depth < 0 || max_depth > ORC_MAX_DEPTH - 1 || split < 0 ||
        (oep_mode != ORC_OEP_NONE && oep_mode != ORC_OEP_EXACT && oep_mode != ORC_OEP_EXACT_LIVE))
        return -1;
    orc_ctx_t ctx;
    if (orc_ctx_init(&ctx, task)) return -1;
    const int T = ctx.num_tests;
    gen_cache_t *g = malloc(sizeof *g);
    if (!g) return -1;
    gen_cache_init(g);
    lvl_t levels[ORC_MAX_DEPTH + 1];
    memset(levels, 0, sizeof levels);
    int built = 0;
    orc_state_t root;
    orc_init_root(&ctx, &root);
    if (lvl_alloc(&levels[0], 1, T)) { free(g); return -1; }
    lvl_put(&levels[0], 0, T, &root, 0, 0);
    uint64_t children[ORC_MAX_DEPTH + 1] = {1};
    int rc = 0;
    uint64_t pruned_cum = 0;
    suffix_t sx = {&ctx, g, NULL, T, 0, {0}, NULL};
    for (int t = 0; t < T; t++) sx.target[t] = task->tests[t].out[0];
    tsols_t *per = calloc((size_t)(nthreads < 1 ? 1 : nthreads), sizeof *per);
    if (!per) { lvl_free(&levels[0]); free(g); return -1; }
    sx.per = per;
    osol_t *all = NULL;
    size_t nall = 0;
    int S = 0;

    /* K = 0: the root itself (tools/enumerate.c:624 starts at depth 0) */
    uint8_t root_sols = matching_regs(&sx, &root, 0);
    if (root_sols) {
        res->optimal_depth = 0;
        for (int r = 1; r < 8; r++) {
            if (!(root_sols >> r & 1)) continue;
            osol_t o;
            memset(&o, 0, sizeof o);
            o.out_reg = (uint8_t)r;
            all = realloc(all, (nall + 1) * sizeof *all);
            all[nall++] = o;
        }
        res->tried[0] = nall;
    }
    for (int K = 1; K <= max_depth && res->optimal_depth < 0; K++) {
        S = K - 1 < split ? K - 1 : split;
        while (built < S) {
            if (build_level(&ctx, g, &levels[built], &levels[built + 1], oep_mode, nthreads,
                            &children[built + 1])) { rc = -1; goto done; }
            built++;
        }
        uint64_t tried = 0;
        for (int j = 1; j <= S; j++) {
            tried += children[j];
            pruned_cum += children[j] - levels[j].n;
        }
        sx.L = &levels[S];
        sx.s = K - S;
        for (int i = 0; i < (nthreads < 1 ? 1 : nthreads); i++) { per[i].n = 0; per[i].children = 0; }
        parallel_for(nthreads, levels[S].n, 64, suffix_range, &sx);
        for (int i = 0; i < (nthreads < 1 ? 1 : nthreads); i++) {
            tried += per[i].children;
            if (per[i].n) {
                all = realloc(all, (nall + per[i].n) * sizeof *all);
                memcpy(all + nall, per[i].v, per[i].n * sizeof *all);
                nall += per[i].n;
            }
        }
        res->tried[K] = tried;
        res->pruned_cum[K] = pruned_cum;
        res->sols_at[K] = (int)nall;
        if (nall) res->optimal_depth = K;
    }
    for (int d = 0; d <= S && d <= built; d++) {
        res->children[d] = children[d];
        res->survivors[d] = levels[d].n;
    }
    res->total_solutions = nall;
    if (nall > 1) qsort(all, nall, sizeof *all, osol_cmp);
    {
        const int K = res->optimal_depth;
        const int s = K > 0 ? K - S : 0;
        int stored = 0;
        for (size_t i = 0; i < nall && stored < sol_cap && sol_progs; i++) {
            uint16_t *p = sol_progs + (size_t)stored * 16;
            memset(p, 0, 32);
            int n = 0;
            for (int q = 0; q < task->num_inputs; q++)
                p[n++] = ENC_I(OP_IN, q + 1, task->input_ports[q]);
            /* prefix: walk the level-S state's parents up to the root */
            uint16_t cidx[ORC_MAX_DEPTH];
            uint32_t at = all[i].state;
            const int prefix = K > 0 ? S : 0;
            for (int d = prefix; d >= 1; d--) {
                cidx[d - 1] = levels[d].cidx[at];
                at = levels[d].parent[at];
            }
            uint8_t live = root.live;
            for (int d = 0; d < prefix; d++) {
                const uint16_t insn = g->cand[(live >> 1) & 127][cidx[d]];
                p[n++] = insn;
                if (I_RD(insn)) live |= (uint8_t)(1u << I_RD(insn));
            }
            for (int d = 0; d < s; d++) {
                const uint16_t insn = g->cand[(live >> 1) & 127][all[i].c[d]];
                p[n++] = insn;
                if (I_RD(insn)) live |= (uint8_t)(1u << I_RD(insn));
            }
            p[n++] = ENC_I(OP_OUT, all[i].out_reg, task->output_ports[0]);
            p[n++] = (uint16_t)(OP_HLT << 11);
            sol_lens[stored] = n;
            stored++;
        }
        res->num_solutions = stored;
    }
done:
    for (int d = 0; d <= ORC_MAX_DEPTH; d++) lvl_free(&levels[d]);
    for (int i = 0; i < (nthreads < 1 ? 1 : nthreads); i++) free(per[i].v);
    free(per);
    free(all);
    free(g);
    return rc;
}
